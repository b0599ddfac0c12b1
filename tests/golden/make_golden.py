"""Generate the golden fixtures in this directory from the reference's own CPU
path (billy-inn/SPME old-version/spme.c + spme_kernel.c compiled by
oracle/Makefile with the project's MKL/DFTI shim and the reference's
sequential spread loop).

Run where the reference sources exist:
    make -C oracle all && python tests/golden/make_golden.py

Each case stores positions, forces, the initial output vectors, alpha/beta
and the reference's vec_out after one compute_spme call, in compute_spme's
layout (nrhs rows of 3N).  Inputs are seeded: positions i.i.d. U[0, L),
forces and initial outputs i.i.d. N(0, 1).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

# name, N, L, K, p, xi, nrhs, seed
CASES = [
    ("c1_n2000_k64_p6", 2000, 50.0, 64, 6, 0.3, 2, 1234),   # first config of the spec
    ("n64_k16_p4", 64, 10.0, 16, 4, 0.5, 1, 7),
    ("n300_k32_p6", 300, 20.0, 32, 6, 0.3, 3, 11),
    ("n200_k24_p4", 200, 30.0, 24, 4, 0.4, 1, 13),
    ("n500_k128_p6", 500, 60.0, 128, 6, 0.3, 1, 17),
]
ALPHA, BETA = 2.1, 2.2  # old-version/main.c:224-225


def make_case(name, n, L, K, p, xi, nrhs, seed, nthreads=4):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, L, size=(n, 3))
    f = rng.standard_normal((nrhs, 3 * n))
    v0 = rng.standard_normal((nrhs, 3 * n))
    ref = oracle.Reference(xi, K, p, n, L, nthreads=nthreads)
    vout = v0.copy()
    ref.compute(pos, nrhs, ALPHA, f, 3 * n, BETA, vout, 3 * n)
    ref.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), pos=pos, f=f, v0=v0, vout=vout,
                        L=L, K=K, p=p, xi=xi, alpha=ALPHA, beta=BETA, seed=seed)


def main():
    oracle.build(reference=True)
    for c in CASES:
        make_case(*c)
        print("wrote", c[0])


if __name__ == "__main__":
    main()
