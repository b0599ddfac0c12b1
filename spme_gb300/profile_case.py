"""A fixed apply for kernel profiling: one engine, seeded uniform positions and
normal forces, a few applies on the current CUDA device.  Small enough for
multi-pass profiler captures (tens of passes per kernel).

  python -m spme_gb300.profile_case --n 100000 --box 480 --mesh 256 --order 6 \\
      --nrhs 4 --terms recip [--tile 16,8,8] [--precision fp32] [--applies 2] [--fft-mode 2]
"""
from __future__ import annotations

import argparse

import numpy as np

from . import TERM_ALL, TERM_REAL, TERM_RECIP, TERM_SELF, Engine

TERMS = {"recip": TERM_RECIP, "real": TERM_REAL | TERM_SELF, "all": TERM_ALL}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--n", type=int, default=100_000)
    ap.add_argument("--box", type=float, default=480.0)
    ap.add_argument("--mesh", type=int, default=256)
    ap.add_argument("--order", type=int, default=6)
    ap.add_argument("--nrhs", type=int, default=4)
    ap.add_argument("--xi", type=float, default=0.3)
    ap.add_argument("--rcut", type=float, default=10.0)
    ap.add_argument("--terms", default="recip", choices=sorted(TERMS))
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--tile", default=None, help="tx,ty,tz")
    ap.add_argument("--applies", type=int, default=2)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--fft-mode", type=int, default=None, help="0, 1 or 2 (see Engine.set_fft_mode)")
    a = ap.parse_args(argv)

    import torch

    rng = np.random.default_rng(a.seed)
    dt = torch.float32 if a.precision == "fp32" else torch.float64
    pos = torch.tensor(rng.uniform(0, a.box, (a.n, 3)), device="cuda")
    f = torch.tensor(rng.standard_normal((a.nrhs, 3 * a.n)), device="cuda", dtype=dt)
    u = torch.zeros_like(f)
    eng = Engine(a.n, a.box, a.xi, a.mesh, a.order, rcut=a.rcut, precision=a.precision,
                 max_nrhs=a.nrhs, terms=TERMS[a.terms])
    eng.set_graphs(False)
    if a.fft_mode is not None:
        eng.set_fft_mode(a.fft_mode)
    if a.tile:
        eng.set_tile(*(int(v) for v in a.tile.split(",")))
    eng.set_positions(pos)
    for _ in range(a.applies):
        eng.apply(f, u)
    torch.cuda.synchronize()
    print(f"ok |u|_1 = {float(u.double().abs().sum()):.6e}")
    eng.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
