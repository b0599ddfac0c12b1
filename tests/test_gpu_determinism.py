"""GPU: run-to-run repeatability.  The position build orders the particles of
every sort key (mesh tile, stencil start, real-space cell) by particle index
after the atomic-count scatter, and no sum over particles or mesh points uses
floating-point atomics, so the same inputs give bitwise the same result on every
run and in every engine built with the same parameters (keys holding more than
16384 particles keep the atomic order)."""
import numpy as np
import pytest

import oracle
import spme_gb300
from conftest import relerr, uniform_case

pytestmark = pytest.mark.gpu


def _clustered(n, L, nclump, width, seed):
    """n particles, nclump of them in one cube of edge `width` (one real-space
    cell, a few mesh tiles and stencil starts hold hundreds to thousands each)."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, L, (n, 3))
    pos[:nclump] = 0.37 * L + rng.uniform(0, width, (nclump, 3))
    rng.shuffle(pos)
    return pos


def _run(pos, f, L, xi, K, p, rc, precision, terms=spme_gb300.TERM_ALL, repeats=2):
    n = pos.shape[0]
    eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, precision=precision,
                            max_nrhs=f.shape[0], terms=terms)
    out = []
    for _ in range(repeats):
        eng.set_positions(pos)
        out.append(eng.apply(f).copy())
    eng.close()
    return out


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_engine_runs_are_bitwise_repeatable(gpu_lib, precision):
    n, L, K, p, xi, rc, R = 20000, 80.0, 64, 6, 0.3, 10.0, 4
    pos, f = uniform_case(n, L, R, seed=21)
    if precision == "fp32":
        f = f.astype(np.float32)
    a = _run(pos, f, L, xi, K, p, rc, precision)
    b = _run(pos, f, L, xi, K, p, rc, precision, repeats=1)
    assert np.array_equal(a[0], a[1])
    assert np.array_equal(a[0], b[0])


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("fp64", 1e-12)])
def test_clustered_particles_repeatable_and_match_oracle(gpu_lib, precision, tol):
    """3000 of 8000 particles in a 2.5-wide cube: long keys in all three sorts and
    a real-space cell with more candidates than the staged path holds."""
    n, L, K, p, xi, rc, R = 8000, 60.0, 48, 6, 0.3, 10.0, 2
    pos = _clustered(n, L, 3000, 2.5, seed=5)
    f = np.random.default_rng(6).standard_normal((R, 3 * n))
    if precision == "fp32":
        f = f.astype(np.float32)
    a = _run(pos, f, L, xi, K, p, rc, precision)
    assert np.array_equal(a[0], a[1])
    ref = oracle.full(pos, L, xi, rc, K, p, f.astype(np.float64), nthreads=4)
    assert relerr(a[0], ref) < tol


def test_real_space_only_repeatable(gpu_lib):
    n, L, xi, rc, R = 30000, 90.0, 0.3, 10.0, 16
    pos = _clustered(n, L, 2000, 4.0, seed=8)
    f = np.random.default_rng(9).standard_normal((R, 3 * n)).astype(np.float32)
    a = _run(pos, f, L, xi, 64, 6, rc, "fp32",
             terms=spme_gb300.TERM_REAL | spme_gb300.TERM_SELF, repeats=3)
    assert np.array_equal(a[0], a[1]) and np.array_equal(a[0], a[2])


def test_batch_runs_are_bitwise_repeatable(gpu_lib):
    import torch
    systems = [dict(N=2500, L=40.0, K=32, p=6, xi=0.3, rc=10.0, radius=1.0),
               dict(N=6000, L=55.0, K=48, p=6, xi=0.3, rc=10.0, radius=1.0),
               dict(N=1200, L=30.0, K=24, p=4, xi=0.35, rc=9.0, radius=1.0)]
    R = 4
    rng = np.random.default_rng(12)
    pos = [rng.uniform(0, s["L"], (s["N"], 3)) for s in systems]
    f = [rng.standard_normal((R, 3 * s["N"])) for s in systems]
    bt = spme_gb300.Batch(systems, nrhs=R, precision="fp32")
    pos_p = spme_gb300.Batch.pack([torch.tensor(x, device="cuda") for x in pos])
    f_p = spme_gb300.Batch.pack([torch.tensor(x, dtype=torch.float32, device="cuda") for x in f])
    outs = []
    for _ in range(2):
        u_p = torch.zeros_like(f_p)
        bt.set_positions(pos_p)
        bt.apply(f_p, u_p)
        bt.synchronize()
        outs.append(u_p.cpu().numpy())
    bt.close()
    assert np.array_equal(outs[0], outs[1])
