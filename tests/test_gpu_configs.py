"""GPU parity at the workload sizes the benchmark and its secondary workloads run,
against the FP64 oracle (the reference's reciprocal path restated + Beenakker's
real-space and self terms), through the C ABI.

* single right-hand side, N = 1e5, L = 220, K = 128, p = 6;
* 16 right-hand sides, N = 2e5, L = 250, K = 160, p = 6;
* 16 right-hand sides, N = 1e6, L = 480, K = 256, p = 6 (the benchmark's system).

All with a = 1, xi = 0.3, rc = 10, uniform positions and N(0,1) forces.
Tolerances (relative L2 over all right-hand sides): the FP64 operator 1e-12,
the FP32 batched operator 1e-5, and the FP32 real-space + self part alone
1e-5 as well (its pair geometry, pair functions and per-batch sums are FP32,
accumulated across batches in compensated FP32; measured about 3e-6 at the
benchmark's size: for overlapping pairs F(r) is a difference of O(1) terms,
so FP32 rounding of those terms is a few 1e-6 of the small result).  Each FP32 result is printed beside the
SPME truncation error at that (xi, K, p): exp(-k_max^2 / 4 xi^2), k_max = pi K / L.

Also: two position builds + applies of the same inputs agree bitwise.  The
counting sorts take slots within a bucket (mesh tile, stencil start cell,
real-space cell) with atomics and then order each bucket's particles by index,
and no sum uses floating-point atomics, so the order of every floating-point
sum is the same on every run."""
import numpy as np
import pytest

import oracle
import spme_gb300
from conftest import relerr, uniform_case

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5
FP32_REAL_TOL = 1e-5
XI, RC, A = 0.3, 10.0, 1.0

# (name, N, L, K, p, R)
CONFIGS = [
    ("single_rhs_n1e5_k128", 100_000, 220.0, 128, 6, 1),
    ("multi_rhs_n2e5_k160", 200_000, 250.0, 160, 6, 16),
    ("large_n1e6_k256", 1_000_000, 480.0, 256, 6, 16),
]


def _truncation(L, K):
    kmax = np.pi * K / L
    return float(np.exp(-kmax ** 2 / (4 * XI ** 2)))


def _apply(N, L, K, p, precision, pos, f, terms=spme_gb300.TERM_ALL):
    import torch
    R = f.shape[0]
    dt = torch.float32 if precision == "fp32" else torch.float64
    eng = spme_gb300.Engine(N, L, XI, K, p, radius=A, rcut=RC, precision=precision,
                            max_nrhs=R, terms=terms)
    try:
        eng.set_positions(torch.tensor(pos, device="cuda"))
        fd = torch.tensor(f, dtype=dt, device="cuda")
        ud = torch.zeros_like(fd)
        eng.apply(fd, ud)
        eng.synchronize()
        return ud.cpu().numpy().astype(np.float64)
    finally:
        eng.close()


@pytest.mark.parametrize("cfg", CONFIGS, ids=[c[0] for c in CONFIGS])
def test_fp64_operator_vs_oracle_at_size(gpu_lib, cfg):
    name, N, L, K, p, R = cfg
    pos, f = uniform_case(N, L, 1, seed=N + K)
    u = _apply(N, L, K, p, "fp64", pos, f)
    ref = oracle.full(pos, L, XI, RC, K, p, f, radius=A)
    err = relerr(u, ref)
    print(f"{name}: FP64 rel-L2 vs oracle {err:.2e}")
    assert err < FP64_TOL


@pytest.mark.parametrize("cfg", CONFIGS, ids=[c[0] for c in CONFIGS])
def test_fp32_batched_vs_oracle_at_size(gpu_lib, cfg):
    """The FP32 engine runs all R right-hand sides in one pass; the oracle checks
    every one of them (R <= 16) except at N = 1e6, where it checks the first 4
    (about a second of oracle time each on the test host)."""
    name, N, L, K, p, R = cfg
    pos, f = uniform_case(N, L, R, seed=2 * N + K)
    u = _apply(N, L, K, p, "fp32", pos, f.astype(np.float32))
    nchk = R if N <= 200_000 else 4
    ref = oracle.full(pos, L, XI, RC, K, p, f[:nchk], radius=A)
    err = relerr(u[:nchk], ref)
    print(f"{name}: FP32 batched (R={R}) rel-L2 vs FP64 oracle {err:.2e}, "
          f"SPME truncation {_truncation(L, K):.1e}")
    assert err < FP32_TOL


def test_fp32_real_space_part_vs_oracle_at_size(gpu_lib):
    """The FP32 real-space + self part alone, N = 1e6 (the benchmark's system)."""
    N, L, R = 1_000_000, 480.0, 4
    pos, f = uniform_case(N, L, R, seed=31)
    u = _apply(N, L, 32, 4, "fp32", pos, f.astype(np.float32),
               terms=spme_gb300.TERM_REAL | spme_gb300.TERM_SELF)
    ref = oracle.real_self(pos, L, XI, RC, f, radius=A)
    err = relerr(u, ref)
    # the pair part alone (the self term is exact up to FP32 rounding of f)
    self_c = oracle.self_coeff(XI, A)
    err_pairs = relerr(u - self_c * f.astype(np.float32), ref - self_c * f)
    print(f"FP32 real-space + self rel-L2 vs oracle {err:.2e} (pairs alone {err_pairs:.2e})")
    assert err < FP32_REAL_TOL
    assert err_pairs < FP32_REAL_TOL


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_run_to_run_bitwise(gpu_lib, precision):
    import torch
    N, L, K, p, R = 200_000, 250.0, 160, 6, 4
    pos, f = uniform_case(N, L, R, seed=5)
    dt = torch.float32 if precision == "fp32" else torch.float64
    eng = spme_gb300.Engine(N, L, XI, K, p, radius=A, rcut=RC, precision=precision,
                            max_nrhs=R, terms=spme_gb300.TERM_ALL)
    pos_d = torch.tensor(pos, device="cuda")
    fd = torch.tensor(f, dtype=dt, device="cuda")
    outs = []
    for _ in range(2):
        ud = torch.zeros_like(fd)
        eng.set_positions(pos_d)
        eng.apply(fd, ud)
        eng.synchronize()
        outs.append(ud.cpu().numpy())
    eng.close()
    assert np.array_equal(outs[0], outs[1])
