"""GPU: the allocation-free real-space + self entry point.

Callers that cannot call cudaMalloc (a pre-reserved device memory pool, or a
time-stepping loop that must not stall on an allocation) use
spme_realspace_apply_noalloc, whose scratch is a fixed array inside the
library.  Through the C ABI, two calls in a row must agree with the engine's
real-space + self apply (the existing entry point) to the FP64 tolerance.
This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import spme_gb300
from conftest import relerr, uniform_case

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
_P = ctypes.c_void_p


def _noalloc(lib):
    fn = lib.spme_realspace_apply_noalloc
    d, i, l = ctypes.c_double, ctypes.c_int, ctypes.c_long
    fn.argtypes = [i, _P, d, d, d, d, i, d, _P, l, d, _P, l, _P]
    fn.restype = i
    return fn


def test_noalloc_matches_engine_twice(gpu_lib):
    import torch
    fn = _noalloc(gpu_lib)
    n, L, xi, rc, a, R = 3000, 50.0, 0.3, 10.0, 1.2, 3
    pos, f1 = uniform_case(n, L, R, seed=41)
    _, f2 = uniform_case(n, L, R, seed=42)
    eng = spme_gb300.Engine(n, L, xi, 32, 4, radius=a, rcut=rc, precision="fp64", max_nrhs=R,
                            terms=spme_gb300.TERM_REAL | spme_gb300.TERM_SELF)
    eng.set_positions(pos)
    pos_d = torch.tensor(pos, device="cuda")
    u0 = np.random.default_rng(5).standard_normal(f1.shape)
    for f, alpha, beta in ((f1, 1.0, 0.0), (f2, 0.8, -0.5)):
        ref = eng.apply(f, u=u0.copy(), alpha=alpha, beta=beta)
        f_d = torch.tensor(f, device="cuda")
        u_d = torch.tensor(u0, device="cuda")
        st = fn(n, pos_d.data_ptr(), L, xi, a, rc, R, alpha, f_d.data_ptr(), 3 * n, beta,
                u_d.data_ptr(), 3 * n, None)
        assert st == 0, spme_gb300.error_string(st)
        torch.cuda.synchronize()
        assert relerr(u_d.cpu().numpy(), ref) < FP64_TOL


def _engine_real_self(n, L, xi, rc, a, R, pos, f, u0, alpha, beta):
    eng = spme_gb300.Engine(n, L, xi, 32, 4, radius=a, rcut=rc, precision="fp64", max_nrhs=R,
                            terms=spme_gb300.TERM_REAL | spme_gb300.TERM_SELF)
    eng.set_positions(pos)
    ref = eng.apply(f, u=u0.copy(), alpha=alpha, beta=beta)
    eng.close()
    return ref


def test_noalloc_sizes_change_between_calls(gpu_lib):
    """The shared array keeps the previous call's contents: calls in a row with
    a zero-size warm-up first, a larger then a smaller problem, a box of fewer
    than 3 cells per axis (one cell, minimum image) and one of more than 32
    (the cell count capped at 32) all match the engine's real-space + self apply."""
    import torch
    fn = _noalloc(gpu_lib)
    # zero-size first call: loads the library's code (and its scratch) on the device
    assert fn(0, None, 50.0, 0.3, 1.0, 10.0, 0, 1.0, None, 0, 0.0, None, 0, None) == 0
    cases = [  # (n, L, xi, rc, a, R)
        (20000, 120.0, 0.3, 10.0, 1.0, 4),
        (900, 40.0, 0.35, 9.0, 1.3, 2),
        (400, 25.0, 0.4, 10.0, 1.0, 3),   # L / rc = 2.5: one cell
        (30000, 200.0, 0.6, 5.0, 1.0, 1),  # L / rc = 40: capped at 32 cells per axis
    ]
    for k, (n, L, xi, rc, a, R) in enumerate(cases):
        pos, f = uniform_case(n, L, R, seed=100 + k)
        u0 = np.random.default_rng(200 + k).standard_normal(f.shape)
        alpha, beta = 1.1, (0.0 if k % 2 == 0 else 0.6)
        ref = _engine_real_self(n, L, xi, rc, a, R, pos, f, u0, alpha, beta)
        pos_d = torch.tensor(pos, device="cuda")
        f_d = torch.tensor(f, device="cuda")
        u_d = torch.tensor(u0, device="cuda")
        st = fn(n, pos_d.data_ptr(), L, xi, a, rc, R, alpha, f_d.data_ptr(), 3 * n, beta,
                u_d.data_ptr(), 3 * n, None)
        assert st == 0, spme_gb300.error_string(st)
        torch.cuda.synchronize()
        assert relerr(u_d.cpu().numpy(), ref) < FP64_TOL, (n, L, rc)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_lib):
    fn = _noalloc(gpu_lib)
    big = 65536 + 1
    st = fn(big, None, 50.0, 0.3, 1.0, 10.0, 1, 1.0, None, 3 * big, 0.0, None, 3 * big, None)
    assert st == 8 and "scratch" in spme_gb300.error_string(st)
    st = fn(100, None, 50.0, 0.3, 1.0, 10.0, 5, 1.0, None, 300, 0.0, None, 300, None)
    assert st == 8
