"""GPU: CUDA-graph replay, the tile autotuner and the Lanczos Brownian sampler."""
import numpy as np
import pytest

import oracle
import spme_gb300
from conftest import relerr, uniform_case

pytestmark = pytest.mark.gpu


def test_graph_replay_matches_oracle(gpu_lib):
    import torch
    n, L, K, p, xi, rc, R = 2500, 45.0, 48, 6, 0.3, 9.0, 4
    pos, f1 = uniform_case(n, L, R, seed=51)
    _, f2 = uniform_case(n, L, R, seed=52)
    eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, precision="fp32", max_nrhs=R)
    eng.set_graphs(True)
    pos_d = torch.tensor(pos, device="cuda")
    fd = torch.zeros((R, 3 * n), dtype=torch.float32, device="cuda")
    ud = torch.zeros_like(fd)
    for f in (f1, f2, f1):  # capture, then replays with new contents of the same buffers
        eng.set_positions(pos_d)
        fd.copy_(torch.tensor(f, dtype=torch.float32))
        eng.apply(fd, ud)
        eng.synchronize()
        ref = oracle.full(pos, L, xi, rc, K, p, f, nthreads=4)
        assert relerr(ud.cpu().numpy(), ref) < 1e-5
    # host-pointer calls run through the captured staging pass as well
    u = eng.apply(f2.astype(np.float32))
    assert relerr(u, oracle.full(pos, L, xi, rc, K, p, f2, nthreads=4)) < 1e-5


def test_autotune_picks_a_working_tile(gpu_lib, tmp_path):
    import torch
    from spme_gb300.autotune import autotune
    n, L, K, p, xi, rc, R = 4000, 60.0, 64, 6, 0.3, 10.0, 4
    pos, f = uniform_case(n, L, R, seed=61)
    eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, precision="fp32", max_nrhs=R)
    pos_d = torch.tensor(pos, device="cuda")
    fd = torch.tensor(f, dtype=torch.float32, device="cuda")
    cache = str(tmp_path / "tune.json")
    tile, timings = autotune(eng, pos_d, fd, reps=2, cache_file=cache)
    assert tile in timings and len(timings) >= 3
    ud = torch.zeros_like(fd)
    eng.apply(fd, ud)
    eng.synchronize()
    assert relerr(ud.cpu().numpy(), oracle.full(pos, L, xi, rc, K, p, f, nthreads=4)) < 1e-5
    tile2, _ = autotune(eng, pos_d, fd, cache_file=cache)  # served from the cache
    assert tile2 == tile


def _dense_mobility(pos, L, xi, rc, K, p):
    n = pos.shape[0]
    eye = np.eye(3 * n)
    return oracle.full(pos, L, xi, rc, K, p, eye, nthreads=4).T


def test_lanczos_sqrt_matches_dense(gpu_lib):
    import torch
    from spme_gb300.bd import sqrt_mobility_apply
    n, L, K, p, xi, rc, R = 40, 14.0, 32, 6, 0.6, 6.5, 3
    pos, _ = uniform_case(n, L, 1, seed=71)
    M = _dense_mobility(pos, L, xi, rc, K, p)
    M = 0.5 * (M + M.T)
    w, Q = np.linalg.eigh(M)
    assert w.min() > 0
    S = (Q * np.sqrt(w)) @ Q.T
    z = np.random.default_rng(3).standard_normal((R, 3 * n))
    eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, precision="fp64", max_nrhs=R)
    eng.set_positions(pos)
    y, iters = sqrt_mobility_apply(eng, torch.tensor(z, device="cuda"), tol=1e-8, max_iter=120)
    assert relerr(y.cpu().numpy(), z @ S.T) < 1e-6
    assert iters < 120


def test_brownian_displacement_statistics(gpu_lib):
    """<dx dx^T> = 2 kT dt M + O(dt^2) drift term: check the covariance of many samples."""
    import torch
    from spme_gb300.bd import brownian_displacements
    n, L, K, p, xi, rc, R = 8, 10.0, 16, 4, 0.8, 4.5, 16
    pos, _ = uniform_case(n, L, 1, seed=81)
    M = _dense_mobility(pos, L, xi, rc, K, p)
    eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, precision="fp64", max_nrhs=R)
    eng.set_positions(pos)
    g = torch.Generator(device="cuda").manual_seed(0)
    samples = []
    F = torch.zeros((R, 3 * n), dtype=torch.float64, device="cuda")
    for _ in range(250):
        dx, _ = brownian_displacements(eng, F, dt=0.5, kT=1.0, generator=g, tol=1e-8)
        samples.append(dx.cpu().numpy())
    X = np.concatenate(samples)
    cov = X.T @ X / X.shape[0]
    assert relerr(cov, 2 * 0.5 * M) < 0.08  # 4000 samples: ~1/sqrt(4000) statistical error


def test_uneven_batch_matches_engines_and_oracle(gpu_lib):
    """The native batch (one persistent launch per stage over all systems, one
    cuFFT plan per distinct K, the step replayed as one CUDA graph) against the
    per-system engines (loop and graph of engines) and the FP64 oracle, on two
    interpolation tiles and every in-step concurrency mode."""
    import torch
    from spme_gb300.batch import SystemBatch, uneven_systems
    systems = uneven_systems(count=6, nmin=500, nmax=3000, seed=9)
    R = 4
    rng = np.random.default_rng(0)
    pos = [rng.uniform(0, s["L"], (s["N"], 3)) for s in systems]
    f = [rng.standard_normal((R, 3 * s["N"])) for s in systems]
    b = SystemBatch(systems, nrhs=R, tune=False)
    pos_d = [torch.tensor(p, device="cuda") for p in pos]
    f_d = [torch.tensor(x, dtype=torch.float32, device="cuda") for x in f]
    u_d = [torch.zeros_like(x) for x in f_d]
    b.bind(pos_d, f_d, u_d)
    b.run_loop()
    torch.cuda.synchronize()
    loop = [u.cpu().numpy().copy() for u in u_d]
    for u in u_d:
        u.zero_()
    b.run_engines_graph()
    torch.cuda.synchronize()
    for k in range(len(systems)):
        assert relerr(u_d[k].cpu().numpy(), loop[k]) < 1e-6
    refs = [oracle.full(pos[k], s["L"], s["xi"], s["rc"], s["K"], s["p"],
                        f[k].astype(np.float32).astype(np.float64), nthreads=4)
            for k, s in enumerate(systems)]
    for tile, overlap in (((8, 8, 8), 0), ((16, 8, 4), 3), ((16, 8, 4), 1), ((16, 8, 4), 2)):
        b.batch.set_tile(*tile)
        b.batch.set_overlap(overlap)
        b.u_p.zero_()
        b.run()
        b.run()  # the captured graph replayed
        b.batch.synchronize()
        got = [x.cpu().numpy() for x in b.results()]
        for k in range(len(systems)):
            assert relerr(got[k], loop[k]) < 2e-6, (tile, overlap, k)
            assert relerr(got[k], refs[k]) < 1e-5, (tile, overlap, k)
    assert b.batch.launch_count() > 0
    b.close()


def test_batch_apply_alpha_beta_fp64(gpu_lib):
    """FP64 batch through set_positions + apply (no graph), u = beta u + alpha M f,
    against the oracle at 1e-12; p = 4, 6, 8 and different K in one batch."""
    import torch
    systems = [dict(N=700, L=36.0, K=24, p=4, xi=0.35, rc=9.0, radius=1.0),
               dict(N=1500, L=45.0, K=30, p=6, xi=0.3, rc=10.0, radius=1.2),
               dict(N=900, L=40.0, K=32, p=8, xi=0.4, rc=8.0, radius=1.0)]
    R = 2
    rng = np.random.default_rng(4)
    pos = [rng.uniform(0, s["L"], (s["N"], 3)) for s in systems]
    f = [rng.standard_normal((R, 3 * s["N"])) for s in systems]
    u0 = [rng.standard_normal((R, 3 * s["N"])) for s in systems]
    bt = spme_gb300.Batch(systems, nrhs=R, precision="fp64")
    pos_p = spme_gb300.Batch.pack([torch.tensor(p, device="cuda") for p in pos])
    f_p = spme_gb300.Batch.pack([torch.tensor(x, device="cuda") for x in f])
    u_p = spme_gb300.Batch.pack([torch.tensor(x, device="cuda") for x in u0])
    bt.set_positions(pos_p)
    bt.apply(f_p, u_p, alpha=0.7, beta=-0.3)
    bt.synchronize()
    got = [x.cpu().numpy() for x in bt.unpack(u_p)]
    for k, s in enumerate(systems):
        ref = oracle.full(pos[k], s["L"], s["xi"], s["rc"], s["K"], s["p"], f[k], alpha=0.7,
                          beta=-0.3, u=u0[k], radius=s["radius"], nthreads=4)
        assert relerr(got[k], ref) < 1e-12, k
    bt.close()


# (K, p, precision, nrhs): even / odd / 5-smooth K, Nyquist planes, R not a
# multiple of anything
FFT_MODE_CASES = [
    (32, 6, "fp64", 3), (25, 4, "fp64", 2), (45, 8, "fp64", 1), (60, 6, "fp32", 5),
    (27, 6, "fp32", 4), (128, 6, "fp64", 2), (8, 4, "fp64", 2),
]


@pytest.mark.parametrize("case", FFT_MODE_CASES)
def test_fused_zfft_matches_3d_fft(gpu_lib, case):
    """The fused z-FFT/influence kernel against cuFFT 3D + the influence
    kernel, and both against the oracle."""
    K, p, prec, R = case
    n, L, xi = 600, 1.1 * K, 0.35
    pos, f = uniform_case(n, L, R, seed=K + p)
    out = {}
    for mode in (0, 1):
        eng = spme_gb300.Engine(n, L, xi, K, p, precision=prec, max_nrhs=R,
                                terms=spme_gb300.TERM_RECIP)
        eng.set_fft_mode(mode)
        eng.set_positions(pos)
        out[mode] = eng.apply(f.astype(eng.dtype))
        eng.close()
    ref = oracle.recip(pos, L, xi, K, p, f, nthreads=4)
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert relerr(out[1], ref) < tol
    assert relerr(out[0], ref) < tol
    assert relerr(out[1], out[0]) < (1e-13 if prec == "fp64" else 2e-6)


def test_fused_mode_unavailable_for_unaligned_fp32_planes(gpu_lib):
    """FP32 K = 25: a z-plane of the half spectrum is 25 x 13 complex values, not
    a multiple of 16 bytes, so the fused kernel's TMA boxes cannot address it:
    mode 1 is refused and the default (3D) path still matches the oracle."""
    K, p, n, L, xi = 25, 4, 300, 30.0, 0.4
    pos, f = uniform_case(n, L, 2, seed=3)
    eng = spme_gb300.Engine(n, L, xi, K, p, precision="fp32", max_nrhs=2,
                            terms=spme_gb300.TERM_RECIP)
    with pytest.raises(spme_gb300.SpmeError) as ei:
        eng.set_fft_mode(1)
    assert ei.value.code == spme_gb300.ERR_UNSUPPORTED
    eng.set_positions(pos)
    u = eng.apply(f.astype(np.float32))
    ref = oracle.recip(pos, L, xi, K, p, f, nthreads=4)
    assert relerr(u, ref) < 1e-5
    eng.close()


def test_overlap_mode_matches_serial(gpu_lib):
    """Real-space sum on a second stream (overlap on) gives the same operator as
    the default serial order, FP32 and FP64, with and without beta."""
    n, L, K, p, R = 1500, 40.0, 32, 6, 4
    pos, f = uniform_case(n, L, R, seed=11)
    for prec, tol in (("fp64", 1e-14), ("fp32", 1e-6)):
        out = {}
        for ov in (0, 1):
            eng = spme_gb300.Engine(n, L, 0.4, K, p, rcut=8.0, precision=prec, max_nrhs=R)
            eng.set_overlap(ov)
            eng.set_positions(pos)
            u0 = np.ones((R, 3 * n), dtype=eng.dtype)
            out[ov] = eng.apply(f.astype(eng.dtype), u0, alpha=0.7, beta=0.5)
            eng.close()
        assert relerr(out[1], out[0]) < tol
    ref = oracle.full(pos, L, 0.4, 8.0, K, p, f, nthreads=4)
    assert relerr((out[0] - 0.5) / 0.7, ref) < 1e-5


@pytest.mark.parametrize("K", [128, 160, 256])
@pytest.mark.parametrize("prec,tol", [("fp32", 2e-6), ("fp64", 1e-13)])
def test_fused_zfft_fixed_sequence_matches_3d_fft(gpu_lib, K, prec, tol):
    """K = 128, 160 and 256 run compile-time pass sequences of the fused kernel
    (where the plan matches); they must agree with cuFFT's 3D path (validated
    against the oracle at other K)."""
    n, L, p, R = 3000, float(K), 6, 3
    pos, f = uniform_case(n, L, R, seed=K)
    out = {}
    for mode in (0, 1):
        eng = spme_gb300.Engine(n, L, 0.4, K, p, precision=prec, max_nrhs=R,
                                terms=spme_gb300.TERM_RECIP)
        eng.set_fft_mode(mode)
        eng.set_positions(pos)
        out[mode] = eng.apply(f.astype(eng.dtype))
        eng.close()
    assert relerr(out[1], out[0]) < tol


@pytest.mark.parametrize("K", [128, 160, 256])
def test_fft2d_one_pass_matches_cufft(gpu_lib, K):
    """fft_mode 2 (one-pass 2D transforms with a cluster exchange, FP32) against
    cuFFT's 2D transforms (mode 1) and the 3D path (mode 0), and the full
    operator against the oracle at K = 128."""
    n, L, p, R = 3000, float(K), 6, 3
    pos, f = uniform_case(n, L, R, seed=K + 1)
    out = {}
    for mode in (0, 1, 2):
        eng = spme_gb300.Engine(n, L, 0.4, K, p, precision="fp32", max_nrhs=R,
                                terms=spme_gb300.TERM_RECIP)
        eng.set_fft_mode(mode)
        eng.set_positions(pos)
        out[mode] = eng.apply(f.astype(eng.dtype))
        eng.close()
    assert relerr(out[2], out[1]) < 2e-6
    assert relerr(out[2], out[0]) < 2e-6
    if K == 128:
        ref = oracle.recip(pos, L, 0.4, K, p, f, nthreads=4)
        assert relerr(out[2], ref) < 1e-5


def test_fft2d_mode_unsupported(gpu_lib):
    """Mode 2 exists only for FP32 and K = 128, 160, 256."""
    pos, f = uniform_case(200, 40.0, 1, seed=3)
    for K, prec in ((200, "fp32"), (256, "fp64")):
        eng = spme_gb300.Engine(200, 40.0, 0.5, K, 4, precision=prec, max_nrhs=1,
                                terms=spme_gb300.TERM_RECIP)
        with pytest.raises(spme_gb300.SpmeError):
            eng.set_fft_mode(2)
        eng.close()


@pytest.mark.parametrize("K,prec,tol", [(320, "fp32", 2e-6), (512, "fp32", 2e-6), (384, "fp64", 1e-13)])
def test_fused_zfft_large_k_matches_3d_fft(gpu_lib, K, prec, tol):
    """K > 256: the fused kernel moves each z column as several TMA boxes
    (z chunks of K/2 or K/4 rows); it must agree with cuFFT's 3D path."""
    n, L, p, R = 2000, float(K), 4, 2
    pos, f = uniform_case(n, L, R, seed=K)
    out = {}
    for mode in (0, 1):
        eng = spme_gb300.Engine(n, L, 0.5, K, p, precision=prec, max_nrhs=R,
                                terms=spme_gb300.TERM_RECIP)
        try:
            eng.set_fft_mode(mode)
        except spme_gb300.SpmeError:
            eng.close()
            pytest.skip(f"K={K} {prec}: no fused configuration")
        eng.set_positions(pos)
        out[mode] = eng.apply(f.astype(eng.dtype))
        eng.close()
    assert relerr(out[1], out[0]) < tol


@pytest.mark.parametrize("R", [8, 10, 12, 16])
def test_host_apply_in_parts_matches_device(gpu_lib, R):
    """Host-buffer applies with 8+ right-hand sides copy the result out in parts of
    4 right-hand sides while the next part is interpolated; the values are those of
    the device-pointer apply (same kernels, bit for bit), with alpha and beta."""
    torch = pytest.importorskip("torch")
    n, L, K, p = 2000, 30.0, 32, 6
    pos, f = uniform_case(n, L, R, seed=R)
    eng = spme_gb300.Engine(n, L, 0.4, K, p, rcut=6.0, precision="fp32", max_nrhs=R)
    eng.set_positions(pos)
    f32 = f.astype(np.float32)
    u0 = np.random.default_rng(R).standard_normal((R, 3 * n)).astype(np.float32)
    uh = eng.apply(f32, u0.copy(), alpha=0.7, beta=0.3)
    fd = torch.tensor(f32, device="cuda")
    ud = torch.tensor(u0, device="cuda")
    eng.apply(fd, ud, alpha=0.7, beta=0.3)
    assert np.array_equal(uh, ud.cpu().numpy())
    # pinned host rows: the forces are packed in place from host memory
    fp = torch.tensor(f32).pin_memory().numpy()
    up = torch.tensor(u0).pin_memory().numpy()
    eng.apply(fp, up, alpha=0.7, beta=0.3)
    assert np.array_equal(up, uh)
    ref = oracle.full(pos, L, 0.4, 6.0, K, p, f, nthreads=4)
    assert relerr((uh - 0.3 * u0) / 0.7, ref) < 1e-5
    eng.close()
