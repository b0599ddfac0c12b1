"""GPU parity: the sm_103a path (through the C ABI) against the reference's
golden vectors and the oracle.  Tolerances: FP64 <= 1e-12 relative L2
(reference and oracle), FP32 batched <= 1e-5 relative L2 vs the FP64 oracle."""
import numpy as np
import pytest

import oracle
import spme_gb300
from conftest import GOLDEN_CASES, load_golden, relerr, uniform_case

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_dropin_matches_reference_golden(gpu_lib, name):
    g = load_golden(name)
    n = g["pos"].shape[0]
    nrhs = g["f"].shape[0]
    h = spme_gb300.create_spme_engine(g["xi"], int(g["K"]), int(g["p"]), n, g["L"], 1)
    try:
        vout = g["v0"].copy()
        spme_gb300.compute_spme(h, g["pos"], nrhs, g["alpha"], g["f"], 3 * n, g["beta"], vout,
                                3 * n)
        assert relerr(vout, g["vout"]) < FP64_TOL
        part = vout - g["beta"] * g["v0"]
        assert relerr(part, g["vout"] - g["beta"] * g["v0"]) < FP64_TOL
        # pos == NULL reuses the positions
        vout2 = g["v0"].copy()
        spme_gb300.compute_spme(h, None, nrhs, g["alpha"], g["f"], 3 * n, g["beta"], vout2,
                                3 * n)
        assert relerr(vout2, g["vout"]) < FP64_TOL
    finally:
        spme_gb300.destroy_spme_engine(h)


def test_dropin_leading_dimensions(gpu_lib):
    g = load_golden("n300_k32_p6")
    n, nrhs = g["pos"].shape[0], g["f"].shape[0]
    ld = 3 * n + 7
    fin = np.zeros((nrhs, ld))
    fin[:, :3 * n] = g["f"]
    vout = np.full((nrhs, ld), 99.0)
    vout[:, :3 * n] = g["v0"]
    h = spme_gb300.create_spme_engine(g["xi"], int(g["K"]), int(g["p"]), n, g["L"], 1)
    try:
        spme_gb300.compute_spme(h, g["pos"], nrhs, g["alpha"], fin, ld, g["beta"], vout, ld)
    finally:
        spme_gb300.destroy_spme_engine(h)
    assert relerr(vout[:, :3 * n], g["vout"]) < FP64_TOL
    assert np.all(vout[:, 3 * n:] == 99.0)  # padding untouched


# (N, L, K, p, xi): odd / 5-smooth K, p = 8, 4p >= K, K not a multiple of the tile
RECIP_CASES = [
    (257, 20.0, 25, 4, 0.5),
    (300, 30.0, 27, 6, 0.4),
    (500, 40.0, 45, 8, 0.3),
    (200, 12.0, 24, 8, 0.6),
    (1000, 50.0, 60, 6, 0.3),
    (128, 16.0, 8, 4, 0.9),
    (999, 35.0, 36, 6, 0.35),
]


@pytest.mark.parametrize("case", RECIP_CASES)
def test_recip_fp64_vs_oracle(gpu_lib, case):
    n, L, K, p, xi = case
    pos, f = uniform_case(n, L, 2, seed=n + K)
    eng = spme_gb300.Engine(n, L, xi, K, p, precision="fp64", max_nrhs=2,
                            terms=spme_gb300.TERM_RECIP)
    eng.set_positions(pos)
    u = eng.apply(f, alpha=1.3)
    ref = oracle.recip(pos, L, xi, K, p, f, alpha=1.3, nthreads=4)
    assert relerr(u, ref) < FP64_TOL


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL)])
def test_small_box_single_cell_real_space(gpu_lib, precision, tol):
    """L < 3 rc: the real-space sum runs over one cell with minimum images (two
    cells per side here, L = 25, rc = 10), full operator against the oracle."""
    n, L, K, p, xi, rc, R = 300, 25.0, 24, 6, 0.35, 10.0, 2
    pos, f = uniform_case(n, L, R, seed=25)
    eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, precision=precision, max_nrhs=R)
    eng.set_positions(pos)
    fin = f.astype(eng.dtype)
    u = eng.apply(fin).astype(np.float64)
    eng.close()
    ref = oracle.full(pos, L, xi, rc, K, p, fin.astype(np.float64), nthreads=4)
    err = relerr(u, ref)
    print(f"single-cell {precision}: rel-L2 vs oracle {err:.2e}")
    assert err < tol


@pytest.mark.parametrize("precision,K,tol", [("fp64", 300, FP64_TOL), ("fp32", 320, 1e-5)])
def test_recip_large_mesh_vs_oracle(gpu_lib, precision, K, tol):
    """K = 300 and 320: the fused z-transform kernel runs its narrow-chunk
    configuration here (2 columns per block in FP64, 4 in FP32, the sizes it
    serves from K = 296 to about 1100), with the runtime radix-3/5 pass sequence
    at K = 300."""
    n, L, p, xi, R = 3000, 60.0, 6, 0.5, 2
    pos, f = uniform_case(n, L, R, seed=K + n)
    eng = spme_gb300.Engine(n, L, xi, K, p, precision=precision, max_nrhs=R,
                            terms=spme_gb300.TERM_RECIP)
    eng.set_positions(pos)
    u = eng.apply(f.astype(eng.dtype)).astype(np.float64)
    eng.close()
    ref = oracle.recip(pos, L, xi, K, p, f.astype(eng.dtype).astype(np.float64))
    err = relerr(u, ref)
    print(f"K={K} {precision}: rel-L2 vs oracle {err:.2e}")
    assert err < tol


@pytest.mark.parametrize("tile", [(4, 4, 4), (8, 8, 8), (16, 8, 4), (16, 16, 4), (8, 16, 8)])
def test_tile_shapes(gpu_lib, tile):
    n, L, K, p, xi = 700, 30.0, 40, 6, 0.4
    pos, f = uniform_case(n, L, 3, seed=5)
    eng = spme_gb300.Engine(n, L, xi, K, p, precision="fp64", max_nrhs=3,
                            terms=spme_gb300.TERM_RECIP, tile=tile)
    eng.set_positions(pos)
    u = eng.apply(f)
    ref = oracle.recip(pos, L, xi, K, p, f, nthreads=4)
    assert relerr(u, ref) < FP64_TOL


def test_tile_too_large_is_rejected(gpu_lib):
    # FP64, p = 8: a 16x16x8 tile's interpolation halo does not fit shared memory
    with pytest.raises(spme_gb300.SpmeError) as ei:
        spme_gb300.Engine(100, 30.0, 0.4, 40, 8, precision="fp64", terms=spme_gb300.TERM_RECIP,
                          tile=(16, 16, 8))
    assert ei.value.code == 2


@pytest.mark.parametrize("radius", [1.0, 1.5])
def test_full_operator_fp64_vs_oracle(gpu_lib, radius):
    n, L, K, p, xi, rc = 2000, 50.0, 64, 6, 0.3, 10.0
    pos, f = uniform_case(n, L, 2, seed=77)
    eng = spme_gb300.Engine(n, L, xi, K, p, radius=radius, rcut=rc, precision="fp64",
                            max_nrhs=2, terms=spme_gb300.TERM_ALL)
    eng.set_positions(pos)
    u0 = np.random.default_rng(1).standard_normal(f.shape)
    u = eng.apply(f, u=u0.copy(), alpha=0.7, beta=-0.4)
    ref = oracle.full(pos, L, xi, rc, K, p, f, alpha=0.7, beta=-0.4, u=u0, radius=radius,
                      nthreads=4)
    assert relerr(u, ref) < FP64_TOL


def test_real_and_self_terms_separately(gpu_lib):
    n, L, K, p, xi, rc = 1500, 40.0, 32, 4, 0.35, 9.0
    pos, f = uniform_case(n, L, 1, seed=8)
    for terms, kw in ((spme_gb300.TERM_REAL, dict(real=True, self_term=False)),
                      (spme_gb300.TERM_SELF, dict(real=False, self_term=True))):
        eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, terms=terms)
        eng.set_positions(pos)
        u = eng.apply(f)
        ref = oracle.real_self(pos, L, xi, rc, f, nthreads=4, **kw)
        assert relerr(u, ref) < FP64_TOL


@pytest.mark.parametrize("nrhs,max_nrhs", [(16, 16), (5, 4), (1, 1)])
def test_fp32_batched_vs_fp64_oracle(gpu_lib, nrhs, max_nrhs):
    n, L, K, p, xi, rc = 3000, 60.0, 64, 6, 0.3, 10.0
    pos, f = uniform_case(n, L, nrhs, seed=3)
    eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, precision="fp32", max_nrhs=max_nrhs,
                            terms=spme_gb300.TERM_ALL)
    eng.set_positions(pos)
    u = eng.apply(f.astype(np.float32))
    ref = oracle.full(pos, L, xi, rc, K, p, f, nthreads=4)
    err = relerr(u, ref)
    assert err < FP32_TOL, err


def test_edge_cases(gpu_lib):
    # one particle; particles on the box faces and outside [0, L) (wrapped)
    L, K, p, xi = 10.0, 16, 4, 0.5
    pos = np.array([[0.0, 0.0, 0.0], [L * (1 - 1e-16), 5.0, 9.999999999], [-3.0, 12.5, 4.0]])
    f = np.random.default_rng(0).standard_normal((1, 9))
    eng = spme_gb300.Engine(3, L, xi, K, p, terms=spme_gb300.TERM_RECIP)
    eng.set_positions(pos)
    u = eng.apply(f)
    ref = oracle.recip(np.mod(pos, L), L, xi, K, p, f, nthreads=1)
    assert relerr(u, ref) < FP64_TOL
    # nrhs == 0 is a no-op
    out = np.ones((1, 9))
    eng.apply(np.zeros((0, 9)), u=np.zeros((0, 9)))
    assert np.all(out == 1.0)
    # a single particle
    e1 = spme_gb300.Engine(1, L, xi, K, p, terms=spme_gb300.TERM_RECIP)
    e1.set_positions(pos[:1])
    u1 = e1.apply(f[:, :3])
    assert relerr(u1, oracle.recip(pos[:1], L, xi, K, p, f[:, :3], nthreads=1)) < FP64_TOL


def test_apply_before_positions_is_an_error(gpu_lib):
    eng = spme_gb300.Engine(10, 10.0, 0.5, 16, 4, terms=spme_gb300.TERM_RECIP)
    with pytest.raises(spme_gb300.SpmeError):
        eng.apply(np.zeros((1, 30)))


def test_device_pointer_api(gpu_lib):
    import torch
    n, L, K, p, xi, rc = 1200, 40.0, 32, 6, 0.35, 9.0
    pos, f = uniform_case(n, L, 4, seed=12)
    eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, precision="fp32", max_nrhs=4)
    eng.set_positions(torch.tensor(pos, device="cuda"))
    fd = torch.tensor(f, dtype=torch.float32, device="cuda")
    ud = torch.zeros_like(fd)
    eng.apply(fd, ud)
    eng.synchronize()
    ref = oracle.full(pos, L, xi, rc, K, p, f, nthreads=4)
    assert relerr(ud.cpu().numpy(), ref) < FP32_TOL


# (N, L, K, p, R): even / odd K, all orders, one and two component chunks
SPREAD_CASES = [
    (800, 40.0, 40, 6, 1),
    (900, 40.0, 32, 6, 4),
    (1200, 50.0, 45, 4, 5),
    (700, 36.0, 36, 8, 16),
    (2000, 60.0, 64, 6, 20),
]


@pytest.mark.parametrize("case", SPREAD_CASES)
def test_column_gather_spread_matches_tile_spread(gpu_lib, case):
    """The column-gather spread and the tile spread give the same operator
    (FP64 to round-off), and both match the oracle."""
    n, L, K, p, R = case
    xi = 0.35
    pos, f = uniform_case(n, L, R, seed=K * p + R)
    out = {}
    for mode in (0, 1):
        eng = spme_gb300.Engine(n, L, xi, K, p, precision="fp64", max_nrhs=R,
                                terms=spme_gb300.TERM_RECIP)
        eng.set_spread_mode(mode)
        eng.set_positions(pos)
        out[mode] = eng.apply(f)
        eng.close()
    assert relerr(out[1], out[0]) < 1e-13
    ref = oracle.recip(pos, L, xi, K, p, f, nthreads=4)
    assert relerr(out[1], ref) < FP64_TOL


@pytest.mark.parametrize("radius", [1.0, 1.5])
def test_fp64_real_space_pairs_across_the_table_ranges(gpu_lib, radius):
    """FP64 engines take F(r), G(r) from a Chebyshev table on [a/2, rc] and from
    the closed form below a/2: pairs placed at separations on both sides of a/2,
    inside and outside the overlap range 2a, and just inside rc, against the
    oracle's closed form (FP64 1e-12)."""
    a, L, rc, xi = radius, 60.0, 9.0, 0.4
    seps = np.array([0.2, 0.49, 0.51, 0.8, 1.5, 1.99, 2.01, 2.5, 4.0, 7.3, 8.99]) * np.array(
        [a] * 8 + [1.0] * 3)
    rng = np.random.default_rng(17)
    pos = []
    for k, s in enumerate(seps):
        c = np.array([5.0 + 11.0 * (k % 5), 5.0 + 11.0 * (k // 5), 30.0])
        d = rng.standard_normal(3)
        d *= s / np.linalg.norm(d)
        pos += [c, c + d]
    pos = np.mod(np.array(pos), L)
    n = pos.shape[0]
    f = rng.standard_normal((2, 3 * n))
    eng = spme_gb300.Engine(n, L, xi, 32, 4, radius=a, rcut=rc, precision="fp64",
                            max_nrhs=2, terms=spme_gb300.TERM_REAL | spme_gb300.TERM_SELF)
    eng.set_positions(pos)
    u = eng.apply(f)
    eng.close()
    ref = oracle.real_self(pos, L, xi, rc, f, radius=a, nthreads=2)
    assert relerr(u, ref) < FP64_TOL
    # the pair part alone (self term removed) at the same tolerance
    self_c = oracle.self_coeff(xi, a)
    assert relerr(u - self_c * f, ref - self_c * f) < 1e-11


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL)])
def test_close_and_coincident_pairs(gpu_lib, precision, tol):
    """Pairs far inside the overlap range (r down to 1e-4 a) and coincident
    particles (r = 0, where the pair has no direction) among random ones: the
    real-space functions for r < 2a are evaluated in a form whose 1/r and 1/r^3
    terms cancel analytically, so FP32 stays within its tolerance and FP64
    within 1e-12 of the oracle."""
    rng = np.random.default_rng(23)
    n0, L, K, p, xi, rc, R = 3000, 60.0, 64, 6, 0.3, 10.0, 3
    pos = rng.uniform(0.0, L, size=(n0, 3))
    seps = [0.0, 1e-4, 1e-3, 0.01, 0.05, 0.2, 0.5, 1.0, 1.9]
    extra = []
    for k, s_ in enumerate(seps):
        d = rng.standard_normal(3)
        d *= s_ / np.linalg.norm(d)
        extra.append(pos[k] + d)
    pos = np.mod(np.vstack([pos, np.array(extra)]), L)
    n = pos.shape[0]
    f = rng.standard_normal((R, 3 * n))
    eng = spme_gb300.Engine(n, L, xi, K, p, rcut=rc, precision=precision, max_nrhs=R,
                            terms=spme_gb300.TERM_ALL)
    eng.set_positions(pos)
    u = eng.apply(f.astype(eng.dtype))
    eng.close()
    ref = oracle.full(pos, L, xi, rc, K, p, f.astype(eng.dtype).astype(np.float64), nthreads=4)
    assert np.all(np.isfinite(u))
    err = relerr(u, ref)
    assert err < tol, err
    # the particles of the close pairs alone, at the same tolerance
    rows = np.concatenate([np.arange(3 * k, 3 * k + 3) for k in
                           list(range(len(seps))) + list(range(n0, n))])
    assert relerr(u[:, rows], ref[:, rows]) < tol


# (N, L, K, p, R): FP32 column-gather spread with 1, 2 and 3 components per lane
# and two component chunks (R = 20: 60 components)
FP32_SPREAD_CASES = [
    (1500, 45.0, 48, 6, 3),
    (1500, 45.0, 40, 4, 8),
    (1200, 40.0, 36, 8, 11),
    (2000, 60.0, 64, 6, 20),
]


@pytest.mark.parametrize("case", FP32_SPREAD_CASES)
def test_fp32_column_gather_spread_vs_oracle(gpu_lib, case):
    """The FP32 column-gather spread (plane pairs with the packed two-lane FMA,
    offset-ranked visits, padded force rows) against the tile spread and the
    FP64 oracle."""
    n, L, K, p, R = case
    xi = 0.35
    pos, f = uniform_case(n, L, R, seed=3 * K + R)
    out = {}
    for mode in (0, 1):
        eng = spme_gb300.Engine(n, L, xi, K, p, precision="fp32", max_nrhs=R,
                                terms=spme_gb300.TERM_RECIP)
        eng.set_spread_mode(mode)
        eng.set_positions(pos)
        out[mode] = eng.apply(f.astype(np.float32))
        eng.close()
    ref = oracle.recip(pos, L, xi, K, p, f.astype(np.float32).astype(np.float64), nthreads=4)
    assert relerr(out[1], out[0]) < 2e-6
    assert relerr(out[1], ref) < FP32_TOL
