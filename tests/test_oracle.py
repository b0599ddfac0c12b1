"""CPU: the oracle pinned against the reference's golden vectors and
known-answer tests (B-splines, moduli, Ewald splitting invariance, Hasimoto's
periodic self-mobility, SPME -> exact Ewald k-sum convergence)."""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN_CASES, load_golden, relerr, uniform_case


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_reference_golden(name):
    g = load_golden(name)
    u = oracle.recip(g["pos"], g["L"], g["xi"], int(g["K"]), int(g["p"]), g["f"],
                     alpha=g["alpha"], beta=g["beta"], u=g["v0"], nthreads=2)
    assert relerr(u, g["vout"]) < 1e-13
    # the operator part alone (beta*v0 removed) must match too
    assert relerr(u - g["beta"] * g["v0"], g["vout"] - g["beta"] * g["v0"]) < 1e-13


@pytest.mark.parametrize("p", [2, 4, 6, 8])
def test_bspline_partition_of_unity_and_values(p):
    for w in [0.0, 0.1, 0.5, 0.77, 0.999]:
        q = oracle.bspline_weights(p, w)
        assert abs(q.sum() - 1.0) < 1e-14
        assert np.all(q >= -1e-15)
    # p=4 closed forms: M4 on [0,1] = x^3/6, on [3,4] = (4-x)^3/6
    q = oracle.bspline_weights(4, 0.3)
    assert abs(q[3] - 0.3 ** 3 / 6) < 1e-15
    assert abs(q[0] - 0.7 ** 3 / 6) < 1e-15


def test_bspline_matches_reference_monomial_table():
    # tab_W of old-version/spme.c:34-39 (p=6) evaluated at g = w - 1/2
    W = np.array([
        [1, -10, 40, -80, 80, -32], [237, -750, 840, -240, -240, 160],
        [1682, -1540, -880, 1120, 160, -320], [1682, 1540, -880, -1120, 160, 320],
        [237, 750, 840, 240, -240, -160], [1, 10, 40, 80, 80, 32]]) / 3840.0
    for w in [0.05, 0.4, 0.93]:
        g = w - 0.5
        q_ref = W @ (g ** np.arange(6))
        assert np.max(np.abs(oracle.bspline_weights(6, w) - q_ref)) < 1e-15


def test_moduli_formula():
    K, p = 16, 6
    b2 = oracle.bspline_moduli2(K, p)
    mp = oracle.bspline_weights(p, 0.0)[::-1]  # mp[j] = M_p(j)
    for m in range(K):
        mm = m if m <= K // 2 else m - K
        phi = 2 * np.pi * mm / K
        den = sum(mp[j + 1] * np.exp(1j * j * phi) for j in range(p - 1))
        assert abs(b2[m] - 1 / abs(den) ** 2) < 1e-12 * b2[m]


def _full_direct(pos, L, xi, rc, f, a=1.0):
    kcut = 2.0 * xi * 6.5  # exp(-kcut^2/4xi^2) = e^-42
    u = oracle.recip_direct(pos, L, xi, kcut, f, radius=a, nthreads=2)
    return oracle.real_self(pos, L, xi, rc, f, beta=1.0, u=u, radius=a, nthreads=2)


def test_ewald_split_independent_of_xi():
    """M = M_real + M_recip + M_self must not depend on the splitting xi."""
    pos, f = uniform_case(40, 12.0, 2, seed=3)
    u1 = _full_direct(pos, 12.0, 0.9, 5.9, f)
    u2 = _full_direct(pos, 12.0, 1.1, 5.9, f)
    assert relerr(u1, u2) < 1e-9


@pytest.mark.parametrize("a", [1.0, 1.7])
def test_hasimoto_periodic_self_mobility(a):
    """One sphere in a periodic box: 6 pi eta a M = 1 - 2.837297 a/L + 4pi/3 (a/L)^3 + O((a/L)^6)."""
    L = 20.0
    pos = np.array([[3.0, 4.0, 5.0]])
    f = np.array([[1.0, 0.0, 0.0]])
    u = _full_direct(pos, L, 0.6, 9.0, f, a=a)
    expect = (1 - 2.837297 * a / L + 4 * np.pi / 3 * (a / L) ** 3) / a
    assert abs(u[0, 0] - expect) < 5e-5 * expect
    assert abs(u[0, 1]) < 1e-12 and abs(u[0, 2]) < 1e-12


def test_rpy_overlap_continuity():
    for xi in [0.3, 0.8]:
        Fm, Gm = oracle.real_FG(2.0 - 1e-9, xi)
        Fp, Gp = oracle.real_FG(2.0 + 1e-9, xi)
        assert abs(Fm - Fp) < 1e-7 and abs(Gm - Gp) < 1e-7


def test_spme_recip_converges_to_exact_ksum():
    pos, f = uniform_case(30, 10.0, 1, seed=5)
    exact = oracle.recip_direct(pos, 10.0, 0.8, 2 * np.pi / 10.0 * 40, f, nthreads=2)
    errs = []
    for K in (16, 32, 64):
        u = oracle.recip(pos, 10.0, 0.8, K, 8, f, nthreads=2)
        errs.append(relerr(u, exact))
    assert errs[2] < 1e-6 and errs[2] < errs[1] < errs[0]


def test_recip_symmetry_and_translation_invariance():
    L, K, p, xi = 15.0, 24, 6, 0.5
    pos, f = uniform_case(80, L, 2, seed=9)
    u = oracle.recip(pos, L, xi, K, p, f, nthreads=2)
    # g^T M f == f^T M g (symmetric operator)
    assert abs(f[1] @ u[0] - f[0] @ u[1]) < 1e-12 * np.linalg.norm(u)
    # shifting every particle by one mesh cell leaves M unchanged
    pos2 = (pos + L / K * np.array([1.0, 2.0, -1.0])) % L
    u2 = oracle.recip(pos2, L, xi, K, p, f, nthreads=2)
    assert relerr(u2, u) < 1e-12


def test_numpy_restatement_agrees():
    """Independent numpy/pocketfft restatement of the reference pipeline."""
    L, K, p, xi = 9.0, 12, 4, 0.7
    pos, f = uniform_case(20, L, 1, seed=21)
    u = oracle.recip(pos, L, xi, K, p, f, nthreads=1)
    grid = np.zeros((3, K, K, K))
    st = []
    for i in range(len(pos)):
        c = pos[i] / L * K
        fl = np.floor(c)
        s0 = (fl.astype(int) - p // 2 + 1) % K
        w = [oracle.bspline_weights(p, c[d] - fl[d]) for d in range(3)]
        st.append((s0, w))
        for z in range(p):
            for y in range(p):
                for x in range(p):
                    idx = ((s0[2] + z) % K, (s0[1] + y) % K, (s0[0] + x) % K)
                    grid[(slice(None),) + idx] += w[2][z] * w[1][y] * w[0][x] * f[0, 3 * i:3 * i + 3]
    G = np.fft.rfftn(grid, axes=(1, 2, 3))
    m = np.arange(K)
    k1 = 2 * np.pi * np.where(m <= K // 2, m, m - K) / L
    kz, ky, kx = np.meshgrid(k1, k1, k1[:K // 2 + 1], indexing="ij")
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    k2[0, 0, 0] = 1.0
    b2 = oracle.bspline_moduli2(K, p)
    S = np.vectorize(lambda k: oracle._load().oracle_scalar_recip(k, xi, 1.0))(np.sqrt(k2))
    m2 = S * b2[None, None, :K // 2 + 1] * b2[None, :, None] * b2[:, None, None] / L ** 3
    kv = [kx, ky, kz]
    out = np.zeros_like(G)
    for a_ in range(3):
        for b_ in range(3):
            B = m2 * ((a_ == b_) - kv[a_] * kv[b_] / k2)
            out[a_] += B * G[b_]
    out[:, 0, 0, 0] = 0
    mesh = np.fft.irfftn(out, s=(K, K, K), axes=(1, 2, 3)) * K ** 3
    un = np.zeros(3 * len(pos))
    for i, (s0, w) in enumerate(st):
        for z in range(p):
            for y in range(p):
                for x in range(p):
                    idx = ((s0[2] + z) % K, (s0[1] + y) % K, (s0[0] + x) % K)
                    un[3 * i:3 * i + 3] += w[2][z] * w[1][y] * w[0][x] * mesh[(slice(None),) + idx]
    assert relerr(un, u[0]) < 1e-13


def test_real_FG_close_pairs_full_precision():
    """For r < 2a the real-space functions combine Beenakker's form with the
    overlap correction; the oracle writes the sum so the 1/r and 1/r^3 terms
    cancel analytically.  Against the textbook form evaluated with 50 digits:
    1e-13 relative (to max |F|, |G|) down to r = 1e-6, finite at r = 0, and
    continuous across r = 2a."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50

    def naive(r, xi, a):
        r, xi, a = mp.mpf(r), mp.mpf(xi), mp.mpf(a)
        rsp = 1 / mp.sqrt(mp.pi)
        x = xi * r
        e, ec = mp.exp(-x * x), mp.erfc(x)
        r2, a3 = r * r, a ** 3
        f = (ec * (mp.mpf(3) / 4 * a / r + a3 / (2 * r ** 3))
             + e * rsp * (4 * xi ** 7 * a3 * r2 * r2 + 3 * xi ** 3 * a * r2
                          - 20 * xi ** 5 * a3 * r2 - mp.mpf(9) / 2 * xi * a + 14 * xi ** 3 * a3
                          + xi * a3 / r2))
        g = (ec * (mp.mpf(3) / 4 * a / r - mp.mpf(3) / 2 * a3 / r ** 3)
             + e * rsp * (-4 * xi ** 7 * a3 * r2 * r2 - 3 * xi ** 3 * a * r2
                          + 16 * xi ** 5 * a3 * r2 + mp.mpf(3) / 2 * xi * a - 2 * xi ** 3 * a3
                          - 3 * xi * a3 / r2))
        if r < 2 * a:
            f += (1 - 9 * r / (32 * a)) - (mp.mpf(3) / 4 * a / r + a3 / (2 * r ** 3))
            g += 3 * r / (32 * a) - (mp.mpf(3) / 4 * a / r - mp.mpf(3) / 2 * a3 / r ** 3)
        return float(f / a), float(g / a)

    for xi, a in ((0.3, 1.0), (0.6, 1.5), (1.0, 1.0)):
        for r in (1e-6, 1e-3, 0.01, 0.1, 0.4 / xi, 0.5 / xi, 0.6 / xi, 1.0, 1.99 * a, 2.5 * a):
            if r > 8.0:
                continue
            F, G = oracle.real_FG(r, xi, a)
            Fn, Gn = naive(r, xi, a)
            scale = max(abs(Fn), abs(Gn))
            assert abs(F - Fn) < 1e-13 * scale and abs(G - Gn) < 1e-13 * scale, (xi, a, r)
        F0, G0 = oracle.real_FG(0.0, xi, a)
        assert np.isfinite(F0) and np.isfinite(G0)
        Fm, Gm = oracle.real_FG(2 * a * (1 - 1e-12), xi, a)
        Fp, Gp = oracle.real_FG(2 * a * (1 + 1e-12), xi, a)
        assert abs(Fm - Fp) < 1e-10 and abs(Gm - Gp) < 1e-10
