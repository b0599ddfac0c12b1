"""CPU: parameter selection and the reference driver's .xyz format."""
import numpy as np
import pytest

import oracle
import spme_gb300
from conftest import relerr, uniform_case


def test_next_smooth():
    assert spme_gb300.next_smooth(1) == 2
    assert spme_gb300.next_smooth(7) == 8
    assert spme_gb300.next_smooth(61) == 64
    assert spme_gb300.next_smooth(97) == 100
    assert spme_gb300.next_smooth(121) == 125


@pytest.mark.parametrize("tol", [1e-3, 1e-5, 1e-7])
def test_suggest_params_meets_its_estimates(tol):
    q = spme_gb300.suggest_params(1000, 40.0, 1.0, tol, 8.0)
    K, xi, p = q["dim"], q["xi"], q["porder"]
    x = xi * 8.0
    assert np.exp(-x * x) * (1 + x ** 4 / 3) == pytest.approx(tol, rel=1e-6)
    y = (np.pi * K / 40.0) ** 2 / (4 * xi * xi)
    assert np.exp(-y) * (1 + y + 2 * y * y) <= tol
    assert spme_gb300.next_smooth(K) == K
    assert p == (4 if tol >= 1e-3 else 6 if tol >= 1e-6 else 8)


def test_suggested_params_reach_target_accuracy():
    """Full operator with suggested parameters vs a much tighter evaluation."""
    L, n = 16.0, 60
    pos, f = uniform_case(n, L, 1, seed=31)
    t = spme_gb300.suggest_params(n, L, 1.0, 1e-10, 7.9)
    ref = oracle.full(pos, L, t["xi"], t["rcut"], t["dim"], t["porder"], f, nthreads=2)
    for tol in (1e-3, 1e-5):
        q = spme_gb300.suggest_params(n, L, 1.0, tol, 7.5)
        u = oracle.full(pos, L, q["xi"], q["rcut"], q["dim"], q["porder"], f, nthreads=2)
        assert relerr(u, ref) < 3 * tol


def test_xyz_round_trip_and_wrap(tmp_path):
    pos = np.array([[1.5, 2.5, 3.5], [-1.0, 11.0, 4.0], [9.999, 0.0, 25.0]])
    path = str(tmp_path / "p.xyz")
    spme_gb300.write_xyz(path, pos, 10.0, radius=1.3)
    got, L, rad = spme_gb300.read_xyz(path)
    assert L == 10.0 and got.shape == (3, 3)
    assert np.allclose(got, np.mod(pos, 10.0))
    assert np.allclose(rad, 1.3)


def test_xyz_reference_style_file(tmp_path):
    path = tmp_path / "ref.xyz"
    path.write_text("# comment\n# another\n3 20.0\nA 1 2 3 1.0\n# mid\nB 4 5 6 1.0\nC 19 21 -1 1.0\n")
    pos, L, rad = spme_gb300.read_xyz(str(path))
    assert L == 20.0
    assert np.allclose(pos, [[1, 2, 3], [4, 5, 6], [19, 1, 19]])


def test_xyz_errors(tmp_path):
    bad = tmp_path / "bad.xyz"
    bad.write_text("2 10.0\nA 1 2 3 1\n")  # one particle short
    with pytest.raises(spme_gb300.SpmeError):
        spme_gb300.read_xyz(str(bad))
    with pytest.raises(spme_gb300.SpmeError):
        spme_gb300.read_xyz(str(tmp_path / "missing.xyz"))


def test_autotune_cache_key_and_round_trip(tmp_path, monkeypatch):
    """The tile autotuner's cache: keys round N up to a power of two and carry the
    rest of the configuration; the file survives a save/load round trip, and an
    unreadable file reads as empty."""
    from spme_gb300 import autotune as at
    k1 = at.config_key("GB300", 1_000_000, 256, 6, 16, "fp32", 7)
    assert k1 == "GB300|N1048576|K256|p6|R16|fp32|t7"
    assert at.config_key("GB300", 600_000, 256, 6, 16, "fp32", 7) == k1
    assert at.config_key("GB300", 1_000_000, 256, 6, 8, "fp32", 7) != k1
    path = tmp_path / "sub" / "autotune.json"
    monkeypatch.setenv("SPME_AUTOTUNE_CACHE", str(path))
    assert at.cache_path() == str(path)
    assert at._load_cache(str(path)) == {}
    at._save_cache(str(path), {k1: [16, 8, 4]})
    assert at._load_cache(str(path)) == {k1: [16, 8, 4]}
    path.write_text("{not json")
    assert at._load_cache(str(path)) == {}


def test_uneven_batch_systems():
    """The uneven-batch workload: N log-uniform in [500, 50000], L for volume
    fraction 0.05, K the smallest 5-smooth size >= 0.6 L (and >= p), p in {4, 6, 8},
    the same list for the same seed."""
    import math

    from spme_gb300.batch import uneven_systems

    def smooth(k):
        for q in (2, 3, 5):
            while k % q == 0:
                k //= q
        return k == 1

    sys_a = uneven_systems(count=64, seed=1234)
    assert sys_a == uneven_systems(count=64, seed=1234)
    assert sys_a != uneven_systems(count=64, seed=99)
    assert len(sys_a) == 64
    for s in sys_a:
        assert 500 <= s["N"] <= 50_000
        assert math.isclose(s["L"], (s["N"] * 4.0 / 3.0 * math.pi / 0.05) ** (1.0 / 3.0))
        assert s["p"] in (4, 6, 8)
        assert smooth(s["K"]) and s["K"] >= max(0.6 * s["L"], s["p"])
        assert not any(smooth(k) for k in range(math.ceil(0.6 * s["L"]), s["K"])) or s["K"] == s["p"]
