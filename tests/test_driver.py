"""The `pme` driver: the reference driver's options and semantics
(old-version/main.c:130-260).  CPU tests cover argument handling; GPU tests
compare its output with the oracle."""
import os
import subprocess

import numpy as np
import pytest

import oracle
import spme_gb300
from conftest import ROOT, relerr, uniform_case

PME = os.path.join(ROOT, "spme_gb300", "pme")


def run(*args, **kw):
    if not os.path.exists(PME):
        pytest.skip("driver not built")
    return subprocess.run([PME, *args], capture_output=True, text=True, timeout=300, **kw)


def test_help_version_and_bad_option():
    r = run("--help")
    assert r.returncode == 0 and "--porder" in r.stderr
    r = run("-v")
    assert r.returncode == 0 and "version" in r.stdout
    r = run("--bogus")
    assert r.returncode == 2


def test_missing_file_and_reference_dim_check(tmp_path):
    r = run("--xyz", str(tmp_path / "none.xyz"))
    assert r.returncode == 1 and "Can not read" in r.stderr
    # old-version/main.c:205-209: dim must exceed 4 * porder
    r = run("--synthetic", "50,10", "--dim", "16", "--porder", "4")
    assert r.returncode == 1 and "dim must be larger than 4 * porder" in r.stderr


def _load(prefix, ext, nrhs):
    return np.loadtxt(prefix + ext).reshape(nrhs, -1)


@pytest.mark.gpu
def test_driver_reference_mode_matches_oracle(gpu_lib, tmp_path):
    n, L = 400, 25.0
    pos, _ = uniform_case(n, L, 1, seed=3)
    xyz = str(tmp_path / "in.xyz")
    spme_gb300.write_xyz(xyz, pos, L)
    out = str(tmp_path / "o")
    r = run("--xyz", xyz, "--dim", "32", "--porder", "6", "--xi", "0.4", "--nrhs", "2",
            "--out", out)
    assert r.returncode == 0, r.stderr
    f, v0, v = _load(out, ".f", 2), _load(out, ".v0", 2), _load(out, ".v", 2)
    ref = oracle.recip(pos, L, 0.4, 32, 6, f, alpha=2.1, beta=2.2, u=v0, nthreads=4)
    assert relerr(v, ref) < 1e-12


@pytest.mark.gpu
def test_driver_full_fp32_matches_oracle(gpu_lib, tmp_path):
    out = str(tmp_path / "o")
    xyz = str(tmp_path / "synth.xyz")
    r = run("--synthetic", "1500,40", "--dim", "48", "--porder", "6", "--xi", "0.3", "--full",
            "--rc", "9", "--precision", "fp32", "--nrhs", "3", "--write-xyz", xyz, "--out", out)
    assert r.returncode == 0, r.stderr
    pos, L, _ = spme_gb300.read_xyz(xyz)
    f, v0, v = _load(out, ".f", 3), _load(out, ".v0", 3), _load(out, ".v", 3)
    ref = oracle.full(pos, L, 0.3, 9.0, 48, 6, f.astype(np.float32).astype(np.float64),
                      alpha=2.1, beta=2.2, u=v0.astype(np.float32).astype(np.float64), nthreads=4)
    assert relerr(v, ref) < 1e-5
