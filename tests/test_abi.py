"""CPU: the C-ABI library loads and exports every entry point the public
headers declare; argument validation happens before any device work."""
import ctypes
import os
import re

import pytest

import spme_gb300
from conftest import ROOT


def header_functions():
    names = set()
    for h in ("spme.h", "spme_gb300.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", text, flags=re.M):
            if m.group(1) not in ("if", "return", "defined"):
                names.add(m.group(1))
    return sorted(names)


def test_headers_declare_reference_entry_points():
    names = header_functions()
    for fn in ("cutoff2xi", "create_spme_engine", "destroy_spme_engine", "compute_spme"):
        assert fn in names


@pytest.mark.parametrize("name", header_functions())
def test_library_exports_symbol(name):
    lib = spme_gb300.load()
    assert hasattr(lib, name), name


def test_invalid_params_rejected_without_device_work():
    lib = spme_gb300.load()
    p = spme_gb300.Params()
    lib.spme_params_init(ctypes.byref(p))
    assert p.radius == 1.0 and p.max_nrhs == 1 and p.terms == spme_gb300.TERM_RECIP
    h = ctypes.c_void_p()
    bad = [dict(dim=1), dict(porder=5), dict(box_size=-1.0), dict(xi=0.0),
           dict(terms=spme_gb300.TERM_ALL, rcut=30.0), dict(max_nrhs=0), dict(dim=4, porder=6)]
    for b in bad:
        q = spme_gb300.Params()
        lib.spme_params_init(ctypes.byref(q))
        q.np, q.dim, q.porder, q.box_size, q.xi = 10, 16, 4, 50.0, 0.3
        for k, v in b.items():
            setattr(q, k, v)
        st = lib.spme_create(ctypes.byref(q), ctypes.byref(h))
        assert st in (1, 2), (b, st)
        assert not h.value


def test_cutoff2xi():
    xi = spme_gb300.cutoff2xi(10.0, 1.2e-4, 50.0)
    assert abs(xi - 0.3004666) < 1e-6
    with pytest.raises(ValueError):
        spme_gb300.cutoff2xi(10.0, 2.0, 50.0)


def test_error_strings():
    assert spme_gb300.error_string(0) == "success"
    assert "invalid" in spme_gb300.error_string(1)
