"""TEST INFRASTRUCTURE ONLY — ctypes access to the oracle.

Two checkers live here:

* ``liboracle`` — the project's FP64 C restatement (``spme_oracle.c``) of the
  reference's SPME-RPY apply (billy-inn/SPME ``old-version/spme.c``,
  ``old-version/spme_kernel.c``) plus Beenakker's real-space and self terms.
  It is built by ``make -C oracle oracle`` on any machine.
* ``Reference`` — the reference's own CPU path compiled from its sources with
  the project's MKL/DFTI shim (``oracle/_ref``).  It exists only where the
  reference sources were present at build time.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
legs may import this package.  The product (``spme_gb300``) never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libspme_ref.so")
REF_COLORED_SO = os.path.join(HERE, "_ref", "libspme_ref_colored.so")

_P = ctypes.c_void_p
_lib = None


def build(reference: bool = False) -> None:
    """Compile the oracle (and, if asked and present, the reference)."""
    target = "all" if reference else "oracle"
    subprocess.check_call(["make", "-s", "-C", HERE, target])


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        lib = ctypes.CDLL(ORACLE_SO)
        i, d, l = ctypes.c_int, ctypes.c_double, ctypes.c_long
        lib.oracle_recip.argtypes = [i, _P, d, d, d, i, i, i, d, _P, l, d, _P, l, i]
        lib.oracle_real_self.argtypes = [i, _P, d, d, d, d, i, d, _P, l, d, _P, l, i, i]
        lib.oracle_recip_direct.argtypes = [i, _P, d, d, d, d, i, d, _P, l, d, _P, l, i]
        lib.oracle_bspline_weights.argtypes = [i, d, _P]
        lib.oracle_bspline_moduli2.argtypes = [i, i, _P]
        lib.oracle_scalar_recip.argtypes = [d, d, d]
        lib.oracle_scalar_recip.restype = d
        lib.oracle_real_FG.argtypes = [d, d, d, _P, _P]
        lib.oracle_self_coeff.argtypes = [d, d]
        lib.oracle_self_coeff.restype = d
        for fn in (lib.oracle_recip, lib.oracle_real_self, lib.oracle_recip_direct):
            fn.restype = i
        _lib = lib
    return _lib


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _ptr(a):
    return a.ctypes.data_as(_P)


def _vec_args(f, u, np_):
    """f, u: arrays (nrhs, 3*np) in the reference's vec layout (ld = 3*np)."""
    f = _c(np.atleast_2d(f))
    nrhs = f.shape[0]
    if u is None:
        u = np.zeros((nrhs, 3 * np_))
    else:
        u = _c(np.atleast_2d(u)).copy()
    return f, u, nrhs


def recip(pos, L, xi, K, p, f, alpha=1.0, beta=0.0, u=None, radius=1.0, nthreads=0):
    """beta*u + alpha*M_recip f (reference semantics); f, u shaped (nrhs, 3N)."""
    pos = _c(pos)
    n = pos.shape[0]
    f, u, nrhs = _vec_args(f, u, n)
    rc = _load().oracle_recip(n, _ptr(pos), L, xi, radius, K, p, nrhs, alpha, _ptr(f),
                              3 * n, beta, _ptr(u), 3 * n, nthreads)
    if rc:
        raise ValueError(f"oracle_recip failed ({rc})")
    return u


def real_self(pos, L, xi, rc, f, alpha=1.0, beta=0.0, u=None, radius=1.0, real=True,
              self_term=True, nthreads=0):
    pos = _c(pos)
    n = pos.shape[0]
    f, u, nrhs = _vec_args(f, u, n)
    flags = (1 if real else 0) | (2 if self_term else 0)
    r = _load().oracle_real_self(n, _ptr(pos), L, xi, radius, rc, nrhs, alpha, _ptr(f), 3 * n,
                                 beta, _ptr(u), 3 * n, flags, nthreads)
    if r:
        raise ValueError(f"oracle_real_self failed ({r})")
    return u


def full(pos, L, xi, rc, K, p, f, alpha=1.0, beta=0.0, u=None, radius=1.0, nthreads=0):
    """beta*u + alpha*(M_recip + M_real + M_self) f."""
    ur = recip(pos, L, xi, K, p, f, alpha=alpha, beta=beta, u=u, radius=radius,
               nthreads=nthreads)
    return real_self(pos, L, xi, rc, f, alpha=alpha, beta=1.0, u=ur, radius=radius,
                     nthreads=nthreads)


def recip_direct(pos, L, xi, kcut, f, alpha=1.0, beta=0.0, u=None, radius=1.0, nthreads=0):
    pos = _c(pos)
    n = pos.shape[0]
    f, u, nrhs = _vec_args(f, u, n)
    r = _load().oracle_recip_direct(n, _ptr(pos), L, xi, radius, kcut, nrhs, alpha, _ptr(f),
                                    3 * n, beta, _ptr(u), 3 * n, nthreads)
    if r:
        raise ValueError(f"oracle_recip_direct failed ({r})")
    return u


def bspline_weights(p, w):
    out = np.zeros(p)
    _load().oracle_bspline_weights(p, float(w), _ptr(out))
    return out


def bspline_moduli2(K, p):
    out = np.zeros(K)
    _load().oracle_bspline_moduli2(K, p, _ptr(out))
    return out


def real_FG(r, xi, a=1.0):
    F, G = ctypes.c_double(), ctypes.c_double()
    _load().oracle_real_FG(float(r), xi, a, ctypes.byref(F), ctypes.byref(G))
    return F.value, G.value


def self_coeff(xi, a=1.0):
    return _load().oracle_self_coeff(xi, a)


class Reference:
    """The reference's own create/compute/destroy_spme_engine (old-version/spme.h:89-97),
    compiled from its sources by ``oracle/Makefile``.  Prints its own phase timers."""

    def __init__(self, xi, dim, porder, np_, box_size, nthreads=0, colored=False):
        so = REF_COLORED_SO if colored else REF_SO
        if not os.path.exists(so):
            raise FileNotFoundError(so)
        lib = ctypes.CDLL(so)
        i, d = ctypes.c_int, ctypes.c_double
        lib.create_spme_engine.argtypes = [d, i, i, i, d, i, ctypes.POINTER(_P)]
        lib.compute_spme.argtypes = [_P, _P, i, d, _P, i, d, _P, i]
        lib.destroy_spme_engine.argtypes = [_P]
        self.lib = lib
        self.np = np_
        nthreads = nthreads or (os.cpu_count() or 1)
        self.nthreads = nthreads
        # the reference sizes per-thread buffers and block ranges by nthreads and
        # indexes them by omp_get_thread_num(): the team size must match exactly
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(nthreads)
        h = _P()
        lib.create_spme_engine(xi, dim, porder, np_, box_size, nthreads, ctypes.byref(h))
        self.h = h

    def compute(self, pos, nrhs, alpha, vec_in, ldin, beta, vec_out, ldout):
        """vec_out (float64, modified in place) = beta*vec_out + alpha*M_recip*vec_in."""
        assert vec_out.dtype == np.float64 and vec_out.flags.c_contiguous
        vin = _c(vec_in)
        pp = _ptr(_c(pos)) if pos is not None else None
        self.lib.compute_spme(self.h, pp, nrhs, alpha, _ptr(vin), ldin, beta, _ptr(vec_out),
                              ldout)
        return vec_out

    def compute_with_timers(self, pos, nrhs, alpha, vec_in, ldin, beta, vec_out, ldout):
        """compute() with the reference's own phase timers (its stdout lines
        "compute P", "srpead", "forward fft", "applying influence", "backward fft",
        "interpolate", "totally takes", old-version/spme.c:168-323,651-724 and
        old-version/spme_kernel.c:41-66,122-224,257-308) captured from file
        descriptor 1 and returned as {phase: seconds} (phases repeat per
        right-hand side and are summed)."""
        import re
        import sys
        import tempfile
        libc = ctypes.CDLL(None)
        sys.stdout.flush()
        libc.fflush(None)
        saved = os.dup(1)
        with tempfile.TemporaryFile(mode="w+b") as tmp:
            os.dup2(tmp.fileno(), 1)
            try:
                self.compute(pos, nrhs, alpha, vec_in, ldin, beta, vec_out, ldout)
                libc.fflush(None)
            finally:
                os.dup2(saved, 1)
                os.close(saved)
            tmp.seek(0)
            text = tmp.read().decode(errors="replace")
        phases, head = {}, None
        for line in text.splitlines():
            m = re.search(r"totally takes\s+([0-9.eE+-]+)", line)
            if m:
                phases["total"] = phases.get("total", 0.0) + float(m.group(1))
                continue
            m = re.search(r"takes\s+([0-9.eE+-]+)\s+secs", line)
            if m and head:
                phases[head] = phases.get(head, 0.0) + float(m.group(1))
                head = None
                continue
            h = line.strip().rstrip(".").strip()
            if h and not h.startswith("Computing"):
                head = {"srpead": "spread"}.get(h, h).replace(" ", "_")
        return vec_out, phases

    def close(self):
        if self.h:
            self.lib.destroy_spme_engine(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
