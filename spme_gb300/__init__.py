"""GB300-native SPME mobility operator for the Rotne-Prager-Yamakawa tensor.

Python host mirror of the C ABI in ``include/spme.h`` / ``include/spme_gb300.h``
(``libspme_gb300.so``, hand-written sm_103a kernels + cuFFT).  Two layers:

* the reference's entry points, same names and argument meaning as
  billy-inn/SPME ``old-version/spme.h:85-97``: ``cutoff2xi``,
  ``create_spme_engine``, ``compute_spme``, ``destroy_spme_engine``;
* :class:`Engine`, the extended operator (full Ewald-split RPY mobility, FP32
  batching of right-hand sides, host numpy arrays or CUDA tensors).

There is no CPU fallback: if the shared library is missing or fails to load,
every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libspme_gb300.so")

SPME_OK = 0
ERR_INVALID, ERR_UNSUPPORTED = 1, 2
SPME_FP64, SPME_FP32 = 0, 1
TERM_RECIP, TERM_REAL, TERM_SELF, TERM_ALL = 1, 2, 4, 7
MEM_HOST, MEM_DEVICE = 0, 1
STAGES = ("pack", "realspace", "spread", "fft_fwd", "influence", "fft_bwd", "interp", "unpack")

_P = ctypes.c_void_p
_lib = None


class SpmeError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        msg = error_string(code) if _lib is not None else str(code)
        super().__init__(f"{what}: {msg} (status {code})" if what else msg)


class Params(ctypes.Structure):
    """Mirror of ``spme_params`` (include/spme_gb300.h)."""

    _fields_ = [
        ("np", ctypes.c_int),
        ("dim", ctypes.c_int),
        ("porder", ctypes.c_int),
        ("box_size", ctypes.c_double),
        ("xi", ctypes.c_double),
        ("radius", ctypes.c_double),
        ("rcut", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("max_nrhs", ctypes.c_int),
        ("terms", ctypes.c_int),
    ]


class BatchSystem(ctypes.Structure):
    """Mirror of ``spme_batch_system`` (include/spme_gb300.h)."""

    _fields_ = [
        ("np", ctypes.c_int),
        ("dim", ctypes.c_int),
        ("porder", ctypes.c_int),
        ("box_size", ctypes.c_double),
        ("xi", ctypes.c_double),
        ("radius", ctypes.c_double),
        ("rcut", ctypes.c_double),
    ]


def load(path: str | None = None):
    """Load libspme_gb300.so (raises if it is absent: no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -m spme_gb300.build` "
            "(nvcc, sm_103a); there is no CPU fallback")
    lib = ctypes.CDLL(path)
    i, d, l = ctypes.c_int, ctypes.c_double, ctypes.c_long
    sig = {
        "spme_params_init": (None, [ctypes.POINTER(Params)]),
        "spme_create": (i, [ctypes.POINTER(Params), ctypes.POINTER(_P)]),
        "spme_destroy": (i, [_P]),
        "spme_set_stream": (i, [_P, _P]),
        "spme_get_stream": (_P, [_P]),
        "spme_set_positions": (i, [_P, _P, i]),
        "spme_apply": (i, [_P, i, d, _P, l, d, _P, l, i]),
        "spme_synchronize": (i, [_P]),
        "spme_set_profiling": (i, [_P, i]),
        "spme_stage_times": (i, [_P, ctypes.POINTER(ctypes.c_float), i]),
        "spme_launch_count": (l, [_P]),
        "spme_set_tile": (i, [_P, i, i, i]),
        "spme_set_graphs": (i, [_P, i]),
        "spme_set_fft_mode": (i, [_P, i]),
        "spme_set_spread_mode": (i, [_P, i]),
        "spme_set_overlap": (i, [_P, i]),
        "spme_last_error": (i, [_P]),
        "spme_error_string": (ctypes.c_char_p, [i]),
        "cutoff2xi": (None, [d, d, d, ctypes.POINTER(d)]),
        "create_spme_engine": (None, [d, i, i, i, d, i, ctypes.POINTER(_P)]),
        "destroy_spme_engine": (None, [_P]),
        "compute_spme": (None, [_P, _P, i, d, _P, i, d, _P, i]),
        "spme_suggest_params": (i, [i, d, d, d, d, ctypes.POINTER(Params)]),
        "spme_next_smooth": (i, [i]),
        "spme_read_xyz": (i, [ctypes.c_char_p, ctypes.POINTER(i), ctypes.POINTER(d),
                              ctypes.POINTER(ctypes.POINTER(d)), ctypes.POINTER(ctypes.POINTER(d))]),
        "spme_write_xyz": (i, [ctypes.c_char_p, i, d, _P, d]),
        "spme_free": (None, [_P]),
        "spme_fma_peak": (i, [i, ctypes.POINTER(d)]),
        "spme_batch_create": (i, [ctypes.POINTER(BatchSystem), i, i, i, ctypes.POINTER(_P)]),
        "spme_batch_destroy": (i, [_P]),
        "spme_batch_set_stream": (i, [_P, _P]),
        "spme_batch_get_stream": (_P, [_P]),
        "spme_batch_set_tile": (i, [_P, i, i, i]),
        "spme_batch_set_positions": (i, [_P, _P]),
        "spme_batch_apply": (i, [_P, d, _P, d, _P]),
        "spme_batch_step": (i, [_P, _P, d, _P, d, _P]),
        "spme_batch_set_graphs": (i, [_P, i]),
        "spme_batch_set_overlap": (i, [_P, i]),
        "spme_batch_synchronize": (i, [_P]),
        "spme_batch_launch_count": (l, [_P]),
        "spme_batch_particles": (l, [_P]),
        "spme_batch_set_profiling": (i, [_P, i]),
        "spme_batch_stage_times": (i, [_P, ctypes.POINTER(ctypes.c_float), i]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def error_string(code: int) -> str:
    return load().spme_error_string(int(code)).decode()


def _check(code: int, what: str):
    if code != SPME_OK:
        raise SpmeError(code, what)


# ---------------------------------------------------------------------------
# reference entry points (old-version/spme.h:85-97)
# ---------------------------------------------------------------------------

def cutoff2xi(rmax: float, ewald_eps: float, box_size: float) -> float:
    """xi with exp(-xi^2 rmax^2) = ewald_eps (old-version/spme.h:85-86, never
    defined in the reference)."""
    out = ctypes.c_double()
    load().cutoff2xi(rmax, ewald_eps, box_size, ctypes.byref(out))
    if out.value <= 0.0:
        raise ValueError("cutoff2xi: need rmax > 0 and 0 < ewald_eps < 1")
    return out.value


def create_spme_engine(xi: float, dim: int, porder: int, np_: int, box_size: float,
                       nthreads: int = 1):
    """Opaque engine handle (old-version/spme.h:89-91).  Reciprocal part only,
    radius 1, FP64 — the reference's operator."""
    h = _P()
    load().create_spme_engine(xi, dim, porder, np_, box_size, nthreads, ctypes.byref(h))
    if not h.value:
        raise SpmeError(1, "create_spme_engine")
    return h


def destroy_spme_engine(h) -> None:
    load().destroy_spme_engine(h)


def compute_spme(h, pos, nrhs: int, alpha: float, vec_in, ldin: int, beta: float, vec_out,
                 ldout: int) -> None:
    """vec_out[r*ldout + 3i + d] = beta*vec_out[...] + alpha*(M_recip vec_in_r)[3i + d]
    (old-version/spme.h:95-97).  numpy float64 host arrays; vec_out updated in place;
    pos None reuses the previous positions."""
    lib = load()
    vin = np.ascontiguousarray(vec_in, dtype=np.float64)
    if not (isinstance(vec_out, np.ndarray) and vec_out.dtype == np.float64
            and vec_out.flags.c_contiguous):
        raise TypeError("vec_out must be a C-contiguous float64 numpy array")
    pp = None
    if pos is not None:
        pp = np.ascontiguousarray(pos, dtype=np.float64)
    lib.compute_spme(h, pp.ctypes.data_as(_P) if pp is not None else None, nrhs, alpha,
                     vin.ctypes.data_as(_P), ldin, beta, vec_out.ctypes.data_as(_P), ldout)
    _check(lib.spme_last_error(h), "compute_spme")


def suggest_params(np_: int, box_size: float, radius: float = 1.0, tol: float = 1e-5,
                   rcut: float = 0.0) -> dict:
    """Ewald parameters (xi, K, p, rc) for a target relative error (host only)."""
    out = Params()
    _check(load().spme_suggest_params(int(np_), float(box_size), float(radius), float(tol),
                                      float(rcut), ctypes.byref(out)), "spme_suggest_params")
    return {"np": out.np, "box_size": out.box_size, "xi": out.xi, "dim": out.dim,
            "porder": out.porder, "radius": out.radius, "rcut": out.rcut}


def fma_peak(precision: str = "fp32") -> float:
    """Measured FMA throughput of the current device in FLOP/s."""
    out = ctypes.c_double()
    _check(load().spme_fma_peak(SPME_FP32 if precision == "fp32" else SPME_FP64,
                                ctypes.byref(out)), "spme_fma_peak")
    return out.value


def next_smooth(n: int) -> int:
    return int(load().spme_next_smooth(int(n)))


def read_xyz(path: str):
    """(positions (N,3) wrapped into [0,L), L, radii) from a reference-format .xyz."""
    lib = load()
    n, L = ctypes.c_int(), ctypes.c_double()
    pp, rp = ctypes.POINTER(ctypes.c_double)(), ctypes.POINTER(ctypes.c_double)()
    _check(lib.spme_read_xyz(path.encode(), ctypes.byref(n), ctypes.byref(L), ctypes.byref(pp),
                             ctypes.byref(rp)), "spme_read_xyz")
    try:
        pos = np.ctypeslib.as_array(pp, shape=(n.value, 3)).copy()
        rad = np.ctypeslib.as_array(rp, shape=(n.value,)).copy()
    finally:
        lib.spme_free(ctypes.cast(pp, _P))
        lib.spme_free(ctypes.cast(rp, _P))
    return pos, L.value, rad


def write_xyz(path: str, pos, box_size: float, radius: float = 1.0) -> None:
    pp = np.ascontiguousarray(pos, dtype=np.float64)
    _check(load().spme_write_xyz(path.encode(), pp.shape[0], float(box_size),
                                 pp.ctypes.data_as(_P), float(radius)), "spme_write_xyz")


# ---------------------------------------------------------------------------
# extended operator
# ---------------------------------------------------------------------------

def _is_torch_cuda(x) -> bool:
    return hasattr(x, "is_cuda") and bool(getattr(x, "is_cuda"))


class Engine:
    """The full Ewald-split RPY mobility M = M_recip + M_real + M_self.

    ``precision`` "fp64" or "fp32"; ``max_nrhs`` right-hand sides go through one
    mesh pass.  Vectors use compute_spme's layout (rows of 3N per right-hand
    side): numpy arrays (host, copied in the call, which returns when the
    result is in place) or CUDA tensors (device; the work is ordered on
    torch's current stream, like any torch operation).
    """

    def __init__(self, np_: int, box_size: float, xi: float, dim: int, porder: int,
                 radius: float = 1.0, rcut: float = 0.0, precision: str = "fp64",
                 max_nrhs: int = 1, terms: int = TERM_ALL, tile=None):
        lib = load()
        p = Params()
        lib.spme_params_init(ctypes.byref(p))
        p.np, p.dim, p.porder = int(np_), int(dim), int(porder)
        p.box_size, p.xi, p.radius, p.rcut = float(box_size), float(xi), float(radius), float(rcut)
        p.precision = SPME_FP32 if precision == "fp32" else SPME_FP64
        p.max_nrhs, p.terms = int(max_nrhs), int(terms)
        self.params = p
        self.np = int(np_)
        self.dtype = np.float32 if precision == "fp32" else np.float64
        h = _P()
        _check(lib.spme_create(ctypes.byref(p), ctypes.byref(h)), "spme_create")
        self.h = h
        self._own_stream = lib.spme_get_stream(h)
        self._stream = self._own_stream
        if tile is not None:
            _check(lib.spme_set_tile(h, *tile), "spme_set_tile")

    # -- lifecycle -----------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            load().spme_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- operations ----------------------------------------------------------
    def set_stream(self, stream_ptr: int | None):
        """Run on the given cudaStream_t handle (0: legacy default stream);
        None returns to the engine's own stream."""
        s = self._own_stream if stream_ptr is None else (stream_ptr or None)
        _check(load().spme_set_stream(self.h, s), "spme_set_stream")
        self._stream = s

    def _follow_torch(self):
        """CUDA-tensor calls are ordered with torch's current stream."""
        import torch
        cur = torch.cuda.current_stream().cuda_stream or None
        if cur != self._stream:
            _check(load().spme_set_stream(self.h, cur), "spme_set_stream")
            self._stream = cur

    def set_positions(self, pos):
        lib = load()
        if _is_torch_cuda(pos):
            import torch
            assert pos.dtype == torch.float64 and pos.is_contiguous()
            self._follow_torch()
            _check(lib.spme_set_positions(self.h, pos.data_ptr(), MEM_DEVICE), "set_positions")
        else:
            pp = np.ascontiguousarray(pos, dtype=np.float64)
            if pp.shape != (self.np, 3):
                raise ValueError(f"positions must be ({self.np}, 3)")
            _check(lib.spme_set_positions(self.h, pp.ctypes.data_as(_P), MEM_HOST),
                   "set_positions")

    def apply(self, f, u=None, alpha: float = 1.0, beta: float = 0.0):
        """u = beta*u + alpha*M f for each row (right-hand side) of f (nrhs, 3N)."""
        lib = load()
        if _is_torch_cuda(f):
            import torch
            self._follow_torch()
            f2 = f.reshape(-1, 3 * self.np)
            if u is None:
                u = torch.zeros_like(f2)
            u2 = u.reshape(-1, 3 * self.np)
            nrhs = f2.shape[0]
            _check(lib.spme_apply(self.h, nrhs, alpha, f2.data_ptr(), f2.stride(0), beta,
                                  u2.data_ptr(), u2.stride(0), MEM_DEVICE), "spme_apply")
            return u
        f2 = np.ascontiguousarray(np.atleast_2d(f), dtype=self.dtype)
        nrhs = f2.shape[0]
        if f2.shape[1] != 3 * self.np:
            raise ValueError("f rows must hold 3N values")
        if u is None:
            u = np.zeros_like(f2)
        if not (u.dtype == self.dtype and u.flags.c_contiguous and u.shape == f2.shape):
            raise TypeError("u must be a C-contiguous array like f")
        _check(lib.spme_apply(self.h, nrhs, alpha, f2.ctypes.data_as(_P), 3 * self.np, beta,
                              u.ctypes.data_as(_P), 3 * self.np, MEM_HOST), "spme_apply")
        return u

    def synchronize(self):
        _check(load().spme_synchronize(self.h), "spme_synchronize")

    def set_profiling(self, level: int = 1):
        """0 off; 1 stage events (real-space still overlapped); 2 stages serialized."""
        load().spme_set_profiling(self.h, int(level))

    def stage_times(self) -> dict:
        buf = (ctypes.c_float * len(STAGES))()
        n = load().spme_stage_times(self.h, buf, len(STAGES))
        return {STAGES[k]: float(buf[k]) for k in range(n)}

    def set_graphs(self, on: bool = True):
        """Replay captured CUDA graphs for repeated passes (see spme_set_graphs)."""
        _check(load().spme_set_graphs(self.h, 1 if on else 0), "spme_set_graphs")

    def set_overlap(self, on: bool):
        """Real-space sum concurrent with the mesh pipeline (True) or before it."""
        _check(load().spme_set_overlap(self.h, 1 if on else 0), "spme_set_overlap")

    def set_spread_mode(self, mode: int):
        """1: column-gather spread (default where it applies); 0: tile spread."""
        _check(load().spme_set_spread_mode(self.h, int(mode)), "spme_set_spread_mode")

    def set_fft_mode(self, mode: int):
        """2: one-pass 2D transforms + fused z-FFT/influence kernel (FP32, K = 128,
        160, 256); 1: 2D cuFFT + fused kernel (the FP32 default where it fits);
        0: 3D cuFFT + influence."""
        _check(load().spme_set_fft_mode(self.h, int(mode)), "spme_set_fft_mode")

    def set_tile(self, tx: int, ty: int, tz: int):
        _check(load().spme_set_tile(self.h, tx, ty, tz), "spme_set_tile")

    def launch_count(self) -> int:
        return int(load().spme_launch_count(self.h))


class Batch:
    """Independent systems (uneven N, L, K, p; same right-hand-side count and
    precision) applied together: every stage is one launch over a packed work
    list of all systems, cuFFT one batched plan per distinct K
    (``spme_batch_*`` in include/spme_gb300.h).  Device (CUDA tensor) data only,
    in the packed layouts: positions ``pack(pos_list)`` (sum N x 3 float64),
    vectors ``pack(f_list)`` with system k's (R, 3 N_k) rows contiguous.  Work
    is ordered on torch's current stream."""

    STAGES = ("positions", "pack", "realspace", "spread", "fft_fwd", "influence", "fft_bwd",
              "interp", "unpack")

    def __init__(self, systems: list, nrhs: int = 4, precision: str = "fp32"):
        lib = load()
        arr = (BatchSystem * len(systems))()
        for k, sy in enumerate(systems):
            arr[k].np, arr[k].dim, arr[k].porder = int(sy["N"]), int(sy["K"]), int(sy["p"])
            arr[k].box_size, arr[k].xi = float(sy["L"]), float(sy["xi"])
            arr[k].radius, arr[k].rcut = float(sy.get("radius", 1.0)), float(sy["rc"])
        h = _P()
        prec = SPME_FP32 if precision == "fp32" else SPME_FP64
        _check(lib.spme_batch_create(arr, len(systems), int(nrhs), prec, ctypes.byref(h)),
               "spme_batch_create")
        self.h = h
        self.systems = list(systems)
        self.nrhs = int(nrhs)
        self.dtype = np.float32 if precision == "fp32" else np.float64
        self._stream = lib.spme_batch_get_stream(h)

    @staticmethod
    def pack(parts):
        """Concatenate per-system tensors (positions (N_k, 3) or vectors (R, 3 N_k))."""
        import torch
        return torch.cat([x.reshape(-1) for x in parts])

    def unpack(self, packed):
        """Per-system views (R, 3 N_k) of a packed vector."""
        out, off = [], 0
        for sy in self.systems:
            m = self.nrhs * 3 * int(sy["N"])
            out.append(packed[off:off + m].view(self.nrhs, 3 * int(sy["N"])))
            off += m
        return out

    def _follow_torch(self):
        import torch
        cur = torch.cuda.current_stream().cuda_stream or None
        if cur != self._stream:
            _check(load().spme_batch_set_stream(self.h, cur), "spme_batch_set_stream")
            self._stream = cur

    def set_positions(self, pos):
        self._follow_torch()
        _check(load().spme_batch_set_positions(self.h, pos.data_ptr()), "spme_batch_set_positions")

    def apply(self, f, u, alpha: float = 1.0, beta: float = 0.0):
        self._follow_torch()
        _check(load().spme_batch_apply(self.h, alpha, f.data_ptr(), beta, u.data_ptr()),
               "spme_batch_apply")
        return u

    def step(self, pos, f, u, alpha: float = 1.0, beta: float = 0.0):
        """Positions then apply; one CUDA graph launch when graphs are on."""
        self._follow_torch()
        _check(load().spme_batch_step(self.h, pos.data_ptr(), alpha, f.data_ptr(), beta,
                                      u.data_ptr()), "spme_batch_step")
        return u

    def set_graphs(self, on: bool = True):
        _check(load().spme_batch_set_graphs(self.h, 1 if on else 0), "spme_batch_set_graphs")

    def set_tile(self, tx: int, ty: int, tz: int):
        _check(load().spme_batch_set_tile(self.h, tx, ty, tz), "spme_batch_set_tile")

    def set_overlap(self, mode: int):
        """1: real-space sum on a second stream; 2: cuFFT groups on four streams."""
        _check(load().spme_batch_set_overlap(self.h, int(mode)), "spme_batch_set_overlap")

    def set_profiling(self, on: bool = True):
        load().spme_batch_set_profiling(self.h, 1 if on else 0)

    def stage_times(self) -> dict:
        buf = (ctypes.c_float * len(self.STAGES))()
        n = load().spme_batch_stage_times(self.h, buf, len(self.STAGES))
        return {self.STAGES[k]: float(buf[k]) for k in range(n)}

    def synchronize(self):
        _check(load().spme_batch_synchronize(self.h), "spme_batch_synchronize")

    def launch_count(self) -> int:
        return int(load().spme_batch_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None):
            load().spme_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
