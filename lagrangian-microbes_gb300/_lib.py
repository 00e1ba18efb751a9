"""ctypes binding of liblmgb300.so (declared in include/lm_api.h).

The library is the only compute path of this package: if it cannot be built or loaded, every
entry point raises. There is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

LM_OK = 0
LM_ERR_ARG = 1
LM_ERR_CUDA = 2
LM_ERR_OOM = 3
LM_ERR_STATE = 4
LM_ERR_OUT_OF_BOUNDS = 5
LM_ERR_NAN = 6
LM_ERR_ROUND_CAP = 7
LM_ERR_TIMEOUT = 8
LM_ERR_TIME = 9
LM_ERR_GRID = 10
LM_ERR_CAPACITY = 11

STEP_ADVECT = 1
STEP_INTERACT = 2
STEP_CENSUS = 4
STEP_LOG_PAIRS = 8
STEP_COUNT_PAIRS = 16

TUNE_ROUNDS_THREADS = 1
TUNE_LONG_BLOCKS_PER_SM = 2
TUNE_ADVECT_THREADS = 3

NORM_INF = 0
NORM_L1 = 1
NORM_L2 = 2


class LMError(RuntimeError):
    """A failing call of liblmgb300 (``code`` is the LM_ERR_* status)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[lm status {code}] {message}")
        self.code = code


class OutOfBoundsError(LMError):
    """Particles left the velocity field's domain (the reference's Parcels run aborts here)."""


class TimeRangeError(LMError):
    """A step needs velocity frames outside the field's time axis."""


_ERRORS = {LM_ERR_OUT_OF_BOUNDS: OutOfBoundsError, LM_ERR_TIME: TimeRangeError}


class Stats(ctypes.Structure):
    _fields_ = [
        ("n_particles", ctypes.c_int64),
        ("pairs", ctypes.c_int64),
        ("rounds", ctypes.c_int64),
        ("max_rounds", ctypes.c_int64),
        ("out_of_bounds", ctypes.c_int64),
        ("step", ctypes.c_int64),
        ("census", ctypes.c_int64 * 4),
        ("adj_capacity", ctypes.c_int64),
        ("regrows", ctypes.c_int64),
        ("pairs_total", ctypes.c_int64),
        ("steps_total", ctypes.c_int64),
        ("cells", ctypes.c_int64),
        ("long_lists", ctypes.c_int64),
        ("n_ensembles", ctypes.c_int64),
        ("rounds_total", ctypes.c_int64),
    ]

    def as_dict(self) -> dict:
        d = {name: getattr(self, name) for name, _ in self._fields_ if name != "census"}
        d["census"] = list(self.census)
        return d


_lock = threading.Lock()
_lib = None

P = ctypes.c_void_p
I32 = ctypes.c_int
I64 = ctypes.c_int64
U32 = ctypes.c_uint32
U64 = ctypes.c_uint64
F64 = ctypes.c_double

# name -> argtypes (all return int status)
SIGNATURES = {
    "lm_version": [],
    "lm_kernel_arch": [ctypes.POINTER(I32)],
    "lm_host_alloc": [ctypes.c_size_t, ctypes.POINTER(P)],
    "lm_host_free": [P],
    "lm_ctx_create": [I32, ctypes.POINTER(P)],
    "lm_ctx_destroy": [P],
    "lm_last_error": [P, ctypes.c_char_p, ctypes.c_size_t],
    "lm_ctx_set_stream": [P, ctypes.c_size_t],
    "lm_sync": [P],
    "lm_field_upload": [P, P, P, I32, I32, I32, P, P, P],
    "lm_field_upload_batch": [P, I32, P, P, I32, I32, I32, P, P, P],
    "lm_ensembles_upload": [P, I32, P, P, P, P],
    "lm_set_ensemble_params": [P, I32, P, P, P, P],
    "lm_set_cell_factor": [P, F64],
    "lm_set_tuning": [P, I32, I32],
    "lm_get_tuning": [P, I32, ctypes.POINTER(I32)],
    "lm_census_get": [P, P, I64],
    "lm_particles_upload": [P, I64, P, P, P],
    "lm_particles_download": [P, P, P, P, P],
    "lm_snapshot_save": [P],
    "lm_snapshot_restore": [P],
    "lm_state_export": [P, P, P, P, P, ctypes.POINTER(I64)],
    "lm_state_import": [P, P, P, P, P, I64],
    "lm_species_upload": [P, I64, P],
    "lm_set_interaction": [P, F64, I32, F64, F64, F64, U64],
    "lm_step": [P, F64, F64, I32, I64, U32, F64, P, P, P, P],
    "lm_query_pairs": [P, I64, P, P, P, P, I64, ctypes.POINTER(I64)],
    "lm_count_pairs": [P, I64, P, P, ctypes.POINTER(I64)],
    "lm_interact": [P, I64, P, P, I64, U32],
    "lm_pairs_get": [P, P, P, P, I64, ctypes.POINTER(I64)],
    "lm_graph_capture": [P, F64, F64, I64, I32, U32, F64],
    "lm_graph_run": [P, I32, I32],
    "lm_set_step": [P, I64],
    "lm_stats_get": [P, ctypes.POINTER(Stats)],
    "lm_stats_reset": [P],
    "lm_profile_enable": [P, I32],
    "lm_profile_get": [P, I32, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(F64), ctypes.POINTER(I64)],
    "lm_profile_count": [],
    "lm_count_pairs_noalloc": [P, P, I64, F64, I32, P, P, ctypes.c_size_t],
    "lm_adjoint_create": [P, ctypes.POINTER(P)],
    "lm_adjoint_destroy": [P],
    "lm_adjoint_set_precision": [P, I32],
    "lm_adjoint_forward": [P, P, P, I32, I32, I32, P, P, P, I64, P, P, F64, F64, I32, I32, P, P],
    "lm_adjoint_backward": [P, P, P, P, P, P, P],
    "lm_adjoint_cell_signature": [P, P],
    "lm_adjoint_final_positions": [P, P, P],
    "lm_distance_histogram": [P, P, P, I64, P, I32, I32, F64, P],
    "lm_debug_inject_wait": [P, F64],
}


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load liblmgb300.so (building it with nvcc first if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise LMError(LM_ERR_STATE, f"{path} is missing: build it with lagrangian_microbes_gb300.build.build()")
        lib = ctypes.CDLL(path)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = lib
        return lib


class _HostBlock:
    """Owns one lm_host_alloc block; freed when the last array viewing it is gone."""

    def __init__(self, lib, nbytes: int):
        self._lib = lib
        p = ctypes.c_void_p()
        rc = lib.lm_host_alloc(nbytes, ctypes.byref(p))
        if rc != LM_OK:
            raise _error(rc, f"page-locked allocation of {nbytes} bytes failed")
        self.addr = p.value
        self.nbytes = nbytes

    def __del__(self):
        if getattr(self, "addr", None):
            self._lib.lm_host_free(ctypes.c_void_p(self.addr))
            self.addr = None


def host_empty(shape, dtype) -> np.ndarray:
    """A C-contiguous numpy array in page-locked host memory (for step records: their copies then
    overlap the following steps instead of holding the calling thread)."""
    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape, dtype=np.int64)) * dtype.itemsize
    block = _HostBlock(load(), nbytes)
    raw = (ctypes.c_uint8 * max(nbytes, 1)).from_address(block.addr)
    raw._block = block  # the ctypes buffer keeps the block alive; numpy keeps the buffer
    return np.frombuffer(raw, dtype=np.uint8, count=nbytes).view(dtype).reshape(shape)


def ptr(a: np.ndarray | None):
    """Host pointer of a C-contiguous numpy array (None -> NULL)."""
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("arrays passed to liblmgb300 must be C-contiguous")
    if not a.dtype.isnative:
        raise ValueError("arrays passed to liblmgb300 must be in native byte order")
    return a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """One liblmgb300 context: a CUDA stream plus the device-resident state of one simulation."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = ctypes.c_void_p()
        rc = self._lib.lm_ctx_create(int(device), ctypes.byref(h))
        if rc != LM_OK:
            raise _error(rc, self._message(None))
        self._h = h
        self.device = device

    def _message(self, h) -> str:
        buf = ctypes.create_string_buffer(512)
        self._lib.lm_last_error(h, buf, len(buf))
        return buf.value.decode(errors="replace")

    def check(self, rc: int) -> None:
        if rc != LM_OK:
            raise _error(rc, self._message(self._h))

    def call(self, name: str, *args) -> None:
        if self._h is None:
            raise LMError(LM_ERR_STATE, "context is closed")
        self.check(getattr(self._lib, name)(self._h, *args))

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self._lib.lm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def stats(self) -> dict:
        s = Stats()
        self.call("lm_stats_get", ctypes.byref(s))
        return s.as_dict()

    def profile_enable(self, on: bool = True) -> None:
        self.call("lm_profile_enable", 1 if on else 0)

    def profile(self) -> dict:
        """kernel name -> (total ms, launches) of the plain launches since profile_enable."""
        out = {}
        for k in range(self._lib.lm_profile_count()):
            name = ctypes.create_string_buffer(64)
            ms = ctypes.c_double()
            n = ctypes.c_int64()
            self.call("lm_profile_get", k, name, len(name), ctypes.byref(ms), ctypes.byref(n))
            out[name.value.decode()] = (ms.value, n.value)
        return out


def _error(code: int, message: str) -> LMError:
    return _ERRORS.get(code, LMError)(code, message)


def exported_symbols() -> list[str]:
    return list(SIGNATURES)
