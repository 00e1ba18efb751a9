"""CPU oracle of the lagrangian-microbes hot path -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py (CPU baseline and the reference
arm), as the checker and the timed CPU restatement; the product package never imports it.

It wraps lm_oracle.c (built by ``build()`` with gcc, -ffp-contract=off so that the float64 pair
test is exactly the reference's) and adds numpy restatements of the reference's lattice helper
(utils.py:25-42, particle_advecter.py:26-35) used to cross-check the package.
"""

from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liblmoracle.so")
SRC = os.path.join(HERE, "lm_oracle.c")
CFLAGS = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]


def build(force: bool = False) -> str:
    """Compile liblmoracle.so from lm_oracle.c (seconds; gcc only)."""
    deps = [SRC, os.path.join(HERE, "lm_oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", *CFLAGS, "-D_GNU_SOURCE", "-I", HERE, SRC, "-o", tmp, "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n$ {' '.join(cmd)}\n{r.stdout}")
    os.replace(tmp, LIB)
    return LIB


class OrcField(ctypes.Structure):
    _fields_ = [("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("nt", ctypes.c_int), ("lon0", ctypes.c_double), ("dlon", ctypes.c_double),
                ("lat0", ctypes.c_double), ("dlat", ctypes.c_double), ("t0", ctypes.c_double),
                ("dT", ctypes.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P, I64, U32, U64, F64, I = (ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint64,
                                    ctypes.c_double, ctypes.c_int)
        sig = {
            "orc_philox4x32_10": (None, [P, P, P]),
            "orc_pair_draw": (None, [U32, U32, U32, U64, P, P]),
            "orc_diffusion_draw": (None, [U32, U32, U64, P, P]),
            "orc_prob_threshold": (U64, [F64]),
            "orc_advect_f64": (I64, [P, I64, P, P, P, F64, F64, I, P, P]),
            "orc_advect_f32": (I64, [P, I64, P, P, P, F64, F64, I, I]),
            "orc_advect_f64d": (I64, [P, I64, P, P, P, F64, F64, I, I, P]),
            "orc_advect_f64d_dir": (I64, [P, P, P, F64, I64, P, P, P, F64, F64, I, I, P]),
            "orc_pairs": (I64, [I64, P, P, F64, I, I, P, P, I64]),
            "orc_count_pairs": (I64, [I64, P, P, F64, I, I]),
            "orc_rps_apply": (None, [P, ctypes.c_int32, ctypes.c_int32, U64, U64, U64, U64]),
            "orc_rps_replay": (None, [P, I64, P, P, U32, U64, U64, U64, U64]),
            "orc_priority_order": (None, [I64, P, P, U32, U64]),
            "orc_pair_prio": (U64, [U32, U32, U32, U64]),
            "orc_interact_step": (I64, [I64, P, P, P, F64, I, U64, U64, U64, U64, U32, I]),
            "orc_run": (I64, [P, I64, P, P, P, P, F64, F64, I, U32, F64, I, U64, U64, U64, U64, I]),
            "orc_haversine": (F64, [F64, F64, F64, F64, F64]),
            "orc_distance_histogram": (None, [I64, P, P, I, F64, F64, I, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def norm_code(p) -> int:
    if p == 2:
        return 2
    if p == 1:
        return 1
    if math.isinf(float(p)):
        return 0
    raise ValueError(p)


# ---------------- random numbers ----------------

def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def pair_draw(i: int, j: int, step: int, seed: int):
    u53 = ctypes.c_uint64()
    prio = ctypes.c_uint64()
    lib().orc_pair_draw(i, j, step, seed & 0xFFFFFFFFFFFFFFFF, ctypes.byref(u53), ctypes.byref(prio))
    return u53.value, prio.value


def pair_uniform(i: int, j: int, step: int, seed: int) -> float:
    """The float64 r in [0, 1) that replaces np.random.rand() for pair (i, j) at `step`."""
    return pair_draw(min(i, j), max(i, j), step, seed)[0] * 2.0 ** -53


def diffusion_draw(p: int, step: int, seed: int):
    a = ctypes.c_float()
    b = ctypes.c_float()
    lib().orc_diffusion_draw(p, step, seed & 0xFFFFFFFFFFFFFFFF, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def prob_threshold(p: float) -> int:
    return lib().orc_prob_threshold(float(p))


# ---------------- lattice (numpy restatement of particle_advecter.py:26-35, utils.py:25-42) ----------------

def lattice_shape(n: int):
    divs = [d for d in range(1, math.isqrt(n) + 1) if n % d == 0]
    a = divs[-1]
    return a, n // a


def lattice(n: int, lat_min, lat_max, lon_min, lon_max):
    n_lat, n_lon = lattice_shape(n)
    lons = np.repeat(np.linspace(lon_min, lon_max, n_lon), n_lat)
    lats = np.tile(np.linspace(lat_min, lat_max, n_lat), n_lon)
    return lons, lats


# ---------------- advection ----------------

def _field_struct(fld):
    u = np.ascontiguousarray(fld.u, dtype=np.float32)
    v = np.ascontiguousarray(fld.v, dtype=np.float32)
    nt, ny, nx = u.shape
    s = OrcField(u.ctypes.data, v.ctypes.data, nx, ny, nt, float(fld.lon[0]), float((fld.lon[-1] - fld.lon[0]) / (nx - 1)),
                 float(fld.lat[0]), float((fld.lat[-1] - fld.lat[0]) / (ny - 1)), float(fld.times[0]),
                 float((fld.times[-1] - fld.times[0]) / (nt - 1)))
    return s, (u, v)


def advect_f64(fld, lons, lats, t0: float, dt: float, n_steps: int, record: bool = False):
    """FP64 RK4 oracle: returns (lon, lat, status[, rec_lon, rec_lat])."""
    s, keep = _field_struct(fld)
    lon = np.array(lons, dtype=np.float64)
    lat = np.array(lats, dtype=np.float64)
    st = np.zeros(lon.size, np.uint8)
    rl = np.empty((n_steps, lon.size)) if record else None
    ra = np.empty((n_steps, lon.size)) if record else None
    bad = lib().orc_advect_f64(ctypes.byref(s), lon.size, _p(lon), _p(lat), _p(st), float(t0), float(dt),
                               int(n_steps), _p(rl), _p(ra))
    if bad < 0:
        raise ValueError("time outside the field's time axis")
    return (lon, lat, st, rl, ra) if record else (lon, lat, st)


def advect_f64_field64(u, v, lon_axis, lat_axis, t_axis, lons, lats, t0: float, dt: float, n_steps: int,
                       n_threads: int = 0, cell_signature: bool = False, du=None, dv=None, s: float = 0.0):
    """FP64 RK4 on a float64 field u, v [nt][ny][nx]: returns (lon, lat, status[, signature]).

    The signature (uint64 per particle) folds the grid cell of every stage evaluation; two runs of
    a particle with equal signatures sampled the same cells, so their difference is smooth.
    With int8 directions du, dv (the field's shape) the run samples u + s du, v + s dv."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    nt, ny, nx = u.shape
    fs = OrcField(u.ctypes.data, v.ctypes.data, nx, ny, nt, float(lon_axis[0]),
                  float((lon_axis[-1] - lon_axis[0]) / (nx - 1)), float(lat_axis[0]),
                  float((lat_axis[-1] - lat_axis[0]) / (ny - 1)), float(t_axis[0]),
                  float((t_axis[-1] - t_axis[0]) / (nt - 1)))
    lon = np.array(lons, dtype=np.float64)
    lat = np.array(lats, dtype=np.float64)
    st = np.zeros(lon.size, np.uint8)
    sig = np.zeros(lon.size, np.uint64) if cell_signature else None
    if du is None:
        bad = lib().orc_advect_f64d(ctypes.byref(fs), lon.size, _p(lon), _p(lat), _p(st), float(t0), float(dt),
                                    int(n_steps), int(n_threads), _p(sig))
    else:
        du = np.ascontiguousarray(du, dtype=np.int8)
        dv = np.ascontiguousarray(dv, dtype=np.int8)
        if du.shape != u.shape or dv.shape != v.shape:
            raise ValueError("directions must have the field's shape")
        bad = lib().orc_advect_f64d_dir(ctypes.byref(fs), _p(du), _p(dv), float(s), lon.size, _p(lon), _p(lat), _p(st),
                                        float(t0), float(dt), int(n_steps), int(n_threads), _p(sig))
    if bad < 0:
        raise ValueError("time outside the field's time axis")
    return (lon, lat, st, sig) if cell_signature else (lon, lat, st)


def advect_f32(fld, lons, lats, t0: float, dt: float, n_steps: int, n_threads: int = 0):
    s, keep = _field_struct(fld)
    lon = np.array(lons, dtype=np.float32)
    lat = np.array(lats, dtype=np.float32)
    st = np.zeros(lon.size, np.uint8)
    bad = lib().orc_advect_f32(ctypes.byref(s), lon.size, _p(lon), _p(lat), _p(st), float(t0), float(dt),
                               int(n_steps), int(n_threads))
    if bad < 0:
        raise ValueError("time outside the field's time axis")
    return lon, lat, st


# ---------------- pairs and interaction ----------------

def pairs(lon, lat, r: float, p=2, n_threads: int = 0):
    lon = np.ascontiguousarray(lon, dtype=np.float32)
    lat = np.ascontiguousarray(lat, dtype=np.float32)
    m = lib().orc_pairs(lon.size, _p(lon), _p(lat), float(r), norm_code(p), int(n_threads), None, None, 0)
    if m < 0:
        raise MemoryError("oracle pair search failed")
    pi = np.empty(m, np.int32)
    pj = np.empty(m, np.int32)
    lib().orc_pairs(lon.size, _p(lon), _p(lat), float(r), norm_code(p), int(n_threads), _p(pi), _p(pj), m)
    return pi.astype(np.int64), pj.astype(np.int64)


def count_pairs(lon, lat, r: float, p=2, n_threads: int = 0) -> int:
    """Number of unordered pairs within r (the count of pairs(), without listing them)."""
    lon = np.ascontiguousarray(lon, dtype=np.float32)
    lat = np.ascontiguousarray(lat, dtype=np.float32)
    m = int(lib().orc_count_pairs(lon.size, _p(lon), _p(lat), float(r), norm_code(p), int(n_threads)))
    if m < 0:
        raise MemoryError("oracle pair count failed")
    return m


def priority_order(pi, pj, step: int, seed: int):
    """Pairs in the GPU's application order (descending 64-bit order hash of (seed, step, i, j))."""
    a = np.ascontiguousarray(pi, dtype=np.int32).copy()
    b = np.ascontiguousarray(pj, dtype=np.int32).copy()
    lib().orc_priority_order(a.size, _p(a), _p(b), int(step), seed & 0xFFFFFFFFFFFFFFFF)
    return a.astype(np.int64), b.astype(np.int64)


def pair_prio(i: int, j: int, step: int, seed: int) -> int:
    return lib().orc_pair_prio(i, j, step, seed & 0xFFFFFFFFFFFFFFFF)


def rps_replay(species, pi, pj, step: int, seed: int, pRS: float, pPR: float, pSP: float):
    """Sequential replay in the given order; returns the new species array."""
    sp = np.array(species, dtype=np.int8)
    a = np.ascontiguousarray(pi, dtype=np.int32)
    b = np.ascontiguousarray(pj, dtype=np.int32)
    lib().orc_rps_replay(_p(sp), a.size, _p(a), _p(b), int(step), seed & 0xFFFFFFFFFFFFFFFF, prob_threshold(pRS),
                         prob_threshold(pPR), prob_threshold(pSP))
    return sp


def interact_step(lon, lat, species, r, p, pRS, pPR, pSP, seed, step, n_threads: int = 0):
    """Pairs + priority-ordered replay: the species the GPU must produce."""
    lon = np.ascontiguousarray(lon, dtype=np.float32)
    lat = np.ascontiguousarray(lat, dtype=np.float32)
    sp = np.array(species, dtype=np.int8)
    m = lib().orc_interact_step(lon.size, _p(lon), _p(lat), _p(sp), float(r), norm_code(p), prob_threshold(pRS),
                                prob_threshold(pPR), prob_threshold(pSP), seed & 0xFFFFFFFFFFFFFFFF, int(step),
                                int(n_threads))
    if m < 0:
        raise MemoryError("oracle interaction failed")
    return sp, m


def run(fld, lon, lat, species, t0, dt, n_steps, step0, r, p, pRS, pPR, pSP, seed, n_threads: int = 0):
    """CPU fused steps (float32 advection + pairs + interaction), in place; returns total pairs."""
    s, keep = _field_struct(fld)
    st = np.zeros(lon.size, np.uint8)
    m = lib().orc_run(ctypes.byref(s), lon.size, _p(lon), _p(lat), _p(st), _p(species), float(t0), float(dt),
                      int(n_steps), int(step0), float(r), norm_code(p), prob_threshold(pRS), prob_threshold(pPR),
                      prob_threshold(pSP), seed & 0xFFFFFFFFFFFFFFFF, int(n_threads))
    if m < 0:
        raise RuntimeError("oracle run failed")
    return m


def great_circle_m(lon1, lat1, lon2, lat2, radius_km: float = 6371.228):
    """Haversine distance in metres (float64)."""
    p1, p2 = np.deg2rad(lat1), np.deg2rad(lat2)
    dphi = p2 - p1
    dl = np.deg2rad(np.asarray(lon2, np.float64) - np.asarray(lon1, np.float64))
    a = np.sin(dphi / 2) ** 2 + np.cos(p1) * np.cos(p2) * np.sin(dl / 2) ** 2
    return 2 * radius_km * 1e3 * np.arcsin(np.sqrt(np.minimum(a, 1.0)))


R_EARTH = 6371.228e3  # the reference's R64 / R32 (sandbox/pairwise_distance_histogram_distributed.jl:94)


def haversine(lat1, lon1, lat2, lon2, radius: float = R_EARTH) -> float:
    """haversine_distance32's formula in float64 (metres)."""
    return float(lib().orc_haversine(float(lat1), float(lon1), float(lat2), float(lon2), float(radius)))


def distance_histogram(lats, lons, bins: int, radius: float = R_EARTH, delta: float = 1e-4, n_threads: int = 0):
    """All-pairs histogram of round(10 log10(max(1, d))): (definite[bins + 1], ambiguous[bins + 1]).

    ambiguous[k] counts pairs within `delta` (in units of 10 log10 d) of the boundary between bins
    k and k + 1, which float32 arithmetic may put on either side; the last column is the overflow."""
    lats = np.ascontiguousarray(lats, dtype=np.float32)
    lons = np.ascontiguousarray(lons, dtype=np.float32)
    d = np.zeros(bins + 1, np.uint64)
    a = np.zeros(bins + 1, np.uint64)
    lib().orc_distance_histogram(lats.size, _p(lats), _p(lons), int(bins), float(radius), float(delta), int(n_threads),
                                 _p(d), _p(a))
    return d.astype(np.int64), a.astype(np.int64)


def histogram_consistent(counts, definite, ambiguous) -> bool:
    """True when counts[bins + 1] is definite plus each ambiguous pair on one side of its boundary:
    for every k, sum(counts[:k+1]) lies between sum(definite[:k+1]) + sum(ambiguous[:k]) and
    sum(definite[:k+1]) + sum(ambiguous[:k+1])."""
    c = np.cumsum(np.asarray(counts, np.int64))
    d = np.cumsum(np.asarray(definite, np.int64))
    a = np.cumsum(np.asarray(ambiguous, np.int64))
    a_before = np.concatenate([[0], a[:-1]])
    return bool(np.all(c >= d + a_before) and np.all(c <= d + a) and c[-1] == d[-1] + a[-1])
