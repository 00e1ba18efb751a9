"""Device-resident fused engine: advect -> bin -> pair -> interact per step on one GPU.

``Simulation`` owns one liblmgb300 context holding the velocity field, the particle state and the
species in HBM. Steps run either as plain per-step launches (``step``) or as a captured CUDA
graph of several steps replayed from the host (``capture`` + ``run_graph``). Nothing here
computes on the CPU: every numeric operation is a kernel of liblmgb300.
"""

from __future__ import annotations

import ctypes
import math
from datetime import datetime, timedelta

import numpy as np

from . import _lib
from ._lib import (NORM_INF, NORM_L1, NORM_L2, STEP_ADVECT, STEP_CENSUS, STEP_COUNT_PAIRS, STEP_INTERACT,
                   STEP_LOG_PAIRS)
from .fields import VelocityField


def norm_code(p) -> int:
    """cKDTree's Minkowski p -> liblmgb300 norm code (only 1, 2 and infinity are supported)."""
    if p == 2:
        return NORM_L2
    if p == 1:
        return NORM_L1
    if p is not None and math.isinf(float(p)) and float(p) > 0:
        return NORM_INF
    raise ValueError(f"interaction_norm must be 1, 2 or inf; got {p!r}")


class Simulation:
    """Fused per-step pipeline over one ensemble of microbes.

    Parameters mirror the reference's call surface: ``radius`` and ``norm`` are the
    ``interaction_radius`` / ``interaction_norm`` of InteractionSimulator (degrees, Minkowski p),
    ``p_rs``, ``p_pr``, ``p_sp`` the forward probabilities of rock_paper_scissors, ``kh`` the
    diffusivity in deg^2/s (the reference converts m^2/s with Kh / 1e10). ``seed`` keys the Philox
    draws (pair uniforms, pair order and diffusion kicks).
    """

    def __init__(self, field: VelocityField, lons, lats, species=None, radius: float = 0.01, norm=2,
                 p_rs: float = 0.5, p_pr: float = 0.5, p_sp: float = 0.5, seed: int = 0, kh: float = 0.0,
                 device: int = 0, ctx: _lib.Context | None = None):
        self.ctx = ctx or _lib.Context(device)
        self.field = field
        self.kh = float(kh)
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.radius = float(radius)
        self.norm = norm
        self.upload_field(field)
        self.upload_particles(lons, lats, species)
        self.set_interaction(radius, norm, p_rs, p_pr, p_sp, seed)
        self.step_index = 0
        self._graph = None

    # ---- uploads ----
    def upload_field(self, fld: VelocityField) -> None:
        nt, ny, nx = fld.u.shape
        self.ctx.call("lm_field_upload", _lib.ptr(fld.u), _lib.ptr(fld.v), nt, ny, nx, _lib.ptr(fld.lon),
                      _lib.ptr(fld.lat), _lib.ptr(fld.times))
        self.field = fld
        self._graph = None  # a captured graph holds the previous field: capture again

    def upload_particles(self, lons, lats, species=None) -> None:
        lons = np.ascontiguousarray(lons, dtype=np.float64).ravel()
        lats = np.ascontiguousarray(lats, dtype=np.float64).ravel()
        if lons.shape != lats.shape:
            raise ValueError("lons and lats must have the same size")
        sp = None if species is None else np.ascontiguousarray(species, dtype=np.int8).ravel()
        if sp is not None and sp.size != lons.size:
            raise ValueError("species must have one entry per particle")
        self.ctx.call("lm_particles_upload", lons.size, _lib.ptr(lons), _lib.ptr(lats), _lib.ptr(sp))
        self.n = lons.size

    def set_interaction(self, radius, norm, p_rs, p_pr, p_sp, seed) -> None:
        self.ctx.call("lm_set_interaction", float(radius), norm_code(norm), float(p_rs), float(p_pr), float(p_sp),
                      int(seed) & 0xFFFFFFFFFFFFFFFF)

    def set_species(self, species) -> None:
        sp = np.ascontiguousarray(species, dtype=np.int8).ravel()
        self.ctx.call("lm_species_upload", sp.size, _lib.ptr(sp))

    def set_cell_factor(self, factor: float) -> None:
        """Binning cell size in units of the radius (>= 1.004; the pair set does not change)."""
        self.ctx.call("lm_set_cell_factor", float(factor))

    # ---- state snapshots, checkpoints, autotuning ----
    def snapshot(self) -> None:
        """Keep a device copy of the state (positions, species, status, step counter)."""
        self.ctx.call("lm_snapshot_save")

    def restore(self) -> None:
        """Return to the last snapshot, bit for bit."""
        self.ctx.call("lm_snapshot_restore")
        self.step_index = int(self.ctx.stats()["step"])

    def export_state(self) -> dict:
        """Exact state for a checkpoint file: float32 offsets from the field origin, species, status, step."""
        n = self.n
        xo = np.empty(n, np.float32)
        yo = np.empty(n, np.float32)
        sp = np.empty(n, np.int8)
        st = np.empty(n, np.uint8)
        step = ctypes.c_int64(0)
        self.ctx.call("lm_state_export", _lib.ptr(xo), _lib.ptr(yo), _lib.ptr(sp), _lib.ptr(st), ctypes.byref(step))
        return {"xo": xo, "yo": yo, "species": sp, "status": st, "step": int(step.value)}

    def import_state(self, state: dict) -> None:
        """Resume from export_state() (same field and particle layout)."""
        arr = lambda k, dt: np.ascontiguousarray(state[k], dtype=dt)
        self.ctx.call("lm_state_import", _lib.ptr(arr("xo", np.float32)), _lib.ptr(arr("yo", np.float32)),
                      _lib.ptr(arr("species", np.int8)), _lib.ptr(arr("status", np.uint8)), int(state["step"]))
        self.step_index = int(state["step"])

    def _time_from_snapshot(self, t0, dt, n_steps, s0, count_pairs, reps):
        """Seconds of n_steps from the snapshot (best of reps, device work included), after one
        untimed step that sizes the buffers for the current settings."""
        import time as _time
        self.restore()
        self.step(t0, dt, 1, step0=s0, count_pairs=count_pairs)
        self.sync()
        best = float("inf")
        for _ in range(reps):
            self.restore()
            t = _time.perf_counter()
            self.step(t0, dt, n_steps, step0=s0, count_pairs=count_pairs)
            self.sync()
            best = min(best, _time.perf_counter() - t)
        return best

    @staticmethod
    def _pick(times: dict, margin: float):
        """The first candidate (the incumbent) unless another is faster by more than margin."""
        keys = list(times)
        best = keys[0]
        for k in keys[1:]:
            if times[k] < times[best] * (1.0 - margin):
                best = k
        return best

    def autotune(self, t0, dt, n_steps: int = 3, factors=(1.004, 1.25, 1.5, 2.0), count_pairs: bool = False,
                 reps: int = 2, margin: float = 0.03):
        """Pick the binning cell size (in units of the radius) that runs n_steps fastest from the
        current state, then return to that state. The first factor is kept unless another is faster
        by more than `margin` (timings of a few steps differ by a few per cent from run to run). The
        pair sets, and so all results, are the same for every cell size; only the speed changes.
        Capture graphs after tuning. Returns (best factor, {factor: seconds})."""
        s0 = self.step_index
        self.snapshot()
        times = {}
        for f in factors:
            self.set_cell_factor(f)
            times[f] = self._time_from_snapshot(t0, dt, n_steps, s0, count_pairs, reps)
        best = self._pick(times, margin)
        self.set_cell_factor(best)
        self.restore()
        self._graph = None
        return best, times

    TUNING_KNOBS = {"rounds_threads": (_lib.TUNE_ROUNDS_THREADS, (1024, 512)),
                    "long_blocks_per_sm": (_lib.TUNE_LONG_BLOCKS_PER_SM, (6, 3, 12)),
                    "advect_threads": (_lib.TUNE_ADVECT_THREADS, (256, 128))}

    def set_tuning(self, knob: str, value: int) -> None:
        """Set a launch-shape knob (TUNING_KNOBS); results never depend on it, only the speed."""
        self.ctx.call("lm_set_tuning", self.TUNING_KNOBS[knob][0], int(value))
        self._graph = None

    def tuning(self) -> dict:
        out = {}
        for name, (code, _) in self.TUNING_KNOBS.items():
            v = ctypes.c_int(0)
            self.ctx.call("lm_get_tuning", code, ctypes.byref(v))
            out[name] = v.value
        return out

    def autotune_all(self, t0, dt, n_steps: int = 3, factors=(1.004, 1.25, 1.5, 2.0), count_pairs: bool = False,
                     reps: int = 2, margin: float = 0.03):
        """The binning cell size (autotune), then each launch-shape knob in turn (block size of the
        interaction and advection kernels, long-list blocks per SM), each value timed over n_steps
        from the current state (best of reps); a knob keeps its first value unless another is faster
        by more than `margin`. The state is returned to where it started. Returns the chosen settings
        with the seconds of every candidate. Tune from a state like the one the run spends its time
        in: the long-list and interaction knobs matter once the flow has clustered the microbes."""
        best_f, ftimes = self.autotune(t0, dt, n_steps, factors, count_pairs, reps, margin)
        s0 = self.step_index
        self.snapshot()
        chosen = {"cell_factor": best_f}
        seconds = {"cell_factor": {str(k): v for k, v in ftimes.items()}}
        for name, (_, values) in self.TUNING_KNOBS.items():
            times = {}
            for v in values:
                self.set_tuning(name, v)
                times[v] = self._time_from_snapshot(t0, dt, n_steps, s0, count_pairs, reps)
            best = self._pick(times, margin)
            self.set_tuning(name, best)
            chosen[name] = best
            seconds[name] = {str(k): v for k, v in times.items()}
        self.restore()
        self._graph = None
        chosen["seconds"] = seconds
        return chosen

    def set_stream(self, stream_handle: int) -> None:
        """Run on an external CUDA stream (e.g. torch.cuda.current_stream().cuda_stream)."""
        self.ctx.call("lm_ctx_set_stream", int(stream_handle))

    # ---- time ----
    def _t(self, t) -> float:
        return self.field.seconds(t)

    @staticmethod
    def _dt(dt) -> float:
        return dt.total_seconds() if isinstance(dt, timedelta) else float(dt)

    # ---- stepping ----
    def step(self, t0, dt, n_steps: int, interact: bool = True, census: bool = False, log_pairs: bool = False,
             record: bool = False, step0: int | None = None, count_pairs: bool = False, out: dict | None = None):
        """Run n_steps plain steps from field time t0. Returns a dict of the requested records.

        ``count_pairs`` replaces the interaction by a count of the pairs within the radius (no lists):
        the count of the last step is ``stats()["pairs"]``, their sum ``stats()["pairs_total"]``.
        ``out`` (with ``record``) supplies the record arrays: {"lon", "lat", "species"} of at least
        [n_steps, N] (float32, float32, int8; C order). Reusing them from call to call saves the
        page faults of fresh host memory, which cost ~10x the copies themselves."""
        n = self.n
        interact = interact and not count_pairs
        flags = STEP_ADVECT | (STEP_INTERACT if interact else 0) | (STEP_CENSUS if census else 0)
        flags |= STEP_COUNT_PAIRS if count_pairs else 0
        flags |= STEP_LOG_PAIRS if log_pairs else 0
        rec_lon = rec_lat = rec_sp = rec_c = None
        if record and out is not None:
            rec_lon, rec_lat, rec_sp = (_record_view(out, k, dt_, n_steps, n) for k, dt_ in
                                        (("lon", np.float32), ("lat", np.float32), ("species", np.int8)))
        elif record:
            rec_lon = np.empty((n_steps, n), np.float32)
            rec_lat = np.empty((n_steps, n), np.float32)
            rec_sp = np.empty((n_steps, n), np.int8)
        if census:
            rec_c = np.empty((n_steps, 4), np.int64)
        s0 = self.step_index if step0 is None else int(step0)
        self.ctx.call("lm_step", self._t(t0), self._dt(dt), int(n_steps), s0, flags, self.kh, _lib.ptr(rec_lon),
                      _lib.ptr(rec_lat), _lib.ptr(rec_sp), _lib.ptr(rec_c))
        self.step_index = s0 + n_steps
        out = {}
        if record:
            out.update(lon=rec_lon, lat=rec_lat, species=rec_sp)
        if census:
            out["census"] = rec_c
        return out

    def record_buffers(self, n_steps: int) -> dict:
        """Record arrays for ``step(..., record=True, out=...)`` in page-locked host memory:
        {"lon", "lat"} float32 and {"species"} int8 of [n_steps, N]. Copies into them run on the
        context's copy stream while the next steps compute; reuse them from call to call."""
        shape = (int(n_steps), self.n)
        return {"lon": _lib.host_empty(shape, np.float32), "lat": _lib.host_empty(shape, np.float32),
                "species": _lib.host_empty(shape, np.int8)}

    def capture(self, t_start, dt, steps_per_graph: int, interact: bool = True, census: bool = False,
                step0: int | None = None, count_pairs: bool = False) -> None:
        """Capture steps_per_graph fused steps as one CUDA graph (time origin t_start at step0)."""
        s0 = self.step_index if step0 is None else int(step0)
        interact = interact and not count_pairs
        flags = STEP_ADVECT | (STEP_INTERACT if interact else 0) | (STEP_CENSUS if census else 0)
        flags |= STEP_COUNT_PAIRS if count_pairs else 0
        self.ctx.call("lm_graph_capture", self._t(t_start), self._dt(dt), s0, int(steps_per_graph), flags, self.kh)
        self.step_index = s0
        self._graph = int(steps_per_graph)

    def run_graph(self, n_launches: int, sync: bool = True) -> None:
        if not self._graph:
            raise RuntimeError("capture() a graph first")
        self.ctx.call("lm_graph_run", int(n_launches), 1 if sync else 0)
        self.step_index += n_launches * self._graph

    def sync(self) -> None:
        self.ctx.call("lm_sync")

    def set_step(self, step: int) -> None:
        self.ctx.call("lm_set_step", int(step))
        self.step_index = int(step)

    # ---- downloads ----
    def state(self):
        """(lon float32[N], lat float32[N], species int8[N], status uint8[N]) of the current state."""
        n = self.n
        lon = np.empty(n, np.float32)
        lat = np.empty(n, np.float32)
        sp = np.empty(n, np.int8)
        st = np.empty(n, np.uint8)
        self.ctx.call("lm_particles_download", _lib.ptr(lon), _lib.ptr(lat), _lib.ptr(sp), _lib.ptr(st))
        return lon, lat, sp, st

    def species(self) -> np.ndarray:
        sp = np.empty(self.n, np.int8)
        self.ctx.call("lm_particles_download", None, None, _lib.ptr(sp), None)
        return sp

    def applied_pairs(self):
        """(i, j, round) of the pairs applied by the last logged step, in application order."""
        return get_pair_log(self.ctx)

    def stats(self) -> dict:
        return self.ctx.stats()

    def census(self) -> np.ndarray:
        """[n_ensembles, 4] species counts after the last step run with census=True."""
        n_ens = max(1, int(self.ctx.stats()["n_ensembles"]))
        out = np.zeros((n_ens, 4), np.int64)
        self.ctx.call("lm_census_get", _lib.ptr(out), out.size)
        return out

    def close(self) -> None:
        self.ctx.close()


def _record_view(out: dict, key: str, dtype, n_steps: int, n: int) -> np.ndarray:
    """The first n_steps rows of a caller-supplied record array, checked."""
    a = out[key]
    if a.dtype != dtype or a.ndim != 2 or a.shape[0] < n_steps or a.shape[1] != n or not a.flags["C_CONTIGUOUS"]:
        raise ValueError(f"out[{key!r}] must be a C-contiguous {np.dtype(dtype).name} array of at least [{n_steps}, {n}]")
    return a[:n_steps]


class EnsembleSimulation(Simulation):
    """Many independent ensembles in one context: every step is one launch sequence for all of them.

    ``fields`` is one VelocityField shared by all ensembles or one per ensemble (same grid);
    ``ensembles`` a list of (lons, lats, species); ``p_rs``/``p_pr``/``p_sp``/``seeds`` scalars or
    one value per ensemble. Microbes of different ensembles never pair, and each ensemble draws
    from its own Philox stream, so every ensemble evolves exactly as it would alone.
    """

    def __init__(self, fields, ensembles, radius: float = 0.01, norm=2, p_rs=0.5, p_pr=0.5, p_sp=0.5, seeds=0,
                 kh: float = 0.0, device: int = 0, ctx: _lib.Context | None = None):
        self.ctx = ctx or _lib.Context(device)
        self.kh = float(kh)
        self.radius = float(radius)
        self.norm = norm
        flds = fields if isinstance(fields, (list, tuple)) else [fields]
        self.field = flds[0]
        self.upload_fields(flds)
        self.upload_ensembles(ensembles)
        e = self.n_ensembles
        as_arr = lambda v, dt: np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=dt), (e,)))
        seeds_u = np.array([int(x) & 0xFFFFFFFFFFFFFFFF for x in np.broadcast_to(np.asarray(seeds, dtype=object), (e,))],
                           dtype=np.uint64)
        self.ctx.call("lm_set_interaction", float(radius), norm_code(norm), 0.5, 0.5, 0.5, 0)
        self.ctx.call("lm_set_ensemble_params", e, _lib.ptr(as_arr(p_rs, np.float64)), _lib.ptr(as_arr(p_pr, np.float64)),
                      _lib.ptr(as_arr(p_sp, np.float64)), _lib.ptr(seeds_u))
        self.step_index = 0
        self._graph = None

    def upload_ensembles(self, ensembles) -> None:
        """(Re)place the microbes of every ensemble: a list of (lons, lats, species)."""
        e = len(ensembles)
        self.counts = np.array([np.asarray(x[0]).size for x in ensembles], dtype=np.int64)
        lons = np.concatenate([np.asarray(x[0], np.float64).ravel() for x in ensembles]) if e else np.zeros(0)
        lats = np.concatenate([np.asarray(x[1], np.float64).ravel() for x in ensembles]) if e else np.zeros(0)
        sp = np.concatenate([np.asarray(x[2], np.int8).ravel() for x in ensembles]) if e else np.zeros(0, np.int8)
        self.ctx.call("lm_ensembles_upload", e, _lib.ptr(self.counts), _lib.ptr(lons), _lib.ptr(lats),
                      _lib.ptr(sp))
        self.n = int(self.counts.sum())
        self.n_ensembles = e

    def upload_fields(self, flds) -> None:
        f0 = flds[0]
        nt, ny, nx = f0.u.shape
        for f in flds[1:]:
            if f.u.shape != f0.u.shape or not (np.array_equal(f.lon, f0.lon) and np.array_equal(f.lat, f0.lat)
                                               and np.array_equal(f.times, f0.times)):
                raise ValueError("ensemble fields must share one grid and time axis")
        u = np.ascontiguousarray(np.stack([f.u for f in flds])) if len(flds) > 1 else f0.u
        v = np.ascontiguousarray(np.stack([f.v for f in flds])) if len(flds) > 1 else f0.v
        self.ctx.call("lm_field_upload_batch", len(flds), _lib.ptr(u), _lib.ptr(v), nt, ny, nx, _lib.ptr(f0.lon),
                      _lib.ptr(f0.lat), _lib.ptr(f0.times))
        self.field = f0
        self._graph = None  # a captured graph holds the previous fields: capture again

    def split(self, flat):
        """Split a per-microbe array (last axis) into a list per ensemble."""
        edges = np.cumsum(self.counts)[:-1]
        return np.split(np.asarray(flat), edges, axis=-1)


def get_pair_log(ctx: _lib.Context):
    n = ctypes.c_int64(0)
    ctx.call("lm_pairs_get", None, None, None, 0, ctypes.byref(n))
    m = n.value
    i = np.empty(m, np.int32)
    j = np.empty(m, np.int32)
    r = np.empty(m, np.int32)
    if m:
        ctx.call("lm_pairs_get", _lib.ptr(i), _lib.ptr(j), _lib.ptr(r), m, ctypes.byref(n))
    return i, j, r


class PairQuery:
    """GPU fixed-radius pair search with cKDTree.query_pairs semantics (interaction_simulator.py:93-98)."""

    def __init__(self, radius: float, norm=2, device: int = 0, ctx: _lib.Context | None = None):
        self.ctx = ctx or _lib.Context(device)
        self.ctx.call("lm_set_interaction", float(radius), norm_code(norm), 0.5, 0.5, 0.5, 0)

    def pairs(self, lon, lat):
        """Unordered pairs (i < j) as two int64 arrays sorted by (i, j)."""
        lon = np.ascontiguousarray(lon, dtype=np.float32).ravel()
        lat = np.ascontiguousarray(lat, dtype=np.float32).ravel()
        n = ctypes.c_int64(0)
        cap = max(16 * lon.size, 1024)
        while True:
            pi = np.empty(cap, np.int32)
            pj = np.empty(cap, np.int32)
            rc = self.ctx._lib.lm_query_pairs(self.ctx.handle, lon.size, _lib.ptr(lon), _lib.ptr(lat), _lib.ptr(pi),
                                              _lib.ptr(pj), cap, ctypes.byref(n))
            if rc == _lib.LM_ERR_CAPACITY and n.value > cap:
                cap = n.value
                continue
            self.ctx.check(rc)
            break
        m = n.value
        return pi[:m].astype(np.int64), pj[:m].astype(np.int64)

    def count(self, lon, lat) -> int:
        """Number of pairs, without listing them (cKDTree.query_pairs' size)."""
        lon = np.ascontiguousarray(lon, dtype=np.float32).ravel()
        lat = np.ascontiguousarray(lat, dtype=np.float32).ravel()
        n = ctypes.c_int64(0)
        self.ctx.call("lm_count_pairs", lon.size, _lib.ptr(lon), _lib.ptr(lat), ctypes.byref(n))
        return int(n.value)
