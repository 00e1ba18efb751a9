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
from ._lib import NORM_INF, NORM_L1, NORM_L2, STEP_ADVECT, STEP_CENSUS, STEP_INTERACT, STEP_LOG_PAIRS
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
             record: bool = False, step0: int | None = None):
        """Run n_steps plain steps from field time t0. Returns a dict of the requested records."""
        n = self.n
        flags = STEP_ADVECT | (STEP_INTERACT if interact else 0) | (STEP_CENSUS if census else 0)
        flags |= STEP_LOG_PAIRS if log_pairs else 0
        rec_lon = rec_lat = rec_sp = rec_c = None
        if record:
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

    def capture(self, t_start, dt, steps_per_graph: int, interact: bool = True, census: bool = False,
                step0: int | None = None) -> None:
        """Capture steps_per_graph fused steps as one CUDA graph (time origin t_start at step0)."""
        s0 = self.step_index if step0 is None else int(step0)
        flags = STEP_ADVECT | (STEP_INTERACT if interact else 0) | (STEP_CENSUS if census else 0)
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

    def close(self) -> None:
        self.ctx.close()


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
