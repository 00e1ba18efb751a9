"""Differentiable RK4 advection: the adjoint tape of liblmgb300 behind torch.autograd.Function.

``advect_rk4(lon0, lat0, u, v, lon_axis, lat_axis, t_axis, t0, dt, n_steps)`` returns the final
positions of microbes advected from (lon0, lat0) through the gridded velocity (u, v), with the
scheme of the fused engine's advection (the reference's Parcels AdvectionRK4 on a spherical
RectilinearZGrid, particle_advecter.py:177-187, 220-223; no diffusion kick), positions carried in
double-float by default (``precision``, see AdjointTape). Its backward gives
dL/d(lon0, lat0) and dL/d(u, v) for any torch loss on the final positions, computed by the
hand-written adjoint kernels (k_adjoint.cu) from checkpoints every ``checkpoint_every`` steps; the
velocity gradient is a deterministic segmented reduction, bit-identical from run to run.

The reference has no differentiation; this module has no reference counterpart. Tensors live on
a CUDA device as float32 (positions: absolute degrees; u, v: m/s, [nt][ny][nx]); the kernels run
on torch's current stream. There is no CPU path: without the CUDA library every call raises.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib

EARTH_RADIUS_M = 6371.228e3


PRECISIONS = {"f32": 0, "f64": 1, "ds": 2}


class AdjointTape:
    """One lm_adjoint tape: the recorded forward run and its backward sweep.

    ``precision="ds"`` (the default) carries every position as a double-float pair of float32
    words, with float32 velocities, Jacobians and adjoint state: over long chaotic runs the
    trajectory does not accumulate float32 position rounding (which the flow amplifies), at
    close to float32 cost. ``"f32"`` keeps float32 state with the engine's arithmetic (final
    positions bit-identical to the fused engine's advection); ``"f64"`` carries float64 state and
    arithmetic over the float32 field. In "ds" and "f64" modes the final positions come back as
    float64 tensors (rounded once from the working state).
    """

    def __init__(self, ctx: _lib.Context | None = None, device: int = 0, precision: str = "ds"):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}; got {precision!r}")
        self.ctx = ctx or _lib.Context(device)
        self._lib = self.ctx._lib
        h = ctypes.c_void_p()
        self.ctx.check(self._lib.lm_adjoint_create(self.ctx.handle, ctypes.byref(h)))
        self._h = h
        self.precision = precision
        self.ctx.check(self._lib.lm_adjoint_set_precision(self._h, PRECISIONS[precision]))
        self.n = 0
        self.field_shape = None

    def _stream(self, dev) -> None:
        self.ctx.call("lm_ctx_set_stream", torch.cuda.current_stream(dev).cuda_stream)

    def forward(self, lon0, lat0, u, v, lon_axis, lat_axis, t_axis, t0: float, dt: float, n_steps: int,
                checkpoint_every: int = 32, allow_out_of_bounds: bool = False):
        """Run and record; returns (lon, lat) float32 device tensors."""
        for name, t in (("lon0", lon0), ("lat0", lat0), ("u", u), ("v", v)):
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
                raise ValueError(f"{name} must be a contiguous float32 CUDA tensor")
        if lon0.shape != lat0.shape or lon0.dim() != 1:
            raise ValueError("lon0 and lat0 must be 1-D of equal length")
        if u.shape != v.shape or u.dim() != 3:
            raise ValueError("u and v must be [nt][ny][nx] of equal shape")
        nt, ny, nx = u.shape
        ax = [np.ascontiguousarray(a, dtype=np.float64) for a in (lon_axis, lat_axis, t_axis)]
        if (ax[0].size, ax[1].size, ax[2].size) != (nx, ny, nt):
            raise ValueError("axes do not match the field shape")
        n = lon0.numel()
        lon = torch.empty_like(lon0)
        lat = torch.empty_like(lat0)
        self._stream(lon0.device)
        rc = self._lib.lm_adjoint_forward(self._h, u.data_ptr(), v.data_ptr(), nt, ny, nx, _lib.ptr(ax[0]),
                                          _lib.ptr(ax[1]), _lib.ptr(ax[2]), n, lon0.data_ptr(), lat0.data_ptr(),
                                          float(t0), float(dt), int(n_steps), int(checkpoint_every),
                                          lon.data_ptr(), lat.data_ptr())
        if not (rc == _lib.LM_ERR_OUT_OF_BOUNDS and allow_out_of_bounds):
            self.ctx.check(rc)
        self.n = n
        self.field_shape = (nt, ny, nx)
        if self.precision in ("f64", "ds"):  # hand back the working state, rounded once to float64
            lon = torch.empty(n, dtype=torch.float64, device=lon0.device)
            lat = torch.empty_like(lon)
            self.ctx.check(self._lib.lm_adjoint_final_positions(self._h, lon.data_ptr(), lat.data_ptr()))
        return lon, lat

    def backward(self, g_lon, g_lat):
        """dL/d(final lon, lat) -> (dL/dlon0, dL/dlat0, dL/du, dL/dv)."""
        g_lon = g_lon.to(torch.float32).contiguous()
        g_lat = g_lat.to(torch.float32).contiguous()
        dev = g_lon.device
        g_lon0 = torch.empty(self.n, dtype=torch.float32, device=dev)
        g_lat0 = torch.empty_like(g_lon0)
        g_u = torch.empty(self.field_shape, dtype=torch.float32, device=dev)
        g_v = torch.empty_like(g_u)
        self._stream(dev)
        self.ctx.check(self._lib.lm_adjoint_backward(self._h, g_lon.data_ptr(), g_lat.data_ptr(), g_lon0.data_ptr(),
                                                     g_lat0.data_ptr(), g_u.data_ptr(), g_v.data_ptr()))
        return g_lon0, g_lat0, g_u, g_v

    def cell_signature(self):
        """uint64 cell-path signature per microbe of the recorded run (as an int64 CUDA tensor)."""
        sig = torch.empty(self.n, dtype=torch.int64, device=torch.device("cuda", self.ctx.device))
        self._stream(sig.device)
        self.ctx.check(self._lib.lm_adjoint_cell_signature(self._h, sig.data_ptr()))
        return sig

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self._lib.lm_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _AdvectRK4(torch.autograd.Function):
    @staticmethod
    def forward(ctx, lon0, lat0, u, v, tape, axes, t0, dt, n_steps, checkpoint_every, allow_oob):
        lon, lat = tape.forward(lon0.detach().contiguous(), lat0.detach().contiguous(), u.detach().contiguous(),
                                v.detach().contiguous(), *axes, t0, dt, n_steps, checkpoint_every, allow_oob)
        ctx.tape = tape
        return lon, lat

    @staticmethod
    def backward(ctx, g_lon, g_lat):
        if g_lon is None:
            g_lon = torch.zeros(ctx.tape.n, dtype=torch.float32, device=g_lat.device)
        if g_lat is None:
            g_lat = torch.zeros(ctx.tape.n, dtype=torch.float32, device=g_lon.device)
        g_lon0, g_lat0, g_u, g_v = ctx.tape.backward(g_lon, g_lat)
        return g_lon0, g_lat0, g_u, g_v, None, None, None, None, None, None, None


def advect_rk4(lon0, lat0, u, v, lon_axis, lat_axis, t_axis, t0: float, dt: float, n_steps: int,
               checkpoint_every: int = 32, tape: AdjointTape | None = None, allow_out_of_bounds: bool = False,
               precision: str = "ds"):
    """Differentiable RK4 advection (float32 CUDA tensors in and out); see the module docstring."""
    tape = tape or AdjointTape(device=lon0.device.index or 0, precision=precision)
    return _AdvectRK4.apply(lon0, lat0, u, v, tape, (lon_axis, lat_axis, t_axis), float(t0), float(dt),
                            int(n_steps), int(checkpoint_every), bool(allow_out_of_bounds))


def great_circle_m(lon1, lat1, lon2, lat2):
    """Haversine distance (m) on a sphere of radius 6371.228 km (torch, any float dtype)."""
    r = math.pi / 180.0
    p1, p2 = lat1 * r, lat2 * r
    h = torch.sin((p2 - p1) / 2) ** 2 + torch.cos(p1) * torch.cos(p2) * torch.sin((lon2 - lon1) * r / 2) ** 2
    return 2 * EARTH_RADIUS_M * torch.asin(torch.sqrt(h.clamp(max=1.0)))


def mean_squared_distance(lon, lat, target_lon, target_lat):
    """Loss of the differentiation benchmark: mean squared great-circle distance (m^2), float64."""
    d = great_circle_m(lon.double(), lat.double(), target_lon.double(), target_lat.double())
    return (d * d).mean()
