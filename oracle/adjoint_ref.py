"""FP64 torch restatement of the advection for the adjoint's checks -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/ and bench.py as the checker of the GPU adjoint (lm_adjoint_*); the
product package never imports it.

The scheme is the FP64 RK4 of lm_oracle.c (orc_advect_f64 / orc_advect_f64d): the reference's
pset.execute(parcels.AdvectionRK4, runtime=dt, dt=dt) on a spherical RectilinearZGrid with linear
interpolation (particle_advecter.py:177-187, 220-223), bilinear in (lon, lat), linear in time,
u / (1852*60*cos(lat)) and v / (1852*60). Written in torch float64 so that torch autograd gives
the FP64 gradient of a loss on final positions with respect to the initial positions and the
gridded u, v. Microbes whose stage leaves the grid are frozen from that step on, as in the
oracle and the GPU forward. Segments of `checkpoint_every` steps go through
torch.utils.checkpoint to bound memory on long runs.

The reference does not differentiate; nothing here has a reference counterpart beyond the
forward scheme.
"""

from __future__ import annotations

import math

import torch
from torch.utils.checkpoint import checkpoint

M_PER_DEG = 1852.0 * 60.0
EARTH_RADIUS_M = 6371.228e3


def bracket(t: float, t0: float, dT: float, nt: int):
    """Frame bracket of time t (the oracle's bracket()); raises outside the time axis."""
    fk = (t - t0) / dT
    if not (fk >= -1e-9 and fk <= (nt - 1) + 1e-9):
        raise ValueError(f"time {t} outside the field's time axis")
    k = int(min(max(math.floor(fk), 0.0), float(nt - 2)))
    w = min(max(fk - k, 0.0), 1.0)
    if w >= 1.0:
        k, w = k + 1, 0.0
    return k, w


class Grid:
    def __init__(self, lon_axis, lat_axis, t_axis):
        self.nx, self.ny, self.nt = len(lon_axis), len(lat_axis), len(t_axis)
        self.lon0 = float(lon_axis[0])
        self.dlon = float((lon_axis[-1] - lon_axis[0]) / (self.nx - 1))
        self.lat0 = float(lat_axis[0])
        self.dlat = float((lat_axis[-1] - lat_axis[0]) / (self.ny - 1))
        self.t0 = float(t_axis[0])
        self.dT = float((t_axis[-1] - t_axis[0]) / (self.nt - 1))


class _Gather(torch.autograd.Function):
    """F.flat[q] for a field F [nt][ny][nx]. Its backward adds the incoming gradient at the sampled
    nodes straight into `sink` (the field's gradient buffer, allocated once per run by advect()),
    the definition of a gather's adjoint, and returns no tensor for F: torch would otherwise build
    a dense field-sized gradient for every lookup, and a 720-step run makes ~10^4 of them."""

    @staticmethod
    def forward(ctx, F, q, sink):
        ctx.save_for_backward(q)
        ctx.sink = sink
        return F.reshape(-1)[q]

    @staticmethod
    def backward(ctx, g):
        (q,) = ctx.saved_tensors
        ctx.sink.view(-1).index_add_(0, q, g)
        return None, None, None


def _node(F, q):
    sink = getattr(F, "_grad_sink", None)
    if sink is None or not torch.is_grad_enabled():
        return F.detach().reshape(-1)[q] if sink is not None else F.reshape(-1)[q]
    return _Gather.apply(F, q, sink)


def _bilinear(F, q, nx, a, b):
    """Bilinear interpolation in the cell whose south-west node has flat index q."""
    return ((1 - a) * (1 - b) * _node(F, q) + a * (1 - b) * _node(F, q + 1) + (1 - a) * b * _node(F, q + nx)
            + a * b * _node(F, q + nx + 1))


def velocity(g: Grid, u, v, k: int, w: float, x, y):
    """(dlon/dt, dlat/dt, inside) in deg/s at absolute positions x, y (float64 tensors)."""
    fx = (x - g.lon0) / g.dlon
    fy = (y - g.lat0) / g.dlat
    inside = (fx >= 0) & (fx <= g.nx - 1) & (fy >= 0) & (fy <= g.ny - 1)
    fxc = fx.clamp(0, g.nx - 1)
    fyc = fy.clamp(0, g.ny - 1)
    i = fxc.detach().floor().long().clamp(max=g.nx - 2)
    j = fyc.detach().floor().long().clamp(max=g.ny - 2)
    a = fxc - i
    b = fyc - j
    q = (k * g.ny + j) * g.nx + i
    U = _bilinear(u, q, g.nx, a, b)
    V = _bilinear(v, q, g.nx, a, b)
    if w != 0.0:
        q1 = q + g.ny * g.nx
        U = (1 - w) * U + w * _bilinear(u, q1, g.nx, a, b)
        V = (1 - w) * V + w * _bilinear(v, q1, g.nx, a, b)
    dlon = U / (M_PER_DEG * torch.cos(y * (math.pi / 180.0)))
    dlat = V / M_PER_DEG
    return dlon, dlat, inside


def rk4_steps(g: Grid, u, v, x, y, active, t_start: float, dt: float, m0: int, m1: int):
    """Steps [m0, m1) from (x, y); `active` (bool) marks microbes that still move."""
    for m in range(m0, m1):
        t = t_start + dt * m
        k0, w0 = bracket(t, g.t0, g.dT, g.nt)
        k1, w1 = bracket(t + 0.5 * dt, g.t0, g.dT, g.nt)
        k2, w2 = bracket(t + dt, g.t0, g.dT, g.nt)
        a1x, a1y, in1 = velocity(g, u, v, k0, w0, x, y)
        a2x, a2y, in2 = velocity(g, u, v, k1, w1, x + 0.5 * dt * a1x, y + 0.5 * dt * a1y)
        a3x, a3y, in3 = velocity(g, u, v, k1, w1, x + 0.5 * dt * a2x, y + 0.5 * dt * a2y)
        a4x, a4y, in4 = velocity(g, u, v, k2, w2, x + dt * a3x, y + dt * a3y)
        ok = active & in1 & in2 & in3 & in4
        nx = x + (a1x + 2 * a2x + 2 * a3x + a4x) * dt / 6.0
        ny = y + (a1y + 2 * a2y + 2 * a3y + a4y) * dt / 6.0
        x = torch.where(ok, nx, x)
        y = torch.where(ok, ny, y)
        active = ok
    return x, y, active


def advect(lon_axis, lat_axis, t_axis, u, v, lon0, lat0, t_start: float, dt: float, n_steps: int,
           checkpoint_every: int = 32):
    """Differentiable FP64 forward: final (lon, lat) of microbes starting at (lon0, lat0)."""
    g = Grid(lon_axis, lat_axis, t_axis)
    for F in (u, v):
        # the field gradient accumulates in F.grad through _Gather (see there); leaves only
        if F.requires_grad:
            if F.grad is None:
                F.grad = torch.zeros_like(F)
            F._grad_sink = F.grad
    x, y = lon0, lat0
    active = torch.isfinite(x) & torch.isfinite(y)
    for m0 in range(0, n_steps, checkpoint_every):
        m1 = min(m0 + checkpoint_every, n_steps)

        def seg(x_, y_, act_, u_, v_, m0=m0, m1=m1):
            return rk4_steps(g, u_, v_, x_, y_, act_, t_start, dt, m0, m1)

        if torch.is_grad_enabled() and n_steps > checkpoint_every:
            x, y, active = checkpoint(seg, x, y, active, u, v, use_reentrant=False)
        else:
            x, y, active = seg(x, y, active, u, v)
    return x, y


def haversine_m(lon1, lat1, lon2, lat2):
    """Great-circle distance (m) on a sphere of radius 6371.228 km, float64 torch."""
    p1 = lat1 * (math.pi / 180.0)
    p2 = lat2 * (math.pi / 180.0)
    dl = (lon2 - lon1) * (math.pi / 180.0)
    h = torch.sin((p2 - p1) / 2) ** 2 + torch.cos(p1) * torch.cos(p2) * torch.sin(dl / 2) ** 2
    return 2 * EARTH_RADIUS_M * torch.asin(torch.sqrt(h.clamp(max=1.0)))


def loss_msd(lon, lat, tlon, tlat):
    """Mean squared great-circle distance (m^2) between final and target positions."""
    return (haversine_m(lon, lat, tlon, tlat) ** 2).mean()
