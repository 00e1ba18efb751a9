"""The adjoint at the differentiation configuration's horizon, against FP64 checkers.

Configuration: a 1000 x 1000 lattice over lon 200-205E, lat 25-30N (every 100th microbe: a
10,000-microbe subset), 720 RK4 steps of 1 h on the 1/12 deg hourly synthetic field, loss = mean
squared great-circle distance to seeded targets (initial positions plus N(0, 20 km) offsets),
checkpoints every 32 steps. The GPU gradients w.r.t. the initial positions and the gridded u, v are
compared with

* an FP64 torch autograd of the same scheme (oracle/adjoint_ref.py) over the microbes whose GPU and
  FP64 runs sample the same grid cells at every stage (the map is piecewise smooth: bilinear pieces
  meet at cell edges), and
* FP64 central finite differences of the C oracle along 64 random directions (normal for the
  positions, h = 1e-6 deg; +-1 m/s per node for u and v, h = 1e-6), over the microbes whose +h and
  -h runs and the GPU run sample the same cells.

"ds" is the tape's default precision (double-float positions, float32 velocities and adjoint
state): its directional derivatives are within 1e-4 of FP64 finite differences (the bar of the
differentiation configuration), and its gradient vectors within 1e-3 of the FP64 autograd (its
trajectories sit a few centimetres from the FP64 ones, and the float32 velocities and Jacobians
leave ~5e-4 per component). "f64" carries float64 state and meets 1e-4 on both. The scheme being
differentiated is the reference's pset.execute(AdvectionRK4) (particle_advecter.py:220-223).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N_FULL, STRIDE, STEPS, K = 1_000_000, 100, 720, 32
KM_PER_DEG = 111.32


@pytest.fixture(scope="module")
def config_d(lm, orc):
    from lagrangian_microbes_gb300.particle_advecter import uniform_particle_locations
    f = lm.synthetic_psi_field(190.0, 215.0, 15.0, 40.0, 1.0 / 12.0, n_frames=STEPS + 1, frame_seconds=3600.0,
                               seed=2024)
    lons, lats = uniform_particle_locations(N_FULL, 25.0, 30.0, 200.0, 205.0)
    rng = np.random.default_rng(7)
    tlon = lons + rng.normal(0, 20.0 / KM_PER_DEG, N_FULL) / np.cos(np.deg2rad(lats))
    tlat = lats + rng.normal(0, 20.0 / KM_PER_DEG, N_FULL)
    sel = slice(None, None, STRIDE)
    lon = lons[sel].astype(np.float32)
    lat = lats[sel].astype(np.float32)
    return f, lon, lat, tlon[sel].copy(), tlat[sel].copy()


@pytest.mark.parametrize("precision", ["ds", "f64"])
def test_config_d_gradients_match_fp64_autograd_and_finite_differences(orc, config_d, precision):
    import adjoint_ref
    from test_gpu_adjoint import _fp64_grads, _fp64_signature, _gpu_grads, _rel

    f, lon, lat, tlon, tlat = config_d
    t0, dt = 0.0, 3600.0
    _, _, _, _, sig = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, STEPS, K, precision=precision)
    same = sig == _fp64_signature(orc, f, lon, lat, t0, dt, STEPS)
    assert same.mean() >= 0.2, same.mean()

    # FP64 autograd of the same scheme, microbe by microbe on the same cell path
    _, _, _, gs, _ = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, STEPS, K, weight=same, precision=precision)
    _, g64 = _fp64_grads(f, lon, lat, tlon, tlat, t0, dt, STEPS, weight=same)
    errs = [_rel(a, b) for a, b in zip(gs, g64)]
    assert max(errs) < (1e-4 if precision == "f64" else 1e-3), errs

    # 64 directions of FP64 central differences (error of the vector of directional derivatives, and
    # the median per direction)
    u64, v64 = f.u.astype(np.float64), f.v.astype(np.float64)
    lon64, lat64 = lon.astype(np.float64), lat.astype(np.float64)
    rng = np.random.default_rng(11)
    h = 1e-6
    ads, fds, kept = [], [], []
    for _ in range(64):
        dl, da = rng.standard_normal(lon.size), rng.standard_normal(lon.size)
        du = (np.frombuffer(rng.bytes(u64.size), np.uint8).reshape(u64.shape) & 1).astype(np.int8) * 2 - 1
        dv = (np.frombuffer(rng.bytes(v64.size), np.uint8).reshape(v64.shape) & 1).astype(np.int8) * 2 - 1
        runs = []
        for s in (h, -h):
            x, y, _, sg = orc.advect_f64_field64(u64, v64, f.lon, f.lat, f.times, lon64 + s * dl, lat64 + s * da, t0,
                                                 dt, STEPS, cell_signature=True, du=du, dv=dv, s=s)
            dd = adjoint_ref.haversine_m(torch.from_numpy(x), torch.from_numpy(y), torch.from_numpy(tlon),
                                         torch.from_numpy(tlat)).numpy()
            runs.append((dd * dd, sg))
        keep = (runs[0][1] == runs[1][1]) & (runs[0][1] == sig)
        kept.append(keep.mean())
        fds.append(float((runs[0][0] - runs[1][0])[keep].sum()) / lon.size / (2 * h))
        _, _, _, gk, _ = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, STEPS, K, weight=keep, precision=precision)
        ads.append(float((gk[0] * dl).sum() + (gk[1] * da).sum() + (gk[2] * du).sum() + (gk[3] * dv).sum()))
    ads, fds = np.array(ads), np.array(fds)
    assert min(kept) >= 0.15, min(kept)
    assert _rel(ads, fds) < 1e-4, (ads, fds)
    assert np.median(np.abs(ads - fds) / np.abs(fds)) < 1e-4
