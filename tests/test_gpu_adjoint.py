"""GPU adjoint of the advection (lm_adjoint_*, k_adjoint.cu) against its FP64 checkers.

* the tape's forward in "f32" precision is bit-identical to the fused engine's advection (lm_step,
  no kick); the default "ds" precision carries positions in double-float;
* dL/d(lon0, lat0) and dL/d(u, v) agree with an FP64 torch autograd of the same scheme
  (oracle/adjoint_ref.py) and with FP64 central finite differences of the C oracle along random
  directions (h = 1e-6 deg for positions, 1e-6 m/s for the field);
* the gradient is deterministic: bit-identical across repeated backward sweeps and across
  checkpoint intervals (the recomputed segments are bit-identical to the forward);
* microbes that leave the domain are frozen and their gradient passes through unchanged.

The loss is the differentiation benchmark's: the mean squared great-circle distance between
final positions and seeded targets (initial positions plus N(0, 20 km) offsets).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

KM_PER_DEG = 111.32


def _case(field, n, seed, box=(199.0, 202.0, 24.0, 27.0)):
    rng = np.random.default_rng(seed)
    lon = (box[0] + (box[1] - box[0]) * rng.random(n)).astype(np.float32)
    lat = (box[2] + (box[3] - box[2]) * rng.random(n)).astype(np.float32)
    tlon = lon.astype(np.float64) + rng.normal(0, 20.0 / KM_PER_DEG, n)
    tlat = lat.astype(np.float64) + rng.normal(0, 20.0 / KM_PER_DEG, n)
    return lon, lat, tlon, tlat


def _gpu_grads(field, lon, lat, tlon, tlat, t0, dt, n_steps, k, allow_oob=False, weight=None, precision="f32"):
    from lagrangian_microbes_gb300.adjoint import AdjointTape, advect_rk4, great_circle_m
    dev = torch.device("cuda:0")
    l0 = torch.from_numpy(lon).to(dev).requires_grad_(True)
    a0 = torch.from_numpy(lat).to(dev).requires_grad_(True)
    u = torch.from_numpy(field.u).to(dev).requires_grad_(True)
    v = torch.from_numpy(field.v).to(dev).requires_grad_(True)
    tape = AdjointTape(precision=precision)
    x, y = advect_rk4(l0, a0, u, v, field.lon, field.lat, field.times, t0, dt, n_steps, checkpoint_every=k,
                      tape=tape, allow_out_of_bounds=allow_oob)
    dist = great_circle_m(x.double(), y.double(), torch.from_numpy(tlon).to(dev), torch.from_numpy(tlat).to(dev))
    w = torch.ones_like(dist) if weight is None else torch.from_numpy(np.asarray(weight, np.float64)).to(dev)
    loss = (w * dist * dist).sum() / dist.numel()  # the mean squared distance (over the weighted microbes)
    loss.backward()
    out = [t.grad.double().cpu().numpy() for t in (l0, a0, u, v)]
    sig = tape.cell_signature().cpu().numpy().view(np.uint64)
    res = (x.detach().cpu().numpy(), y.detach().cpu().numpy(), float(loss.detach()), out, sig)
    tape.close()
    tape.ctx.close()
    return res


def _fp64_grads(field, lon, lat, tlon, tlat, t0, dt, n_steps, weight=None):
    import adjoint_ref
    tl = [torch.from_numpy(np.asarray(a, np.float64).copy()).requires_grad_(True)
          for a in (lon, lat, field.u, field.v)]
    x, y = adjoint_ref.advect(field.lon, field.lat, field.times, tl[2], tl[3], tl[0], tl[1], t0, dt, n_steps,
                              checkpoint_every=16)
    dist = adjoint_ref.haversine_m(x, y, torch.from_numpy(tlon), torch.from_numpy(tlat))
    w = torch.ones_like(dist) if weight is None else torch.from_numpy(np.asarray(weight, np.float64))
    loss = (w * dist * dist).sum() / dist.numel()
    loss.backward()
    return float(loss.detach()), [t.grad.numpy() for t in tl]


def _fp64_signature(orc, f, lon, lat, t0, dt, n_steps):
    return orc.advect_f64_field64(f.u, f.v, f.lon, f.lat, f.times, np.asarray(lon, np.float64),
                                  np.asarray(lat, np.float64), t0, dt, n_steps, cell_signature=True)[3]


def central_difference(orc, f, lon, lat, tlon, tlat, t0, dt, n_steps, d, h=1e-6, path=None):
    """FP64 central difference of the loss along direction d = (d_lon0, d_lat0, d_u, d_v), over the
    microbes whose two runs sample the same grid cells at every stage (the others straddle an edge
    of the piecewise-bilinear field, where the derivative jumps) and, with `path`, the cells of the
    GPU run too. Returns (fd, keep mask)."""
    import adjoint_ref
    runs = []
    for s in (h, -h):
        x, y, _, sig = orc.advect_f64_field64(f.u.astype(np.float64) + s * d[2], f.v.astype(np.float64) + s * d[3],
                                              f.lon, f.lat, f.times, lon.astype(np.float64) + s * d[0],
                                              lat.astype(np.float64) + s * d[1], t0, dt, n_steps, cell_signature=True)
        dd = adjoint_ref.haversine_m(torch.from_numpy(x), torch.from_numpy(y), torch.from_numpy(tlon),
                                     torch.from_numpy(tlat)).numpy()
        runs.append((dd * dd, sig))
    keep = runs[0][1] == runs[1][1]
    if path is not None:
        keep &= runs[0][1] == path
    fd = float((runs[0][0] - runs[1][0])[keep].sum()) / lon.size / (2 * h)
    return fd, keep


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_adjoint_forward_bit_identical_to_engine_advection(lm, small_field):
    f = small_field
    lon, lat, _, _ = _case(f, 5000, 1)
    t0, dt, n_steps = float(f.times[0]), 3600.0, 40
    sim = lm.Simulation(f, lon.astype(np.float64), lat.astype(np.float64), np.ones(lon.size, np.int8), kh=0.0)
    sim.step(t0, dt, n_steps, interact=False)
    want_lon, want_lat, _, st = sim.state()
    sim.close()
    assert (st == 0).all()
    x, y, _, _, _ = _gpu_grads(f, lon, lat, lon.astype(np.float64), lat.astype(np.float64), t0, dt, n_steps, 7)
    np.testing.assert_array_equal(x, want_lon)
    np.testing.assert_array_equal(y, want_lat)


@pytest.mark.parametrize("precision", ["f32", "ds"])
def test_adjoint_matches_fp64_autograd_and_finite_differences(lm, orc, small_field, precision):
    """Gradients within 1e-4 relative of the FP64 scheme, microbe by microbe on the same cell path.

    The map is piecewise smooth: moving a start by 0.1 m moves the FP64 gradient itself by ~1e-4
    when a stage crosses a cell edge, and the float32 trajectory sits ~0.1-1 m from the FP64 one.
    The comparison therefore keeps the microbes whose GPU and FP64 runs sample the same cells (the
    GPU reports its path, lm_adjoint_cell_signature) and reports how many that is."""
    f = small_field
    lon, lat, tlon, tlat = _case(f, 3000, 2)
    t0, dt, n_steps = float(f.times[0]), 3600.0, 48
    _, _, loss32, g, sig = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 16, precision=precision)
    same = sig == _fp64_signature(orc, f, lon, lat, t0, dt, n_steps)
    assert same.mean() >= 0.97, same.mean()
    loss64, g64 = _fp64_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps)
    assert abs(loss32 - loss64) <= 1e-5 * loss64
    errs = [_rel(a, b) for a, b in zip(g, g64)]
    assert max(errs) < 1e-3, errs  # all microbes, cell-edge crossings included
    _, _, _, gs, _ = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 16, weight=same, precision=precision)
    _, g64s = _fp64_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, weight=same)
    errs = [_rel(a, b) for a, b in zip(gs, g64s)]
    assert max(errs) < 1e-4, errs
    # directional derivatives vs FP64 central differences of the C oracle on a float64 field
    # (error of the vector of 16 directional derivatives: a single direction whose derivative happens
    # to be near zero would inflate a per-direction ratio without any loss of accuracy)
    rng = np.random.default_rng(5)
    ads, fds, dropped = [], [], 0
    for _ in range(16):
        d = [rng.standard_normal(a.shape) for a in (lon, lat, f.u, f.v)]
        fd, keep = central_difference(orc, f, lon, lat, tlon, tlat, t0, dt, n_steps, d, path=sig)
        dropped = max(dropped, int((~keep).sum()))
        _, _, _, gk, _ = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 16, weight=keep, precision=precision)
        ads.append(sum(float((gg * dd).sum()) for gg, dd in zip(gk, d)))
        fds.append(fd)
    ads, fds = np.array(ads), np.array(fds)
    assert dropped <= lon.size * 3 // 100
    assert _rel(ads, fds) < 1e-4, (ads, fds)
    assert np.median(np.abs(ads - fds) / np.abs(fds)) < 1e-4


@pytest.mark.parametrize("precision", ["f32", "ds"])
def test_adjoint_gradient_is_deterministic_across_runs_and_checkpoint_intervals(lm, small_field, precision):
    f = small_field
    lon, lat, tlon, tlat = _case(f, 20000, 3)
    t0, dt, n_steps = float(f.times[0]), 3600.0, 30
    ref = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 30, precision=precision)
    for k in (30, 1, 7):
        got = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, k, precision=precision)
        np.testing.assert_array_equal(got[0], ref[0])
        for a, b in zip(got[3], ref[3]):
            np.testing.assert_array_equal(a, b)


def test_adjoint_repeated_backward_is_bit_identical(lm, small_field):
    from lagrangian_microbes_gb300.adjoint import AdjointTape
    f = small_field
    lon, lat, _, _ = _case(f, 10000, 4)
    dev = torch.device("cuda:0")
    tape = AdjointTape()
    tape.forward(torch.from_numpy(lon).to(dev), torch.from_numpy(lat).to(dev), torch.from_numpy(f.u).to(dev),
                 torch.from_numpy(f.v).to(dev), f.lon, f.lat, f.times, float(f.times[0]), 3600.0, 20, 8)
    g = torch.randn(2, lon.size, device=dev)
    first = [t.cpu().numpy() for t in tape.backward(g[0], g[1])]
    second = [t.cpu().numpy() for t in tape.backward(g[0], g[1])]
    for a, b in zip(first, second):
        np.testing.assert_array_equal(a, b)
    tape.close()


def test_adjoint_frozen_microbes_pass_their_gradient_through(lm, orc, small_field):
    f = small_field
    # a strip hugging the eastern edge: some microbes leave the grid and freeze
    lon, lat, tlon, tlat = _case(f, 2000, 6, box=(205.85, 206.0, 24.0, 27.0))
    t0, dt, n_steps = float(f.times[0]), 3600.0, 24
    _, _, st = orc.advect_f64(f, lon, lat, t0, dt, n_steps)
    assert 0 < int((st != 0).sum()) < lon.size  # some froze, some stayed
    sig64 = _fp64_signature(orc, f, lon, lat, t0, dt, n_steps)
    _, _, _, _, sig = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 8, allow_oob=True)
    same = sig == sig64
    assert same.mean() >= 0.97
    _, _, _, g, _ = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 8, allow_oob=True, weight=same)
    _, g64 = _fp64_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, weight=same)
    errs = [_rel(a, b) for a, b in zip(g, g64)]
    assert max(errs) < 1e-4, errs


def test_adjoint_time_window_outside_field_raises(lm, small_field):
    from lagrangian_microbes_gb300 import TimeRangeError
    from lagrangian_microbes_gb300.adjoint import AdjointTape
    f = small_field
    dev = torch.device("cuda:0")
    z = torch.zeros(4, device=dev) + 200.0
    tape = AdjointTape()
    with pytest.raises(TimeRangeError):
        tape.forward(z, z - 175.0, torch.from_numpy(f.u).to(dev), torch.from_numpy(f.v).to(dev), f.lon, f.lat, f.times,
                     float(f.times[-1]), 3600.0, 5)
    tape.close()


def test_adjoint_f64_trajectories_track_the_fp64_scheme(lm, orc, small_field):
    """FP64 mode: positions within 1e-9 deg of the FP64 oracle and gradients within 1e-5 of the FP64
    autograd on every microbe (no cell-path selection needed), deterministic across intervals."""
    f = small_field
    lon, lat, tlon, tlat = _case(f, 3000, 8)
    t0, dt, n_steps = float(f.times[0]), 3600.0, 48
    x, y, loss, g, sig = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 16, precision="f64")
    x64, y64, _, sig64 = orc.advect_f64_field64(f.u, f.v, f.lon, f.lat, f.times, lon.astype(np.float64),
                                                lat.astype(np.float64), t0, dt, n_steps, cell_signature=True)
    # final positions come back as float64 in this mode
    assert x.dtype == np.float64 and np.abs(x - x64).max() <= 1e-9 and np.abs(y - y64).max() <= 1e-9
    assert (sig == sig64).all()
    loss64, g64 = _fp64_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps)
    errs = [_rel(a, b) for a, b in zip(g, g64)]
    assert max(errs) < 1e-5, errs
    again = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 5, precision="f64")
    for a, b in zip(again[3], g):
        np.testing.assert_array_equal(a, b)


def test_adjoint_steps_longer_than_a_cell_fall_back_to_the_record_form(lm, orc):
    """Stages that leave the 3 x 3 cells around a step's start (a fine grid, fast flow) switch the
    backward to sorting the stage records themselves; the gradient still matches the FP64 scheme
    and is deterministic."""
    f = lm.synthetic_psi_field(199.0, 203.0, 24.0, 28.0, 0.02, n_frames=8, frame_seconds=3600.0, rms_speed=2.0,
                               seed=3)
    lon, lat, tlon, tlat = _case(f, 2000, 9, box=(200.5, 201.5, 25.5, 26.5))
    t0, dt, n_steps = float(f.times[0]), 3600.0, 6
    _, _, _, g, sig = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 4)
    same = sig == _fp64_signature(orc, f, lon, lat, t0, dt, n_steps)
    assert same.mean() >= 0.9
    _, _, _, gs, _ = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 4, weight=same)
    _, g64 = _fp64_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, weight=same)
    errs = [_rel(a, b) for a, b in zip(gs, g64)]
    assert max(errs) < 1e-4, errs
    again = _gpu_grads(f, lon, lat, tlon, tlat, t0, dt, n_steps, 3)
    for a, b in zip(again[3], g):
        np.testing.assert_array_equal(a, b)
