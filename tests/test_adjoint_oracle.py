"""The FP64 checkers of the adjoint, pinned on the CPU.

adjoint_ref (FP64 torch restatement of the advection) must reproduce the FP64 C oracle's forward,
and its autograd gradient must agree with central finite differences of the C oracle's FP64
forward on an FP64 field. Only then is it a checker for the GPU adjoint (tests/test_gpu_adjoint.py).
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _case(lm, field, n=600, seed=3, box=(199.0, 202.0, 24.0, 27.0)):
    rng = np.random.default_rng(seed)
    lon = box[0] + (box[1] - box[0]) * rng.random(n)
    lat = box[2] + (box[3] - box[2]) * rng.random(n)
    tlon = lon + rng.normal(0, 0.2, n)
    tlat = lat + rng.normal(0, 0.2, n)
    return lon, lat, tlon, tlat


def _losses64(orc, field, u, v, lon, lat, tlon, tlat, t0, dt, n_steps):
    """Per-microbe squared distances of the FP64 forward and the cell-path signatures."""
    import adjoint_ref
    x, y, _, sig = orc.advect_f64_field64(u, v, field.lon, field.lat, field.times, lon, lat, t0, dt, n_steps,
                                          n_threads=4, cell_signature=True)
    d = adjoint_ref.haversine_m(torch.from_numpy(x), torch.from_numpy(y), torch.from_numpy(tlon),
                                torch.from_numpy(tlat)).numpy()
    return d * d, sig


def test_fp64_torch_forward_matches_c_oracle(lm, orc, small_field):
    import adjoint_ref
    f = small_field
    lon, lat, _, _ = _case(lm, f, n=2000)
    t0, dt, n_steps = float(f.times[0]), 3600.0, 24
    want_x, want_y, want_st = orc.advect_f64(f, lon, lat, t0, dt, n_steps)
    with torch.no_grad():
        x, y = adjoint_ref.advect(f.lon, f.lat, f.times, torch.from_numpy(f.u.astype(np.float64)),
                                  torch.from_numpy(f.v.astype(np.float64)), torch.from_numpy(lon),
                                  torch.from_numpy(lat), t0, dt, n_steps, checkpoint_every=8)
    np.testing.assert_allclose(x.numpy(), want_x, rtol=0, atol=1e-10)
    np.testing.assert_allclose(y.numpy(), want_y, rtol=0, atol=1e-10)
    # the float64-field forward of the finite differences is the same scheme
    x2, y2, st2 = orc.advect_f64_field64(f.u, f.v, f.lon, f.lat, f.times, lon, lat, t0, dt, n_steps)
    np.testing.assert_array_equal(x2, want_x)
    np.testing.assert_array_equal(st2, want_st)


def test_fp64_autograd_matches_central_differences(lm, orc, small_field):
    """dL/d(lon0, lat0, u, v) of the FP64 scheme vs central FD (h = 1e-6 deg, 1e-6 m/s) along random directions."""
    import adjoint_ref
    f = small_field
    lon, lat, tlon, tlat = _case(lm, f, n=400)
    t0, dt, n_steps = float(f.times[0]), 3600.0, 12
    u = f.u.astype(np.float64)
    v = f.v.astype(np.float64)
    rng = np.random.default_rng(11)
    h = 1e-6
    for _ in range(6):
        d = [rng.standard_normal(a.shape) for a in (lon, lat, u, v)]
        lp, sp = _losses64(orc, f, u + h * d[2], v + h * d[3], lon + h * d[0], lat + h * d[1], tlon, tlat, t0, dt,
                           n_steps)
        lm_, sm = _losses64(orc, f, u - h * d[2], v - h * d[3], lon - h * d[0], lat - h * d[1], tlon, tlat, t0, dt,
                            n_steps)
        keep = sp == sm  # both runs sampled the same cells: the difference quotient is smooth
        assert keep.sum() >= lon.size - 4
        fd = float((lp - lm_)[keep].sum()) / lon.size / (2 * h)
        tl = [torch.from_numpy(a.copy()).requires_grad_(True) for a in (lon, lat, u, v)]
        x, y = adjoint_ref.advect(f.lon, f.lat, f.times, tl[2], tl[3], tl[0], tl[1], t0, dt, n_steps,
                                  checkpoint_every=5)
        dist = adjoint_ref.haversine_m(x, y, torch.from_numpy(tlon), torch.from_numpy(tlat))
        loss = (torch.from_numpy(keep.astype(np.float64)) * dist * dist).sum() / lon.size
        loss.backward()
        ad = sum(float((t.grad.numpy() * dd).sum()) for t, dd in zip(tl, d))
        assert abs(fd - ad) <= 1e-6 * abs(ad) + 1e-9, (fd, ad)


def test_cell_signature_flags_edge_straddling_differences(lm, orc, small_field):
    """A difference quotient across a cell edge is flagged: same cells -> equal signatures, else not."""
    f = small_field
    dlon = float(f.lon[1] - f.lon[0])
    edge = float(f.lon[20])
    lon = np.array([edge - 1e-7, edge + 1e-7, edge + 0.3 * dlon])
    lat = np.full(3, 25.1)
    _, _, _, sig = orc.advect_f64_field64(f.u, f.v, f.lon, f.lat, f.times, lon, lat, float(f.times[0]), 60.0, 1,
                                          cell_signature=True)
    assert sig[0] != sig[1]
    _, _, _, sig2 = orc.advect_f64_field64(f.u, f.v, f.lon, f.lat, f.times, lon + 1e-9, lat, float(f.times[0]), 60.0,
                                           1, cell_signature=True)
    assert sig2[2] == sig[2]
