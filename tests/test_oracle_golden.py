"""Pins the CPU oracle (and the package's host helpers) to the reference's own outputs.

Golden fixtures come from running the reference's code (tests/golden/make_golden.py): its
lattice helpers, scipy's cKDTree.query_pairs as it calls it, its rock_paper_scissors_interaction
and its InteractionSimulator.time_step.
"""

import hashlib

import numpy as np
import pytest
from conftest import golden


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_philox_known_answers(orc):
    # Random123 known-answer vectors of Philox4x32-10
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in kat:
        assert list(orc.philox4x32_10(ctr, key)) == want


def test_oracle_diffusion_draws_are_uniform(orc):
    # the kick's two draws (lat, then lon) per microbe and step are U(-1, 1): range, mean 0,
    # variance 1/3, no correlation between them or between neighbouring microbes (5 standard errors)
    n = 20_000
    d = np.array([orc.diffusion_draw(p, 7, 99) for p in range(n)], dtype=np.float64)
    assert np.all(np.abs(d) <= 1.0)
    for u in (d[:, 0], d[:, 1]):
        assert abs(u.mean()) < 5 * np.sqrt(1 / 3 / n)
        assert abs(u.var() - 1 / 3) < 5 * np.sqrt(4 / 45 / n)
    assert abs(np.corrcoef(d[:, 0], d[:, 1])[0, 1]) < 5 / np.sqrt(n)
    assert abs(np.corrcoef(d[:-1, 0], d[1:, 0])[0, 1]) < 5 / np.sqrt(n)
    # another step draws afresh
    e = np.array([orc.diffusion_draw(p, 8, 99)[0] for p in range(n)], dtype=np.float64)
    assert abs(np.corrcoef(d[:, 0], e)[0, 1]) < 5 / np.sqrt(n)


def test_factorization_matches_reference(lm, orc):
    g = golden("lattice.npz")
    for n, (a, b) in zip(g["ns"], g["factorization"]):
        assert lm.most_symmetric_integer_factorization(int(n)) == (a, b)
        assert orc.lattice_shape(int(n)) == (a, b)


def test_lattice_matches_reference(orc):
    from lagrangian_microbes_gb300.particle_advecter import uniform_particle_locations
    g = golden("lattice.npz")
    for k in range(3):
        n, a, b, c, d = g[f"small{k}_args"]
        lons, lats = uniform_particle_locations(int(n), a, b, c, d)
        np.testing.assert_array_equal(lons, g[f"small{k}_lons"])
        np.testing.assert_array_equal(lats, g[f"small{k}_lats"])
        lo2, la2 = orc.lattice(int(n), a, b, c, d)
        np.testing.assert_array_equal(lo2, g[f"small{k}_lons"])
        np.testing.assert_array_equal(la2, g[f"small{k}_lats"])
    for (n, a, b, c, d), (dl, da) in zip(g["big_args"], g["big_digests"]):
        lons, lats = uniform_particle_locations(int(n), a, b, c, d)
        assert _digest(lons) == dl and _digest(lats) == da


def test_oracle_pairs_match_ckdtree_cases(orc):
    g = golden("kdtree_cases.npz")
    for k in range(int(g["n_cases"])):
        X, r, p = g[f"c{k}_X"], float(g[f"c{k}_r"]), float(g[f"c{k}_p"])
        pi, pj = orc.pairs(X[:, 0], X[:, 1], r, p)
        want = g[f"c{k}_pairs"]
        got = np.stack([pi, pj], -1) if pi.size else np.zeros((0, 2), np.int64)
        np.testing.assert_array_equal(got, want, err_msg=str(g[f"c{k}_name"]))


def test_oracle_pairs_match_ckdtree_lattices(orc):
    g = golden("kdtree_lattice.npz")
    for (n, a, b, c, d), count, dig in zip(g["configs"], g["counts"], g["digests"]):
        lons, lats = orc.lattice(int(n), a, b, c, d)
        pi, pj = orc.pairs(lons.astype(np.float32), lats.astype(np.float32), 0.01, 2)
        assert pi.size == count
        if count:
            packed = (pi.astype(np.uint64) << np.uint64(32)) | pj.astype(np.uint64)
            assert _digest(packed) == dig


def test_oracle_rps_rule_matches_reference(orc):
    g = golden("rps_rule.npz")
    pRS, pPR, pSP = g["params"]
    t = [orc.prob_threshold(pRS), orc.prob_threshold(pPR), orc.prob_threshold(pSP)]
    L = orc.lib()
    for s1, s2, u53, o1, o2, calls in g["rows"].astype(np.int64):
        sp = np.array([s1, s2], np.int8)
        L.orc_rps_apply(sp.ctypes.data, 0, 1, int(u53), *t)
        assert (sp[0], sp[1]) == (o1, o2), (s1, s2, u53)
        assert calls == (1 if s1 != s2 else 0)  # the reference draws only when species differ


def test_oracle_replay_matches_reference(orc):
    g = golden("rps_replay.npz")
    out = orc.rps_replay(g["species0"], g["pi"], g["pj"], int(g["step"]), int(g["seed"]), *g["params"])
    np.testing.assert_array_equal(out, g["species1"])


def test_oracle_matches_reference_interaction_simulator(orc):
    """The reference's InteractionSimulator, step by step, with its own set order and Philox uniforms."""
    g = golden("interaction_sim.npz")
    lon, lat, order = g["lon"], g["lat"], g["order"]
    sp = g["species0"].copy()
    r = float(g["radius"])
    for step in range(lon.shape[1]):
        rows = order[order[:, 0] == step]
        # same pair set as cKDTree at this step
        pi, pj = orc.pairs(lon[:, step], lat[:, step], r, 2)
        got = set(zip(pi.tolist(), pj.tolist()))
        assert got == set(zip(rows[:, 1].tolist(), rows[:, 2].tolist()))
        sp = orc.rps_replay(sp, rows[:, 1], rows[:, 2], step, int(g["seed"]), *g["params"])
        np.testing.assert_array_equal(sp, g["species"][:, step])


def test_priority_order_is_a_linear_extension(orc):
    """Replaying in priority order = replaying the order's rounds (pairs of a round are disjoint)."""
    g = golden("interaction_sim.npz")
    lon, lat = g["lon"][:, 0], g["lat"][:, 0]
    pi, pj = orc.pairs(lon, lat, float(g["radius"]), 2)
    a, b = orc.priority_order(pi, pj, 0, 99)
    # build rounds greedily from the priority order and check the replay is unchanged
    level = {}
    rnd = np.empty(a.size, np.int64)
    for k, (x, y) in enumerate(zip(a.tolist(), b.tolist())):
        rnd[k] = max(level.get(x, -1), level.get(y, -1)) + 1
        level[x] = level[y] = rnd[k]
    o = np.lexsort((b, a, rnd))
    sp0 = g["species0"]
    s1 = orc.rps_replay(sp0, a, b, 0, 99, 0.6, 0.7, 0.8)
    s2 = orc.rps_replay(sp0, a[o], b[o], 0, 99, 0.6, 0.7, 0.8)
    np.testing.assert_array_equal(s1, s2)


def test_advection_uniform_flow_known_answer(lm, orc):
    fld = lm.uniform_field(190, 215, 15, 40, 0.5, n_frames=4, u0=0.3, v0=0.0)
    lons = np.array([200.0, 201.5, 205.25])
    lats = np.array([25.0, 30.0, 35.5])
    lon, lat, st = orc.advect_f64(fld, lons, lats, 0.0, 3600.0, 3)
    u32 = float(np.float32(0.3))  # the field stores float32
    want = lons + u32 * 3 * 3600.0 / (111120.0 * np.cos(np.deg2rad(lats)))
    np.testing.assert_allclose(lon, want, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(lat, lats)
    assert not st.any()


def test_advection_time_linear_field_known_answer(lm, orc):
    # v = a + b t everywhere: RK4 integrates a linear-in-time field exactly
    fld = lm.uniform_field(190, 215, 15, 40, 0.5, n_frames=5, u0=0.0, v0=0.0)
    a, b = 0.1, 0.2 / (4 * 3600.0)
    fld.v[:] = (a + b * fld.times)[:, None, None].astype(np.float32)
    a32 = float(np.float32(a))
    lat0 = np.array([20.0, 30.0])
    lon, lat, st = orc.advect_f64(fld, np.array([200.0, 200.0]), lat0, 0.0, 3600.0, 4)
    vv = fld.v[:, 0, 0].astype(np.float64)
    # exact integral of the piecewise-linear interpolant over 4 frames (trapezoid per frame)
    disp = sum(0.5 * (vv[k] + vv[k + 1]) * 3600.0 for k in range(4)) / 111120.0
    np.testing.assert_allclose(lat, lat0 + disp, rtol=0, atol=1e-11)
    assert a32 > 0 and not st.any()


def test_advection_oob_flagged(lm, orc):
    fld = lm.uniform_field(200, 201, 25, 26, 0.1, n_frames=3, u0=5.0)
    lon, lat, st = orc.advect_f64(fld, np.array([200.99, 200.1]), np.array([25.5, 25.5]), 0.0, 3600.0, 2)
    assert st[0] == 1 and st[1] == 0


def test_oracle_f32_vs_f64_small_config(lm, orc, small_field):
    lons, lats = orc.lattice(10000, 25, 26, 200, 201)
    l64, a64, _ = orc.advect_f64(small_field, lons, lats, 0.0, 3600.0, 24)
    l32, a32, _ = orc.advect_f32(small_field, lons, lats, 0.0, 3600.0, 24)
    d = orc.great_circle_m(l64, a64, l32.astype(np.float64), a32.astype(np.float64))
    assert d.max() < 50.0  # absolute-float32 CPU loop (the Parcels-like baseline), informative bound


def test_synthetic_field_properties(lm):
    fld, modes = lm.synthetic_psi_field(190, 215, 15, 40, 1 / 12, n_frames=3, seed=5, with_modes=True)
    speed2 = fld.u[0].astype(np.float64) ** 2 + fld.v[0].astype(np.float64) ** 2
    assert abs(np.sqrt(speed2.mean()) - 0.2) < 1e-6
    # analytic re-evaluation agrees with the gridded frames
    j, i = 37, 101
    u, v = modes.velocity(fld.lon[i], fld.lat[j], fld.times[2])
    assert abs(u - fld.u[2, j, i]) < 1e-6 and abs(v - fld.v[2, j, i]) < 1e-6
    # 10-day phase period
    fld2 = lm.synthetic_psi_field(190, 215, 15, 40, 1.0, n_frames=2, frame_seconds=10 * 86400.0, seed=5)
    np.testing.assert_allclose(fld2.u[0], fld2.u[1], atol=1e-6)
