"""CUDA path (through the C-ABI) against the oracle and the reference's golden outputs."""

import hashlib

import numpy as np
import pytest
from conftest import golden

pytestmark = pytest.mark.gpu


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def engine():
    from lagrangian_microbes_gb300 import engine as eng
    return eng


# ---------------- pairs (K2 + K3) ----------------

def test_gpu_pairs_match_ckdtree_cases(engine):
    g = golden("kdtree_cases.npz")
    for k in range(int(g["n_cases"])):
        X, r, p = g[f"c{k}_X"], float(g[f"c{k}_r"]), float(g[f"c{k}_p"])
        q = engine.PairQuery(r, p)
        pi, pj = q.pairs(X[:, 0], X[:, 1])
        q.ctx.close()
        got = np.stack([pi, pj], -1) if pi.size else np.zeros((0, 2), np.int64)
        np.testing.assert_array_equal(got, g[f"c{k}_pairs"], err_msg=str(g[f"c{k}_name"]))


def test_gpu_pairs_match_ckdtree_full_size_lattices(engine, orc):
    """The 10k / 490k / 1M lattices at r = 0.01: counts and digests of cKDTree's pair sets."""
    g = golden("kdtree_lattice.npz")
    q = engine.PairQuery(0.01, 2)
    for (n, a, b, c, d), count, dig in zip(g["configs"], g["counts"], g["digests"]):
        lons, lats = orc.lattice(int(n), a, b, c, d)
        pi, pj = q.pairs(lons.astype(np.float32), lats.astype(np.float32))
        assert pi.size == count
        if count:
            packed = (pi.astype(np.uint64) << np.uint64(32)) | pj.astype(np.uint64)
            assert _digest(packed) == dig


@pytest.mark.parametrize("p", [2, 1, np.inf])
def test_gpu_pairs_match_oracle_random(engine, orc, p):
    rng = np.random.default_rng(5)
    for n, box, r in [(20000, 0.5, 0.01), (5000, 0.05, 0.01), (3000, 3.0, 0.2)]:
        lon = (200 + rng.random(n) * box).astype(np.float32)
        lat = (25 + rng.random(n) * box).astype(np.float32)
        q = engine.PairQuery(r, p)
        gi, gj = q.pairs(lon, lat)
        q.ctx.close()
        oi, oj = orc.pairs(lon, lat, r, p)
        np.testing.assert_array_equal(gi, oi)
        np.testing.assert_array_equal(gj, oj)


def test_gpu_pairs_empty_and_nonfinite(engine):
    q = engine.PairQuery(0.01, 2)
    pi, pj = q.pairs(np.zeros(0, np.float32), np.zeros(0, np.float32))
    assert pi.size == 0
    lon = np.array([200.0, 200.001, np.nan, 200.002], np.float32)
    lat = np.array([25.0, 25.0, 25.0, np.inf], np.float32)
    pi, pj = q.pairs(lon, lat)
    assert list(zip(pi, pj)) == [(0, 1)]


def test_gpu_dense_cluster_regrows_neighbour_lists(engine, orc):
    # ~1500 neighbours per particle: far above the initial 16 per particle capacity
    rng = np.random.default_rng(9)
    n = 3000
    lon = (200 + rng.normal(0, 0.004, n)).astype(np.float32)
    lat = (25 + rng.normal(0, 0.004, n)).astype(np.float32)
    q = engine.PairQuery(0.01, 2)
    gi, gj = q.pairs(lon, lat)
    oi, oj = orc.pairs(lon, lat, 0.01, 2)
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gj, oj)
    assert q.ctx.stats()["regrows"] >= 1


# ---------------- interaction (K4 + K5) ----------------

def _interact(engine, lon, lat, species, r, p, probs, seed, step, log=True):
    from lagrangian_microbes_gb300 import _lib
    ctx = _lib.Context(0)
    ctx.call("lm_set_interaction", float(r), engine.norm_code(p), *map(float, probs), seed)
    sp = np.ascontiguousarray(species, np.int8)
    ctx.call("lm_species_upload", sp.size, _lib.ptr(sp))
    lon = np.ascontiguousarray(lon, np.float32)
    lat = np.ascontiguousarray(lat, np.float32)
    ctx.call("lm_interact", lon.size, _lib.ptr(lon), _lib.ptr(lat), step, _lib.STEP_LOG_PAIRS if log else 0)
    out = np.empty_like(sp)
    ctx.call("lm_particles_download", None, None, _lib.ptr(out), None)
    log_ = engine.get_pair_log(ctx) if log else None
    stats = ctx.stats()
    ctx.close()
    return out, log_, stats


def test_gpu_interaction_matches_oracle_and_reference_rule(engine, orc):
    g = golden("interaction_sim.npz")
    probs = g["params"]
    seed = int(g["seed"])
    sp = g["species0"].copy()
    for step in range(g["lon"].shape[1]):
        lon, lat = g["lon"][:, step], g["lat"][:, step]
        got, (li, lj, lr), stats = _interact(engine, lon, lat, sp, 0.02, 2, probs, seed, step)
        # 1. the oracle's priority-ordered replay gives the same species
        want, m = orc.interact_step(lon, lat, sp, 0.02, 2, *probs, seed, step)
        np.testing.assert_array_equal(got, want)
        # 2. the applied pairs are exactly cKDTree's set, each once
        assert li.size == m == stats["pairs"]
        oi, oj = orc.pairs(lon, lat, 0.02, 2)
        assert set(zip(li.tolist(), lj.tolist())) == set(zip(oi.tolist(), oj.tolist()))
        # 3. every round is a matching (no microbe in two pairs of one round)
        for r in np.unique(lr):
            ends = np.concatenate([li[lr == r], lj[lr == r]])
            assert np.unique(ends).size == ends.size
        # 4. replaying the GPU's own application order with the reference's rule reproduces it
        np.testing.assert_array_equal(orc.rps_replay(sp, li, lj, step, seed, *probs), got)
        sp = got


def test_gpu_interaction_large_random(engine, orc):
    rng = np.random.default_rng(21)
    n = 200000
    lon = (200 + rng.random(n) * 2.0).astype(np.float32)
    lat = (25 + rng.random(n) * 2.0).astype(np.float32)
    sp = rng.integers(1, 4, n).astype(np.int8)
    probs = (0.6, 0.7, 0.55)
    got, _, stats = _interact(engine, lon, lat, sp, 0.01, 2, probs, 1234, 7, log=False)
    want, m = orc.interact_step(lon, lat, sp, 0.01, 2, *probs, 1234, 7)
    assert stats["pairs"] == m
    np.testing.assert_array_equal(got, want)


def test_gpu_interaction_dense_lists_match_oracle(engine, orc):
    # blob A (sigma 0.004 deg): ~2,000-3,000 neighbours per microbe, lists ordered in global memory;
    # blob B (sigma 0.02 deg): 10 to ~375 neighbours, lists bucket-sorted in shared memory with
    # several entries per bucket. The species depend on every list's order.
    rng = np.random.default_rng(31)
    lon = np.concatenate([200.0 + rng.normal(0, 0.004, 3000), 200.5 + rng.normal(0, 0.02, 3000)]).astype(np.float32)
    lat = np.concatenate([25.0 + rng.normal(0, 0.004, 3000), 25.5 + rng.normal(0, 0.02, 3000)]).astype(np.float32)
    sp = rng.integers(1, 4, lon.size).astype(np.int8)
    probs = (0.6, 0.7, 0.55)
    got, _, stats = _interact(engine, lon, lat, sp, 0.01, 2, probs, 77, 3, log=False)
    want, m = orc.interact_step(lon, lat, sp, 0.01, 2, *probs, 77, 3)
    assert stats["pairs"] == m > 3_000_000
    np.testing.assert_array_equal(got, want)


def test_gpu_interaction_other_species_values_unchanged(engine, orc):
    rng = np.random.default_rng(3)
    n = 2000
    lon = (200 + rng.random(n) * 0.1).astype(np.float32)
    lat = (25 + rng.random(n) * 0.1).astype(np.float32)
    sp = rng.integers(0, 5, n).astype(np.int8)  # 0 and 4 are outside the rule's table
    got, _, _ = _interact(engine, lon, lat, sp, 0.01, 2, (0.5, 0.5, 0.5), 5, 0, log=False)
    want, _ = orc.interact_step(lon, lat, sp, 0.01, 2, 0.5, 0.5, 0.5, 5, 0)
    np.testing.assert_array_equal(got, want)


# ---------------- advection (K1) ----------------

def test_gpu_advection_uniform_flow(engine, lm, orc):
    fld = lm.uniform_field(190, 215, 15, 40, 0.5, n_frames=6, u0=0.3, v0=-0.1)
    lons = np.array([200.0, 201.5, 205.25, 210.0])
    lats = np.array([25.0, 30.0, 35.5, 20.0])
    sim = engine.Simulation(fld, lons, lats, None, radius=0.0)
    sim.step(0.0, 3600.0, 5, interact=False)
    lon, lat, _, st = sim.state()
    l64, a64, _ = orc.advect_f64(fld, lons, lats, 0.0, 3600.0, 5)
    d = orc.great_circle_m(l64, a64, lon.astype(np.float64), lat.astype(np.float64))
    assert d.max() < 1.0 and not st.any()
    sim.close()


def test_gpu_advection_within_10m_of_fp64_after_24h(engine, lm, orc, small_field):
    """Configuration S: 10k lattice, 0.25 deg 6-hourly psi field, dt = 1 h, 24 h (and 48 h)."""
    lons, lats = orc.lattice(10000, 25, 26, 200, 201)
    sim = engine.Simulation(small_field, lons, lats, None, radius=0.0)
    rec = sim.step(0.0, 3600.0, 48, interact=False, record=True)
    _, _, _, rl, ra = orc.advect_f64(small_field, lons, lats, 0.0, 3600.0, 48, record=True)
    d24 = orc.great_circle_m(rl[23], ra[23], rec["lon"][23].astype(np.float64), rec["lat"][23].astype(np.float64))
    d48 = orc.great_circle_m(rl[47], ra[47], rec["lon"][47].astype(np.float64), rec["lat"][47].astype(np.float64))
    assert d24.max() <= 10.0, d24.max()
    assert d48.max() <= 20.0, d48.max()
    sim.close()


def test_gpu_advection_1_12_degree_hourly_24h(engine, lm, orc):
    """490k configuration's field (1/12 deg, hourly) on a 40k sub-lattice: <= 10 m after 24 h."""
    fld = lm.synthetic_psi_field(190, 215, 15, 40, 1 / 12, n_frames=26, seed=2)
    lons, lats = orc.lattice(40000, 25, 30, 200, 205)
    sim = engine.Simulation(fld, lons, lats, None, radius=0.0)
    sim.step(0.0, 3600.0, 24, interact=False)
    lon, lat, _, st = sim.state()
    l64, a64, st64 = orc.advect_f64(fld, lons, lats, 0.0, 3600.0, 24)
    d = orc.great_circle_m(l64, a64, lon.astype(np.float64), lat.astype(np.float64))
    assert d.max() <= 10.0, d.max()
    np.testing.assert_array_equal(st, st64)
    sim.close()


def test_gpu_advection_out_of_domain_is_flagged(engine, lm):
    from lagrangian_microbes_gb300 import OutOfBoundsError
    fld = lm.uniform_field(200, 201, 25, 26, 0.1, n_frames=4, u0=5.0)
    sim = engine.Simulation(fld, np.array([200.99, 200.1]), np.array([25.5, 25.5]), None, radius=0.0)
    with pytest.raises(OutOfBoundsError):
        sim.step(0.0, 3600.0, 2, interact=False)
    _, _, _, st = sim.state()
    assert st[0] == 1 and st[1] == 0
    sim.close()


def test_gpu_diffusion_kick_matches_philox(engine, lm, orc):
    fld = lm.uniform_field(190, 215, 15, 40, 0.5, n_frames=4, u0=0.0, v0=0.0)
    lons = np.linspace(200, 205, 64)
    lats = np.linspace(25, 30, 64)
    kh = 100 / 1e10  # the reference's Kh = 100 m^2/s in deg^2/s
    sim = engine.Simulation(fld, lons, lats, None, radius=0.0, kh=kh, seed=77)
    sim.step(0.0, 3600.0, 1, interact=False, step0=3)
    lon, lat, _, _ = sim.state()
    amp = np.float32(np.sqrt(6 * 3600.0 * kh))
    for p in range(64):
        ulat, ulon = orc.diffusion_draw(p, 3, 77)
        assert abs(float(lat[p]) - (lats[p] + ulat * float(amp))) < 2e-5
        assert abs(float(lon[p]) - (lons[p] + ulon * float(amp))) < 3e-5
    sim.close()


def test_gpu_diffusion_kick_statistics(engine, lm):
    # particle_advecter.py:239-244: lat += U(-1, 1) * sqrt(6 |dt| Kh), then lon likewise. Over many
    # microbes in a still field the kick has mean 0, variance amp^2 / 3, |kick| <= amp, and the two
    # draws are uncorrelated (bounds: 5 standard errors).
    fld = lm.uniform_field(190, 215, 15, 40, 0.5, n_frames=4, u0=0.0, v0=0.0)
    n = 200_000
    rng = np.random.default_rng(5)
    lons = 200 + 5 * rng.random(n)
    lats = 25 + 5 * rng.random(n)
    kh = 100 / 1e10
    sim = engine.Simulation(fld, lons, lats, None, radius=0.0, kh=kh, seed=1234)
    sim.step(0.0, 3600.0, 1, interact=False)
    lon, lat, _, _ = sim.state()
    amp = float(np.sqrt(6 * 3600.0 * kh))
    for dx in (lat.astype(np.float64) - lats.astype(np.float32).astype(np.float64),
               lon.astype(np.float64) - lons.astype(np.float32).astype(np.float64)):
        u = dx / amp
        assert np.abs(u).max() <= 1.0 + 1e-3  # float32 rounding of the moved position
        assert abs(u.mean()) < 5 * np.sqrt(1 / 3 / n)
        # var(U^2) of U(-1, 1) is 4/45; the standard error of the variance estimate is sqrt(4/45/n)
        assert abs(u.var() - 1 / 3) < 5 * np.sqrt(4 / 45 / n)
    ulat = (lat.astype(np.float64) - lats.astype(np.float32)) / amp
    ulon = (lon.astype(np.float64) - lons.astype(np.float32)) / amp
    assert abs(np.corrcoef(ulat, ulon)[0, 1]) < 5 / np.sqrt(n)
    sim.close()


# ---------------- fused steps and graphs ----------------

def _fused_setup(lm, orc, n=40000, seed=3):
    fld = lm.synthetic_psi_field(190, 215, 15, 40, 1 / 12, n_frames=30, seed=seed)
    lons, lats = orc.lattice(n, 25, 27, 200, 202)
    rng = np.random.default_rng(seed)
    sp = rng.integers(1, 4, n).astype(np.int8)
    return fld, lons, lats, sp


def test_gpu_fused_steps_match_oracle_every_step(engine, lm, orc):
    fld, lons, lats, sp0 = _fused_setup(lm, orc)
    probs = (0.7, 0.7, 0.7)
    sim = engine.Simulation(fld, lons, lats, sp0, radius=0.01, p_rs=probs[0], p_pr=probs[1], p_sp=probs[2], seed=42)
    rec = sim.step(0.0, 3600.0, 12, record=True, census=True)
    sp = sp0.copy()
    for s in range(12):
        sp, m = orc.interact_step(rec["lon"][s], rec["lat"][s], sp, 0.01, 2, *probs, 42, s)
        np.testing.assert_array_equal(rec["species"][s], sp, err_msg=f"step {s}")
        cnt = np.bincount(sp, minlength=4)
        np.testing.assert_array_equal(rec["census"][s], cnt[:4])
    sim.close()


def test_gpu_graph_equals_plain(engine, lm, orc):
    fld, lons, lats, sp0 = _fused_setup(lm, orc, n=30000, seed=4)
    a = engine.Simulation(fld, lons, lats, sp0, radius=0.01, p_rs=0.6, p_pr=0.7, p_sp=0.8, seed=9)
    a.step(0.0, 3600.0, 16)
    b = engine.Simulation(fld, lons, lats, sp0, radius=0.01, p_rs=0.6, p_pr=0.7, p_sp=0.8, seed=9)
    b.capture(0.0, 3600.0, steps_per_graph=4)
    b.run_graph(4)
    la, aa, sa, _ = a.state()
    lb, ab, sb, _ = b.state()
    np.testing.assert_array_equal(la, lb)
    np.testing.assert_array_equal(aa, ab)
    np.testing.assert_array_equal(sa, sb)
    assert b.stats()["step"] == 16
    a.close()
    b.close()


def test_gpu_graph_recovers_from_neighbour_overflow(engine, lm, orc):
    # a dense blob: the first captured step overflows the initial neighbour capacity
    fld = lm.uniform_field(190, 215, 15, 40, 0.5, n_frames=10, u0=0.05, v0=0.02)
    rng = np.random.default_rng(8)
    n = 4000
    lons = 200 + rng.normal(0, 0.004, n)
    lats = 25 + rng.normal(0, 0.004, n)
    sp0 = rng.integers(1, 4, n).astype(np.int8)
    a = engine.Simulation(fld, lons, lats, sp0, radius=0.01, seed=1)
    a.capture(0.0, 3600.0, steps_per_graph=2)
    a.run_graph(3)
    b = engine.Simulation(fld, lons, lats, sp0, radius=0.01, seed=1)
    rec = b.step(0.0, 3600.0, 6, record=True)
    _, _, sa, _ = a.state()
    np.testing.assert_array_equal(sa, rec["species"][-1])
    assert a.stats()["regrows"] >= 1
    a.close()
    b.close()


def test_gpu_490k_lattice_first_step_pairs(engine, lm, orc):
    """Full-size property: one fused step at 490k; pair count equals the oracle's on the same positions."""
    fld = lm.synthetic_psi_field(190, 215, 15, 40, 1 / 12, n_frames=4, seed=0)
    lons, lats = orc.lattice(490000, 25, 30, 200, 205)
    sp0 = np.random.default_rng(0).integers(1, 4, lons.size).astype(np.int8)
    sim = engine.Simulation(fld, lons, lats, sp0, radius=0.01, p_rs=0.7, p_pr=0.7, p_sp=0.7, seed=11)
    rec = sim.step(0.0, 3600.0, 1, record=True)
    want, m = orc.interact_step(rec["lon"][0], rec["lat"][0], sp0, 0.01, 2, 0.7, 0.7, 0.7, 11, 0)
    assert sim.stats()["pairs"] == m
    np.testing.assert_array_equal(rec["species"][0], want)
    sim.close()


# ---------------- batched ensembles ----------------

def _batched_setup(lm, orc, E=5, seed=12):
    rng = np.random.default_rng(seed)
    fields = [lm.synthetic_psi_field(195, 215, 20, 35, 1 / 12, n_frames=14, seed=100 + e) for e in range(E)]
    ens = []
    for e in range(E):
        n = int(np.exp(rng.uniform(np.log(1000), np.log(20000))))
        side = rng.uniform(0.5, 1.5)
        x0, y0 = rng.uniform(198, 210), rng.uniform(23, 31)
        lons, lats = orc.lattice(n, y0, y0 + side, x0, x0 + side)
        ens.append((lons, lats, rng.integers(1, 4, lons.size).astype(np.int8)))
    p = rng.uniform(0.5, 0.9, E)
    seeds = rng.integers(1, 2**62, E)
    return fields, ens, p, seeds


def test_gpu_batched_ensembles_equal_single_runs(engine, lm, orc):
    fields, ens, p, seeds = _batched_setup(lm, orc)
    bat = engine.EnsembleSimulation(fields, ens, radius=0.01, p_rs=p, p_pr=p, p_sp=p, seeds=seeds)
    rec = bat.step(0.0, 3600.0, 10, record=True, census=True)
    lon_e = bat.split(rec["lon"])
    sp_e = bat.split(rec["species"])
    cen = bat.census()
    for e, (lons, lats, sp0) in enumerate(ens):
        one = engine.Simulation(fields[e], lons, lats, sp0, radius=0.01, p_rs=p[e], p_pr=p[e], p_sp=p[e],
                                seed=int(seeds[e]))
        r1 = one.step(0.0, 3600.0, 10, record=True)
        np.testing.assert_array_equal(lon_e[e], r1["lon"], err_msg=f"ensemble {e}")
        np.testing.assert_array_equal(sp_e[e], r1["species"], err_msg=f"ensemble {e}")
        np.testing.assert_array_equal(cen[e], np.bincount(r1["species"][-1], minlength=4)[:4])
        one.close()
    # and the oracle on one ensemble, step by step
    lons, lats, sp = ens[1]
    for s in range(10):
        sp, _ = orc.interact_step(lon_e[1][s], bat.split(rec["lat"])[1][s], sp, 0.01, 2, p[1], p[1], p[1],
                                  int(seeds[1]), s)
        np.testing.assert_array_equal(sp_e[1][s], sp)
    bat.close()


def test_gpu_batched_beyond_one_tile_pass_equals_single_runs(engine, lm):
    # 1.2M microbes in 6 ensembles: more than the blocks' shared memory holds at once (304 x 2048),
    # so the interaction runs in groups of whole ensembles; one ensemble is dense (long lists)
    fld = lm.synthetic_psi_field(195.0, 206.0, 20.0, 31.0, 1.0 / 12.0, n_frames=4, frame_seconds=3600.0, seed=4)
    rng = np.random.default_rng(17)
    ens = []
    for e, (n, side) in enumerate([(250_000, 2.0), (40_000, 0.3), (300_000, 3.0), (260_000, 2.5), (200_000, 2.0),
                                   (150_000, 1.5)]):
        x0, y0 = 197.0 + (e % 3) * 2.5, 23.0 + (e // 3) * 3.0
        ens.append(((x0 + side * rng.random(n)), (y0 + side * rng.random(n)), rng.integers(1, 4, n).astype(np.int8)))
    p = [0.55, 0.6, 0.65, 0.7, 0.75, 0.8]
    seeds = [11, 12, 13, 14, 15, 16]
    bat = engine.EnsembleSimulation([fld] * len(ens), ens, radius=0.01, p_rs=p, p_pr=p, p_sp=p, seeds=seeds)
    rec = bat.step(0.0, 3600.0, 2, record=True)
    sp_e = bat.split(rec["species"])
    assert bat.stats()["pairs"] > 1_000_000
    for e, (lons, lats, sp0) in enumerate(ens):
        one = engine.Simulation(fld, lons, lats, sp0, radius=0.01, p_rs=p[e], p_pr=p[e], p_sp=p[e], seed=seeds[e])
        r1 = one.step(0.0, 3600.0, 2, record=True)
        np.testing.assert_array_equal(sp_e[e], r1["species"], err_msg=f"ensemble {e}")
        one.close()
    bat.close()


def test_gpu_batched_more_ensembles_than_the_ranking_block_equals_single_runs(engine, lm):
    # 1,100 small dense ensembles: more than the one block that orders key ranges by density handles
    # (1,024), so the key ranges stay in ensemble order; sampled ensembles against single runs
    fld = lm.synthetic_psi_field(195.0, 206.0, 20.0, 31.0, 1.0 / 12.0, n_frames=5, frame_seconds=3600.0, seed=9)
    rng = np.random.default_rng(23)
    E = 1100
    ens = []
    for e in range(E):
        n = int(rng.integers(30, 200))
        side = rng.uniform(0.02, 0.1)
        x0, y0 = rng.uniform(197.0, 204.0), rng.uniform(22.0, 29.0)
        ens.append((x0 + side * rng.random(n), y0 + side * rng.random(n), rng.integers(1, 4, n).astype(np.int8)))
    p = rng.uniform(0.5, 0.9, E)
    seeds = rng.integers(1, 2**62, E)
    bat = engine.EnsembleSimulation(fld, ens, radius=0.01, p_rs=p, p_pr=p, p_sp=p, seeds=seeds)
    rec = bat.step(0.0, 3600.0, 3, record=True)
    assert bat.stats()["pairs"] > 10_000
    sp_e = bat.split(rec["species"])
    lon_e = bat.split(rec["lon"])
    for e in (0, 1, 517, 1023, 1024, 1099):
        lons, lats, sp0 = ens[e]
        one = engine.Simulation(fld, lons, lats, sp0, radius=0.01, p_rs=p[e], p_pr=p[e], p_sp=p[e], seed=int(seeds[e]))
        r1 = one.step(0.0, 3600.0, 3, record=True)
        np.testing.assert_array_equal(lon_e[e], r1["lon"], err_msg=f"ensemble {e}")
        np.testing.assert_array_equal(sp_e[e], r1["species"], err_msg=f"ensemble {e}")
        one.close()
    bat.close()


def test_gpu_batched_graph_equals_plain(engine, lm, orc):
    fields, ens, p, seeds = _batched_setup(lm, orc, E=7, seed=4)
    a = engine.EnsembleSimulation(fields, ens, radius=0.01, p_rs=p, p_pr=p, p_sp=p, seeds=seeds)
    a.step(0.0, 3600.0, 12)
    b = engine.EnsembleSimulation(fields, ens, radius=0.01, p_rs=p, p_pr=p, p_sp=p, seeds=seeds)
    b.capture(0.0, 3600.0, steps_per_graph=4)
    b.run_graph(3)
    for x, y in zip(a.state(), b.state()):
        np.testing.assert_array_equal(x, y)
    a.close()
    b.close()


def test_gpu_cell_factor_does_not_change_results(engine, lm, orc):
    fld, lons, lats, sp0 = _fused_setup(lm, orc, n=20000, seed=6)
    out = []
    for f in (1.004, 2.0, 3.5):
        sim = engine.Simulation(fld, lons, lats, sp0, radius=0.01, p_rs=0.7, p_pr=0.7, p_sp=0.7, seed=3)
        sim.set_cell_factor(f)
        rec = sim.step(0.0, 3600.0, 5, record=True)
        out.append(rec["species"])
        sim.close()
    np.testing.assert_array_equal(out[0], out[1])
    np.testing.assert_array_equal(out[0], out[2])
