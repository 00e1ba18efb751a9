"""Parity at the configured sizes: the CUDA path against the oracle on the benchmark workloads.

* the 490k README-scale run (700 x 700 lattice, 1/12 deg hourly field, r = 0.01, p = 0.7): the
  first three fused steps and three steps of the last simulated day, when the flow has clustered
  the microbes (tens of thousands of lists longer than 8 entries, the long-list kernel and its
  overflow area in use). Pair sets, pair counts and species, step by step;
* the small configuration end to end through the reference's two-phase call surface
  (rock_paper_scissors_example.py:22-36): 10k lattice, 0.25 deg 6-hourly field, 48 hourly steps,
  r = 0.01 with interaction;
* the batching configuration: all 256 ensembles of the benchmark in one context against each
  ensemble run alone, and the densest ensemble against the oracle, on its first steps and on its
  last simulated day (reached through one-day field windows).

The oracle replays each step's pairs in the GPU's application order with a restatement of the
reference's pair rule (interaction_simulator.py:98-105, interactions.py:13-40), so equal species
mean equal pair sets applied in an order equal in effect.
"""

import hashlib
import os
import sys
from datetime import datetime, timedelta

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import bench
    return bench


def _packed_digest(pi, pj):
    packed = (np.asarray(pi, np.uint64) << np.uint64(32)) | np.asarray(pj, np.uint64)
    return hashlib.sha256(np.ascontiguousarray(packed).tobytes()).hexdigest()


def _check_steps(engine, orc, rec, sp_in, step0, probs, seed, r=0.01):
    """Species of every recorded step against the oracle's replay, and the pair set of the first
    recorded step against the oracle's (both as digests of the sorted (i, j) lists)."""
    sp = sp_in.copy()
    for s in range(rec["species"].shape[0]):
        lon, lat = rec["lon"][s], rec["lat"][s]
        sp, m = orc.interact_step(lon, lat, sp, r, 2, *probs, seed, step0 + s, 0)
        np.testing.assert_array_equal(rec["species"][s], sp, err_msg=f"step {step0 + s}")
        if s == 0:
            q = engine.PairQuery(r, 2)
            gi, gj = q.pairs(lon, lat)
            q.ctx.close()
            oi, oj = orc.pairs(lon, lat, r, 2)
            assert gi.size == oi.size == m
            assert _packed_digest(gi, gj) == _packed_digest(oi, oj)
    return sp


def test_490k_first_and_last_simulated_day_match_oracle(lm, orc):
    from lagrangian_microbes_gb300 import engine
    bench = _bench()
    fld, lons, lats, sp0 = bench.make_inputs(702)
    probs = (bench.P_WIN,) * 3
    sim = engine.Simulation(fld, lons, lats, sp0, radius=bench.RADIUS, p_rs=probs[0], p_pr=probs[1],
                            p_sp=probs[2], seed=bench.SEED)
    rec = sim.step(0.0, bench.DT, 3, record=True, step0=0)
    _check_steps(engine, orc, rec, sp0, 0, probs, bench.SEED)
    # advance through the captured graph (the benchmark's form) to step 696, then three recorded steps
    sim.capture(3 * bench.DT, bench.DT, 21, step0=3)
    sim.run_graph(33)  # steps 3 .. 695
    assert sim.step_index == 696
    sp_late = sim.species()
    rec = sim.step(696 * bench.DT, bench.DT, 3, record=True, step0=696)
    st = sim.stats()
    assert st["long_lists"] > 10_000, st  # the clustered regime: many lists longer than 8 entries
    _check_steps(engine, orc, rec, sp_late, 696, probs, bench.SEED)
    sim.close()


def test_small_configuration_end_to_end_through_the_drop_in(lm, orc, small_field, tmp_path):
    """10k lattice over lon 200-201E, lat 25-26N; 48 hourly steps; r = 0.01; p = 0.7."""
    from lagrangian_microbes_gb300.interaction_simulator import InteractionSimulator
    from lagrangian_microbes_gb300.ncio import read_particle_file
    from lagrangian_microbes_gb300.particle_advecter import ParticleAdvecter, uniform_particle_locations

    N, steps = 10000, 48
    start, dt = datetime(2017, 1, 1), timedelta(hours=1)
    end = start + steps * dt
    out = str(tmp_path)
    lons, lats = uniform_particle_locations(N_particles=N, lat_min=25, lat_max=26, lon_min=200, lon_max=201)
    pa = ParticleAdvecter(lons, lats, N_procs=4, velocity_field=small_field, output_dir=out, output_chunk_iters=10,
                          Kh=0)
    pa.time_step(start, end, dt)
    pa.create_netcdf_file(start, end, dt)
    data = read_particle_file(os.path.join(out, "particle_data.nc"))
    assert data["longitude"].shape == (N, steps)
    _, _, _, rl, ra = orc.advect_f64(small_field, lons, lats, 0.0, 3600.0, steps, record=True)
    d24 = orc.great_circle_m(rl[23], ra[23], data["longitude"][:, 23].astype(np.float64),
                             data["latitude"][:, 23].astype(np.float64))
    assert d24.max() <= 10.0, d24.max()

    rps = lm.rock_paper_scissors(N_microbes=N, pRS=0.7, pPR=0.7, pSP=0.7, seed=2024)
    sp = rps[2]["species"].copy()
    InteractionSimulator(pair_interaction=rps, interaction_radius=0.01, advection_dir=out,
                         output_dir=out).time_step(start, end, dt)
    m = read_particle_file(os.path.join(out, "microbe_data.nc"))
    seed = rps[1]["seed"]
    total = 0
    for s in range(steps):
        sp, k = orc.interact_step(data["longitude"][:, s], data["latitude"][:, s], sp, 0.01, 2, 0.7, 0.7, 0.7, seed, s)
        total += k
        np.testing.assert_array_equal(m["species"][:, s], sp, err_msg=f"step {s}")
    assert total > 0  # the flow brings lattice neighbours within the radius during the two days
    np.testing.assert_array_equal(rps[2]["species"], sp)


def test_batching_configuration_all_256_ensembles(lm, orc):
    from lagrangian_microbes_gb300 import engine
    bench = _bench()
    fields, ens, ps, seeds = bench.make_ensembles(bench.B_ENSEMBLES, 4)
    bat = engine.EnsembleSimulation(fields, ens, radius=bench.RADIUS, p_rs=ps, p_pr=ps, p_sp=ps, seeds=seeds)
    rec = bat.step(0.0, bench.DT, 2, record=True)
    assert bat.stats()["pairs"] > 10_000_000
    lon_e, lat_e, sp_e = bat.split(rec["lon"]), bat.split(rec["lat"]), bat.split(rec["species"])
    bat.close()
    for e, (lons, lats, sp0) in enumerate(ens):
        one = engine.Simulation(fields[e], lons, lats, sp0, radius=bench.RADIUS, p_rs=ps[e], p_pr=ps[e], p_sp=ps[e],
                                seed=int(seeds[e]))
        r1 = one.step(0.0, bench.DT, 2, record=True)
        one.close()
        np.testing.assert_array_equal(lon_e[e], r1["lon"], err_msg=f"ensemble {e}")
        np.testing.assert_array_equal(sp_e[e], r1["species"], err_msg=f"ensemble {e}")
    # the densest ensemble (most microbes per area: the longest lists) against the oracle
    dens = [x[0].size / max((np.ptp(x[0]) * np.ptp(x[1])), 1e-9) for x in ens]
    e = int(np.argmax(dens))
    sp = ens[e][2].copy()
    for s in range(2):
        sp, _ = orc.interact_step(lon_e[e][s], lat_e[e][s], sp, bench.RADIUS, 2, ps[e], ps[e], ps[e], int(seeds[e]), s)
        np.testing.assert_array_equal(sp_e[e][s], sp, err_msg=f"densest ensemble {e}, step {s}")


def test_batching_configuration_last_simulated_day(lm, orc):
    """The batching configuration at the end of its 240 steps: the batch advanced to step 216
    through one-day field windows, then two recorded steps. The densest ensembles (and two others)
    run alone from the batch's exported state give the same records bit for bit, and the densest
    ensemble that kept all its microbes on the grid matches the oracle's replay."""
    from lagrangian_microbes_gb300 import engine
    bench = _bench()
    bases = bench.ensemble_bases(bench.B_ENSEMBLES)
    fields, ens, ps, seeds = bench.make_ensembles(bench.B_ENSEMBLES, bench.B_STEPS + 1, bases=bases)
    bat = engine.EnsembleSimulation(fields, ens, radius=bench.RADIUS, p_rs=ps, p_pr=ps, p_sp=ps, seeds=seeds)
    late, dt = bench.B_TOTAL_STEPS - bench.B_STEPS, bench.DT
    for d in range(0, late, bench.B_STEPS):
        if d:
            bat.upload_fields([b.frames(d, bench.B_STEPS + 1) for b in bases])
        bench._oob_ok(bat.step, d * dt, dt, bench.B_STEPS, step0=d)
    bat.upload_fields([b.frames(late, 4) for b in bases])
    state = bat.export_state()
    assert state["step"] == late
    bufs = bat.record_buffers(2)
    bench._oob_ok(bat.step, late * dt, dt, 2, record=True, step0=late, out=bufs)  # records kept in bufs
    lon_e, lat_e, sp_e = bat.split(bufs["lon"]), bat.split(bufs["lat"]), bat.split(bufs["species"])
    edges = np.concatenate([[0], np.cumsum([x[0].size for x in ens])])
    on_grid = [bool((state["status"][edges[e]:edges[e + 1]] == 0).all()) for e in range(len(ens))]
    dens = np.array([x[0].size / max(np.ptp(x[0]) * np.ptp(x[1]), 1e-9) for x in ens])
    order = [int(e) for e in np.argsort(-dens)]
    chosen = order[:3] + order[len(order) // 2:len(order) // 2 + 2]
    for e in chosen:
        a, b = edges[e], edges[e + 1]
        one = engine.Simulation(bases[e].frames(late, 4), ens[e][0], ens[e][1], ens[e][2], radius=bench.RADIUS,
                                p_rs=ps[e], p_pr=ps[e], p_sp=ps[e], seed=int(seeds[e]))
        one.import_state({k: (v[a:b] if k != "step" else v) for k, v in state.items()})
        ob = one.record_buffers(2)
        bench._oob_ok(one.step, late * dt, dt, 2, record=True, step0=late, out=ob)
        one.close()
        np.testing.assert_array_equal(lon_e[e], ob["lon"], err_msg=f"ensemble {e}")
        np.testing.assert_array_equal(lat_e[e], ob["lat"], err_msg=f"ensemble {e}")
        np.testing.assert_array_equal(sp_e[e], ob["species"], err_msg=f"ensemble {e}")
    bat.close()
    e = next(e for e in order if on_grid[e])
    sp = state["species"][edges[e]:edges[e + 1]].copy()
    for s in range(2):
        sp, m = orc.interact_step(lon_e[e][s], lat_e[e][s], sp, bench.RADIUS, 2, ps[e], ps[e], ps[e], int(seeds[e]),
                                  late + s)
        assert m > 0
        np.testing.assert_array_equal(sp_e[e][s], sp, err_msg=f"densest on-grid ensemble {e}, step {late + s}")
