"""The reference's two-phase workflow through the drop-in modules, on the GPU.

Mirrors rock_paper_scissors_example.py:22-36: uniform_particle_locations -> ParticleAdvecter
(.time_step, .create_netcdf_file) -> rock_paper_scissors -> InteractionSimulator.time_step.
"""

import glob
import os
from datetime import datetime, timedelta

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_two_phase_workflow_matches_oracle(lm, orc, small_field, tmp_path):
    from lagrangian_microbes_gb300.interaction_simulator import InteractionSimulator
    from lagrangian_microbes_gb300.ncio import read_particle_file
    from lagrangian_microbes_gb300.particle_advecter import ParticleAdvecter, uniform_particle_locations

    N = 10000
    start = datetime(2017, 1, 1)
    end = start + timedelta(hours=12)
    dt = timedelta(hours=1)
    out = str(tmp_path)
    lons, lats = uniform_particle_locations(N_particles=N, lat_min=25, lat_max=26, lon_min=200, lon_max=201)
    pa = ParticleAdvecter(lons, lats, N_procs=4, velocity_field=small_field, output_dir=out, output_chunk_iters=5,
                          Kh=0)
    pa.time_step(start, end, dt)
    chunks = sorted(glob.glob(os.path.join(out, "particle_locations_*.pickle")))
    assert len(chunks) == 3 * 4  # 5 + 5 + 2 iterations, 4 tiles
    assert os.path.basename(chunks[0]) == "particle_locations_00000_00005_tile00.pickle"
    pa.create_netcdf_file(start, end, dt)
    assert not glob.glob(os.path.join(out, "particle_locations_*.pickle"))
    data = read_particle_file(os.path.join(out, "particle_data.nc"))
    assert data["longitude"].shape == (N, 12)

    # column n holds the position after step n + 1 (the reference's labelling); compare with FP64
    _, _, _, rl, ra = orc.advect_f64(small_field, lons, lats, 0.0, 3600.0, 12, record=True)
    d = orc.great_circle_m(rl[11], ra[11], data["longitude"][:, 11].astype(np.float64),
                           data["latitude"][:, 11].astype(np.float64))
    assert d.max() <= 10.0

    np.random.seed(1)
    rps = lm.rock_paper_scissors(N_microbes=N, pRS=0.6, pPR=0.7, pSP=0.8)
    species0 = rps[2]["species"].copy()
    isim = InteractionSimulator(pair_interaction=rps, interaction_radius=0.012, advection_dir=out, output_dir=out)
    isim.time_step(start, end, dt)
    m = read_particle_file(os.path.join(out, "microbe_data.nc"))
    sp = species0
    seed = rps[1]["seed"]
    for s in range(12):
        sp, _ = orc.interact_step(data["longitude"][:, s], data["latitude"][:, s], sp, 0.012, 2, 0.6, 0.7, 0.8, seed, s)
        np.testing.assert_array_equal(m["species"][:, s], sp, err_msg=f"step {s}")
    np.testing.assert_array_equal(rps[2]["species"], sp)  # updated in place, like the reference
    np.testing.assert_array_equal(m["longitude"], data["longitude"])


def test_fused_engine_equals_two_phase(lm, orc, small_field, tmp_path):
    """The fused per-step engine gives the same positions and species as the two-phase workflow."""
    from lagrangian_microbes_gb300.engine import Simulation
    from lagrangian_microbes_gb300.interaction_simulator import InteractionSimulator
    from lagrangian_microbes_gb300.ncio import read_particle_file
    from lagrangian_microbes_gb300.particle_advecter import ParticleAdvecter, uniform_particle_locations

    N = 4096
    start = datetime(2017, 1, 1)
    dt = timedelta(hours=1)
    end = start + 8 * dt
    lons, lats = uniform_particle_locations(N, 25, 25.5, 200, 200.5)
    out = str(tmp_path)
    pa = ParticleAdvecter(lons, lats, N_procs=1, velocity_field=small_field, output_dir=out)
    pa.time_step(start, end, dt)
    pa.create_netcdf_file(start, end, dt)
    rps = lm.rock_paper_scissors(N, 0.7, 0.7, 0.7, seed=123)
    sp0 = rps[2]["species"].copy()
    InteractionSimulator(rps, 0.01, advection_dir=out, output_dir=out).time_step(start, end, dt)
    m = read_particle_file(os.path.join(out, "microbe_data.nc"))

    sim = Simulation(small_field, lons, lats, sp0, radius=0.01, p_rs=0.7, p_pr=0.7, p_sp=0.7, seed=123)
    rec = sim.step(start, dt, 8, record=True)
    np.testing.assert_array_equal(rec["lon"].T, m["longitude"])
    np.testing.assert_array_equal(rec["lat"].T, m["latitude"])
    np.testing.assert_array_equal(rec["species"].T, m["species"])
    sim.close()


def test_killed_run_resumes_from_its_chunk_files(lm, orc, small_field, tmp_path):
    # a run stopped after 10 h (its process gone, its chunk files kept) and resumed by a new
    # ParticleAdvecter from the files ends where an uninterrupted run ends (within float32
    # rounding of the stored positions, amplified by 10 more hours of flow)
    import pickle
    from lagrangian_microbes_gb300.particle_advecter import ParticleAdvecter, _chunk_name, uniform_particle_locations
    start, dt = datetime(2017, 1, 1), timedelta(hours=1)
    lons, lats = uniform_particle_locations(N_particles=4000, lat_min=25, lat_max=26, lon_min=200, lon_max=201)
    mk = lambda d: ParticleAdvecter(lons, lats, N_procs=4, velocity_field=small_field, output_dir=str(tmp_path / d),
                                    output_chunk_iters=5, Kh=0)
    whole = mk("whole")
    whole.time_step(start, start + 10 * dt, dt)
    whole.time_step(start + 10 * dt, start + 20 * dt, dt)
    first = mk("resumed")
    first.time_step(start, start + 10 * dt, dt)
    del first
    again = mk("resumed")
    assert again.restore_from_disk() == 10
    again.time_step(start + 10 * dt, start + 20 * dt, dt)
    for tile_id in range(4):
        chunk = {}
        for d in ("whole", "resumed"):
            with open(os.path.join(str(tmp_path / d), _chunk_name(15, 20, tile_id)), "rb") as f:
                chunk[d] = pickle.load(f)
        a, b = chunk["whole"], chunk["resumed"]
        dist = orc.great_circle_m(a["lon"][-1].astype(np.float64), a["lat"][-1].astype(np.float64),
                                  b["lon"][-1].astype(np.float64), b["lat"][-1].astype(np.float64))
        assert dist.max() <= 10.0, (tile_id, dist.max())
