"""Time the reference's own CPU interaction step on the 490k workload (writes reference_cpu_timing.json).

Runs ali-ramadhan/lagrangian-microbes' InteractionSimulator.time_step (interaction_simulator.py:54-122:
cKDTree build + query_pairs + the Python loop calling rock_paper_scissors_interaction) unmodified, on
a single thread as the reference does, for a few hourly steps of the benchmark's 490,000-microbe
700 x 700 lattice (r = 0.01 deg, p = 0.7). Positions come from the oracle's float32 RK4 on the
benchmark's synthetic field (Parcels, the reference's advection, is not installable here). The
xarray / parcels imports are stubbed exactly as in make_golden.py; the reference is read from
LM_REFERENCE_DIR. The reference's advection phase is not timed (no Parcels), so the figure covers
pairs + interaction only and flatters the CPU path.

The reference cannot run on the GPU host, so bench.py reports this committed measurement beside
its live CPU baseline (the oracle's port), with the machine it was taken on.

  LM_REFERENCE_DIR=<checkout> python tests/golden/time_reference_cpu.py [steps]
"""

import json
import os
import platform
import sys
import time
from datetime import datetime, timedelta

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)
import make_golden  # noqa: E402  (stubs and the reference import; needs LM_REFERENCE_DIR)


def main(steps: int = 3):
    import bench  # workload constants and inputs

    _, interactions, _, isim = make_golden._import_reference()
    import oracle
    fld, lons, lats, _ = bench.make_inputs(steps + 2)
    lon = lons.astype(np.float32)
    lat = lats.astype(np.float32)
    plon = np.empty((lon.size, steps), np.float32)
    plat = np.empty((lon.size, steps), np.float32)
    for s in range(steps):  # the positions the reference stores after each advection step
        lon, lat, _ = oracle.advect_f32(fld, lon, lat, s * bench.DT, bench.DT, 1)
        plon[:, s], plat[:, s] = lon, lat
    xr = sys.modules["xarray"]
    adv = os.getcwd()
    xr.Dataset({"longitude": (["particle number", "time"], plon),
                "latitude": (["particle number", "time"], plat)}).to_netcdf(os.path.join(adv, "particle_data.nc"))
    np.random.seed(bench.SEED)
    rps = interactions.rock_paper_scissors(lon.size, bench.P_WIN, bench.P_WIN, bench.P_WIN)
    sim = isim.InteractionSimulator(pair_interaction=rps, interaction_radius=bench.RADIUS, advection_dir=adv,
                                    output_dir=adv)
    start = datetime(2017, 1, 1)
    t0 = time.perf_counter()
    sim.time_step(start, start + steps * timedelta(hours=1), timedelta(hours=1))
    wall = time.perf_counter() - t0
    out = {"what": "reference InteractionSimulator.time_step (cKDTree pairs + Python RPS loop), unmodified",
           "workload": bench.WORKLOAD, "microbes": int(lon.size), "steps": steps, "seconds": wall,
           "value": lon.size * steps / wall, "unit": "microbe-steps/s (pairs + interaction only; advection not timed)",
           "cores": 1, "machine": f"{platform.machine()}, {os.cpu_count()} cores, {platform.processor() or 'cpu'}",
           "python": platform.python_version(), "numpy": np.__version__,
           "scipy": __import__("scipy").__version__,
           "command": "LM_REFERENCE_DIR=<checkout> python tests/golden/time_reference_cpu.py " + str(steps)}
    with open(os.path.join(HERE, "reference_cpu_timing.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 3)
