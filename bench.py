#!/usr/bin/env python
"""Throughput benchmark of the fused advect -> bin -> pair -> interact step (microbe-steps/s).

Workload (the README-scale configuration): 490,000 microbes on a 700 x 700 lattice over
lon 200-205E, lat 25-30N, species i.i.d. uniform over {rock, paper, scissors}, p = 0.7,
a seeded synthetic 32-mode streamfunction field on a 1/12 deg grid over lon 190-215E,
lat 15-40N with hourly frames, RK4 dt = 1 h, interaction radius 0.01 deg (1 km), 720 steps.

One bench step = one CUDA-graph launch of 24 fused steps (one simulated day); K = 30 bench steps
run the configuration's 720 steps. Between timed bench steps a 512 MiB buffer is written to flush
the 129 MB L2. Timing uses CUDA events on the stream the library launches on. Per-kernel times
(CUDA events around plain launches) are reported for the first simulated day (`kernels`, which the
roofline uses) and for four steps of the last one (`kernels_last_day`), when the flow has
clustered the microbes.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU restatement of the reference's path (the oracle: float32 RK4 over
threads, cell-list fixed-radius pairs, sequential rock-paper-scissors replay) on the host cores.
With --gpus N > 1 (torchrun), every rank runs an independent replica (the path has no exchange).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_MICROBES = 490_000
LAT = (25.0, 30.0)
LON = (200.0, 205.0)
FIELD_BOX = (190.0, 215.0, 15.0, 40.0)
RES = 1.0 / 12.0
DT = 3600.0
RADIUS = 0.01
P_WIN = 0.7
SEED = 2024
STEPS_PER_LAUNCH = 24
TUNE_DAY = 3  # the autotuner times steps from the state after this many simulated days
WORKLOAD = "490k microbes, 700x700 lattice lon 200-205E lat 25-30N, 1/12 deg hourly psi field, RK4 dt=1h, r=0.01 deg, p=0.7"


METRIC = "microbe-steps/s (advect+interact), batched+graphed vs plain, 1 GB300, <=10 m err"
DTYPE = "f32 (positions), f64 (pair-boundary refine), int8 (species)"


def bench_config(world: int) -> dict:
    """The workload both arms report (the same dict, so the two lines compare like for like)."""
    return {"workload": WORKLOAD, "microbes": N_MICROBES, "parallelism": f"replicas x{world}",
            "l2": "flushed: a 512 MiB buffer is written between timed GPU bench steps"}


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def make_inputs(n_frames: int):
    import numpy as np

    import lagrangian_microbes_gb300 as lm
    from lagrangian_microbes_gb300.particle_advecter import uniform_particle_locations
    fld = lm.synthetic_psi_field(*FIELD_BOX, RES, n_frames=n_frames, frame_seconds=DT, seed=SEED)
    lons, lats = uniform_particle_locations(N_MICROBES, LAT[0], LAT[1], LON[0], LON[1])
    species = np.random.default_rng(SEED).integers(1, 4, N_MICROBES).astype(np.int8)
    return fld, lons, lats, species


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clocks not sampled"], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# Algorithmic bytes of one launch of each kernel: n = microbes, p = unordered pairs of the step,
# g = grid nodes per frame, frames = distinct frames read per step, cells = binning cells used.
def kernel_bytes(name: str, n: int, p: float, g: int, frames: int, cells: float) -> float:
    if name == "k_advect":
        # read offsets 8 + status 1, write offsets 8 + recorded position 8; plus the frames read
        return 25.0 * n + 8.0 * g * frames
    if name == "k_keys":
        return 17.0 * n  # read position 8 + status 1, write key + rank 8
    if name == "k_cscan":
        return 12.0 * cells  # read counts (twice: reduce + scan) and write starts, 4 B per cell each
    if name == "k_scatter":
        return 40.0 * n  # read key, rank, position, cell start; write id, key, ensemble, position
    if name == "k_sweep":
        return 36.0 * n + 2 * p * 4.0  # vertex reads 20 + per-vertex state writes 16, list entries 4 B
    if name == "k_rounds":
        # list entries once (two per pair); per microbe its state word 8, slot id 4, degree 4, species 1
        return 2 * p * 4.0 + 17.0 * n
    if name == "k_census":
        return 2.0 * n
    return 0.0


def run_gb300(args):
    import numpy as np
    import torch

    from lagrangian_microbes_gb300.engine import Simulation

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    K, W, spg = args.steps, args.warmup, STEPS_PER_LAUNCH
    n_frames = max(K, W, TUNE_DAY + 1) * spg + 2
    fld, lons, lats, species = make_inputs(n_frames)
    n = lons.size

    sim = Simulation(fld, lons, lats, species, radius=RADIUS, p_rs=P_WIN, p_pr=P_WIN, p_sp=P_WIN, seed=SEED,
                     device=local)
    # one dedicated stream shared by torch (events, L2 flush) and the library's launches
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim.set_stream(stream.cuda_stream)
    # cell size and launch shapes (results do not depend on them), tuned on the fourth simulated day:
    # the long-list and interaction kernels matter once the flow has begun to cluster the microbes
    # (profile runs, for ncu launch lists, keep the default settings and launch only the warm-up and
    # timed graphs)
    tuned = {"seconds": None, **sim.tuning(), "cell_factor": 1.004}
    if not args.profile_run:
        sim.capture(0.0, DT, spg, step0=0)
        sim.run_graph(TUNE_DAY, sync=True)
        tuned = sim.autotune_all(TUNE_DAY * spg * DT, DT, 4)
        sim.upload_particles(lons, lats, species)
        sim.set_step(0)
    cell_factor = tuned["cell_factor"]
    sim.capture(0.0, DT, spg, step0=0)
    sim.run_graph(W, sync=True)  # warm-up (also grows neighbour lists if needed)

    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def reset():
        sim.upload_particles(lons, lats, species)
        sim.set_step(0)
        sim.ctx.call("lm_stats_reset")

    reset()
    depth_first = dependency_depth(sim, 0)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for k in range(K):
            flush.zero_()
            starts[k].record(stream)
            sim.run_graph(1, sync=False)
            ends[k].record(stream)
        torch.cuda.synchronize()
    sim.sync()  # raises on any device-side error of the timed region
    total_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    stats = sim.stats()
    if args.profile_run:  # ncu launch lists: warm-up + timed graph launches only
        sim.close()
        return
    if world > 1:
        t = torch.tensor([total_ms], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    sim_steps = K * spg
    value = world * n * sim_steps / (total_ms / 1e3)
    pairs_per_step = stats["pairs_total"] / max(stats["steps_total"], 1)

    # ---- plain per-step launches (the drop-in form), same workload and step count ----
    reset()
    plain_steps = min(sim_steps, args.plain_steps)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    p0.record(stream)
    sim.step(0.0, DT, plain_steps, step0=0)
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1)
    plain_value = n * plain_steps / (plain_ms / 1e3)

    # ---- per-kernel timing (plain launches with CUDA events) for the roofline ----
    reset()
    sim.ctx.profile_enable(True)
    prof_steps = min(48, sim_steps)
    sim.step(0.0, DT, prof_steps, step0=0)
    prof = sim.ctx.profile()
    sim.ctx.profile_enable(False)
    g = fld.u.shape[1] * fld.u.shape[2]
    kernels = {}
    cells = float(sim.stats()["cells"])
    for name, (ms, cnt) in prof.items():
        if cnt:
            kernels[name] = {"launches": cnt, "total_ms": ms, "avg_us": 1e3 * ms / cnt,
                             "bytes_per_launch": kernel_bytes(name, n, pairs_per_step, g, 2, cells)}
    total_k = sum(v["total_ms"] for v in kernels.values()) or 1.0
    for v in kernels.values():
        v["share"] = v["total_ms"] / total_k
    dom = max(kernels, key=lambda k: kernels[k]["total_ms"])
    peak, peak_kind = measured_peaks()
    dk = kernels[dom]
    achieved = dk["bytes_per_launch"] / (dk["avg_us"] * 1e-6) / 1e9 if dk["bytes_per_launch"] else None
    traffic = None
    if args.traffic_json and os.path.exists(args.traffic_json):
        with open(args.traffic_json) as f:
            traffic = json.load(f).get(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": dk["bytes_per_launch"], "avg_launch_us": dk["avg_us"]}
    step_bytes = 42.0 * n + 16.0 * pairs_per_step + 8.0 * g * 2
    whole = {"bytes_per_step": step_bytes, "gbs": step_bytes * sim_steps / (total_ms / 1e3) / 1e9}

    # ---- the same per-kernel timing in the last simulated day: by then the flow has clustered the
    # microbes (longer neighbour lists, longer dependency chains, a wider cell grid) ----
    reset()
    late_step = (K - 1) * spg
    if late_step:
        sim.run_graph(K - 1, sync=True)
    depth_late = dependency_depth(sim, late_step)
    sim.ctx.profile_enable(True)
    sim.step(late_step * DT, DT, 4, step0=late_step)
    prof_late = sim.ctx.profile()
    st_late = sim.stats()
    sim.ctx.profile_enable(False)
    last_day = {"after_steps": late_step, "steps": 4, "long_lists": st_late["long_lists"], "cells": st_late["cells"],
                "pairs": st_late["pairs"],
                "us_per_launch": {k: 1e3 * ms / cnt for k, (ms, cnt) in prof_late.items() if cnt}}

    # ---- end to end through the public API from host buffers ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(fld, lons, lats, species, K, spg, local, stream)

    batched = adjoint = stress = histogram = dropin = None
    if rank == 0 and not args.no_dropin:
        dropin = run_dropin(fld, lons, lats, species, local, stream)
    if rank == 0 and not args.no_batched:
        batched = run_batched(local, stream)
    if rank == 0 and not args.no_stress:
        stress = run_stress(fld, local)
    if rank == 0 and not args.no_adjoint:
        adjoint = run_adjoint(local)
    if rank == 0 and not args.no_histogram:
        histogram = run_histogram(lons, lats, species)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(fld, lons, lats, species, args.cpu_seconds)
    clk = clocks.summary()
    launches_per_step = (sum(v["launches"] for v in kernels.values()) / prof_steps) * spg
    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value, "unit": "microbe-steps/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPE, "data": "synthetic",
            "config": bench_config(world),
            "run": {"sim_steps_per_bench_step": spg, "sim_steps_timed": sim_steps, "form": "cuda-graph, 24 steps/launch",
                    "tuning": {k: v for k, v in tuned.items() if k != "seconds"}, "autotune_s": tuned["seconds"]},
            "pairs_per_step": pairs_per_step,
            "plain": {"value": plain_value, "unit": "microbe-steps/s", "sim_steps": plain_steps,
                      "graph_speedup": value / world / plain_value},
            "roofline": roofline, "whole_step": whole, "kernels": kernels, "kernels_last_day": last_day,
            "e2e": e2e, "cpu_baseline": cpu, "clocks": clk, "dropin": dropin, "batched": batched, "adjoint": adjoint,
            "stress": stress,
            "distance_histogram": histogram,
            "gpu_launches": int(round(launches_per_step * K)),
            "dependency_depth": {"first_step": depth_first, f"step_{late_step}": depth_late,
                                 "what": "longest chain of pairs that share a microbe, in application order "
                                         "(levels of one logged step, replayed from the same state)"},
            "cpu_baseline_reference": reference_cpu_timing(),
        }
        print(json.dumps(line), flush=True)
    sim.close()
    if world > 1:
        torch.distributed.destroy_process_group()


DROPIN_STEPS = 48


def run_dropin(fld, lons, lats, species, local: int, stream):
    """The reference's own two-phase call surface on the 490k workload (rock_paper_scissors_example.py:
    22-36): ParticleAdvecter.time_step over 48 hourly steps writing per-tile chunk pickles every 24
    steps, create_netcdf_file, then InteractionSimulator.time_step over the same 48 steps (wall
    clock, files in a temporary directory). Beside it, the fused engine's plain steps with and
    without per-step records (positions and species copied to host arrays)."""
    import shutil
    import tempfile
    from datetime import timedelta

    import numpy as np
    import torch

    import lagrangian_microbes_gb300 as lm
    from lagrangian_microbes_gb300.engine import Simulation
    from lagrangian_microbes_gb300.interaction_simulator import InteractionSimulator
    from lagrangian_microbes_gb300.particle_advecter import ParticleAdvecter
    n, steps = lons.size, DROPIN_STEPS
    start, dt = fld.epoch, timedelta(seconds=DT)
    out = tempfile.mkdtemp(prefix="lm_dropin_")
    try:
        t0 = time.perf_counter()
        pa = ParticleAdvecter(lons, lats, N_procs=4, velocity_field=fld, output_dir=out, output_chunk_iters=24,
                              seed=SEED, device=local)
        pa._engine()  # context, field and particle upload
        t1 = time.perf_counter()
        pa.time_step(start, start + steps * dt, dt)
        t2 = time.perf_counter()
        pa.create_netcdf_file(start, start + steps * dt, dt)
        t3 = time.perf_counter()
        rps = lm.rock_paper_scissors(n, P_WIN, P_WIN, P_WIN, seed=SEED)
        rps[2]["species"][:] = species
        InteractionSimulator(rps, RADIUS, advection_dir=out, output_dir=out, device=local).time_step(
            start, start + steps * dt, dt)
        t4 = time.perf_counter()
    finally:
        shutil.rmtree(out, ignore_errors=True)
    # the fused engine from one state: plain steps without and with records
    sim = Simulation(fld, lons, lats, species, radius=RADIUS, p_rs=P_WIN, p_pr=P_WIN, p_sp=P_WIN, seed=SEED,
                     device=local)
    sim.set_stream(stream.cuda_stream)
    sim.step(0.0, DT, 2, step0=0)  # warm-up (list capacities, the record ring)
    sim.upload_particles(lons, lats, species)
    sim.snapshot()
    bufs = sim.record_buffers(steps)
    walls = {}
    for mode in ("plain", "reused", "fresh", "plain", "reused", "fresh"):
        sim.restore()
        torch.cuda.synchronize()
        a = time.perf_counter()
        sim.step(0.0, DT, steps, step0=0, record=mode != "plain", out=bufs if mode == "reused" else None)
        torch.cuda.synchronize()
        walls[mode] = min(walls.get(mode, 1e9), time.perf_counter() - a)
    sim.close()
    ms = n * steps
    return {"workload": "490k lattice, 48 hourly steps through ParticleAdvecter (4 tiles, chunks of 24) + "
                        "create_netcdf_file + InteractionSimulator (r = 0.01, p = 0.7), files on local disk",
            "advect": {"value": ms / (t2 - t1), "unit": "microbe-steps/s", "seconds": t2 - t1,
                       "setup_s": t1 - t0},
            "netcdf_s": t3 - t2,
            "interact": {"value": ms / (t4 - t3), "unit": "microbe-steps/s", "seconds": t4 - t3},
            "two_phase": {"value": ms / (t4 - t1), "unit": "microbe-steps/s (advect + netcdf + interact)"},
            "fused_plain": {"unrecorded_ms_per_step": 1e3 * walls["plain"] / steps,
                            "recorded_ms_per_step": 1e3 * walls["reused"] / steps,
                            "recorded_over_unrecorded": walls["reused"] / walls["plain"],
                            "recorded_into_fresh_arrays_ms_per_step": 1e3 * walls["fresh"] / steps,
                            "record_bytes_per_step": 9 * n,
                            "note": "records copied on a second stream into reused page-locked host arrays "
                                    "(Simulation.record_buffers); fresh pageable arrays pay the page faults of new "
                                    "host memory and hold the host thread for every copy"}}


def dependency_depth(sim, step: int) -> int:
    """Levels of the interaction at `step` from the current state (a logged step, then the state
    is restored): the critical path of the interaction kernel."""
    sim.snapshot()
    sim.step(step * DT, DT, 1, step0=step, log_pairs=True)
    depth = int(sim.stats()["rounds"])
    sim.restore()
    return depth


def reference_cpu_timing():
    """The reference's own CPU interaction step (cKDTree + Python loop) on this workload, measured by
    tests/golden/time_reference_cpu.py where the reference is available (it is not on the GPU host)."""
    path = os.path.join(REPO, "tests", "golden", "reference_cpu_timing.json")
    try:
        with open(path) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    d["source"] = "recorded by tests/golden/time_reference_cpu.py on the machine named in 'machine', not on this host"
    return d


def run_e2e(fld, lons, lats, species, K, spg, local, stream):
    """Same job through the public API: host field/particles in, final state out, all timed."""
    import numpy as np
    import torch

    from lagrangian_microbes_gb300 import _lib
    from lagrangian_microbes_gb300.engine import Simulation
    from lagrangian_microbes_gb300.fields import VelocityField

    def pinned(a):  # a page-locked copy, made before the timed region (a caller's staging buffer)
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

    fld = VelocityField(fld.lon, fld.lat, fld.times, pinned(fld.u), pinned(fld.v), fld.epoch)
    lons, lats, species = pinned(lons), pinned(lats), pinned(species)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim = Simulation.__new__(Simulation)  # the constructor's calls, timed one by one
    sim.ctx = _lib.Context(local)
    tc0 = time.perf_counter()
    sim.field, sim.kh, sim.seed, sim.radius, sim.norm, sim._graph, sim.step_index = fld, 0.0, SEED, RADIUS, 2, None, 0
    sim.upload_field(fld)
    tf = time.perf_counter()
    sim.upload_particles(lons, lats, species)
    tp = time.perf_counter()
    sim.set_interaction(RADIUS, 2, P_WIN, P_WIN, P_WIN, SEED)
    ta = time.perf_counter()
    sim.capture(0.0, DT, spg, step0=0)
    tb = time.perf_counter()
    sim.run_graph(K, sync=True)
    tc = time.perf_counter()
    lon, lat, sp, st = sim.state()
    t1 = time.perf_counter()
    sim.close()
    n = lons.size
    h2d = fld.u.nbytes + fld.v.nbytes + lons.nbytes + lats.nbytes + species.nbytes
    d2h = lon.nbytes + lat.nbytes + sp.nbytes + st.nbytes
    return {"value": n * K * spg / (t1 - t0), "unit": "microbe-steps/s", "h2d_bytes_per_step": h2d / K,
            "d2h_bytes_per_step": d2h / K, "seconds": t1 - t0,
            "phases_s": {"context": tc0 - t0, "field": tf - tc0, "particles": tp - tf, "params": ta - tp,
                         "capture": tb - ta, "steps": tc - tb, "download": t1 - tc},
            "note": "setup (field + particles upload from page-locked host buffers, graph capture) + 720 steps + "
                    "state download, wall clock"}


B_ENSEMBLES = 256
B_STEPS = 24
B_TOTAL_STEPS = 240
B_BOX = (195.0, 215.0, 20.0, 35.0)
B_WORKLOAD = ("256 ensembles, counts log-uniform in [1e3, 2e5] (rounded to square-ish lattices), patches of 0.5-3 deg side within lon "
              "195-215E lat 20-35N, p ~ U[0.5, 0.9], own seed and own 32-mode psi field each on a shared 1/12 deg "
              "hourly grid, RK4 dt=1h, r=0.01 deg; timed on the first and on the last simulated day of the 240 steps")


def ensemble_bases(n_ens: int):
    """The per-ensemble synthetic fields of the batching configuration, before sampling in time
    (frames are sampled window by window: a 240-step run never holds all 256 x 241 frames)."""
    from lagrangian_microbes_gb300.fields import psi_basis
    return [psi_basis(*B_BOX, RES, frame_seconds=DT, seed=SEED + 1 + e) for e in range(n_ens)]


def make_ensembles(n_ens: int, n_frames: int, seed: int = 2025, bases=None):
    """The batching configuration: per-ensemble lattices, probabilities, seeds and fields (seeded)."""
    import numpy as np

    from lagrangian_microbes_gb300.particle_advecter import uniform_particle_locations
    rng = np.random.default_rng(seed)
    raw = np.exp(rng.uniform(np.log(1e3), np.log(2e5), n_ens))
    # square-ish lattices: the count is rounded to rows x columns with rows = round(sqrt(count)), so
    # that the lattice helper's factorisation never degenerates into a single dense line
    rows = np.maximum(1, np.rint(np.sqrt(raw))).astype(np.int64)
    counts = rows * np.maximum(1, np.rint(raw / rows)).astype(np.int64)
    sides = rng.uniform(0.5, 3.0, n_ens)
    margin = 0.5  # keeps a day of drift inside the field
    lon0 = rng.uniform(B_BOX[0] + margin, B_BOX[1] - margin - sides)
    lat0 = rng.uniform(B_BOX[2] + margin, B_BOX[3] - margin - sides)
    ps = rng.uniform(0.5, 0.9, n_ens)
    seeds = rng.integers(0, 2 ** 62, n_ens)
    ens = []
    for e in range(n_ens):
        lons, lats = uniform_particle_locations(int(counts[e]), lat0[e], lat0[e] + sides[e], lon0[e], lon0[e] + sides[e])
        sp = np.random.default_rng(int(seeds[e])).integers(1, 4, lons.size).astype(np.int8)
        ens.append((lons, lats, sp))
    bases = bases or ensemble_bases(n_ens)
    fields = [b.frames(0, n_frames) for b in bases]
    return fields, ens, ps, seeds


def _oob_ok(fn, *args, **kw):
    """Run fn; microbes that leave the shared grid are frozen and excluded (the engine reports it
    once, as OutOfBoundsError, after the call has completed). Returns True when that happened."""
    from lagrangian_microbes_gb300 import OutOfBoundsError
    try:
        fn(*args, **kw)
        return False
    except OutOfBoundsError:
        return True


def _time_graph(sim, stream, reps: int = 3) -> float:
    """Median ms of one graph launch, each from the snapshot taken before (CUDA events)."""
    import numpy as np
    import torch
    times = []
    for _ in range(reps):
        sim.restore()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        sim.run_graph(1, sync=False)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
        _oob_ok(sim.sync)
    return float(np.median(times))


def _time_plain_per_ensemble(bases, ens, ps, seeds, first: int, local: int, state=None) -> float:
    """Wall ms of B_STEPS plain steps of every ensemble alone (its own context), ensembles one after
    another, from step `first` (state: the exact state of every ensemble there, or the lattices)."""
    import numpy as np
    import torch

    from lagrangian_microbes_gb300.engine import Simulation
    sims = []
    edges = np.concatenate([[0], np.cumsum([x[0].size for x in ens])])
    for e in range(len(ens)):
        one = Simulation(bases[e].frames(first, B_STEPS + 2), ens[e][0], ens[e][1], ens[e][2], radius=RADIUS,
                         p_rs=ps[e], p_pr=ps[e], p_sp=ps[e], seed=int(seeds[e]), device=local)
        if state is not None:
            a, b = edges[e], edges[e + 1]
            one.import_state({k: (v[a:b] if k != "step" else v) for k, v in state.items()})
        one.snapshot()
        _oob_ok(one.step, first * DT, DT, 1, step0=first)  # warm-up (list capacities), then back
        one.restore()
        sims.append(one)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for one in sims:
        _oob_ok(one.step, first * DT, DT, B_STEPS, step0=first)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3
    for one in sims:
        one.close()
    return ms


def profile_batched(steps: int) -> None:
    """Plain steps of the batching workload and nothing else: a short program for ncu captures of
    its kernels (k_advect reads 256 different fields there, which do not fit L2 together)."""
    from lagrangian_microbes_gb300.engine import EnsembleSimulation
    fields, ens, ps, seeds = make_ensembles(B_ENSEMBLES, steps + 2)
    sim = EnsembleSimulation(fields, ens, radius=RADIUS, p_rs=ps, p_pr=ps, p_sp=ps, seeds=seeds)
    sim.step(0.0, DT, steps, step0=0)
    sim.sync()
    sim.close()


def run_batched(local: int, stream):
    """Config B: all ensembles in one context (CUDA graph of B_STEPS fused steps) against plain
    per-step launches of each ensemble alone (its own context), the same simulated steps: the
    first simulated day, and the last one (steps 216-239) reached by streaming the fields in
    one-day windows."""
    from lagrangian_microbes_gb300.engine import EnsembleSimulation
    t_start = t_gen = time.perf_counter()
    bases = ensemble_bases(B_ENSEMBLES)
    fields, ens, ps, seeds = make_ensembles(B_ENSEMBLES, B_STEPS + 2, bases=bases)
    t_gen = time.perf_counter() - t_gen
    total = int(sum(x[0].size for x in ens))
    sim = EnsembleSimulation(fields, ens, radius=RADIUS, p_rs=ps, p_pr=ps, p_sp=ps, seeds=seeds, device=local)
    sim.set_stream(stream.cuda_stream)
    tuned = sim.autotune_all(0.0, DT, 2)
    cell_factor = tuned["cell_factor"]
    # per-kernel time of two plain steps (CUDA events around each launch)
    sim.upload_ensembles(ens)
    sim.ctx.profile_enable(True)
    sim.step(0.0, DT, 2, step0=0)
    prof = sim.ctx.profile()
    sim.ctx.profile_enable(False)
    kernels_ms = {k: ms / 2 for k, (ms, cnt) in prof.items() if cnt}
    # first simulated day
    sim.upload_ensembles(ens)
    sim.set_step(0)
    sim.snapshot()
    sim.capture(0.0, DT, B_STEPS, step0=0)
    sim.run_graph(1, sync=True)  # warm-up: sizes the long neighbour lists for this workload
    sim.ctx.call("lm_stats_reset")
    graph_ms = _time_graph(sim, stream)
    st = sim.stats()
    plain_ms = _time_plain_per_ensemble(bases, ens, ps, seeds, 0, local)
    # last simulated day: advance through one-day field windows, then the same two timings
    late = B_TOTAL_STEPS - B_STEPS
    sim.restore()
    for d in range(0, late, B_STEPS):
        sim.upload_fields([b.frames(d, B_STEPS + 1) for b in bases])
        _oob_ok(sim.step, d * DT, DT, B_STEPS, step0=d)
    sim.upload_fields([b.frames(late, B_STEPS + 2) for b in bases])
    sim.snapshot()
    sim.ctx.profile_enable(True)
    _oob_ok(sim.step, late * DT, DT, 2, step0=late)
    prof_late = sim.ctx.profile()
    sim.ctx.profile_enable(False)
    sim.restore()
    sim.capture(late * DT, DT, B_STEPS, step0=late)
    _oob_ok(sim.run_graph, 1, sync=True)
    sim.ctx.call("lm_stats_reset")
    graph_late_ms = _time_graph(sim, stream)
    st_late = sim.stats()
    sim.restore()
    state = sim.export_state()
    frozen = int((state["status"] != 0).sum())
    sim.close()
    plain_late_ms = _time_plain_per_ensemble(bases, ens, ps, seeds, late, local, state=state)

    def part(g_ms, p_ms, stats, prof_ms, first):
        gv = total * B_STEPS / (g_ms / 1e3)
        pv = total * B_STEPS / (p_ms / 1e3)
        return {"steps": [first, first + B_STEPS - 1],
                "pairs_per_step": stats["pairs_total"] / max(stats["steps_total"], 1),
                "long_lists": stats["long_lists"],
                "graph": {"value": gv, "unit": "microbe-steps/s", "ms_per_sim_step": g_ms / B_STEPS,
                          "form": "one context, one CUDA graph of 24 fused steps for all ensembles",
                          "tuning": {k: v for k, v in tuned.items() if k != "seconds"}},
                "plain_per_ensemble": {"value": pv, "unit": "microbe-steps/s", "ms_per_sim_step": p_ms / B_STEPS,
                                       "form": "one context per ensemble, per-step launches, ensembles one after another"},
                "batched_over_plain": gv / pv, "kernels_ms_per_step": prof_ms}

    first = part(graph_ms, plain_ms, st, kernels_ms, 0)
    last = part(graph_late_ms, plain_late_ms, st_late,
                {k: ms / 2 for k, (ms, cnt) in prof_late.items() if cnt}, late)
    return {"workload": B_WORKLOAD, "ensembles": B_ENSEMBLES, "microbes": total, "sim_steps": B_STEPS,
            "first_day": first, "last_day": last,
            "left_the_grid_by_step_216": frozen,  # frozen and excluded from pairing, like every microbe that leaves
            # the headline of the configuration: both timed days together
            "graph": {"value": total * 2 * B_STEPS / ((graph_ms + graph_late_ms) / 1e3), "unit": "microbe-steps/s"},
            "batched_over_plain": (plain_ms + plain_late_ms) / (graph_ms + graph_late_ms),
            "field_generation_s": t_gen, "seconds": time.perf_counter() - t_start}


def run_adjoint(local: int):
    """Config D timing: 1M microbes on a 1000x1000 lattice, 720 steps, checkpoints every 32, the
    mean squared great-circle distance to seeded targets, forward + backward (both precisions). The
    721-frame field is generated here, whatever the number of bench steps."""
    import numpy as np
    import torch

    import lagrangian_microbes_gb300 as lm
    from lagrangian_microbes_gb300.adjoint import AdjointTape, advect_rk4, mean_squared_distance
    from lagrangian_microbes_gb300.particle_advecter import uniform_particle_locations
    n, steps, k = 1_000_000, 720, 32
    fld = lm.synthetic_psi_field(*FIELD_BOX, RES, n_frames=steps + 1, frame_seconds=DT, seed=SEED)
    lons, lats = uniform_particle_locations(n, LAT[0], LAT[1], LON[0], LON[1])
    rng = np.random.default_rng(7)
    dev = torch.device("cuda", local)
    tl = torch.from_numpy(lons + rng.normal(0, 20.0 / 111.32, n) / np.cos(np.deg2rad(lats))).to(dev)
    ta = torch.from_numpy(lats + rng.normal(0, 20.0 / 111.32, n)).to(dev)
    u = torch.from_numpy(fld.u[: steps + 1]).to(dev).requires_grad_(True)
    v = torch.from_numpy(fld.v[: steps + 1]).to(dev).requires_grad_(True)
    out = {"workload": "1M microbes, 1000x1000 lattice lon 200-205E lat 25-30N, 720 RK4 steps dt=1h on the 1/12 deg "
                       "hourly field, checkpoints every 32 steps, loss = mean squared great-circle distance to "
                       "targets x0 + N(0, 20 km)", "microbes": n, "sim_steps": steps}
    for prec in ("ds", "f32", "f64"):
        tape = AdjointTape(device=local, precision=prec)
        res = []
        for _ in range(3):
            l0 = torch.from_numpy(lons.astype(np.float32)).to(dev).requires_grad_(True)
            a0 = torch.from_numpy(lats.astype(np.float32)).to(dev).requires_grad_(True)
            u.grad = v.grad = None
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            torch.cuda.synchronize()
            ev[0].record()
            x, y = advect_rk4(l0, a0, u, v, fld.lon, fld.lat, fld.times[: steps + 1], 0.0, DT, steps,
                              checkpoint_every=k, tape=tape)
            ev[1].record()
            loss = mean_squared_distance(x, y, tl, ta)
            loss.backward()
            ev[2].record()
            torch.cuda.synchronize()
            res.append((ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])))
        tape.close()
        fwd = float(np.median([r[0] for r in res]))
        bwd = float(np.median([r[1] for r in res]))
        out[prec] = {"forward_ms": fwd, "backward_ms": bwd,
                     "value": n * steps / ((fwd + bwd) / 1e3), "unit": "microbe-steps/s (forward + backward)",
                     "loss_m2": float(loss.detach())}
    return out


X_MICROBES = 16_000_000
X_CLUSTERS = 2000
X_STEPS = 3
X_WORKLOAD = ("16M microbes in 2,000 Gaussian clusters (sigma 0.03 deg = 3 km at 100 km/deg, centres uniform over "
              "200-210E x 25-35N, sizes rank-size Zipf(1.2) normalised to 16M), 1/12 deg hourly psi field, RK4 dt=1h, "
              "r=0.01 deg, count-only pairs (no lists, no interaction)")


def make_clusters(n: int = X_MICROBES, k: int = X_CLUSTERS, seed: int = 2026):
    """The neighbour-search stress configuration's positions (seeded)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    w = np.arange(1, k + 1, dtype=np.float64) ** -1.2
    sizes = np.floor(n * w / w.sum()).astype(np.int64)
    sizes[: n - sizes.sum()] += 1  # exactly n
    cx = rng.uniform(200.0, 210.0, k)
    cy = rng.uniform(25.0, 35.0, k)
    lon = np.repeat(cx, sizes) + 0.03 * rng.standard_normal(n)
    lat = np.repeat(cy, sizes) + 0.03 * rng.standard_normal(n)
    return lon, lat, sizes


def run_stress(fld, local: int):
    """Config X: advect -> bin -> count pairs, per-kernel CUDA events; binning HBM GB/s."""
    import numpy as np

    from lagrangian_microbes_gb300.engine import Simulation
    lons, lats, sizes = make_clusters()
    n = lons.size
    sim = Simulation(fld, lons, lats, np.ones(n, np.int8), radius=RADIUS, device=local)
    sim.step(0.0, DT, 1, step0=0, count_pairs=True)  # warm-up
    sim.upload_particles(lons, lats, np.ones(n, np.int8))
    sim.ctx.call("lm_stats_reset")
    sim.ctx.profile_enable(True)
    t0 = time.perf_counter()
    sim.step(0.0, DT, X_STEPS, step0=0, count_pairs=True)
    wall = time.perf_counter() - t0
    prof = sim.ctx.profile()
    sim.ctx.profile_enable(False)
    st = sim.stats()
    cells = float(st["cells"])
    sim.close()
    per = {k: 1e3 * ms / cnt for k, (ms, cnt) in prof.items() if cnt}
    bin_kernels = ("k_grid", "k_keys", "k_cscan", "k_scatter")
    bin_us = sum(per.get(k, 0.0) for k in bin_kernels)
    bin_bytes = sum(kernel_bytes(k, n, 0.0, 0, 2, cells) for k in bin_kernels)
    peak, kind = measured_peaks()
    pairs = st["pairs_total"] / max(st["steps_total"], 1)
    return {"workload": X_WORKLOAD, "microbes": n, "largest_cluster": int(sizes.max()), "sim_steps": X_STEPS,
            "pairs_per_step": pairs, "ms_per_step": 1e3 * wall / X_STEPS,
            "value": n * X_STEPS / wall, "unit": "microbe-steps/s (count-only pipeline, plain launches)",
            "kernels_us": per,
            "binning": {"kernels": list(bin_kernels), "us_per_step": bin_us, "algorithmic_bytes": bin_bytes,
                        "gbs": bin_bytes / (bin_us * 1e-6) / 1e9 if bin_us else None, "peak_gbs": peak,
                        "frac": (bin_bytes / (bin_us * 1e-6) / 1e9) / peak if bin_us else None, "peak_source": kind},
            "count": {"us_per_step": per.get("k_count_pairs"),
                      "pairs_per_s": pairs / (per["k_count_pairs"] * 1e-6) if per.get("k_count_pairs") else None}}


def run_histogram(lons, lats, species):
    """Pairwise distance histograms per species of the 490k lattice (sandbox/pairwise_distance_
    histogram_distributed.jl:133-147, 70 bins) through the public API from host arrays; the oracle
    (float64, all host threads) on a bounded sample of the same pairs beside it."""
    import numpy as np

    from lagrangian_microbes_gb300 import _lib
    from lagrangian_microbes_gb300.pairwise_distance_histogram import species_distance_histograms
    ctx = _lib.Context(0)
    sizes = [int(np.count_nonzero(species == k)) for k in (1, 2, 3)]
    pairs = sum(m * (m - 1) // 2 for m in sizes)
    species_distance_histograms(lons, lats, species, 70, ctx=ctx)  # warm-up
    t0 = time.perf_counter()
    got = species_distance_histograms(lons, lats, species, 70, ctx=ctx)
    wall = time.perf_counter() - t0
    ctx.close()
    assert sum(int(c.sum()) + o for c, o in got.values()) == pairs
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    sel = np.flatnonzero(species == 1)[:20_000]
    la, lo = np.asarray(lats, np.float32)[sel], np.asarray(lons, np.float32)[sel]
    oracle.distance_histogram(la[:2000], lo[:2000], 70)  # build, threads up
    t0 = time.perf_counter()
    oracle.distance_histogram(la, lo, 70)
    cpu_wall = time.perf_counter() - t0
    cpu_pairs = sel.size * (sel.size - 1) // 2
    return {"workload": "one histogram per species of the 490k lattice (i.i.d. species), 70 bins of "
                        "round(10 log10(max(1 m, d))), float32 haversine",
            "pairs": pairs, "ms": 1e3 * wall, "value": pairs / wall,
            "unit": "pairs/s (public API, host arrays in and out)",
            "cpu_baseline": {"value": cpu_pairs / cpu_wall, "unit": "pairs/s", "cores": cpu_threads(), "kind": "port",
                             "sample": f"all pairs of the first {sel.size} rock microbes (float64 oracle)"},
            "reference_published": {"pairs_per_s_1_process": 5e7 / 4.035, "pairs_per_s_60_processes": 5e7 / 0.268,
                                    "source": "timing comment of sandbox/pairwise_distance_histogram_distributed.jl "
                                              "(10,000 random points)"}}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(fld, lons, lats, species, seconds):
    """The oracle's fused CPU steps on the full 490k workload, as many steps as fit in ~`seconds`."""
    import numpy as np
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.build()
    threads = cpu_threads()
    lon = lons.astype(np.float32)
    lat = lats.astype(np.float32)
    sp = species.copy()
    steps, t0 = 0, time.perf_counter()
    while True:
        oracle.run(fld, lon, lat, sp, DT * steps, DT, 1, steps, RADIUS, 2, P_WIN, P_WIN, P_WIN, SEED, threads)
        steps += 1
        if time.perf_counter() - t0 > seconds or steps >= 720:
            break
    dt = time.perf_counter() - t0
    return {"value": lons.size * steps / dt, "unit": "microbe-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} fused steps of the full 490k workload (float32 RK4 on {threads} threads, "
                      f"cell-list pairs, sequential RPS replay)", "seconds": dt}


def run_reference(args):
    rank, world, local = env_rank()
    if rank != 0:
        return
    import numpy as np
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.build()
    K, W = args.steps, args.warmup
    fld, lons, lats, species = make_inputs(K + W + 2)
    threads = cpu_threads()
    lon = lons.astype(np.float32)
    lat = lats.astype(np.float32)
    sp = species.copy()
    for s in range(W):
        oracle.run(fld, lon, lat, sp, DT * s, DT, 1, s, RADIUS, 2, P_WIN, P_WIN, P_WIN, SEED, threads)
    times = []
    for s in range(W, W + K):
        t0 = time.perf_counter()
        oracle.run(fld, lon, lat, sp, DT * s, DT, 1, s, RADIUS, 2, P_WIN, P_WIN, P_WIN, SEED, threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = lons.size * K / total
    line = {"impl": "reference", "metric": METRIC,
            "value": value, "unit": "microbe-steps/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * total / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPE, "data": "synthetic",
            "config": bench_config(world),
            "run": {"sim_steps_per_bench_step": 1, "form": "the oracle's fused CPU step on all host threads"},
            "cpu_baseline": {"value": value, "unit": "microbe-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{K} fused steps of the full 490k workload (one step per bench step)"},
            "e2e": {"value": value, "unit": "microbe-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--plain-steps", type=int, default=720, help="plain steps (the same steps the graph runs)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-dropin", action="store_true", help="skip the two-phase drop-in measurement")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-ensemble batching measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint (differentiation) timing")
    ap.add_argument("--no-stress", action="store_true", help="skip the 16M clustered count-only measurement")
    ap.add_argument("--no-histogram", action="store_true", help="skip the pairwise distance histogram measurement")
    ap.add_argument("--profile-run", action="store_true", help="only the warm-up and timed graph launches")
    ap.add_argument("--profile-batched", type=int, default=0, metavar="STEPS",
                    help="only STEPS plain steps of the 256-ensemble batching workload (for ncu captures)")
    ap.add_argument("--traffic-json", default=os.path.join(REPO, "profiles", "traffic.json"))
    args = ap.parse_args()
    if args.warmup < 0 or args.steps < 1:
        ap.error("--steps >= 1 and --warmup >= 0")
    if args.impl == "reference":
        run_reference(args)
    elif args.profile_batched:
        profile_batched(args.profile_batched)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
