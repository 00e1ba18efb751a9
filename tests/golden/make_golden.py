"""Generate the golden fixtures of tests/golden/ by running the reference's own code.

Run where a checkout of the reference is available, named by the LM_REFERENCE_DIR environment
variable (there is no default). The reference's Python modules are imported unmodified
with stub modules for the packages that are absent here (xarray, parcels); scipy's cKDTree is
the installed one. Outputs (small .npz files) are committed and read by the CPU tests; nothing at
test time reads the reference.

Fixtures:
  lattice.npz          utils.most_symmetric_integer_factorization and
                       particle_advecter.uniform_particle_locations (arrays or sha256 digests)
  kdtree_lattice.npz   cKDTree(X).query_pairs(r=0.01) pair counts + digests on the lattices
                       of the 10k / 490k / 1M configurations (float32 positions)
  kdtree_cases.npz     query_pairs on random, clustered, duplicate and boundary (+-ulp) cases,
                       p in {1, 2, inf}
  rps_rule.npz         rock_paper_scissors_interaction on every species pair and uniforms
                       around each threshold (np.random.rand patched)
  rps_replay.npz       sequential replay of a random pair list with Philox uniforms
  interaction_sim.npz  InteractionSimulator.time_step end to end (5 steps) with the pair order
                       and uniforms recorded
"""

from __future__ import annotations

import hashlib
import os
import shutil
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE = os.environ.get("LM_REFERENCE_DIR")
if not REFERENCE or not os.path.isdir(REFERENCE):
    raise SystemExit("set LM_REFERENCE_DIR to a checkout of ali-ramadhan/lagrangian-microbes")
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle  # noqa: E402  (Philox uniforms keyed by (seed, step, i, j))

_registry: dict = {}


def _install_stubs():
    xr = types.ModuleType("xarray")

    class Dataset:
        def __init__(self, data_vars=None, coords=None):
            self.vars = {k: v[1] for k, v in (data_vars or {}).items()}
            self.coords = coords or {}

        def __getitem__(self, k):
            return self.vars[k]

        def to_netcdf(self, path):
            _registry[os.path.abspath(path)] = self

    def open_dataset(path):
        return _registry[os.path.abspath(path)]

    xr.Dataset = Dataset
    xr.open_dataset = open_dataset
    sys.modules["xarray"] = xr
    sys.modules["parcels"] = types.ModuleType("parcels")


def _import_reference():
    work = tempfile.mkdtemp(prefix="lm_golden_")
    shutil.copy(os.path.join(REFERENCE, "logging.ini"), work)
    os.chdir(work)  # logging.ini opens its log file in the working directory
    _install_stubs()
    sys.path.insert(0, REFERENCE)
    import logging

    import interaction_simulator
    import interactions
    import particle_advecter
    import utils
    logging.disable(logging.CRITICAL)
    return utils, interactions, particle_advecter, interaction_simulator


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def packed_pairs(P) -> np.ndarray:
    arr = np.array(sorted(P), dtype=np.int64).reshape(-1, 2)
    return (arr[:, 0].astype(np.uint64) << np.uint64(32)) | arr[:, 1].astype(np.uint64)


def make_lattice(utils, pa):
    ns = [1, 2, 3, 7, 12, 36, 97, 100, 1000, 4096, 9991, 10000, 123456, 490000, 1000000]
    fac = np.array([utils.most_symmetric_integer_factorization(n) for n in ns], dtype=np.int64)
    out = {"ns": np.array(ns), "factorization": fac}
    small = [(12, 25, 26, 200, 201), (97, 20, 21, 195, 196), (10000, 25, 26, 200, 201)]
    for k, (n, a, b, c, d) in enumerate(small):
        lons, lats = pa.uniform_particle_locations(n, a, b, c, d)
        out[f"small{k}_args"] = np.array([n, a, b, c, d], dtype=np.float64)
        out[f"small{k}_lons"] = lons
        out[f"small{k}_lats"] = lats
    big = [(490000, 25, 30, 200, 205), (1000000, 25, 30, 200, 205)]
    digs = []
    for n, a, b, c, d in big:
        lons, lats = pa.uniform_particle_locations(n, a, b, c, d)
        digs.append([digest(lons), digest(lats)])
    out["big_args"] = np.array(big, dtype=np.float64)
    out["big_digests"] = np.array(digs)
    np.savez_compressed(os.path.join(HERE, "lattice.npz"), **out)


def make_kdtree_lattice(pa):
    from scipy.spatial import cKDTree
    cfg = [(10000, 25, 26, 200, 201), (490000, 25, 30, 200, 205), (1000000, 25, 30, 200, 205)]
    counts, digs = [], []
    for n, a, b, c, d in cfg:
        lons, lats = pa.uniform_particle_locations(n, a, b, c, d)
        X = np.stack((lons.astype(np.float32), lats.astype(np.float32)), axis=-1)
        P = cKDTree(np.array(X)).query_pairs(r=0.01, p=2)
        counts.append(len(P))
        digs.append(digest(packed_pairs(P)) if P else "")
    np.savez_compressed(os.path.join(HERE, "kdtree_lattice.npz"), configs=np.array(cfg, dtype=np.float64),
                        counts=np.array(counts, dtype=np.int64), digests=np.array(digs))


def boundary_points(rng, n_pairs, r, p, x0=(200.0, 25.0)):
    """Point pairs placed at distance ~r with +-few-ulp jitter (float32 coordinates)."""
    pts = []
    for _ in range(n_pairs):
        ax = np.float32(x0[0] + rng.random() * 5)
        ay = np.float32(x0[1] + rng.random() * 5)
        th = rng.random() * 2 * np.pi
        if p == 2:
            bx, by = ax + r * np.cos(th), ay + r * np.sin(th)
        elif p == 1:
            t = rng.random()
            bx, by = ax + r * t * np.sign(np.cos(th)), ay + r * (1 - t) * np.sign(np.sin(th))
        else:
            bx, by = ax + r * np.sign(np.cos(th)), ay + r * rng.uniform(-1, 1)
        bx = np.float32(bx)
        by = np.float32(by)
        for _ in range(int(rng.integers(-3, 4))):
            bx = np.nextafter(bx, np.float32(np.inf) if rng.random() < 0.5 else np.float32(-np.inf))
        for _ in range(int(rng.integers(-3, 4))):
            by = np.nextafter(by, np.float32(np.inf) if rng.random() < 0.5 else np.float32(-np.inf))
        pts += [(ax, ay), (bx, by)]
    return np.array(pts, dtype=np.float32)


def make_kdtree_cases():
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(20240601)
    cases = []
    for p in (2, 1, np.inf):
        X = np.stack([200 + rng.random(3000) * 0.2, 25 + rng.random(3000) * 0.2], -1).astype(np.float32)
        cases.append(("uniform", X, 0.01, p))
    for p in (2, 1, np.inf):
        cases.append(("boundary", boundary_points(rng, 1500, 0.01, p), 0.01, p))
    centers = np.stack([200 + rng.random(8) * 0.5, 25 + rng.random(8) * 0.5], -1)
    X = (centers[rng.integers(0, 8, 2000)] + rng.normal(0, 0.015, (2000, 2))).astype(np.float32)
    cases.append(("clustered", X, 0.01, 2))
    X = np.repeat(np.array([[201.0, 26.0], [201.005, 26.0], [201.02, 26.0]], np.float32), [5, 3, 2], axis=0)
    cases.append(("duplicates", X, 0.005, 2))
    cases.append(("single", np.array([[200.0, 25.0]], np.float32), 0.01, 2))
    X = np.stack([195 + rng.random(2000) * 20, 20 + rng.random(2000) * 15], -1).astype(np.float32)
    cases.append(("sparse_wide", X, 0.05, 2))
    out = {"n_cases": np.array(len(cases))}
    for k, (name, X, r, p) in enumerate(cases):
        P = cKDTree(np.array(X)).query_pairs(r=r, p=p)
        arr = np.array(sorted(P), dtype=np.int64).reshape(-1, 2)
        out[f"c{k}_name"] = np.array(name)
        out[f"c{k}_X"] = X
        out[f"c{k}_r"] = np.array(r)
        out[f"c{k}_p"] = np.array(p)
        out[f"c{k}_pairs"] = arr
    np.savez_compressed(os.path.join(HERE, "kdtree_cases.npz"), **out)


class _RandPatch:
    """np.random.rand replacement: returns the uniform of the pair currently being applied."""

    def __init__(self):
        self.value = None
        self.calls = 0

    def __call__(self, *args):
        assert not args and self.value is not None
        self.calls += 1
        return self.value


def make_rps_rule(interactions):
    patch = _RandPatch()
    orig = np.random.rand
    np.random.rand = patch
    try:
        params = {"pRS": 0.5, "pPR": 0.7, "pSP": 0.6}
        rows = []
        for s1 in (1, 2, 3):
            for s2 in (1, 2, 3):
                for p in (0.5, 0.7, 0.6):
                    t = oracle.prob_threshold(p)
                    for u53 in sorted({0, t - 1, t, t + 1, (1 << 53) - 1, 1 << 52}):
                        if not 0 <= u53 < (1 << 53):
                            continue
                        sp = np.array([s1, s2], dtype=np.int8)
                        patch.value = u53 * 2.0 ** -53
                        patch.calls = 0
                        interactions.rock_paper_scissors_interaction(params, {"species": sp}, 0, 1)
                        rows.append([s1, s2, u53, sp[0], sp[1], patch.calls])
    finally:
        np.random.rand = orig
    np.savez_compressed(os.path.join(HERE, "rps_rule.npz"), params=np.array([0.5, 0.7, 0.6]),
                        rows=np.array(rows, dtype=np.uint64))


def make_rps_replay(interactions):
    rng = np.random.default_rng(7)
    n, m, step, seed = 500, 3000, 17, 0x1234_5678_9ABC_DEF0
    species = rng.integers(1, 4, n).astype(np.int8)
    i = rng.integers(0, n, m)
    j = rng.integers(0, n, m)
    keep = i != j
    pi, pj = np.minimum(i, j)[keep], np.maximum(i, j)[keep]
    params = {"pRS": 0.55, "pPR": 0.8, "pSP": 0.65}
    patch = _RandPatch()
    orig = np.random.rand
    np.random.rand = patch
    try:
        sp = species.copy()
        for a, b in zip(pi, pj):
            patch.value = oracle.pair_uniform(int(a), int(b), step, seed)
            interactions.rock_paper_scissors_interaction(params, {"species": sp}, int(a), int(b))
    finally:
        np.random.rand = orig
    np.savez_compressed(os.path.join(HERE, "rps_replay.npz"), species0=species, pi=pi, pj=pj, step=np.array(step),
                        seed=np.array(seed, dtype=np.uint64), params=np.array([0.55, 0.8, 0.65]), species1=sp)


def make_interaction_sim(interactions, isim_mod):
    from datetime import datetime, timedelta
    rng = np.random.default_rng(11)
    n, nt = 400, 5
    lon = np.empty((n, nt), np.float32)
    lat = np.empty((n, nt), np.float32)
    x = 200 + rng.random(n) * 0.15
    y = 25 + rng.random(n) * 0.15
    for t in range(nt):
        x = x + rng.normal(0, 0.004, n)
        y = y + rng.normal(0, 0.004, n)
        lon[:, t] = x
        lat[:, t] = y
    ds = sys.modules["xarray"].Dataset({"longitude": (["particle number", "time"], lon),
                                        "latitude": (["particle number", "time"], lat)})
    adv = tempfile.mkdtemp(prefix="lm_adv_")
    ds.to_netcdf(os.path.join(adv, "particle_data.nc"))
    np.random.seed(3)
    fn, params, props = interactions.rock_paper_scissors(n, 0.6, 0.7, 0.8)
    species0 = props["species"].copy()
    seed = 0xC0FFEE
    patch = _RandPatch()
    order = []
    state = {"step": 0}

    def recording_rule(parameters, microbe_properties, p1, p2):
        order.append((state["step"], int(p1), int(p2)))
        patch.value = oracle.pair_uniform(int(p1), int(p2), state["step"], seed)
        return fn(parameters, microbe_properties, p1, p2)

    sim = isim_mod.InteractionSimulator(pair_interaction=(recording_rule, params, props), interaction_radius=0.02,
                                        advection_dir=adv, output_dir=adv)
    orig_rand = np.random.rand
    np.random.rand = patch
    # track the step index the reference is on while its loop runs
    orig_stack = np.stack

    def stack_and_mark(arrs, axis=0):
        state["step"] = sim.iteration
        return orig_stack(arrs, axis=axis)

    isim_mod.stack = stack_and_mark
    try:
        start = datetime(2017, 1, 1)
        sim.time_step(start, start + nt * timedelta(hours=1), timedelta(hours=1))
    finally:
        np.random.rand = orig_rand
        isim_mod.stack = orig_stack
    out = _registry[os.path.abspath(os.path.join(adv, "microbe_data.nc"))]
    order = np.array(order, dtype=np.int64).reshape(-1, 3)
    np.savez_compressed(os.path.join(HERE, "interaction_sim.npz"), lon=lon, lat=lat, species0=species0,
                        species=out["species"], order=order, radius=np.array(0.02), seed=np.array(seed, np.uint64),
                        params=np.array([0.6, 0.7, 0.8]))


def main():
    utils, interactions, pa, isim = _import_reference()
    make_lattice(utils, pa)
    make_kdtree_lattice(pa)
    make_kdtree_cases()
    make_rps_rule(interactions)
    make_rps_replay(interactions)
    make_interaction_sim(interactions, isim)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
