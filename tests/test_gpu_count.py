"""Count-only pair search (lm_count_pairs, LM_STEP_COUNT_PAIRS): the clustered stress workload.

The count must equal the size of cKDTree.query_pairs (golden lattice counts and boundary cases)
and the oracle's count on clustered positions whose cells hold thousands of microbes (the
shared-memory tiles of k_count_pairs), and the fused count step must count the pairs of exactly
the positions it advected.
"""

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from lagrangian_microbes_gb300 import engine as e
    return e


def clusters(rng, n_clusters, per, sigma, box=(200.0, 203.0, 25.0, 28.0)):
    cx = box[0] + (box[1] - box[0]) * rng.random(n_clusters)
    cy = box[2] + (box[3] - box[2]) * rng.random(n_clusters)
    sizes = np.maximum(1, (per * (np.arange(1, n_clusters + 1) ** -1.2) / np.mean(np.arange(1, n_clusters + 1) ** -1.2)).astype(int))
    lon = np.concatenate([c + sigma * rng.standard_normal(s) for c, s in zip(cx, sizes)])
    lat = np.concatenate([c + sigma * rng.standard_normal(s) for c, s in zip(cy, sizes)])
    return lon.astype(np.float32), lat.astype(np.float32)


def test_count_matches_ckdtree_lattices(engine, orc):
    g = golden("kdtree_lattice.npz")
    q = engine.PairQuery(0.01, 2)
    for (n, a, b, c, d), count in zip(g["configs"], g["counts"]):
        lons, lats = orc.lattice(int(n), a, b, c, d)
        assert q.count(lons.astype(np.float32), lats.astype(np.float32)) == count
    q.ctx.close()


def test_count_matches_ckdtree_boundary_cases(engine):
    g = golden("kdtree_cases.npz")
    for k in range(int(g["n_cases"])):
        X, r, p = g[f"c{k}_X"], float(g[f"c{k}_r"]), float(g[f"c{k}_p"])
        q = engine.PairQuery(r, p)
        assert q.count(X[:, 0], X[:, 1]) == len(g[f"c{k}_pairs"]), str(g[f"c{k}_name"])
        q.ctx.close()


@pytest.mark.parametrize("p", [2, 1, np.inf])
def test_count_dense_clusters_match_oracle(engine, orc, p):
    rng = np.random.default_rng(41)
    # Zipf-sized Gaussian clusters, sigma = 3 km: cores hold thousands of microbes per 0.01 deg cell
    lon, lat = clusters(rng, 40, 8000, 0.03)
    lon[::4001] = np.nan  # non-finite points are never paired
    q = engine.PairQuery(0.01, p)
    got = q.count(lon, lat)
    q.ctx.close()
    assert got == orc.count_pairs(lon, lat, 0.01, p)
    assert got > 1_000_000


def test_count_agrees_with_listed_pairs(engine, orc):
    rng = np.random.default_rng(43)
    lon, lat = clusters(rng, 12, 2500, 0.02)
    q = engine.PairQuery(0.01, 2)
    pi, pj = q.pairs(lon, lat)
    assert q.count(lon, lat) == pi.size == orc.count_pairs(lon, lat, 0.01, 2)
    q.ctx.close()


def test_fused_count_step_counts_the_advected_positions(engine, lm, orc, small_field):
    rng = np.random.default_rng(44)
    lon, lat = clusters(rng, 20, 3000, 0.03, box=(199.0, 202.0, 24.0, 27.0))
    sim = engine.Simulation(small_field, lon.astype(np.float64), lat.astype(np.float64),
                            np.ones(lon.size, np.int8), radius=0.01)
    totals = []
    for k in range(3):
        rec = sim.step(float(small_field.times[0]) + 3600.0 * k, 3600.0, 1, record=True, count_pairs=True)
        want = orc.count_pairs(rec["lon"][0], rec["lat"][0], 0.01, 2)
        st = sim.stats()
        assert st["pairs"] == want
        totals.append(want)
    assert sim.stats()["pairs_total"] == sum(totals)
    _, _, sp, _ = sim.state()
    assert (sp == 1).all()  # counting leaves the species alone
    sim.close()
