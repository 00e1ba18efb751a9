"""Pairwise distance histogram on the GPU (lm_distance_histogram) against the oracle.

The GPU evaluates haversine_distance32 in float32 (as the reference); the oracle in float64 marks
the pairs within 1e-4 (in units of 10 log10 d) of a bin boundary as ambiguous, and the GPU
histogram must put every other pair in the oracle's bin and each ambiguous pair on one side of its
boundary (histogram_consistent). At sizes the oracle cannot finish, size-independent properties:
the total is n (n - 1) / 2 per segment, repeated calls agree, and shuffling the points moves a
few pairs by one bin at most (the float32 formula is not symmetric in its two points).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pdh():
    from lagrangian_microbes_gb300 import pairwise_distance_histogram as m
    return m


def _points(rng, n, box=(20.0, 40.0, 20.0, 40.0)):
    # the reference's random_points: lats and lons uniform in [20, 40) degrees
    lat = (box[0] + (box[1] - box[0]) * rng.random(n)).astype(np.float32)
    lon = (box[2] + (box[3] - box[2]) * rng.random(n)).astype(np.float32)
    return lat, lon


def _full(counts, overflow):
    return np.concatenate([counts, [overflow]])


def test_random_points_match_oracle(pdh, orc):
    rng = np.random.default_rng(11)
    lat, lon = _points(rng, 3000)
    counts, over = pdh.pairwise_distance_histogram(lat, lon, 70)
    d, a = orc.distance_histogram(lat, lon, 70)
    assert orc.histogram_consistent(_full(counts, over), d, a)
    assert counts.sum() + over == 3000 * 2999 // 2


def test_patch_with_duplicates_and_close_points_match_oracle(pdh, orc):
    rng = np.random.default_rng(12)
    # a 5-degree patch like the 490k lattice, with exact duplicates and sub-metre neighbours
    lat, lon = _points(rng, 2500, box=(25.0, 30.0, 200.0, 205.0))
    lat[100:140] = lat[99]
    lon[100:140] = lon[99]
    lat[200:260] = lat[199] + np.float32(3e-6) * np.arange(60, dtype=np.float32)
    lon[200:260] = lon[199]
    counts, over = pdh.pairwise_distance_histogram(lat, lon, 70)
    d, a = orc.distance_histogram(lat, lon, 70)
    assert orc.histogram_consistent(_full(counts, over), d, a)
    assert counts[0] >= 41 * 40 // 2


def test_whole_globe_overflow_and_small_bin_counts(pdh, orc):
    rng = np.random.default_rng(13)
    lat = rng.uniform(-89, 89, 1500).astype(np.float32)
    lon = rng.uniform(-180, 180, 1500).astype(np.float32)
    lat[:2] = [0, 0]
    lon[:2] = [0, 180]  # antipodal: a = 1, d = pi R
    for bins in (70, 72, 1, 256):
        counts, over = pdh.pairwise_distance_histogram(lat, lon, bins)
        d, a = orc.distance_histogram(lat, lon, bins)
        assert orc.histogram_consistent(_full(counts, over), d, a), bins
        if bins == 70:
            assert over > 0  # bins 70-73 (d >= 9.7e6 m) exist on the whole globe
        if bins == 256:
            assert over == 0


def test_species_histograms_are_per_species_pairs(pdh, orc):
    rng = np.random.default_rng(14)
    lat, lon = _points(rng, 2400, box=(25.0, 30.0, 200.0, 205.0))
    species = rng.integers(1, 4, lat.size).astype(np.int8)
    got = pdh.species_distance_histograms(lon, lat, species, 70)
    for k in (1, 2, 3):
        sel = species == k
        d, a = orc.distance_histogram(lat[sel], lon[sel], 70)
        counts, over = got[k]
        assert orc.histogram_consistent(_full(counts, over), d, a), k
        c1, o1 = pdh.pairwise_distance_histogram(lat[sel], lon[sel], 70)
        np.testing.assert_array_equal(c1, counts)  # one segment alone gives the same bins
        assert o1 == over


def test_edge_cases(pdh, lm):
    for n in (0, 1):
        counts, over = pdh.pairwise_distance_histogram(np.zeros(n, np.float32), np.zeros(n, np.float32), 70)
        assert counts.sum() == 0 and over == 0
    counts, over = pdh.pairwise_distance_histogram(np.full(300, 10, np.float32), np.full(300, 20, np.float32), 70)
    assert counts[0] == 300 * 299 // 2 and counts[1:].sum() == 0 and over == 0
    lat = np.array([1.0, np.nan], np.float32)
    with pytest.raises(lm.LMError):
        pdh.pairwise_distance_histogram(lat, np.zeros(2, np.float32), 70)
    with pytest.raises(lm.LMError):
        pdh.pairwise_distance_histogram(np.zeros(4, np.float32), np.zeros(4, np.float32), 0)
    with pytest.raises(lm.LMError):
        pdh.pairwise_distance_histogram(np.zeros(4, np.float32), np.zeros(4, np.float32), 257)


def test_large_totals_and_shuffle_invariance(pdh):
    rng = np.random.default_rng(15)
    n = 200_000  # 2.0e10 pairs
    lat, lon = _points(rng, n, box=(25.0, 30.0, 200.0, 205.0))
    counts, over = pdh.pairwise_distance_histogram(lat, lon, 70)
    assert counts.sum() + over == n * (n - 1) // 2
    again, o_again = pdh.pairwise_distance_histogram(lat, lon, 70)
    np.testing.assert_array_equal(counts, again)
    assert over == o_again
    # haversine_distance32 takes the lower index first and is not symmetric in float32 (the
    # products c1 c2 round in order), so shuffling may move a pair to the next bin: only a few,
    # only across one boundary
    p = rng.permutation(n)
    c2, o2 = pdh.pairwise_distance_histogram(lat[p], lon[p], 70)
    moved = np.abs(np.cumsum(np.concatenate([counts - c2, [over - o2]])))
    assert moved[-1] == 0 and moved.max() <= 1e-7 * n * (n - 1) / 2
    # segments: the three species' pairs plus the cross pairs make all pairs
    species = rng.integers(1, 4, n).astype(np.int8)
    got = pdh.species_distance_histograms(lon, lat, species, 70)
    sizes = [int((species == k).sum()) for k in (1, 2, 3)]
    for k, m in zip((1, 2, 3), sizes):
        assert got[k][0].sum() + got[k][1] == m * (m - 1) // 2


def test_short_route_gives_the_reference_chain_bins(pdh, monkeypatch):
    """Most pairs take the short route (polynomial sin/asin, hardware log2) unless they lie near a
    bin boundary or outside its range; the bins must be exactly those of the reference chain for
    every pair (LM_HIST_EXACT=1 makes every pair take the reference chain)."""
    rng = np.random.default_rng(16)
    cases = [_points(rng, 20_000, box=(25.0, 30.0, 200.0, 205.0)),                      # 2e8 pairs, all short
             (rng.uniform(-89, 89, 6000).astype(np.float32), rng.uniform(-180, 180, 6000).astype(np.float32)),
             ((30 + 1e-4 * rng.random(3000)).astype(np.float32), (150 + 1e-4 * rng.random(3000)).astype(np.float32))]
    for lat, lon in cases:  # a 5-degree patch, the whole globe, a sub-10-m cluster (d around 1-15 m)
        fast = pdh.pairwise_distance_histogram(lat, lon, 80)
        monkeypatch.setenv("LM_HIST_EXACT", "1")
        exact = pdh.pairwise_distance_histogram(lat, lon, 80)
        monkeypatch.delenv("LM_HIST_EXACT")
        np.testing.assert_array_equal(fast[0], exact[0])
        assert fast[1] == exact[1]
