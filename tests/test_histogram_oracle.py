"""Oracle of the pairwise distance histogram (sandbox/pairwise_distance_histogram_distributed.jl).

Pins orc_haversine to known distances and to an independent float64 formula (the atan2 form of
the haversine), and the all-pairs histogram to a numpy brute force; checks the consistency rule
that the GPU tests apply (every ambiguous pair on one side of its boundary).
"""

import math

import numpy as np
import pytest

R = 6371.228e3


def _atan2_haversine(lat1, lon1, lat2, lon2):
    p1, p2 = np.radians(lat1), np.radians(lat2)
    dp, dl = p2 - p1, np.radians(lon2 - lon1)
    a = np.sin(dp / 2) ** 2 + np.cos(p1) * np.cos(p2) * np.sin(dl / 2) ** 2
    return R * 2 * np.arctan2(np.sqrt(a), np.sqrt(1 - a))


def test_haversine_known_distances(orc):
    assert orc.haversine(0, 0, 0, 1) == pytest.approx(R * math.pi / 180, rel=1e-13)
    assert orc.haversine(10, 30, 11, 30) == pytest.approx(R * math.pi / 180, rel=1e-13)
    assert orc.haversine(0, 0, 0, 180) == pytest.approx(R * math.pi, rel=1e-13)
    assert orc.haversine(45, 7, 45, 7) == 0.0
    # the two distances the reference's plotting marks (plot_pairwise_histogram, :148-149)
    assert orc.haversine(30, -150, 30, -150.01) == pytest.approx(963.0108, abs=1e-3)
    assert orc.haversine(25, -145, 35, -155) == pytest.approx(1469218.09, abs=0.1)


def test_haversine_matches_the_atan2_form(orc):
    rng = np.random.default_rng(3)
    for _ in range(200):
        la1, la2 = rng.uniform(-80, 80, 2)
        lo1, lo2 = rng.uniform(-180, 180, 2)
        want = float(_atan2_haversine(la1, lo1, la2, lo2))
        assert orc.haversine(la1, lo1, la2, lo2) == pytest.approx(want, rel=1e-9, abs=1e-6)


def test_histogram_matches_brute_force(orc):
    rng = np.random.default_rng(5)
    n, bins = 300, 70
    lat = (20 + 20 * rng.random(n)).astype(np.float32)
    lon = (20 + 20 * rng.random(n)).astype(np.float32)
    lat[:5] = lat[5]  # duplicates: distance 0 -> bin 0
    lon[:5] = lon[5]
    i, j = np.triu_indices(n, 1)
    d = _atan2_haversine(lat[i].astype(np.float64), lon[i].astype(np.float64), lat[j].astype(np.float64),
                         lon[j].astype(np.float64))
    x = 10 * np.log10(np.maximum(1.0, d))
    want = np.bincount(np.minimum(np.rint(x).astype(np.int64), bins), minlength=bins + 1)
    definite, amb = orc.distance_histogram(lat, lon, bins, delta=1e-4)
    assert definite.sum() + amb.sum() == n * (n - 1) // 2
    assert orc.histogram_consistent(want, definite, amb)
    assert definite[0] >= 10  # the 15 pairs among the 6 equal points
    # the rule rejects a histogram with one pair moved where no boundary is ambiguous
    bad = want.copy()
    bad[0] -= 1
    bad[1] += 1
    assert amb[0] == 0 and not orc.histogram_consistent(bad, definite, amb)
    bad = want.copy()
    bad[-1] += 1  # a pair too many
    assert not orc.histogram_consistent(bad, definite, amb)


def test_histogram_overflow_and_ambiguity(orc):
    lat = np.array([0, 0, 0], np.float32)
    lon = np.array([0, 180, 90], np.float32)  # pi R (bin 73) once, pi R / 2 (bin 70) twice
    definite, amb = orc.distance_histogram(lat, lon, 72, delta=1e-4)
    assert definite[72] == 1 and definite[70] == 2  # bin 73 is past a 72-bin histogram: overflow
    assert amb.sum() == 0
    # x = 70.0034 lies within 1e-2 of no boundary, 73.0137 neither
    definite, amb = orc.distance_histogram(lat, lon, 80, delta=0.6)
    assert amb[69] + amb[70] == 2 and amb[72] + amb[73] == 1  # a wide band makes every pair ambiguous
