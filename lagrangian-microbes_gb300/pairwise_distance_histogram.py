"""Pairwise great-circle distance histograms on the GPU.

Counterpart of the reference's sandbox scripts sandbox/pairwise_distance_histogram_distributed.jl
(haversine_distance32 :35-46, pairwise_distance_histogram_1point / _parallel :56-76, one
histogram per species in plot_pairwise_histogram :93-147) and
sandbox/pairwise_distance_histogram_gpu.jl. Every unordered pair of points (of one species) gets
the float32 haversine distance d of haversine_distance32 and is counted in bin
round(10 log10(max(1, d))) (ties to even, as Julia's round), i.e. tenths of a decade in metres.

Bins: ``counts[k]`` holds bin k for 0 <= k < bins, and the returned ``overflow`` the pairs whose bin
is bins or more. The Julia code stores bin k at its 1-based index k, so its array equals
``counts[1:bins]`` followed by nothing for bin 0 (it writes bin 0 and bins past the end out of
bounds); pass bins one larger to cover its last index.

All pairs are computed by lm_distance_histogram (csrc/k_hist.cu); there is no CPU path.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .interactions import PAPER, ROCK, SCISSORS

R64 = 6371.228e3  # mean Earth radius of the reference [m]
R32 = np.float32(6371.228e3)


def _histograms(lats, lons, seg, bins: int, radius: float, device: int, ctx):
    lats = np.ascontiguousarray(lats, dtype=np.float32).ravel()
    lons = np.ascontiguousarray(lons, dtype=np.float32).ravel()
    if lats.size != lons.size:
        raise ValueError("lats and lons differ in length")
    seg = np.ascontiguousarray(seg, dtype=np.int64)
    n_seg = seg.size - 1
    counts = np.zeros((n_seg, bins + 1), np.uint64)
    own = ctx is None
    ctx = ctx or _lib.Context(device)
    try:
        ctx.call("lm_distance_histogram", _lib.ptr(lats), _lib.ptr(lons), lats.size, _lib.ptr(seg), n_seg, int(bins),
                 float(radius), _lib.ptr(counts))
    finally:
        if own:
            ctx.close()
    return counts.astype(np.int64)


def pairwise_distance_histogram(lats, lons, bins: int = 70, radius: float = R32, *, device: int = 0,
                                ctx: _lib.Context | None = None):
    """Histogram of all pairwise distances: (counts[bins], overflow). Latitude first, as the reference."""
    n = np.asarray(lats).size
    c = _histograms(lats, lons, [0, n], bins, radius, device, ctx)[0]
    return c[:bins], int(c[bins])


def pairwise_distance_histogram_parallel(lats, lons, bins: int, R: float = R32):
    """The reference's name (sandbox/pairwise_distance_histogram_distributed.jl:68): the summed
    histogram of all pairs, bins 0 .. bins-1 (pairs past the last bin are dropped, as there)."""
    return pairwise_distance_histogram(lats, lons, bins, R)[0]


def species_distance_histograms(lons, lats, species, bins: int = 70, radius: float = R32, *, device: int = 0,
                                ctx: _lib.Context | None = None):
    """One histogram per species (rock, paper, scissors), pairs within a species only, as
    plot_pairwise_histogram (:130-147); one launch for the three. Returns {species: (counts, overflow)}."""
    lons = np.asarray(lons, dtype=np.float32).ravel()
    lats = np.asarray(lats, dtype=np.float32).ravel()
    species = np.asarray(species).ravel()
    if not (lons.size == lats.size == species.size):
        raise ValueError("lons, lats and species differ in length")
    kinds = (ROCK, PAPER, SCISSORS)
    order = np.concatenate([np.flatnonzero(species == k) for k in kinds])
    sizes = [int(np.count_nonzero(species == k)) for k in kinds]
    seg = np.concatenate([[0], np.cumsum(sizes)])
    c = _histograms(lats[order], lons[order], seg, bins, radius, device, ctx)
    return {k: (c[s, :bins], int(c[s, bins])) for s, k in enumerate(kinds)}
