"""Pair counting for callers that cannot allocate device memory.

lm_count_pairs_noalloc serves hosts whose device memory all belongs to their own pool allocator
and plugins that may not allocate after start-up: it takes device pointers from its caller (here
torch tensors stand in for a host application's own buffers) and allocates nothing; its scratch
is a fixed array inside the library. Its counts must equal those of the allocating pair query,
lm_query_pairs, on every call, also when the same scratch is reused by a second call with
different inputs, and those of scipy's cKDTree on the golden cases (all three norms, boundary,
clustered and duplicate points).
"""

import numpy as np
import pytest
from conftest import golden

pytestmark = pytest.mark.gpu


def _noalloc(lib, torch, lon, lat, r, p, stream):
    from lagrangian_microbes_gb300 import _lib
    from lagrangian_microbes_gb300.engine import norm_code
    n = lon.size
    d_lon = torch.from_numpy(np.ascontiguousarray(lon, np.float32)).cuda()
    d_lat = torch.from_numpy(np.ascontiguousarray(lat, np.float32)).cuda()
    d_deg = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    d_pairs = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.lm_count_pairs_noalloc(d_lon.data_ptr(), d_lat.data_ptr(), n, r, norm_code(p), d_deg.data_ptr(),
                                    d_pairs.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    assert rc == _lib.LM_OK
    return int(d_pairs.item()), d_deg.cpu().numpy()[:n]


def _reference_counts(lon, lat, r, p):
    from lagrangian_microbes_gb300.engine import PairQuery
    q = PairQuery(r, p)
    pi, pj = q.pairs(lon, lat)
    q.ctx.close()
    n = lon.size
    return pi.size, np.bincount(pi, minlength=n) + np.bincount(pj, minlength=n)


def test_noalloc_pair_count_matches_query_pairs_on_two_calls():
    torch = pytest.importorskip("torch")
    from lagrangian_microbes_gb300 import _lib
    from lagrangian_microbes_gb300.engine import norm_code

    lib = _lib.load()
    rng = np.random.default_rng(17)
    stream = torch.cuda.Stream()
    cases = [(60000, 0.5, 0.01, 2), (30000, 0.25, 0.008, 1)]  # two calls in a row, different inputs
    for n, box, r, p in cases:
        lon = (200 + rng.random(n) * box).astype(np.float32)
        lat = (25 + rng.random(n) * box).astype(np.float32)
        lon[::997] = np.nan  # non-finite points are never paired
        d_lon = torch.from_numpy(lon).cuda()
        d_lat = torch.from_numpy(lat).cuda()
        d_deg = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        d_pairs = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.lm_count_pairs_noalloc(d_lon.data_ptr(), d_lat.data_ptr(), n, r, norm_code(p), d_deg.data_ptr(),
                                        d_pairs.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        assert rc == _lib.LM_OK
        want_pairs, want_deg = _reference_counts(lon, lat, r, p)
        assert int(d_pairs.item()) == want_pairs
        np.testing.assert_array_equal(d_deg.cpu().numpy(), want_deg)


def test_noalloc_rejects_more_points_than_its_scratch_holds():
    torch = pytest.importorskip("torch")
    import ctypes

    from lagrangian_microbes_gb300 import _lib

    lib = _lib.load()
    d_pairs = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = lib.lm_count_pairs_noalloc(None, None, 70000, 0.01, 2, None, d_pairs.data_ptr(), 0)
    assert rc == _lib.LM_ERR_ARG
    buf = ctypes.create_string_buffer(256)
    lib.lm_last_error(None, buf, 256)
    assert b"65536" in buf.value


def test_noalloc_pair_count_matches_ckdtree_golden_cases():
    torch = pytest.importorskip("torch")
    from lagrangian_microbes_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.Stream()
    g = golden("kdtree_cases.npz")
    for k in range(int(g["n_cases"])):
        X, r, p = g[f"c{k}_X"], float(g[f"c{k}_r"]), float(g[f"c{k}_p"])
        want = g[f"c{k}_pairs"]
        n = X.shape[0]
        pairs, deg = _noalloc(lib, torch, X[:, 0], X[:, 1], r, p, stream)
        assert pairs == want.shape[0], str(g[f"c{k}_name"])
        np.testing.assert_array_equal(deg, np.bincount(want.ravel(), minlength=n), err_msg=str(g[f"c{k}_name"]))


def test_noalloc_call_leaves_free_device_memory_unchanged():
    torch = pytest.importorskip("torch")
    from lagrangian_microbes_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(3)
    lon = (200 + rng.random(50000) * 0.5).astype(np.float32)
    lat = (25 + rng.random(50000) * 0.5).astype(np.float32)
    want, _ = _reference_counts(lon, lat, 0.01, np.inf)
    d_lon = torch.from_numpy(lon).cuda()
    d_lat = torch.from_numpy(lat).cuda()
    d_deg = torch.zeros(lon.size, dtype=torch.int32, device="cuda")
    d_pairs = torch.zeros(1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    counts = []
    free = []
    for _ in range(3):
        free.append(torch.cuda.mem_get_info()[0])
        rc = lib.lm_count_pairs_noalloc(d_lon.data_ptr(), d_lat.data_ptr(), lon.size, 0.01, _lib.NORM_INF,
                                        d_deg.data_ptr(), d_pairs.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        assert rc == _lib.LM_OK
        counts.append(int(d_pairs.item()))
    free.append(torch.cuda.mem_get_info()[0])
    assert counts == [want] * 3
    assert len(set(free[1:])) == 1, free  # after the first call's set-up nothing is allocated
