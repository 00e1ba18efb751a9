"""Pair counting for callers that cannot allocate device memory.

lm_count_pairs_noalloc takes device pointers from its caller (here torch tensors stand in for a
host application's own buffers) and allocates nothing; its scratch is a fixed array inside the
library. Its counts must equal those of the allocating pair query, lm_query_pairs, on every call,
also when the same scratch is reused by a second call with different inputs.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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
