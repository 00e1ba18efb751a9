"""Host-side logic and the C-ABI library surface (no GPU needed)."""

import ctypes
import os
import re
from datetime import datetime, timedelta

import numpy as np
import pytest
from conftest import REPO


def _declared_symbols():
    with open(os.path.join(REPO, "include", "lm_api.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^int\s+(lm_\w+)\s*\(", text, flags=re.M)))


def test_library_builds_and_exports_every_declared_symbol(lm):
    from lagrangian_microbes_gb300 import _lib
    lib = _lib.load()
    declared = _declared_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(_lib.SIGNATURES), "ctypes signatures must cover exactly the header"
    assert lib.lm_version() == 1


def _header_text():
    with open(os.path.join(REPO, "include", "lm_api.h")) as f:
        return re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)


def test_python_binding_matches_the_header(lm):
    # every declared entry is bound with as many arguments as the header declares (no drift
    # between include/lm_api.h and the ctypes binding)
    from lagrangian_microbes_gb300 import _lib
    protos = {}
    for m in re.finditer(r"^int\s+(lm_\w+)\s*\((.*?)\)\s*;", _header_text(), flags=re.M | re.S):
        args = m.group(2).strip()
        protos[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    assert set(protos) == set(_lib.SIGNATURES), sorted(set(protos) ^ set(_lib.SIGNATURES))
    for name, argtypes in _lib.SIGNATURES.items():
        assert len(argtypes) == protos[name], name


def test_stats_struct_matches_the_header(lm):
    from lagrangian_microbes_gb300 import _lib
    body = re.search(r"typedef struct lm_stats \{(.*?)\} lm_stats;", _header_text(), flags=re.S).group(1)
    fields = re.findall(r"int64_t\s+(\w+)(?:\[(\d+)\])?;", body)
    assert [(n, int(k or 1)) for n, k in fields] == [
        (n, getattr(t, "_length_", 1)) for n, t in _lib.Stats._fields_]
    assert ctypes.sizeof(_lib.Stats) == 8 * sum(int(k or 1) for _, k in fields)


def test_missing_library_fails_loudly(lm, monkeypatch, tmp_path):
    # no CPU fallback: without the CUDA library every entry point raises
    from lagrangian_microbes_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib._build, "LIB_PATH", str(tmp_path / "liblmgb300.so"))
    with pytest.raises(_lib.LMError, match="missing"):
        _lib.load(build_if_missing=False)


def test_library_is_built_for_sm103a_only(lm):
    # one -gencode, sm_103a, for every translation unit and the link (the GPU tests check at run
    # time that the loaded kernels report binary version 103: test_gpu_state.py)
    from lagrangian_microbes_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert not any("gencode" in f or "arch=" in f for f in build.NVCC_FLAGS)


def test_context_without_gpu_fails_cleanly(lm):
    from lagrangian_microbes_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.lm_ctx_create(0, ctypes.byref(h))
    if rc == _lib.LM_OK:
        lib.lm_ctx_destroy(h)
        pytest.skip("a GPU is present")
    assert rc in (_lib.LM_ERR_CUDA, _lib.LM_ERR_ARG)
    buf = ctypes.create_string_buffer(256)
    lib.lm_last_error(None, buf, 256)
    assert buf.value
    with pytest.raises(_lib.LMError):
        _lib.Context(0)


def test_null_context_is_rejected(lm):
    from lagrangian_microbes_gb300 import _lib
    lib = _lib.load()
    assert lib.lm_sync(None) == _lib.LM_ERR_ARG
    assert lib.lm_step(None, 0.0, 1.0, 1, 0, 1, 0.0, None, None, None, None) == _lib.LM_ERR_ARG


def test_norm_codes(lm):
    from lagrangian_microbes_gb300.engine import norm_code
    assert norm_code(2) == 2 and norm_code(1) == 1 and norm_code(np.inf) == 0 and norm_code(float("inf")) == 0
    with pytest.raises(ValueError):
        norm_code(3)


def test_rock_paper_scissors_surface(lm):
    np.random.seed(0)
    fn, params, props = lm.rock_paper_scissors(1000, 0.5, 0.6, 0.7)
    sp = props["species"]
    assert sp.dtype == np.int8 and set(np.unique(sp)) <= {1, 2, 3}
    assert (params["pRS"], params["pPR"], params["pSP"]) == (0.5, 0.6, 0.7)
    np.random.seed(0)
    fn2, params2, props2 = lm.rock_paper_scissors(1000, 0.5, 0.6, 0.7)
    np.testing.assert_array_equal(sp, props2["species"])
    assert params["seed"] == params2["seed"]
    assert fn is lm.rock_paper_scissors_interaction
    with pytest.raises(NotImplementedError):
        fn(params, props, 0, 1)
    assert (lm.ROCK, lm.PAPER, lm.SCISSORS) == (1, 2, 3)


def test_interaction_simulator_rejects_other_rules(lm, tmp_path):
    from lagrangian_microbes_gb300.interaction_simulator import InteractionSimulator
    with pytest.raises(NotImplementedError):
        InteractionSimulator((lambda *a: None, {}, {"species": np.zeros(3, np.int8)}), 0.01, output_dir=str(tmp_path))
    with pytest.raises(ValueError):
        InteractionSimulator(lm.rock_paper_scissors(3, .5, .5, .5), 0.01, interaction_norm=3, output_dir=str(tmp_path))


def test_particle_advecter_argument_checks(lm, tmp_path):
    from lagrangian_microbes_gb300.particle_advecter import ParticleAdvecter, distribute_particles_across_tiles
    fld = lm.uniform_field(195, 206, 20, 31, 0.25, 4)
    lons, lats = np.linspace(200, 201, 12), np.linspace(25, 26, 12)
    with pytest.raises(NotImplementedError):
        ParticleAdvecter(lons, lats, N_procs=1, velocity_field="OSCAR", output_dir=str(tmp_path))
    with pytest.raises(AssertionError):
        ParticleAdvecter(lons, lats, N_procs=1, velocity_field="HYCOM", output_dir=str(tmp_path))
    with pytest.raises(AssertionError):
        ParticleAdvecter(lons, lats, N_procs=0, velocity_field=fld, output_dir=str(tmp_path))
    with pytest.raises(AssertionError):
        ParticleAdvecter(lons, lats, N_procs=5, velocity_field=fld, output_dir=str(tmp_path))
    pa = ParticleAdvecter(lons, lats, N_procs=3, velocity_field=fld, output_dir=str(tmp_path / "out"), Kh=100)
    assert pa.N_procs == min(3, os.cpu_count()) and pa.particles_per_tile * pa.N_procs == 12
    assert pa.Kh == pytest.approx(1e-8) and os.path.isdir(tmp_path / "out")
    tl, ta = distribute_particles_across_tiles(lons, lats, 4)
    assert len(tl) == 4 and all(t.size == 3 for t in tl)
    np.testing.assert_array_equal(np.concatenate(tl), lons)
    with pytest.raises(AssertionError):
        distribute_particles_across_tiles(lons, lats, 5)


def _write_chunks(pa, spans, rng):
    import pickle
    from lagrangian_microbes_gb300.particle_advecter import _chunk_name
    rows = {}
    for i0, i1 in spans:
        for tile_id in range(pa.N_procs):
            lon = rng.random((i1 - i0, pa.particles_per_tile)).astype(np.float32) + 200
            lat = rng.random((i1 - i0, pa.particles_per_tile)).astype(np.float32) + 25
            with open(os.path.join(pa.output_dir, _chunk_name(i0, i1, tile_id)), "wb") as f:
                pickle.dump({"time": list(range(i0, i1)), "lat": lat, "lon": lon}, f)
            rows[(i0, i1, tile_id)] = (lon[-1], lat[-1])
    return rows


def test_restore_reads_the_newest_complete_chunk(lm, tmp_path):
    # the resume path after a killed run (particle_advecter.py:124-138): the last row of every tile
    # of the newest chunk, and the iteration it ends at
    from lagrangian_microbes_gb300.particle_advecter import ParticleAdvecter
    fld = lm.uniform_field(195, 206, 20, 31, 0.25, 4)
    pa = ParticleAdvecter(np.linspace(200, 201, 12), np.linspace(25, 26, 12), N_procs=3, velocity_field=fld,
                          output_dir=str(tmp_path))
    rows = _write_chunks(pa, [(0, 5), (5, 10), (10, 12)], np.random.default_rng(1))
    lons, lats, it = pa.newest_stored_positions()
    assert it == 12
    for t in range(3):
        np.testing.assert_array_equal(lons[4 * t:4 * t + 4], rows[(10, 12, t)][0])
        np.testing.assert_array_equal(lats[4 * t:4 * t + 4], rows[(10, 12, t)][1])


def test_restore_rejects_missing_corrupt_and_misshapen_checkpoints(lm, tmp_path):
    import pickle
    from lagrangian_microbes_gb300.particle_advecter import ParticleAdvecter, _chunk_name
    fld = lm.uniform_field(195, 206, 20, 31, 0.25, 4)
    mk = lambda d: ParticleAdvecter(np.linspace(200, 201, 12), np.linspace(25, 26, 12), N_procs=3,
                                    velocity_field=fld, output_dir=str(tmp_path / d))
    with pytest.raises(FileNotFoundError):  # nothing stored yet
        mk("empty").newest_stored_positions()
    # a tile file of the newest chunk is missing: an error, not the older chunk's row for that tile
    pa = mk("missing")
    _write_chunks(pa, [(0, 5), (5, 10)], np.random.default_rng(2))
    os.remove(os.path.join(pa.output_dir, _chunk_name(5, 10, 1)))
    with pytest.raises(FileNotFoundError, match=r"tile\(s\) \[1\]"):
        pa.newest_stored_positions()
    # a truncated file (a write cut short when the process was killed)
    pa = mk("truncated")
    _write_chunks(pa, [(0, 5)], np.random.default_rng(3))
    path = os.path.join(pa.output_dir, _chunk_name(0, 5, 2))
    with open(path, "rb") as f:
        data = f.read()
    with open(path, "wb") as f:
        f.write(data[: len(data) // 2])
    with pytest.raises(ValueError, match="unreadable"):
        pa.newest_stored_positions()
    # positions of the wrong shape, and a file that is not a chunk of this run's name pattern
    pa = mk("shape")
    _write_chunks(pa, [(0, 5)], np.random.default_rng(4))
    with open(os.path.join(pa.output_dir, _chunk_name(0, 5, 0)), "wb") as f:
        pickle.dump({"time": [], "lat": np.zeros((5, 3), np.float32), "lon": np.zeros((5, 3), np.float32)}, f)
    with pytest.raises(ValueError, match="expected"):
        pa.newest_stored_positions()
    pa = mk("name")
    _write_chunks(pa, [(0, 5)], np.random.default_rng(5))
    open(os.path.join(pa.output_dir, "particle_locations_x_y_tilez.pickle"), "wb").close()
    with pytest.raises(ValueError, match="not a chunk file name"):
        pa.newest_stored_positions()


def test_velocity_field_descending_latitude_is_flipped(lm):
    lon = np.array([0.0, 1.0, 2.0])
    lat = np.array([2.0, 1.0])
    u = np.arange(12, dtype=np.float32).reshape(2, 2, 3)
    f = lm.VelocityField(lon, lat, np.array([0.0, 3600.0]), u, -u)
    assert f.lat[0] == 1.0
    np.testing.assert_array_equal(f.u[:, 0, :], u[:, 1, :])
    assert f.seconds(f.epoch + timedelta(hours=2)) == 7200.0


def test_netcdf_roundtrip(tmp_path):
    from lagrangian_microbes_gb300.ncio import read_particle_file, write_particle_file
    lon = np.random.default_rng(0).random((7, 4)).astype(np.float32)
    sp = np.arange(28, dtype=np.int8).reshape(7, 4)
    path = str(tmp_path / "m.nc")
    write_particle_file(path, {"longitude": lon, "species": sp}, datetime(2017, 1, 1), np.arange(4) * 3600.0)
    d = read_particle_file(path)
    np.testing.assert_array_equal(d["longitude"], lon)
    np.testing.assert_array_equal(d["species"], sp)
    np.testing.assert_array_equal(d["particle number"], np.arange(1, 8))
    np.testing.assert_array_equal(d["time"], np.arange(4) * 3600.0)
    assert all(a.dtype.isnative for a in d.values())  # NetCDF is big-endian on disk


def test_shard_partitions(lm):
    from lagrangian_microbes_gb300.replicas import shard, shard_weighted
    for n in (0, 1, 7, 256):
        for w in (1, 2, 3, 8):
            parts = [list(shard(n, w, r)) for r in range(w)]
            assert sorted(sum(parts, [])) == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1
    weights = np.random.default_rng(1).random(50).tolist()
    got = sorted(sum((shard_weighted(weights, 4, r) for r in range(4)), []))
    assert got == list(range(50))
