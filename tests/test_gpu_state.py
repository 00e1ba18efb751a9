"""Device snapshots, exact checkpoints and the cell-size autotuner.

A run rewound to a snapshot, or resumed in a new context from an exported state, must continue
bit-identically; the autotuner must return the state it started from and change nothing but the
speed (the pair sets do not depend on the cell size).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(lm, orc, field, n=30000, seed=9):
    rng = np.random.default_rng(seed)
    lons, lats = orc.lattice(n, 25.0, 26.0, 200.0, 201.0)
    sp = rng.integers(1, 4, lons.size).astype(np.int8)
    return lm.Simulation(field, lons, lats, sp, radius=0.01, p_rs=0.7, p_pr=0.6, p_sp=0.8, seed=5), (lons, lats, sp)


def test_snapshot_restore_continues_bit_identically(lm, orc, small_field):
    sim, _ = _sim(lm, orc, small_field)
    t0 = float(small_field.times[0])
    sim.step(t0, 3600.0, 4, step0=0)
    sim.snapshot()
    sim.step(t0 + 4 * 3600.0, 3600.0, 5, step0=4)
    a = sim.state()
    sim.restore()
    assert sim.step_index == 4
    sim.step(t0 + 4 * 3600.0, 3600.0, 5, step0=4)
    b = sim.state()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    sim.close()


def test_exported_state_resumes_in_a_new_context(lm, orc, small_field):
    t0 = float(small_field.times[0])
    sim, _ = _sim(lm, orc, small_field)
    sim.step(t0, 3600.0, 7, step0=0)
    want = sim.state()
    sim.close()
    sim, _ = _sim(lm, orc, small_field)
    sim.step(t0, 3600.0, 3, step0=0)
    ck = sim.export_state()
    assert ck["step"] == 3
    sim.close()
    other, _ = _sim(lm, orc, small_field, seed=123)  # same layout, other species: overwritten by the import
    other.import_state(ck)
    other.step(t0 + 3 * 3600.0, 3600.0, 4, step0=3)
    got = other.state()
    for x, y in zip(want, got):
        np.testing.assert_array_equal(x, y)
    other.close()


def test_autotune_changes_speed_only(lm, orc, small_field):
    t0 = float(small_field.times[0])
    ref, _ = _sim(lm, orc, small_field)
    ref.step(t0, 3600.0, 6, step0=0)
    want = ref.state()
    ref.close()
    sim, _ = _sim(lm, orc, small_field)
    best, times = sim.autotune(t0, 3600.0, n_steps=2, factors=(1.004, 1.7, 3.0))
    assert best in (1.004, 1.7, 3.0) and len(times) == 3
    assert sim.step_index == 0
    sim.step(t0, 3600.0, 6, step0=0)
    got = sim.state()
    for x, y in zip(want, got):
        np.testing.assert_array_equal(x, y)
    sim.close()


def test_loaded_kernels_are_sm103a(lm):
    import ctypes

    from lagrangian_microbes_gb300 import _lib
    sm = ctypes.c_int(0)
    assert _lib.load().lm_kernel_arch(ctypes.byref(sm)) == _lib.LM_OK
    assert sm.value == 103


def test_field_window_upload_keeps_the_state_and_drops_the_graph(lm, orc):
    """A long run can stream its field in windows of frames: uploading the next window keeps the
    microbes (same grid, same origin) and forgets the captured graph, whose steps hold the old
    field; after capturing again the run continues exactly as with the whole field."""
    from lagrangian_microbes_gb300 import LMError
    from lagrangian_microbes_gb300.fields import psi_basis
    basis = psi_basis(190.0, 215.0, 15.0, 40.0, 1.0 / 12.0, seed=3)
    lons, lats = orc.lattice(20000, 25.0, 26.0, 200.0, 201.0)
    sp = np.random.default_rng(2).integers(1, 4, lons.size).astype(np.int8)
    whole = lm.Simulation(basis.frames(0, 14), lons, lats, sp, radius=0.01, p_rs=0.7, p_pr=0.6, p_sp=0.8, seed=5)
    whole.capture(0.0, 3600.0, 4, step0=0)
    whole.run_graph(3)
    win = lm.Simulation(basis.frames(0, 7), lons, lats, sp, radius=0.01, p_rs=0.7, p_pr=0.6, p_sp=0.8, seed=5)
    win.capture(0.0, 3600.0, 6, step0=0)
    win.run_graph(1)
    win.upload_field(basis.frames(6, 7))
    with pytest.raises(LMError, match="no captured graph"):
        win.ctx.call("lm_graph_run", 1, 1)
    win.capture(6 * 3600.0, 3600.0, 6, step0=6)
    win.run_graph(1)
    for a, b in zip(whole.state(), win.state()):
        np.testing.assert_array_equal(a, b)
    whole.close()
    win.close()


def test_launch_shape_knobs_change_speed_only(lm, orc, small_field):
    """Every value of every tuning knob gives the same trajectory and species, bit for bit; the
    full autotuner returns to the state it started from."""
    t0 = float(small_field.times[0])
    ref, _ = _sim(lm, orc, small_field)
    ref.step(t0, 3600.0, 5, step0=0)
    want = ref.state()
    ref.close()
    for name, (_, values) in lm.Simulation.TUNING_KNOBS.items():
        for v in values:
            sim, _ = _sim(lm, orc, small_field)
            sim.set_tuning(name, v)
            assert sim.tuning()[name] == v
            sim.step(t0, 3600.0, 5, step0=0)
            for x, y in zip(want, sim.state()):
                np.testing.assert_array_equal(x, y, err_msg=f"{name}={v}")
            sim.close()
    sim, _ = _sim(lm, orc, small_field)
    chosen = sim.autotune_all(t0, 3600.0, n_steps=1, factors=(1.004, 2.0))
    assert set(chosen) >= {"cell_factor", *lm.Simulation.TUNING_KNOBS}
    assert sim.step_index == 0
    sim.step(t0, 3600.0, 5, step0=0)
    for x, y in zip(want, sim.state()):
        np.testing.assert_array_equal(x, y)
    sim.close()


def test_page_locked_record_buffers_hold_the_same_records(lm, orc, small_field):
    """Records copied into page-locked buffers (asynchronous copies on the copy stream) equal the
    records copied into fresh numpy arrays, step by step, over calls that reuse the buffers."""
    t0 = float(small_field.times[0])
    a, _ = _sim(lm, orc, small_field)
    b, _ = _sim(lm, orc, small_field)
    bufs = b.record_buffers(4)
    assert all(not v.flags["OWNDATA"] and v.flags["C_CONTIGUOUS"] for v in bufs.values())
    for call in range(3):
        want = a.step(t0 + 4 * call * 3600.0, 3600.0, 4, record=True, step0=4 * call)
        got = b.step(t0 + 4 * call * 3600.0, 3600.0, 4, record=True, step0=4 * call, out=bufs)
        for k in ("lon", "lat", "species"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"call {call}, {k}")
    a.close()
    b.close()
    del bufs, got  # the blocks are freed with the last array that views them


def test_field_from_page_locked_arrays_equals_staged_upload(lm, orc, small_field):
    """A field whose u and v live in page-locked memory is read by the device directly; the run is
    bit-identical to one whose field went through the staging copies."""
    from lagrangian_microbes_gb300 import _lib
    t0 = float(small_field.times[0])
    u = _lib.host_empty(small_field.u.shape, np.float32)
    v = _lib.host_empty(small_field.v.shape, np.float32)
    u[...] = small_field.u
    v[...] = small_field.v
    pinned = lm.VelocityField(small_field.lon, small_field.lat, small_field.times, u, v, small_field.epoch)
    assert pinned.u is u or np.shares_memory(pinned.u, u)
    states = []
    for fld in (small_field, pinned):
        sim, _ = _sim(lm, orc, fld)
        sim.step(t0, 3600.0, 6, step0=0)
        states.append(sim.state())
        sim.close()
    for x, y in zip(*states):
        np.testing.assert_array_equal(x, y)


def test_particles_from_page_locked_arrays_equal_host_conversion(lm, orc, small_field):
    """Particles whose positions and species live in page-locked memory are converted to the slot
    layout on the device; the state equals the host conversion bit for bit, before and after steps."""
    from lagrangian_microbes_gb300 import _lib
    t0 = float(small_field.times[0])
    rng = np.random.default_rng(21)
    lons, lats = orc.lattice(30000, 25.0, 26.0, 200.0, 201.0)
    sp = rng.integers(1, 4, lons.size).astype(np.int8)

    def pinned(a):
        out = _lib.host_empty(a.shape, a.dtype)
        out[...] = a
        return out

    states = []
    for args in ((lons, lats, sp), (pinned(lons), pinned(lats), pinned(sp))):
        sim = lm.Simulation(small_field, *args, radius=0.01, p_rs=0.7, p_pr=0.6, p_sp=0.8, seed=5)
        first = sim.export_state()
        sim.step(t0, 3600.0, 4, step0=0)
        states.append((first, sim.export_state()))
        sim.close()
    for a, b in zip(*states):
        for k in ("xo", "yo", "species", "status"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
