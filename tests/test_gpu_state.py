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
