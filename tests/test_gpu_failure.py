"""Failure detection without a GPU fault: an injected stall of the interaction kernel.

lm_debug_inject_wait makes the next interaction kernel wait on a device flag that nothing sets,
as a stalled dependency would. The wait is bounded like every wait of that kernel: it gives up,
records the timeout, the call returns LM_ERR_TIMEOUT, and the context goes on working. The
failed step advected the microbes but applied no pair, so the same context then matches a second
context that ran that step without interaction, bit for bit.
"""

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_injected_stall_times_out_and_the_context_stays_usable(lm, small_field):
    from lagrangian_microbes_gb300 import _lib, engine
    rng = np.random.default_rng(61)
    n = 6000
    lons = 200.0 + 0.8 * rng.random(n)
    lats = 25.0 + 0.8 * rng.random(n)
    sp0 = rng.integers(1, 4, n).astype(np.int8)
    t0, dt = float(small_field.times[0]), 3600.0
    a = engine.Simulation(small_field, lons, lats, sp0, radius=0.02, seed=3)
    b = engine.Simulation(small_field, lons, lats, sp0, radius=0.02, seed=3)
    for sim in (a, b):
        sim.step(t0, dt, 1, step0=0)
    a.ctx.call("lm_debug_inject_wait", 0.05)
    start = time.perf_counter()
    with pytest.raises(lm.LMError) as err:
        a.step(t0 + dt, dt, 1, step0=1)
    assert err.value.code == _lib.LM_ERR_TIMEOUT
    assert time.perf_counter() - start < 5.0  # the bound (50 ms), not a hang
    b.step(t0 + dt, dt, 1, step0=1, interact=False)  # the same step without its pairs
    for x, y in zip(a.state(), b.state()):
        np.testing.assert_array_equal(x, y)
    # the injection was one step only, and the context is usable: later steps agree bit for bit
    ra = a.step(t0 + 2 * dt, dt, 3, step0=2, record=True)
    rb = b.step(t0 + 2 * dt, dt, 3, step0=2, record=True)
    for k in ("lon", "lat", "species"):
        np.testing.assert_array_equal(ra[k], rb[k])
    assert a.stats()["pairs"] > 0
    a.close()
    b.close()


def test_injection_rejects_bad_bounds(lm):
    from lagrangian_microbes_gb300 import _lib
    ctx = _lib.Context(0)
    for bad in (0.0, -1.0, 11.0, float("nan")):
        with pytest.raises(lm.LMError):
            ctx.call("lm_debug_inject_wait", bad)
    ctx.close()
