"""Per-phase timing of the real substep (cosmosim_phase_times): CUDA events
between the phases of the same kernels a substep always runs, read back per
substep. Timing must not change any result, and the phases must account for
the substep's time."""
import ctypes

import numpy as np
import pytest

from conftest import same_bytes
from cosmosim_gb300.abi import NODE_DTYPE

pytestmark = pytest.mark.gpu

MAIN = ("kick_drift_ms", "build_ms", "gravity_ms", "kick_ms", "cooling_ms")


@pytest.mark.parametrize("sph,prec", [(True, 1), (False, 0)])
def test_phase_times_cover_the_substep_and_change_nothing(lib, sph, prec):
    b = lib.generate_ics(1, 20000, 31)
    kw = dict(softening=0.01, sph=sph, precision=prec)
    timed = lib.Sim.from_bodies(b, **kw)
    plain = lib.Sim.from_bodies(b, **kw)
    timed.enable_phase_timing(True)
    timed.substeps_async(4)
    plain.substeps_async(4)
    timed.sync()
    plain.sync()
    assert same_bytes(timed.bodies(), plain.bodies())  # same kernels, same bits
    t = timed.phase_times()
    assert t["substeps"] == 4
    for k in ("kick_drift_ms", "build_ms", "gravity_ms", "kick_ms", "substep_ms"):
        assert t[k] > 0.0, k
    # without SPH those phases hold no kernel: only the events' own overhead
    assert (t["sph_ms"] > 0.05 * t["gravity_ms"]) == sph
    assert (t["cooling_ms"] > 0.0) and (t["cooling_ms"] < 0.05 * t["substep_ms"])
    # the build's parts follow one another inside the build
    parts = sum(t[k] for k in ("build_keys_ms", "build_sort_ms", "build_cells_ms",
                               "build_moments_ms", "build_rest_ms"))
    assert 0.9 * t["build_ms"] <= parts <= 1.001 * t["build_ms"]
    assert min(t["build_sort_ms"], t["build_moments_ms"]) > 0.0
    # the phases on the main stream follow one another inside the substep
    assert sum(t[k] for k in MAIN) <= t["substep_ms"] * 1.001
    if not sph:
        assert sum(t[k] for k in MAIN) >= 0.9 * t["substep_ms"]
    # off: graph replays again, the sums stay for reading
    timed.enable_phase_timing(False)
    timed.substeps_async(2)
    plain.substeps_async(2)
    timed.sync()
    plain.sync()
    assert same_bytes(timed.bodies(), plain.bodies())
    assert timed.phase_times() == t
    timed.close()
    plain.close()


def test_free_function_phase_times(lib):
    L = lib.load()
    b = lib.generate_ics(1, 5000, 32)
    pool = np.zeros(8 * len(b), dtype=NODE_DTYPE)
    lib.integrator_init_accelerations(b, 1.0, 0.01, 0.5, pool)
    assert L.csg_enable_phase_timing(1) == 0
    for _ in range(3):
        lib.integrator_step(b, 1e-3, 1.0, 0.01, 0.5, pool, 1)
    t = lib.CsgPhaseTimes()
    assert L.csg_phase_times(ctypes.byref(t)) == 0
    assert L.csg_enable_phase_timing(0) == 0
    assert t.substeps == 3 and t.substep_ms > 0.0 and t.gravity_ms > 0.0 and t.sph_ms > 0.0
