"""Failure paths, exercised without faulting the GPU.

Each failure is made on the host or by a bounded device wait running out:
  * non-finite positions or masses: the tree's bounding-box pass rejects them
    (CSG_ERR_BAD_ARG) before any key is formed; the free functions leave the
    caller's arrays as they were (the reference has no error channel and
    would build a tree of NaNs);
  * device waits: the walks' producer/consumer waits with their limit lowered
    to one poll give up and report CSG_ERR_DEVICE_WAIT; the sort's look-back
    wait gives up on a status word that nothing publishes; in both cases the
    context stays usable;
  * allocation failures, injected on the host (csg_inject_alloc_failure):
    creating a handle, stepping one (SPH buffers are allocated on first use)
    and the free functions report CSG_ERR_NOMEM, change nothing, and work
    again once memory is available.
Error codes: 2 NOMEM, 4 BAD_ARG, 9 DEVICE_WAIT.
"""
import ctypes

import numpy as np
import pytest

from conftest import same_bytes
from cosmosim_gb300.abi import NODE_DTYPE, ptr

pytestmark = pytest.mark.gpu

NOMEM, BAD_ARG, DEVICE_WAIT = 2, 4, 9


def _code(exc):
    return int(str(exc).rsplit("code ", 1)[1].rstrip(")"))


@pytest.fixture
def clean(lib):
    """Leaves the calling thread's state and the injection as they were."""
    L = lib.load()
    yield L
    L.csg_inject_alloc_failure(-1)
    L.csg_set_wait_limit(0)
    lib.set_precision(lib.PREC_FP64)


@pytest.mark.parametrize("field,value", [("x", np.nan), ("z", np.inf), ("y", -np.inf),
                                         ("mass", np.nan), ("mass", np.inf)])
def test_non_finite_input_is_rejected_and_changes_nothing(lib, clean, field, value):
    b = lib.generate_ics(1, 3000, 21)
    b[field][1234] = value
    before = b.copy()
    pool = np.zeros(8 * len(b), dtype=NODE_DTYPE)
    pool_before = pool.copy()
    for call in (lambda: lib.integrator_step(b, 1e-3, 1.0, 0.01, 0.5, pool, 1),
                 lambda: lib.integrator_init_accelerations(b, 1.0, 0.01, 0.5, pool),
                 lambda: lib.octree_build(b, pool)):
        with pytest.raises(lib.CudaError) as e:
            call()
        assert _code(e.value) == BAD_ARG
        assert same_bytes(b, before)
        assert same_bytes(pool, pool_before)
    # a handle cannot be created over such bodies
    with pytest.raises(lib.CudaError):
        lib.Sim.from_bodies(b, softening=0.01)
    assert clean.csg_last_error() == BAD_ARG
    # the same bodies with the bad one dead (mass 0, position anything) are fine
    if field != "mass":
        b["mass"][1234] = 0.0
        lib.integrator_step(b, 1e-3, 1.0, 0.01, 0.5, pool, 1)
        assert np.isfinite(b["ax"][b["mass"] > 0]).all()


def test_handle_fails_its_step_on_non_finite_bodies(lib, clean):
    b = lib.generate_ics(0, 5000, 3)
    sim = lib.Sim.from_bodies(b, softening=0.01)
    start = sim.bodies()  # with the initial accelerations
    bad = start.copy()
    bad["x"][77] = np.nan
    sim.set_bodies(bad)
    sim.substeps_async(2)
    with pytest.raises(lib.CudaError) as e:
        sim.sync()
    assert _code(e.value) == BAD_ARG
    sim.set_bodies(start)  # usable again with good bodies
    sim.substeps_async(1)
    sim.sync()
    ref = lib.Sim.from_bodies(b, softening=0.01)
    ref.substeps_async(1)
    ref.sync()
    assert same_bytes(sim.bodies(), ref.bodies())
    sim.close()
    ref.close()


def test_look_back_wait_gives_up_on_an_unpublished_status(lib, clean):
    for polls in (1, 64, 4096):
        st = ctypes.c_int(-1)
        assert clean.csg_check_device_wait(polls, ctypes.byref(st)) == 0
        assert st.value == DEVICE_WAIT
    # the context is still usable: a step matches a fresh state's
    b = lib.generate_ics(0, 2000, 4)
    pool = np.zeros(8 * len(b), dtype=NODE_DTYPE)
    lib.integrator_init_accelerations(b, 1.0, 0.01, 0.5, pool)
    assert np.isfinite(b["ax"]).all()


def test_walk_wait_expiry_is_reported_and_the_handle_recovers(lib, clean):
    """FP64 walk: the consumer warp's first wait for the producer's cells
    finds none; with a limit of one poll it gives up (both warps leave the
    task) and the step reports CSG_ERR_DEVICE_WAIT."""
    b = lib.generate_ics(0, 20000, 5)
    sim = lib.Sim.from_bodies(b, softening=0.01, precision=lib.PREC_FP64)
    start = sim.bodies()  # with the initial accelerations
    assert clean.cosmosim_set_wait_limit(sim.h, 1) == 0
    sim.substeps_async(1)
    with pytest.raises(lib.CudaError) as e:
        sim.sync()
    assert _code(e.value) == DEVICE_WAIT
    # default limit again: the handle steps normally, as a fresh one does
    assert clean.cosmosim_set_wait_limit(sim.h, 0) == 0
    sim.set_bodies(start)
    sim.substeps_async(2)
    sim.sync()
    ref = lib.Sim.from_bodies(b, softening=0.01, precision=lib.PREC_FP64)
    ref.substeps_async(2)
    ref.sync()
    assert same_bytes(sim.bodies(), ref.bodies())
    sim.close()
    ref.close()


def test_walk_wait_expiry_in_a_free_function_leaves_the_arrays(lib, clean):
    b = lib.generate_ics(0, 20000, 6)
    pool = np.zeros(8 * len(b), dtype=NODE_DTYPE)
    lib.integrator_init_accelerations(b, 1.0, 0.01, 0.5, pool)
    before, pool_before = b.copy(), pool.copy()
    lib.set_precision(lib.PREC_FP64)
    clean.csg_set_wait_limit(1)
    with pytest.raises(lib.CudaError) as e:
        lib.integrator_step(b, 1e-3, 1.0, 0.01, 0.5, pool, 0)
    assert _code(e.value) == DEVICE_WAIT
    assert same_bytes(b, before) and same_bytes(pool, pool_before)
    clean.csg_set_wait_limit(0)
    lib.integrator_step(b, 1e-3, 1.0, 0.01, 0.5, pool, 0)
    assert np.isfinite(b["x"]).all()


def _params(lib, sph):
    return lib.CsgSimParams(1.0, 0.01, 0.5, 1e-3, 1, int(sph), lib.PREC_FP64)


def test_handle_creation_reports_allocation_failure(lib, clean):
    """Every allocation a handle's creation makes is made to fail in turn:
    each attempt returns NULL with CSG_ERR_NOMEM; then creation succeeds."""
    b = lib.generate_ics(1, 3000, 7)
    p = _params(lib, True)
    for allow in range(0, 200):
        clean.csg_inject_alloc_failure(allow)
        h = clean.cosmosim_create_from_bodies(ptr(b), len(b), ctypes.byref(p))
        clean.csg_inject_alloc_failure(-1)
        if h:
            clean.cosmosim_destroy(h)
            break
        assert clean.csg_last_error() == NOMEM, allow
    else:
        pytest.fail("creation never succeeded")
    assert allow > 10  # the device state and every body buffer were hit


def test_handle_step_reports_allocation_failure_and_changes_nothing(lib, clean):
    """SPH buffers are allocated at a handle's first SPH substep: with no
    allocation allowed the step fails before any kernel, the bodies stay as
    they were, and the next step (memory available) runs normally."""
    b = lib.generate_ics(1, 3000, 8)
    sim = lib.Sim.from_bodies(b, softening=0.01, sph=True)
    start = sim.bodies()
    clean.csg_inject_alloc_failure(0)
    rc = clean.cosmosim_substeps_async(sim.h, 1)
    clean.csg_inject_alloc_failure(-1)
    assert rc == NOMEM
    with pytest.raises(lib.CudaError):
        sim.sync()  # the recorded error is collected once
    assert same_bytes(sim.bodies(), start)
    sim.substeps_async(1)
    sim.sync()
    ref = lib.Sim.from_bodies(b, softening=0.01, sph=True)
    ref.substeps_async(1)
    ref.sync()
    assert same_bytes(sim.bodies(), ref.bodies())
    sim.close()
    ref.close()


def test_free_function_reports_allocation_failure(lib, clean):
    """integrator_step on a fresh thread state, every allocation made to fail
    in turn: CSG_ERR_NOMEM and untouched arrays, until it succeeds."""
    b = lib.generate_ics(1, 3000, 9)
    pool = np.zeros(8 * len(b), dtype=NODE_DTYPE)
    for allow in range(0, 200):
        clean.csg_release_thread_state()
        work, wpool = b.copy(), pool.copy()
        clean.csg_inject_alloc_failure(allow)
        try:
            lib.integrator_step(work, 1e-3, 1.0, 0.01, 0.5, wpool, 1)
            ok = True
        except lib.CudaError as e:
            ok = False
            assert _code(e) == NOMEM, allow
            assert same_bytes(work, b) and same_bytes(wpool, pool)
        finally:
            clean.csg_inject_alloc_failure(-1)
        if ok:
            break
    else:
        pytest.fail("integrator_step never succeeded")
    assert allow > 10
    clean.csg_release_thread_state()
