"""Leapfrog and the handle API on the GPU against the reference (through the C-ABI).

Tolerance: positions, velocities, accelerations and SPH fields after each
step within 1e-9 relative (scaled by each field's largest magnitude) of the
reference's own outputs — the only source of difference is the gravity
walk's 1e-13-level rounding (cell moments summed in a different order); the
kick/drift and SPH arithmetic are bit-identical.
Known-answer tests mirror tests/test_physics.c:274-343 and :1048-1137.
"""
import numpy as np
import pytest

from conftest import fields, golden
from cosmosim_gb300.abi import BODY_DTYPE, NODE_DTYPE

pytestmark = pytest.mark.gpu

OUT = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "density", "pressure",
       "internal_energy", "smoothing_h"]


def close(got, want, rtol=1e-9):
    scale = np.maximum(np.abs(want).max(axis=0), 1e-300)
    err = np.abs(got - want) / scale
    assert err.max() <= rtol, err.max(axis=0)


def test_leapfrog_with_sph_matches_reference(lib):
    g = golden("kdk_1500.npz")
    b = g["bodies"].copy()
    pool = np.zeros(8 * len(b), dtype=NODE_DTYPE)
    lib.integrator_init_accelerations(b, 1.0, 0.01, 0.5, pool)
    close(fields(b, OUT), g["init"])
    want = dict(zip(g["step_numbers"].tolist(), g["steps"]))
    for step in range(1, 9):
        lib.integrator_step(b, 1e-3, 1.0, 0.01, 0.5, pool, 1)
        if step in want:
            close(fields(b, OUT), want[step])


def test_energy_conservation_kat(lib, orc):  # :274-304
    M, r = 100.0, 5.0
    b = np.zeros(2, dtype=BODY_DTYPE)
    b["mass"] = [M, 1.0]
    b["x"][1] = r
    b["vy"][1] = np.sqrt(M / r)
    pool = np.zeros(16, dtype=NODE_DTYPE)
    lib.integrator_init_accelerations(b, 1.0, 0.01, 0.0, pool)
    e0 = orc.total_energy(b, 1.0, 0.01)
    for _ in range(2000):
        lib.integrator_step(b, 0.001, 1.0, 0.01, 0.0, pool, 0)
    e1 = orc.total_energy(b, 1.0, 0.01)
    assert abs((e1 - e0) / e0) < 0.01


def test_momentum_conservation_kat(lib):  # :306-343
    b = np.zeros(4, dtype=BODY_DTYPE)
    b["x"], b["y"], b["z"] = [1, -1, 0, 0], [0, 0, 2, -2], [0, 0, 1, -1]
    b["vx"], b["vy"], b["vz"] = [0, 0, -0.5, 0.5], [1, -1, 0, 0], [0, 0, 0.3, -0.3]
    b["mass"] = [2.0, 2.0, 3.0, 1.0]
    pool = np.zeros(32, dtype=NODE_DTYPE)
    lib.integrator_init_accelerations(b, 1.0, 0.1, 0.0, pool)
    p0 = (b["mass"][:, None] * fields(b, ("vx", "vy", "vz"))).sum(0)
    for _ in range(500):
        lib.integrator_step(b, 0.002, 1.0, 0.1, 0.0, pool, 0)
    p1 = (b["mass"][:, None] * fields(b, ("vx", "vy", "vz"))).sum(0)
    assert np.all(np.abs(p1 - p0) < 1e-10)


def test_api_create_destroy_kat(lib):  # :1048-1073
    L = lib.load()
    cfg = L.cosmosim_default_config()
    cfg.n_bodies = 1000
    s = lib.Sim(L.cosmosim_create(cfg))
    assert s.count == 1000
    assert s.active_count == 1000
    assert abs(s.sim_time) < 1e-15
    v = s.get_bodies_view()
    assert v["mass"].sum() > 0
    s.close()


def test_api_step_kat(lib):  # :1075-1103
    L = lib.load()
    cfg = L.cosmosim_default_config()
    cfg.n_bodies = 500
    s = lib.Sim(L.cosmosim_create(cfg))
    s.step()
    assert abs(s.sim_time - cfg.dt * cfg.substeps) < 1e-12
    v = s.get_bodies_view()
    assert np.any((v["vx"] != 0) | (v["vy"] != 0) | (v["vz"] != 0))
    s.close()


def test_api_quasar_runs_without_the_cpu_quasar_code(lib):
    """Quasar mode runs its quasar step on the GPU and restates the
    reference's quasar initial conditions: create succeeds without the
    reference's CPU units."""
    L = lib.load()
    cfg = L.cosmosim_default_config()
    cfg.n_bodies = 1000
    cfg.merger = 1
    cfg.quasar = 1
    s = lib.Sim(L.cosmosim_create(cfg))
    v = s.get_bodies_view()
    assert (v["type"] == 2).sum() == 2  # two SMBHs
    s.step()
    assert s.sim_time > 0
    s.close()


def test_api_null_handle_is_a_no_op(lib):  # src/cosmosim_api.c:117-183
    L = lib.load()
    L.cosmosim_step(None)
    assert L.cosmosim_get_bodies(None) is None
    assert L.cosmosim_get_count(None) == 0
    assert L.cosmosim_get_active_count(None) == 0
    assert L.cosmosim_get_sim_time(None) == 0.0
    L.cosmosim_destroy(None)


@pytest.mark.parametrize("sph", [False, True])
def test_resident_handle_matches_reference_steps(lib, orc, sph):
    """Device-resident substeps (no host copies between them) equal the
    reference's integrator_step sequence."""
    b = lib.generate_ics(1, 4000, 21)
    if not sph:
        b["type"] = 0
    s = lib.Sim.from_bodies(b, softening=0.01, theta=0.5, dt=1e-3, substeps=1, sph=sph)
    ref = b.copy()
    pool = np.zeros(8 * len(b), dtype=NODE_DTYPE)
    orc.integrator_init_accelerations(ref, 1.0, 0.01, 0.5, pool)
    s.substeps_async(5)
    s.sync()
    for _ in range(5):
        orc.integrator_step(ref, 1e-3, 1.0, 0.01, 0.5, pool, int(sph))
    close(fields(s.bodies(), OUT), fields(ref, OUT))
    s.close()


def test_fp32_mixed_handle_tracks_fp64(lib):
    b = lib.generate_ics(0, 20000, 1)
    r64 = lib.Sim.from_bodies(b, softening=0.01, theta=0.5, dt=1e-3)
    r32 = lib.Sim.from_bodies(b, softening=0.01, theta=0.5, dt=1e-3, precision=lib.PREC_FP32_MIXED)
    for s in (r64, r32):
        s.substeps_async(20)
        s.sync()
    a, c = r64.bodies(), r32.bodies()
    dx = np.sqrt(sum((a[f] - c[f]) ** 2 for f in ("x", "y", "z")))
    assert np.median(dx) < 1e-9 and dx.max() < 1e-6
    r64.close()
    r32.close()


def test_graph_replay_equals_direct_launches(lib):
    """Substeps replayed from the captured CUDA graph are bit-identical to the
    same substeps launched one kernel at a time (every kernel is deterministic)."""
    b = lib.generate_ics(1, 20000, 8)
    out = []
    for graphs in (True, False):
        s = lib.Sim.from_bodies(b, softening=0.01, theta=0.5, dt=1e-3, sph=True,
                                precision=lib.PREC_FP32_MIXED)
        s.enable_graphs(graphs)
        s.substeps_async(4)
        s.sync()
        out.append(fields(s.bodies(), OUT))
        s.close()
    np.testing.assert_array_equal(out[0], out[1])


def test_energy_drift_bound_and_precision(lib):
    """Energy drift over 1000 substeps (disk + SMBH, 4000 bodies, dt 1e-3):
    below 2e-2 for both walks, and the FP32-mixed walk adds no drift of its
    own (|drift32 - drift64| <= 1e-5)."""
    b = lib.generate_ics(0, 4000, 42)
    drifts = []
    for prec in (lib.PREC_FP64, lib.PREC_FP32_MIXED):
        s = lib.Sim.from_bodies(b, softening=0.01, theta=0.5, dt=1e-3, precision=prec)
        e0 = sum(s.energy())
        s.substeps_async(1000)
        s.sync()
        e1 = sum(s.energy())
        drifts.append(abs((e1 - e0) / e0))
        s.close()
    assert max(drifts) < 2e-2, drifts
    assert abs(drifts[0] - drifts[1]) <= 1e-5, drifts


@pytest.mark.parametrize("sph", [0, 1])
def test_integrator_step_pinned_pool_equals_pageable(lib, sph):
    """A pinned (mapped) pool is written by the export kernels beside the walk,
    a pageable one by a copy after the substep: bodies and pools must agree
    bit for bit, step after step."""
    torch = pytest.importorskip("torch")
    b = lib.generate_ics(1, 3000, 5)
    n = len(b)
    page_b, page_pool = b.copy(), np.zeros(8 * n, dtype=NODE_DTYPE)
    pin_b = torch.empty(n * b.dtype.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(b.dtype)
    pin_b[:] = b
    pin_pool = torch.zeros(8 * n * NODE_DTYPE.itemsize, dtype=torch.uint8,
                           pin_memory=True).numpy().view(NODE_DTYPE)
    for step in range(4):
        lib.integrator_step(page_b, 1e-3, 1.0, 0.01, 0.5, page_pool, sph)
        lib.integrator_step(pin_b, 1e-3, 1.0, 0.01, 0.5, pin_pool, sph)
        assert page_b.tobytes() == pin_b.tobytes(), step
        assert page_pool.tobytes() == pin_pool.tobytes(), step
