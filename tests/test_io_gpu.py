"""Snapshot export (cosmosim_snapshot_f32) and device compaction
(cosmosim_compact) on the GPU, against numpy restatements of the reference's
host loops: the Unreal plugin's SnapshotToBuffer
(ue/CosmosimPlugin/Source/CosmosimPlugin/Private/CosmosimSubsystem.cpp:12-43),
the renderer's vertex upload (src/renderer.c:348-365) and quasar_compact
(src/quasar.c:511-523). Float records are bit-exact (the same FP64 -> FP32
conversions); compaction is exact.
"""
import numpy as np
import pytest

from conftest import fields
from cosmosim_gb300.abi import BODY_DTYPE

pytestmark = pytest.mark.gpu

UE = ["x", "y", "z", "mass", "vx", "vy", "vz", "type", "internal_energy", "density", "lifetime",
      "luminosity", "spin_x", "spin_y", "spin_z"]
RENDER = ["x", "y", "z", "mass", "vx", "vy", "vz", "type", "internal_energy", "density"]


def snapshot_ref(b, names, cap):
    keep = ~(b["mass"] <= 0.0)  # the reference skips mass <= 0.0; NaN is kept
    sel = b[keep][:cap]
    cols = [sel[f].astype(np.float64).astype(np.float32) for f in names]
    if len(names) == 15:
        cols.append(np.zeros(len(sel), np.float32))
    return np.stack(cols, axis=1) if len(sel) else np.zeros((0, len(cols)), np.float32)


def bodies_with_dead(lib, n=5000, seed=3):
    b = lib.generate_ics(1, n, seed)
    rng = np.random.default_rng(seed)
    b["lifetime"] = rng.random(n)
    b["luminosity"] = rng.random(n)
    b["spin_x"], b["spin_y"], b["spin_z"] = rng.random(n), rng.random(n), rng.random(n)
    b["mass"][rng.random(n) < 0.05] = 0.0
    b["mass"][rng.random(n) < 0.02] = -1.0
    return b


@pytest.mark.parametrize("fmt,names", [(0, UE), (1, RENDER)])
def test_snapshot_matches_host_loops(lib, fmt, names):
    b = bodies_with_dead(lib)
    s = lib.Sim.from_bodies(b, softening=0.01)
    s.substeps_async(3)
    s.sync()
    state = s.bodies()
    alive = int((~(state["mass"] <= 0)).sum())
    for cap in (len(b), alive - 7, 1):
        got = s.snapshot(fmt, cap)
        want = snapshot_ref(state, names, cap)
        assert got.shape == want.shape
        np.testing.assert_array_equal(got, want)
    s.close()


def test_snapshot_into_a_device_buffer(lib):
    torch = pytest.importorskip("torch")
    b = bodies_with_dead(lib, 3000, 4)
    s = lib.Sim.from_bodies(b, softening=0.01)
    buf = torch.zeros((len(b), 16), dtype=torch.float32, device="cuda")
    k = s.snapshot(0, len(b), device_out=buf.data_ptr())
    np.testing.assert_array_equal(buf[:k].cpu().numpy(), snapshot_ref(s.bodies(), UE, len(b)))
    s.close()


def test_compaction_matches_quasar_compact_and_keeps_stepping(lib):
    b = bodies_with_dead(lib, 6000, 5)
    s = lib.Sim.from_bodies(b, softening=0.01, sph=True)
    s.substeps_async(2)
    s.sync()
    before = s.bodies()
    before["mass"][17] = np.nan  # quasar_compact keeps mass > 0.0 only
    s.set_bodies(before)
    k = s.compact()
    keep = before["mass"] > 0.0
    assert k == int(keep.sum()) and s.count == k
    after = s.bodies()
    np.testing.assert_array_equal(after.view(np.uint8).reshape(k, -1)[:, :80],
                                  before[keep].view(np.uint8).reshape(k, -1)[:, :80])
    np.testing.assert_array_equal(fields(after, ["spin_x", "lifetime", "density", "smoothing_h"]),
                                  fields(before[keep], ["spin_x", "lifetime", "density",
                                                        "smoothing_h"]))
    # stepping on: equal to a handle created over the compacted bodies
    t = lib.Sim.from_bodies(before[keep].astype(BODY_DTYPE), softening=0.01, sph=True)
    t.set_bodies(before[keep].astype(BODY_DTYPE))
    for h in (s, t):
        h.substeps_async(3)
        h.sync()
    out = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "density", "internal_energy"]
    np.testing.assert_array_equal(fields(s.bodies(), out), fields(t.bodies(), out))
    s.close()
    t.close()
