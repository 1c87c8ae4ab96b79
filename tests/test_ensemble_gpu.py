"""Batched ensembles (cosmosim_create_ensemble) on the GPU.

An ensemble handle holds several independent systems; each gets the octree
the reference would build for it alone, and the walks never cross systems.
So every system's accelerations and orbits must be BIT-IDENTICAL to those of
a handle created over that system alone (same cells, same moments summed in
the same octant order, same per-body interaction order) — in FP64 and in
FP32-mixed, through graph replays, for every walk launch shape.
"""
import numpy as np
import pytest

from conftest import fields

pytestmark = pytest.mark.gpu

OUT = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"]


def _systems(lib, sizes, seed0=100):
    parts = [lib.generate_ics(3, n, seed0 + g) if n > 0 else lib.generate_ics(3, 1, 1)[:0]
             for g, n in enumerate(sizes)]
    return parts


def _concat(parts):
    from cosmosim_gb300.abi import BODY_DTYPE
    return np.concatenate([p.astype(BODY_DTYPE) for p in parts]).astype(BODY_DTYPE)


# uneven sizes, a single body, an empty system and one whose bodies are all dead
SIZES = [2000, 517, 1, 0, 4096, 33, 12000, 64]


def _make(lib, sizes=SIZES, dead=5):
    parts = _systems(lib, sizes)
    if dead is not None and dead < len(parts):
        parts[dead]["mass"] = 0.0
    return parts


@pytest.mark.parametrize("prec,sizes", [(0, SIZES), (1, SIZES),
                                        # 42.5k bodies: the FP64 walk of the ensemble takes the
                                        # two-pairs-per-block layout, each system alone one pair
                                        (0, [30000, 517, 12000]),
                                        # FP64 with one system above the split size (about 58k
                                        # bodies on 152 SMs): one launch of each form
                                        (0, [70000, 2000, 517]),
                                        # FP64, 121k bodies of small systems: the ensemble's
                                        # pairs walk eight root children each, the systems alone
                                        # two or one
                                        (0, [30000, 29000, 31000, 30500, 700]),
                                        # 74.5k bodies: the FP32 ensemble is walked one warp per
                                        # task, the small systems alone eight warps per task
                                        (1, [60000, 2000, 517, 12000])])
def test_ensemble_equals_separate_handles(lib, prec, sizes):
    parts = _make(lib, sizes)
    allb = _concat(parts)
    kw = dict(softening=0.01, theta=0.5, dt=1e-3, precision=prec)
    ens = lib.Sim.ensemble(allb, [len(p) for p in parts], **kw)
    assert ens.system_count == len(parts)
    init = ens.bodies()
    ens.substeps_async(6)
    ens.sync()
    got = ens.bodies()
    ens.close()
    off = 0
    for p in parts:
        n = len(p)
        if n == 0:
            continue
        one = lib.Sim.from_bodies(p, **kw)
        np.testing.assert_array_equal(fields(init[off:off + n], OUT), fields(one.bodies(), OUT))
        one.substeps_async(6)
        one.sync()
        np.testing.assert_array_equal(fields(got[off:off + n], OUT), fields(one.bodies(), OUT))
        one.close()
        off += n


@pytest.mark.parametrize("prec", [0, 1])
def test_walk_shapes_give_identical_results(lib, prec):
    parts = _make(lib)
    allb = _concat(parts)
    ens = lib.Sim.ensemble(allb, [len(p) for p in parts], softening=0.01, precision=prec)
    ref = None
    for shape in [(8, 0, 0), (4, 0, 0), (8, 1, 3), (8, 4, 2), (4, 2, 6), (4, 1, 2)]:
        ens.set_walk_shape(*shape)
        ens.build_tree_async()
        ens.gravity_async()
        ens.sync()
        acc = fields(ens.bodies(), ("ax", "ay", "az"))
        if ref is None:
            ref = acc
        else:
            np.testing.assert_array_equal(acc, ref)
    ens.close()


def test_autotune_keeps_bodies_and_picks_a_candidate(lib):
    parts = _make(lib)
    allb = _concat(parts)
    ens = lib.Sim.ensemble(allb, [len(p) for p in parts], softening=0.01, precision=1)
    before = ens.bodies()
    best, cand = ens.autotune_walk(reps=2)
    assert len(cand) == 20
    assert all(c["ms"] > 0 for c in cand)
    assert best["ms"] == min(c["ms"] for c in cand)
    assert ens.walk_shape()["warps_per_block"] == best["warps_per_block"]
    np.testing.assert_array_equal(fields(ens.bodies(), OUT), fields(before, OUT))
    ens.substeps_async(2)
    ens.sync()
    ens.close()


def test_ensemble_direct_sum_stays_inside_each_system(lib):
    parts = _make(lib, [3000, 1500, 700])
    allb = _concat(parts)
    ens = lib.Sim.ensemble(allb, [len(p) for p in parts], softening=0.01)
    rng = np.random.default_rng(3)
    off = 0
    for p in parts:
        idx = rng.choice(len(p), size=64, replace=False)
        one = lib.Sim.from_bodies(p, softening=0.01)
        want = one.direct_forces(idx)
        got = ens.direct_forces(idx + off)
        err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
        assert err.max() < 1e-12
        one.close()
        off += len(p)
    ens.close()


def test_ensemble_interaction_count_is_the_sum_of_its_systems(lib):
    parts = _make(lib, [2500, 900, 4000])
    allb = _concat(parts)
    ens = lib.Sim.ensemble(allb, [len(p) for p in parts], softening=0.01, precision=1)
    ens.set_walk_shape(8, 2, 3)
    ens.enable_stats(True)
    ens.build_tree_async()
    ens.gravity_async()
    total = ens.interactions()
    ens.close()
    want = 0
    for p in parts:
        one = lib.Sim.from_bodies(p, softening=0.01, precision=1)
        one.enable_stats(True)
        one.build_tree_async()
        one.gravity_async()
        want += one.interactions()
        one.close()
    assert total == want


def test_set_bodies_replaces_the_state_and_keeps_the_systems(lib):
    parts = _make(lib, [1500, 2500], dead=None)
    allb = _concat(parts)
    ens = lib.Sim.ensemble(allb, [1500, 2500], softening=0.01, precision=1)
    other = _concat(_systems(lib, [1500, 2500], seed0=500))
    ens.set_bodies(other)
    ens.sync()
    np.testing.assert_array_equal(fields(ens.bodies(), OUT), fields(other, OUT))
    assert ens.system_count == 2
    ens.substeps_async(2)
    ens.sync()
    got = ens.bodies()
    ens.close()
    off = 0
    for p in _systems(lib, [1500, 2500], seed0=500):
        one = lib.Sim.from_bodies(p, softening=0.01, precision=1)
        one.set_bodies(p)  # same accelerations as uploaded into the ensemble
        one.substeps_async(2)
        one.sync()
        np.testing.assert_array_equal(fields(got[off:off + len(p)], OUT), fields(one.bodies(), OUT))
        one.close()
        off += len(p)
