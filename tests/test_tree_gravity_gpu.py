"""Tree build and gravity walk on the GPU against the reference (through the C-ABI).

Tolerances (written per test):
  - tree structure and geometry (body_index, children, centres, half sizes,
    node numbering): bit-exact — index work;
  - cell mass / centre of mass: 1e-13 relative (the reference sums cells in
    insertion order, this library bottom-up);
  - FP64 walk on the reference's own pool, EXACT mode: bit-exact;
  - FP64 walk (fast 1/r^3): per-body |da|/|a| <= 1e-13 on the reference pool,
    <= 1e-11 on this library's own pool;
  - FP32-mixed walk vs FP64 walk, same tree: p99 <= 1e-5, max <= 1e-4.
The known-answer tests mirror the reference's tests/test_physics.c:87-270,
396-421 with the same tolerances.
"""
import numpy as np
import pytest

from conftest import (assert_moments_close, assert_same_topology, fields, golden, rel_err,
                      same_bytes)
from cosmosim_gb300.abi import BODY_DTYPE, NODE_DTYPE

pytestmark = pytest.mark.gpu


def body(x, y, z, m, vx=0.0, vy=0.0, vz=0.0):
    b = np.zeros(1, dtype=BODY_DTYPE)
    b["x"], b["y"], b["z"], b["mass"] = x, y, z, m
    b["vx"], b["vy"], b["vz"] = vx, vy, vz
    return b


def bodies(*rows):
    # concatenate repacks padded dtypes; restore the 168-byte Body layout
    return np.concatenate([body(*r) for r in rows]).astype(BODY_DTYPE)


# ---- known-answer tests (reference tests/test_physics.c) ----

def test_single_body(lib):  # :87-104
    pool, ps = lib.octree_build(body(3.0, 4.0, 5.0, 7.0), np.zeros(8, dtype=NODE_DTYPE))
    assert ps >= 1
    assert abs(pool[0]["total_mass"] - 7.0) < 1e-12
    assert (pool[0]["cx"], pool[0]["cy"], pool[0]["cz"]) == (3.0, 4.0, 5.0)


def test_two_bodies_com(lib):  # :106-124
    pool, _ = lib.octree_build(bodies((1, 0, 0, 1.0), (-1, 0, 0, 3.0)),
                               np.zeros(16, dtype=NODE_DTYPE))
    assert abs(pool[0]["total_mass"] - 4.0) < 1e-12
    assert abs(pool[0]["cx"] + 0.5) < 1e-12
    assert abs(pool[0]["cy"]) < 1e-12 and abs(pool[0]["cz"]) < 1e-12


def test_mass_conservation(lib):  # :126-148
    g = golden("edge_cases.npz")
    b = g["lattice_bodies"]
    pool, _ = lib.octree_build(b)
    assert abs(pool[0]["total_mass"] - b["mass"].sum()) < 1e-8


def test_two_body_force_direction(lib):  # :152-175
    b = bodies((0, 0, 0, 1.0), (5.0, 0, 0, 1.0))
    pool, _ = lib.octree_build(b, np.zeros(16, dtype=NODE_DTYPE))
    lib.octree_compute_forces(pool, b, 1.0, 0.01, 0.0)
    assert b[0]["ax"] > 0 and b[1]["ax"] < 0
    assert abs(b[0]["ay"]) < 1e-12 and abs(b[0]["az"]) < 1e-12
    assert abs(b[1]["ay"]) < 1e-12 and abs(b[1]["az"]) < 1e-12


def test_newton3(lib):  # :177-199
    b = bodies((0, 0, 0, 2.0), (3.0, 4.0, 0, 5.0))
    pool, _ = lib.octree_build(b, np.zeros(16, dtype=NODE_DTYPE))
    lib.octree_compute_forces(pool, b, 1.0, 0.01, 0.0)
    f0 = b[0]["mass"] * fields(b)[0]
    f1 = b[1]["mass"] * fields(b)[1]
    assert np.all(np.abs(f0 + f1) < 1e-10)


def test_inverse_square(lib):  # :201-232
    a = []
    for d in (5.0, 10.0):
        b = bodies((0, 0, 0, 1.0), (d, 0, 0, 1.0))
        pool, _ = lib.octree_build(b, np.zeros(16, dtype=NODE_DTYPE))
        lib.octree_compute_forces(pool, b, 1.0, 0.0001, 0.0)
        a.append(abs(b[0]["ax"]))
    assert abs(a[0] / a[1] - 4.0) < 0.01


def test_vs_direct_sum_golden(lib, orc):  # :234-270 (golden vector)
    g = golden("kat_8body.npz")
    b = g["bodies"].copy()
    pool, ps = lib.octree_build(b)
    assert_same_topology(pool[:ps], g["pool"])
    lib.octree_compute_forces(pool, b, 1.0, 0.1, 0.0)
    direct = orc.direct_forces(g["bodies"], 1.0, 0.1)
    assert np.max(np.abs(fields(b) - direct)) < 1e-10
    assert np.max(np.abs(fields(b) - g["forces"])) < 1e-12


def test_dead_body_skipping(lib):  # :396-421
    b = bodies((0, 0, 0, 10.0), (5.0, 0, 0, 0.0), (-5.0, 0, 0, 3.0))
    pool, _ = lib.octree_build(b, np.zeros(24, dtype=NODE_DTYPE))
    assert abs(pool[0]["total_mass"] - 13.0) < 1e-12
    b["ax"][1] = 123.0  # dead bodies must come back with a = 0
    lib.octree_compute_forces(pool, b, 1.0, 0.01, 0.0)
    assert b[0]["ax"] < 0
    assert b[1]["ax"] == 0.0 and b[1]["ay"] == 0.0 and b[1]["az"] == 0.0


# ---- parity against the reference's outputs ----

def test_tree_matches_reference_pool(lib):
    g = golden("disk_3000.npz")
    pool, ps = lib.octree_build(g["bodies"])
    ref = g["pool"]
    assert ps == len(ref)
    assert_same_topology(pool[:ps], ref)  # numbering included: reference allocation order
    assert_moments_close(pool[:ps], ref)


@pytest.mark.parametrize("case", ["one", "two", "all_dead", "close", "lattice"])
def test_edge_case_trees_and_forces(lib, case):
    """One body, two, no alive body, bodies closer than 2^-21 of the root cube
    and exactly coincident ones (depth-64 leaf), a lattice."""
    g = golden("edge_cases.npz")
    b = g[f"{case}_bodies"].copy()
    pool, ps = lib.octree_build(b)
    ref = g[f"{case}_pool"]
    assert ps == len(ref)
    assert_same_topology(pool[:ps], ref)
    assert_moments_close(pool[:ps], ref)
    lib.octree_compute_forces(pool, b, 1.0, 0.01, 0.5)
    want = g[f"{case}_forces"]
    err = rel_err(fields(b), want)
    assert np.all(err <= 1e-11), (case, err.max())


@pytest.mark.parametrize("theta", [3, 5, 7])
def test_exact_walk_on_reference_pool_is_bitwise(lib, theta):
    """Walking the reference's own pool with the reference's operation
    sequence reproduces its accelerations bit for bit."""
    g = golden("disk_3000.npz")
    b = g["bodies"].copy()
    lib.octree_compute_forces(g["pool"], b, 1.0, 0.01, theta / 10, exact=True)
    np.testing.assert_array_equal(fields(b), g[f"forces_t{theta}"])


@pytest.mark.parametrize("theta", [3, 5, 7])
def test_fp64_walk_on_reference_pool(lib, theta):
    g = golden("disk_3000.npz")
    b = g["bodies"].copy()
    lib.octree_compute_forces(g["pool"], b, 1.0, 0.01, theta / 10)
    err = rel_err(fields(b), g[f"forces_t{theta}"])
    assert err.max() <= 1e-13, err.max()


@pytest.mark.parametrize("theta", [3, 5, 7])
def test_fp64_walk_on_own_tree(lib, theta):
    g = golden("disk_3000.npz")
    b = g["bodies"].copy()
    pool, _ = lib.octree_build(b)
    lib.octree_compute_forces(pool, b, 1.0, 0.01, theta / 10)
    err = rel_err(fields(b), g[f"forces_t{theta}"])
    assert err.max() <= 1e-11, err.max()


def test_fp32_mixed_precision_error(lib):
    g = golden("disk_3000.npz")
    pool = g["pool"]
    b64 = g["bodies"].copy()
    lib.octree_compute_forces(pool, b64, 1.0, 0.01, 0.5)
    b32 = g["bodies"].copy()
    lib.set_precision(lib.PREC_FP32_MIXED)
    try:
        lib.octree_compute_forces(pool, b32, 1.0, 0.01, 0.5)
    finally:
        lib.set_precision(lib.PREC_FP64)
    alive = g["bodies"]["mass"] > 0
    err = rel_err(fields(b32)[alive], fields(b64)[alive])
    assert np.quantile(err, 0.99) <= 1e-5, np.quantile(err, 0.99)
    assert err.max() <= 1e-4, err.max()


def test_oracle_agrees_on_random_trees(lib, orc):
    """Fresh random inputs (not in any fixture): tree and forces vs the oracle
    (60,000 bodies: the FP64 walk's two-pairs-per-block layout)."""
    rng = np.random.default_rng(99)
    for n in (5, 64, 777, 20000, 60000):
        b = np.zeros(n, dtype=BODY_DTYPE)
        b["x"] = rng.standard_cauchy(n) * 0.3
        b["y"] = rng.normal(0, 1, n)
        b["z"] = rng.uniform(-0.1, 0.1, n)
        b["mass"] = rng.uniform(0.1, 1.0, n)
        b["mass"][rng.random(n) < 0.05] = 0.0
        pool, ps = lib.octree_build(b)
        opool, ops = orc.octree_build(b)
        assert ps == ops
        assert_same_topology(pool[:ps], opool[:ops])
        assert_moments_close(pool[:ps], opool[:ops], rel=1e-12)
        fb, ob = b.copy(), b.copy()
        lib.octree_compute_forces(pool, fb, 1.0, 0.01, 0.6)
        orc.octree_compute_forces(opool, ob, 1.0, 0.01, 0.6)
        alive = b["mass"] > 0
        err = rel_err(fields(fb)[alive], fields(ob)[alive])
        assert err.max() <= 1e-10, (n, err.max())
        assert np.all(fields(fb)[~alive] == 0.0)


@pytest.mark.parametrize("precision", [0, 1])
def test_interaction_count_matches_oracle(lib, orc, precision):
    """Both walks (FP64 producer/consumer, FP32-mixed) give every body the
    reference's interaction set: the totals equal the oracle's count."""
    from cosmosim_gb300.lib import Sim

    g = golden("disk_3000.npz")
    b = g["bodies"]
    s = Sim.from_bodies(b, softening=0.01, theta=0.5, precision=precision)
    s.enable_stats(True)
    s.gravity_async()
    got = s.interactions()
    pool, _ = orc.octree_build(b)
    want, _ = orc.count_interactions(pool, b, 0.5)
    assert got == want
    s.close()


def test_pool_numbering_is_reference_allocation_order(lib):
    """Reference numbering holds even when bodies arrive in a shuffled order."""
    rng = np.random.default_rng(3)
    g = golden("disk_3000.npz")
    b = g["bodies"][rng.permutation(len(g["bodies"]))]
    from oracle.orc import Oracle

    opool, ops = Oracle().octree_build(b)
    pool, ps = lib.octree_build(b)
    assert ps == ops
    assert_same_topology(pool[:ps], opool[:ops])


def test_bad_pool_is_reported_not_walked(lib):
    """A pool with a cycle is rejected with an error; bodies stay untouched."""
    b = bodies((0, 0, 0, 1.0), (1, 0, 0, 1.0))
    pool = np.zeros(4, dtype=NODE_DTYPE)
    pool["children"] = -1
    pool["body_index"] = -1
    pool[0]["total_mass"] = 2.0
    pool[0]["half_size"] = 1.0
    pool[0]["children"][0] = 1
    pool[1]["total_mass"] = 1.0
    pool[1]["half_size"] = 0.5
    pool[1]["children"][3] = 0  # back to the root
    before = b.copy()
    with pytest.raises(lib.CudaError):
        lib.octree_compute_forces(pool, b, 1.0, 0.01, 0.5)
    assert same_bytes(b, before)


@pytest.mark.parametrize("n", [3000, 20000, 70000])
def test_handle_walks_match_oracle(lib, orc, n):
    """A handle's walks on its own tree against the oracle's walk on the
    oracle's tree. Up to ~58k bodies the FP64 walk is split by the root's
    children (a producer/consumer pair per child subtree, partials added in
    child order), above it one pair per task; the FP32-mixed walk is split the
    same way while the launch has few tasks. FP64: <= 1e-11 per body (own
    tree); FP32-mixed against that FP64: p99 <= 1e-5, max <= 1e-4; the
    interaction totals equal the oracle's."""
    from cosmosim_gb300.lib import Sim

    b = lib.generate_ics(0, n, 321)
    b["mass"][::53] = 0.0  # dead bodies get no force and exert none
    pool, _ = orc.octree_build(b)
    want = b.copy()
    orc.octree_compute_forces(pool, want, 1.0, 0.01, 0.5)
    count, _ = orc.count_interactions(pool, b, 0.5)
    alive = b["mass"] > 0
    got = {}
    for prec in (0, 1):
        s = Sim.from_bodies(b, softening=0.01, theta=0.5, precision=prec)
        got[prec] = s.bodies()
        s.enable_stats(True)
        s.gravity_async()
        assert s.interactions() == count, prec
        s.close()
    err64 = rel_err(fields(got[0])[alive], fields(want)[alive])
    assert err64.max() <= 1e-11, err64.max()
    assert np.all(fields(got[0])[~alive] == 0.0)
    err32 = rel_err(fields(got[1])[alive], fields(got[0])[alive])
    assert np.quantile(err32, 0.99) <= 1e-5 and err32.max() <= 1e-4, err32.max()
