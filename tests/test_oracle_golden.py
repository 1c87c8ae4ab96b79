"""The CPU oracle reproduces the reference's outputs bit for bit (CPU).

Fixtures in tests/golden/ were produced by cosmosim's own compiled sources
(tests/golden/make_golden.py). The oracle is compiled with -ffp-contract=off,
like the fixtures' library, so every comparison here is exact.
"""
import numpy as np

from conftest import fields, golden
from cosmosim_gb300.abi import NODE_DTYPE

OUT_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "density", "pressure",
              "internal_energy", "smoothing_h"]


def same_pool(a, b):
    assert len(a) == len(b)
    for f in a.dtype.names:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


def test_kat_8body(orc):
    g = golden("kat_8body.npz")
    b = g["bodies"].copy()
    pool, ps = orc.octree_build(b)
    same_pool(pool[:ps], g["pool"])
    orc.octree_compute_forces(pool, b, 1.0, 0.1, 0.0)
    np.testing.assert_array_equal(fields(b), g["forces"])
    # and the reference test's own check: theta=0 equals the direct sum to 1e-10
    direct = orc.direct_forces(g["bodies"], 1.0, 0.1)
    assert np.max(np.abs(direct - g["forces"])) < 1e-10


def test_disk_tree_and_forces(orc):
    g = golden("disk_3000.npz")
    b = g["bodies"]
    pool, ps = orc.octree_build(b)
    same_pool(pool[:ps], g["pool"])
    for th in (3, 5, 7):
        f = b.copy()
        orc.octree_compute_forces(pool, f, 1.0, 0.01, th / 10)
        np.testing.assert_array_equal(fields(f), g[f"forces_t{th}"])


def test_edge_cases(orc):
    g = golden("edge_cases.npz")
    for name in ("one", "two", "all_dead", "close", "lattice"):
        b = g[f"{name}_bodies"]
        pool, ps = orc.octree_build(b)
        same_pool(pool[:ps], g[f"{name}_pool"])
        f = b.copy()
        orc.octree_compute_forces(pool, f, 1.0, 0.01, 0.5)
        np.testing.assert_array_equal(fields(f), g[f"{name}_forces"], err_msg=name)


def test_sph(orc):
    g = golden("sph_3000.npz")
    b = g["bodies"]
    pool = g["pool"]
    for k, c in enumerate(g["queries"]):
        full = orc.octree_find_neighbors(pool, b, c, 0.3, 128)
        np.testing.assert_array_equal(full, g["nb_full"][k][: g["nb_full_n"][k]])
        cap = orc.octree_find_neighbors(pool, b, c, 0.3, 7)
        np.testing.assert_array_equal(cap, g["nb_cap"][k][: g["nb_cap_n"][k]])
    names = ("density", "pressure", "smoothing_h", "internal_energy", "ax", "ay", "az")
    d = b.copy()
    orc.sph_compute_density(d, pool)
    np.testing.assert_array_equal(fields(d, names), g["density"])
    d["ax"] = d["ay"] = d["az"] = 0.0
    orc.sph_compute_forces(d, pool)
    np.testing.assert_array_equal(fields(d, names), g["forces"])
    for _ in range(5):
        orc.sph_apply_cooling(d, 0.01)
    np.testing.assert_array_equal(fields(d, names), g["cooled"])


def test_leapfrog_with_sph(orc):
    g = golden("kdk_1500.npz")
    b = g["bodies"].copy()
    pool = np.zeros(8 * len(b), dtype=NODE_DTYPE)
    orc.integrator_init_accelerations(b, 1.0, 0.01, 0.5, pool)
    np.testing.assert_array_equal(fields(b, OUT_FIELDS), g["init"])
    want = dict(zip(g["step_numbers"].tolist(), g["steps"]))
    for step in range(1, 9):
        orc.integrator_step(b, 1e-3, 1.0, 0.01, 0.5, pool, 1)
        if step in want:
            np.testing.assert_array_equal(fields(b, OUT_FIELDS), want[step], err_msg=f"step {step}")


def test_interaction_count_matches_walk(orc):
    """The oracle's counter counts exactly the terms the walk sums."""
    g = golden("disk_3000.npz")
    b = g["bodies"]
    pool, _ = orc.octree_build(b)
    total, per = orc.count_interactions(pool, b, 0.0)
    alive = b["mass"] > 0
    # theta = 0 opens every cell: each alive body meets every other alive leaf
    assert np.all(per[alive] == alive.sum() - 1)
    assert total == per.sum()


def quasar_cfg(g):
    from cosmosim_gb300.abi import QuasarConfig

    cfg = QuasarConfig.from_buffer_copy(g["cfg"].tobytes())
    cfg.jet_count = 40
    cfg.max_bodies = len(g["bodies"])
    return cfg


def test_quasar_step(orc):
    """Six quasar steps (accretion, feedback, jet decay into lobes, recycling,
    spawning with the reference's random stream) equal the reference's."""
    g = golden("quasar_3000.npz")
    names = [str(x) for x in g["out_fields"]]
    b = g["bodies"].copy()
    cfg = quasar_cfg(g)
    orc.quasar_seed(1, 0)
    n = int(g["n0"])
    want = dict(zip(g["step_numbers"].tolist(), g["steps"]))
    for step in range(1, 7):
        n = orc.quasar_step(b, n, cfg, float(g["dt"]))
        assert (n, cfg.jet_count) == tuple(g["counts"][step - 1])
        if step in want:
            np.testing.assert_array_equal(fields(b[:n], names), want[step][:n])
