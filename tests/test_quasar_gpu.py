"""The quasar step on the GPU (csg_quasar_step and handles in quasar mode)
against the reference (src/quasar.c:477-509).

csg_quasar_step vs the reference's own outputs (tests/golden/quasar_3000.npz,
six steps from the generator state the reference starts with): body counts,
live jet counts, types and masses equal; every field within 1e-12 of the
field's largest magnitude (sin, cos and log are CUDA's, within 2 ulp of the C
library's: they enter the positions and velocities of spawned and recycled
jets).
"""
import numpy as np
import pytest

from conftest import fields, golden
from cosmosim_gb300.abi import BODY_DTYPE, QuasarConfig

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def close(got, want, rtol=RTOL):
    scale = np.maximum(np.abs(want).max(axis=0), 1e-300)
    err = np.abs(got - want) / scale
    assert err.max() <= rtol, err.max(axis=0)


def test_quasar_step_matches_reference(lib):
    g = golden("quasar_3000.npz")
    names = [str(x) for x in g["out_fields"]]
    b = g["bodies"].copy()
    cfg = QuasarConfig.from_buffer_copy(g["cfg"].tobytes())
    cfg.jet_count = 40
    cfg.max_bodies = len(b)
    lib.quasar_seed(1, 0)
    n = int(g["n0"])
    want = dict(zip(g["step_numbers"].tolist(), g["steps"]))
    for step in range(1, 7):
        n = lib.quasar_step(b, n, cfg, float(g["dt"]))
        assert (n, cfg.jet_count) == tuple(g["counts"][step - 1])
        if step in want:
            got = fields(b[:n], names)
            w = want[step][:n]
            for f in ("type", "mass"):
                k = names.index(f)
                np.testing.assert_array_equal(got[:, k], w[:, k])
            close(got, w)


def test_quasar_handle_matches_oracle_substeps(lib, orc):
    """A handle in quasar mode (device substep + device quasar step) equals the
    oracle's integrator_step + quasar_step sequence."""
    L = lib.load()
    cfg = L.cosmosim_default_config()
    cfg.n_bodies = 3000
    cfg.merger = 1
    cfg.quasar = 1
    cfg.substeps = 1
    s = lib.Sim(L.cosmosim_create(cfg))
    ref = s.get_bodies_view()
    n = s.count
    qc = L.csg_quasar_default_config()
    qc.accretion_radius = cfg.accretion_radius
    qc.jet_speed = cfg.jet_speed
    qc.feedback_strength = cfg.feedback_strength
    qc.jet_cap = cfg.n_bodies // 10
    n_alloc = cfg.n_bodies + cfg.n_bodies // 5 + cfg.n_bodies // 4
    qc.max_bodies = n_alloc
    buf = np.zeros(n_alloc, dtype=BODY_DTYPE)
    buf[:n] = ref
    pool = np.zeros(8 * n_alloc, dtype=NODE_DTYPE_())
    orc.quasar_seed(1, 0)
    out = ["x", "y", "z", "vx", "vy", "vz", "mass", "type", "density", "internal_energy"]
    for _ in range(3):
        s.step()
        w = buf[:n].copy()
        orc.integrator_step(w, cfg.dt, 1.0, 1.5, cfg.theta, pool, 1)
        buf[:n] = w
        n = orc.quasar_step(buf, n, qc, cfg.dt)
        assert s.count == n
        close(fields(s.bodies(), out), fields(buf[:n], out), 1e-9)
    s.close()


def NODE_DTYPE_():
    from cosmosim_gb300.abi import NODE_DTYPE
    return NODE_DTYPE


def test_quasar_handle_runs_and_compacts_on_the_device(lib):
    """Quasar merger with dust, 61 steps: jets spawn, bodies die, the step-60
    compaction drops the dead ones; the body array stays consistent."""
    L = lib.load()
    cfg = L.cosmosim_default_config()
    cfg.n_bodies = 4000
    cfg.merger = 1
    cfg.quasar = 1
    s = lib.Sim(L.cosmosim_create(cfg))
    n0 = s.count
    for _ in range(59):
        s.step()
    before = s.bodies()
    s.step()  # the 60th step compacts
    after = s.bodies()
    assert s.count == len(after) <= len(before) + 2 * 8 * cfg.substeps * 20
    assert np.all(after["mass"] > 0) or s.count < len(before)
    assert np.isfinite(fields(after, ["x", "y", "z"])).all()
    assert s.count != n0 or (before["type"] == 3).any()
    s.close()


# ---- adversarial cases against the oracle (orc_quasar_step, pinned to the
# reference's golden vector in test_oracle_golden.py) -------------------------

QUASAR_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "mass", "spin_x", "spin_y",
                 "spin_z", "accretion_rate", "luminosity", "lifetime", "density", "pressure",
                 "internal_energy", "smoothing_h"]


def _scene(seed, n_smbh, n_field, n_jets, n_lobes, spare, dead_first=False, far_jets=0.1):
    """SMBHs 1.5 apart (overlapping accretion spheres), stars, gas and dust
    around them (some inside the swallow radius and the ISCO), jets and lobes
    with lifetimes around one step, some jets far out (recycled)."""
    rng = np.random.default_rng(seed)
    n = n_smbh + n_field + n_jets + n_lobes
    b = np.zeros(n + spare, dtype=BODY_DTYPE)
    order = rng.permutation(n)  # interleave the kinds in index order
    kinds = np.r_[np.full(n_smbh, 2), np.zeros(n_field, int), np.full(n_jets, 3),
                  np.full(n_lobes, 5)][order]
    centres = np.stack([1.5 * np.arange(n_smbh), 0.2 * np.arange(n_smbh), np.zeros(n_smbh)], 1)
    host = rng.integers(0, max(n_smbh, 1), n)
    for f in ("x", "y", "z"):
        b[f][:n] = rng.normal(0, 1.2, n)
    if n_smbh:
        b["x"][:n] += centres[host, 0]
        b["y"][:n] += centres[host, 1]
    for f in ("vx", "vy", "vz"):
        b[f][:n] = rng.normal(0, 2.0, n)
    b["mass"][:n] = rng.uniform(0.05, 1.0, n)
    b["type"][:n] = kinds
    field = kinds == 0
    b["type"][:n][field] = rng.choice([0, 1, 4], field.sum(), p=[0.5, 0.4, 0.1])
    gas = b["type"][:n] == 1
    b["smoothing_h"][:n][gas] = rng.uniform(0.0, 0.5, gas.sum())
    b["internal_energy"][:n][gas] = rng.uniform(0.0, 2.0, gas.sum())
    smbh = np.nonzero(kinds == 2)[0]
    b["x"][smbh], b["y"][smbh], b["z"][smbh] = centres.T
    b["mass"][smbh] = rng.uniform(30.0, 60.0, len(smbh))
    b["accretion_rate"][smbh] = rng.uniform(0.0, 50.0, len(smbh))
    b["luminosity"][smbh] = rng.uniform(0.0, 600.0, len(smbh))
    sp = rng.normal(size=(len(smbh), 3))
    sp /= np.linalg.norm(sp, axis=1, keepdims=True)
    if len(smbh):
        sp[0] = (0.0, 0.05, 0.9987)  # spin along z: the other jet frame
    b["spin_x"][smbh], b["spin_y"][smbh], b["spin_z"][smbh] = sp.T
    if dead_first and len(smbh):
        b["mass"][smbh[0]] = 0.0
    jets = np.nonzero(kinds == 3)[0]
    b["lifetime"][jets] = rng.uniform(-0.01, 0.06, len(jets))
    far = jets[rng.random(len(jets)) < far_jets]
    b["x"][far] += 40.0
    lobes = np.nonzero(kinds == 5)[0]
    b["lifetime"][lobes] = rng.uniform(-0.01, 0.06, len(lobes))
    return b, n, int(len(jets))


def _run_both(lib, orc, b, n, cfg, steps, dt=0.02, seed=(99, 0)):
    """Steps the GPU and the oracle from the same bodies and generator state;
    every step starts both from the oracle's bodies. (Recycled jets land at
    exactly the accretion radius of the first SMBH, where the candidate test
    of the next step is decided by the last bit of a position that went
    through sin and cos: CUDA's and the C library's may differ there by an
    ulp. Within one step no transcendental result feeds a decision.)"""
    import copy
    g, c = b.copy(), b.copy()
    cg, cc = copy.copy(cfg), copy.copy(cfg)
    lib.quasar_seed(*seed)
    orc.quasar_seed(*seed)
    ng = nc = n
    for _ in range(steps):
        ng = lib.quasar_step(g, ng, cg, dt)
        nc = orc.quasar_step(c, nc, cc, dt)
        assert (ng, cg.jet_count) == (nc, cc.jet_count)
        np.testing.assert_array_equal(g["type"][:ng], c["type"][:nc])
        np.testing.assert_array_equal(g["mass"][:ng], c["mass"][:nc])
        close(fields(g[:ng], QUASAR_FIELDS), fields(c[:nc], QUASAR_FIELDS))
        g[:] = c
    return g[:ng], ng


@pytest.mark.parametrize("case", ["overlapping", "dead_first", "tight_room", "tight_cap",
                                  "burst", "no_smbh", "many_smbh", "no_ring"])
def test_quasar_step_matches_oracle(lib, orc, case):
    cfg = QuasarConfig.from_buffer_copy(bytes(104))
    for k, v in dict(accretion_radius=3.0, swallow_radius=0.3, isco_radius=0.5,
                     viscosity_alpha=0.05, jet_speed=20.0, jet_mass=0.5, jet_lifetime=0.05,
                     feedback_strength=1.0, eta_eff=0.1, eddington_k=0.5,
                     accretion_smoothing=0.95).items():
        setattr(cfg, k, v)
    cfg.jet_ring_count = 4
    seed = (99, 0)
    kw = dict(n_smbh=3, n_field=3000, n_jets=300, n_lobes=150, spare=4000)
    if case == "dead_first":
        kw["dead_first"] = True
    if case == "tight_room":
        kw["spare"] = 60  # the spawns run out of body capacity mid-ring
    if case == "no_smbh":
        kw["n_smbh"] = 0
    if case == "many_smbh":
        kw.update(n_smbh=40, n_field=6000)
    if case == "burst":
        seed = (12345, 9)  # knot phase 10..: speed modulation above 1.35
    if case == "no_ring":
        cfg.jet_ring_count = 0
    b, n, jets = _scene(7 + len(case), **kw)
    cfg.jet_count = jets
    cfg.jet_cap = jets + {"tight_cap": -130, "many_smbh": 25}.get(case, 100000)
    cfg.max_bodies = len(b)
    out, n_end = _run_both(lib, orc, b, n, cfg, steps=4, seed=seed)
    if case in ("overlapping", "many_smbh"):
        assert n_end > n  # jets were spawned


def test_quasar_step_rejects_too_many_smbhs_and_changes_nothing(lib):
    b, n, jets = _scene(3, n_smbh=1025, n_field=100, n_jets=10, n_lobes=0, spare=100)
    cfg = lib.load().csg_quasar_default_config()
    cfg.jet_count = jets
    before = b.copy()
    L = lib.load()
    import ctypes
    from cosmosim_gb300.abi import ptr
    nn = ctypes.c_int(n)
    L.csg_quasar_step(ptr(b), ctypes.byref(nn), len(b), ctypes.byref(cfg), 0.01)
    assert L.csg_last_error() == 8  # CSG_ERR_UNSUPPORTED
    assert nn.value == n and cfg.jet_count == jets
    from conftest import same_bytes
    assert same_bytes(b, before)
