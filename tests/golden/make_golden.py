"""Generates the golden fixtures in tests/golden/ from cosmosim's own code.

Run with CSG_REFERENCE_DIR naming a cosmosim checkout (it compiles its
sources with `make -C oracle ref REF=$CSG_REFERENCE_DIR`, i.e. cosmosim's
src/*.c built where they lie, into oracle/_ref/libcosmosim_ref.so) and commit
the .npz files it writes:

    CSG_REFERENCE_DIR=<cosmosim checkout> python tests/golden/make_golden.py

Every output below is what the reference library itself returned on the
stored seeded inputs. Inputs are drawn with numpy's PCG64 from fixed seeds.
The 8-body case is the golden vector of the reference's own test suite
(tests/test_physics.c:234-270).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cosmosim_gb300.abi import BODY_DTYPE, BODY_GAS, NODE_DTYPE  # noqa: E402
from oracle import orc  # noqa: E402


def disk(rng, n, gas_frac=0.0, dead_frac=0.0, h=0.2):
    b = np.zeros(n, dtype=BODY_DTYPE)
    r = rng.exponential(1.0, n)
    th = rng.uniform(0, 2 * np.pi, n)
    b["x"] = r * np.cos(th)
    b["y"] = r * np.sin(th)
    b["z"] = rng.normal(0, 0.1, n)
    vc = np.sqrt((1 - np.exp(-r) * (1 + r)) / np.maximum(r, 1e-3))
    b["vx"] = -vc * np.sin(th) + rng.normal(0, 0.02, n)
    b["vy"] = vc * np.cos(th) + rng.normal(0, 0.02, n)
    b["vz"] = rng.normal(0, 0.005, n)
    b["mass"] = 1.0 / n * rng.uniform(0.5, 1.5, n)
    if dead_frac:
        b["mass"][rng.random(n) < dead_frac] = 0.0
    g = rng.random(n) < gas_frac
    b["type"][g] = BODY_GAS
    b["internal_energy"][g] = rng.uniform(0.2, 1.0, g.sum())
    b["smoothing_h"][g] = h
    return b


OUT_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "density", "pressure",
              "internal_energy", "smoothing_h"]


def fields(b, names=("ax", "ay", "az")):
    """The output fields of a Body array as one (n, k) float64 array."""
    return np.stack([b[f] for f in names], axis=1)


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name), **arrays)


def main():
    orc.build(quiet=False)
    ref = orc.reference()
    if ref is None:
        raise SystemExit("reference library not built (needs the reference sources)")

    # 1. the reference test suite's 8-body golden vector (theta 0, eps 0.1)
    pos = np.array([[1, 2, 3], [-4, 5, -1], [7, -3, 2], [0, 0, 0],
                    [-2, -6, 4], [3, 1, -5], [-1, 8, 0], [6, -2, -3]], dtype=float)
    mas = np.array([1, 3, 2, 5, 1, 4, 2, 3], dtype=float)
    b8 = np.zeros(8, dtype=BODY_DTYPE)
    b8["x"], b8["y"], b8["z"] = pos.T
    b8["mass"] = mas
    pool, ps = ref.octree_build(b8)
    f8 = b8.copy()
    ref.octree_compute_forces(pool, f8, 1.0, 0.1, 0.0)
    save("kat_8body.npz", bodies=b8, pool=pool[:ps], forces=fields(f8))

    # 2. seeded disks: tree and forces at several theta
    rng = np.random.default_rng(20260101)
    b = disk(rng, 3000, dead_frac=0.01)
    pool, ps = ref.octree_build(b)
    res = {"bodies": b, "pool": pool[:ps]}
    for th in (0.3, 0.5, 0.7):
        f = b.copy()
        ref.octree_compute_forces(pool, f, 1.0, 0.01, th)
        res[f"forces_t{int(th * 10)}"] = fields(f)
    save("disk_3000.npz", **res)

    # 3. edge cases: one body, two, all dead, near/exactly coincident bodies
    cases = {}
    one = np.zeros(1, dtype=BODY_DTYPE)
    one["x"], one["y"], one["z"], one["mass"] = 3.0, 4.0, 5.0, 7.0
    cases["one"] = one
    two = np.zeros(2, dtype=BODY_DTYPE)
    two["x"] = [1.0, -1.0]
    two["mass"] = [1.0, 3.0]
    cases["two"] = two
    dead = disk(rng, 16)
    dead["mass"] = 0.0
    cases["all_dead"] = dead
    close = disk(rng, 400)
    close[1]["x"], close[1]["y"], close[1]["z"] = close[0]["x"] + 1e-9, close[0]["y"], close[0]["z"]
    for k in (3, 4, 5):  # three bodies at one point
        close[k]["x"], close[k]["y"], close[k]["z"] = close[2]["x"], close[2]["y"], close[2]["z"]
    close[7]["x"] = close[6]["x"] + 3e-7
    close[7]["y"] = close[6]["y"] - 2e-8
    close[7]["z"] = close[6]["z"]
    cases["close"] = close
    lattice = np.zeros(100, dtype=BODY_DTYPE)  # reference tests/test_physics.c:126-148
    i = np.arange(100)
    lattice["x"] = (i * 17 % 97) - 48.0
    lattice["y"] = (i * 31 % 89) - 44.0
    lattice["z"] = (i * 13 % 73) - 36.0
    lattice["mass"] = 1.0 + (i % 5)
    cases["lattice"] = lattice
    edge = {}
    for name, bb in cases.items():
        pool, ps = ref.octree_build(bb)
        f = bb.copy()
        ref.octree_compute_forces(pool, f, 1.0, 0.01, 0.5)
        edge[f"{name}_bodies"] = bb
        edge[f"{name}_pool"] = pool[:ps]
        edge[f"{name}_forces"] = fields(f)
    save("edge_cases.npz", **edge)

    # 4. SPH: gas/star mix, neighbour lists (full and tiny cap), density, forces, cooling
    rng = np.random.default_rng(7)
    b = disk(rng, 3000, gas_frac=0.3, dead_frac=0.01, h=0.15)
    pool, ps = ref.octree_build(b)
    q = rng.normal(0, 0.7, (24, 3))
    nb_full, nb_cap = [], []
    for c in q:
        nb_full.append(ref.octree_find_neighbors(pool, b, c, 0.3, 128))
        nb_cap.append(ref.octree_find_neighbors(pool, b, c, 0.3, 7))
    dens = b.copy()
    ref.sph_compute_density(dens, pool)
    frc = dens.copy()
    frc["ax"] = frc["ay"] = frc["az"] = 0.0
    ref.sph_compute_forces(frc, pool)
    cool = frc.copy()
    for _ in range(5):
        ref.sph_apply_cooling(cool, 0.01)
    pad = lambda lists: np.array([np.pad(x, (0, 128 - len(x)), constant_values=-1) for x in lists])
    sph_f = ("density", "pressure", "smoothing_h", "internal_energy", "ax", "ay", "az")
    save("sph_3000.npz", bodies=b, pool=pool[:ps], queries=q,
         nb_full=pad(nb_full), nb_full_n=np.array([len(x) for x in nb_full]),
         nb_cap=pad(nb_cap), nb_cap_n=np.array([len(x) for x in nb_cap]),
         density=fields(dens, sph_f), forces=fields(frc, sph_f), cooled=fields(cool, sph_f))

    # 5. leapfrog with SPH: 8 reference integrator steps
    rng = np.random.default_rng(11)
    b = disk(rng, 1500, gas_frac=0.2, dead_frac=0.01, h=0.15)
    pool = np.zeros(8 * len(b), dtype=NODE_DTYPE)
    s = b.copy()
    ref.integrator_init_accelerations(s, 1.0, 0.01, 0.5, pool)
    init = s.copy()
    steps = []
    for _ in range(8):
        ref.integrator_step(s, 1e-3, 1.0, 0.01, 0.5, pool, 1)
        steps.append(fields(s, OUT_FIELDS))
    keep = [0, 3, 7]  # states after steps 1, 4 and 8
    save("kdk_1500.npz", bodies=b, init=fields(init, OUT_FIELDS),
         steps=np.array([steps[k] for k in keep]), step_numbers=np.array(keep) + 1,
         out_fields=np.array(OUT_FIELDS))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


QUASAR_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "mass", "type", "spin_x",
                 "spin_y", "spin_z", "accretion_rate", "luminosity", "lifetime", "density",
                 "pressure", "internal_energy", "smoothing_h"]


def quasar_bodies(rng, n=3000, extra=600):
    """Two SMBHs with stars and gas around them (some inside the swallow and
    ISCO radii), jets about to expire or far enough to be recycled, lobes,
    dust and dead bodies; room for `extra` appended bodies."""
    from cosmosim_gb300.abi import BODY_DUST, BODY_JET, BODY_LOBE, BODY_SMBH

    b = np.zeros(n + extra, dtype=BODY_DTYPE)
    c = np.array([[0.0, 0.0, 0.0], [12.0, 0.0, 0.0]])
    b["type"][:2] = BODY_SMBH
    b["mass"][:2] = [5.0, 3.0]
    b["x"][:2], b["y"][:2], b["z"][:2] = c[:, 0], c[:, 1], c[:, 2]
    b["vx"][:2] = [0.05, -0.08]
    b["spin_x"][:2], b["spin_y"][:2], b["spin_z"][:2] = [0.0, 0.1], [0.7071, 0.1], [0.7071, 0.99]
    b["accretion_rate"][:2] = [2.0, 0.5]
    b["luminosity"][:2] = [5.0, 1.0]
    m = n - 2 - 40 - 10 - 20
    host = rng.integers(0, 2, m)
    r = rng.exponential(1.6, m)
    th = rng.uniform(0, 2 * np.pi, m)
    k = slice(2, 2 + m)
    b["x"][k] = c[host, 0] + r * np.cos(th)
    b["y"][k] = c[host, 1] + r * np.sin(th)
    b["z"][k] = rng.normal(0, 0.2, m)
    vc = np.sqrt(np.where(host == 0, 5.0, 3.0) / np.maximum(r, 0.05)) * rng.uniform(0.2, 1.2, m)
    b["vx"][k] = -vc * np.sin(th) + rng.normal(0, 0.1, m)
    b["vy"][k] = vc * np.cos(th) + rng.normal(0, 0.1, m)
    b["vz"][k] = rng.normal(0, 0.05, m)
    b["mass"][k] = rng.uniform(0.001, 0.01, m)
    gas = rng.random(m) < 0.3
    b["type"][k] = np.where(gas, BODY_GAS, 0)
    b["internal_energy"][k] = np.where(gas & (rng.random(m) < 0.8), rng.uniform(0.1, 1.0, m), 0.0)
    b["smoothing_h"][k] = np.where(gas & (rng.random(m) < 0.8), 0.2, 0.0)
    b["mass"][k][rng.random(m) < 0.02] = 0.0
    j = slice(2 + m, 2 + m + 40)
    b["type"][j] = BODY_JET
    b["mass"][j] = rng.choice([0.5, 0.3, 0.15], 40)
    b["lifetime"][j] = rng.uniform(-0.01, 0.1, 40)
    far = rng.random(40) < 0.3
    rj = np.where(far, rng.uniform(31.0, 40.0, 40), rng.uniform(0.5, 20.0, 40))
    pj = rng.normal(0, 1, (40, 3))
    pj /= np.linalg.norm(pj, axis=1)[:, None]
    b["x"][j], b["y"][j], b["z"][j] = (rj[:, None] * pj).T
    b["vx"][j], b["vy"][j], b["vz"][j] = rng.normal(0, 5.0, (3, 40))
    lo = slice(2 + m + 40, 2 + m + 50)
    b["type"][lo] = BODY_LOBE
    b["mass"][lo] = 0.25
    b["lifetime"][lo] = rng.uniform(-0.01, 0.08, 10)
    b["x"][lo] = rng.uniform(-20, 20, 10)
    du = slice(2 + m + 50, n)
    b["type"][du] = BODY_DUST
    b["mass"][du] = rng.uniform(0.4, 1.0, n - (2 + m + 50))
    b["x"][du] = rng.uniform(-5, 15, n - (2 + m + 50))
    b["y"][du] = rng.uniform(-3, 3, n - (2 + m + 50))
    return b, n


def quasar_golden():
    """Runs in a fresh process: the reference's quasar_step keeps its random
    generator and knot phase in file statics that start at 1 and 0."""
    import ctypes

    from cosmosim_gb300.abi import QuasarConfig

    orc.build()
    ref = orc.reference()
    ref.lib.quasar_default_config.restype = QuasarConfig
    rng = np.random.default_rng(21)
    b0, n0 = quasar_bodies(rng)
    cfg = ref.lib.quasar_default_config()
    cfg.jet_count = 40
    cfg.max_bodies = len(b0)
    s, n = b0.copy(), n0
    steps, counts = [], []
    for _ in range(6):
        n = ref.quasar_step(s, n, cfg, 0.02)
        steps.append(fields(s, QUASAR_FIELDS))
        counts.append((n, cfg.jet_count))
    keep = [0, 5]  # states after steps 1 and 6 (bodies in use at the end)
    save("quasar_3000.npz", bodies=b0, n0=n0, dt=0.02,
         steps=np.array([steps[k][:n] for k in keep]), step_numbers=np.array(keep) + 1,
         counts=np.array(counts), out_fields=np.array(QUASAR_FIELDS),
         cfg=np.frombuffer(bytes(ref.lib.quasar_default_config()), dtype=np.uint8))
    del ctypes


if __name__ == "__main__":
    if sys.argv[1:] == ["--quasar"]:
        quasar_golden()
    else:
        main()
        import subprocess

        subprocess.run([sys.executable, __file__, "--quasar"], check=True)
