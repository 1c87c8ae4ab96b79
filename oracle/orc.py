"""ctypes binding of the CPU oracle (test infrastructure only).

Loads ``oracle/liborc.so`` (the C restatement in orc.c) and, when it was built
in this tree, ``oracle/_ref/libcosmosim_ref.so`` (cosmosim's own sources).
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs use
this module; the product library never does.
"""
import ctypes
import os
import subprocess

import numpy as np

from cosmosim_gb300.abi import BODY_DTYPE, NODE_DTYPE, ptr

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_SO = os.path.join(HERE, "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libcosmosim_ref.so")

_c_int_p = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_d = ctypes.c_double
_i = ctypes.c_int


def reference_dir():
    """The cosmosim checkout named by CSG_REFERENCE_DIR, when it holds the
    sources; None otherwise (there is no default location)."""
    ref = os.environ.get("CSG_REFERENCE_DIR")
    if ref and os.path.isdir(os.path.join(ref, "src")):
        return ref
    return None


def build(quiet=True):
    """Compile liborc.so (and the reference library when CSG_REFERENCE_DIR
    names a cosmosim checkout)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE, "liborc.so"], check=True, stdout=out)
    ref = reference_dir()
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True, stdout=out)


def _bind(lib, prefix):
    f = getattr(lib, prefix + "octree_build")
    f.argtypes = [_vp, _c_int_p, _vp, _i]
    f.restype = None
    f = getattr(lib, prefix + "octree_compute_forces")
    f.argtypes = [_vp, _i, _vp, _i, _d, _d, _d]
    f.restype = None
    f = getattr(lib, prefix + "octree_find_neighbors")
    f.argtypes = [_vp, _i, _vp, _i, _d, _d, _d, _d, _vp, _i]
    f.restype = _i
    for name in ("sph_compute_density", "sph_compute_forces"):
        f = getattr(lib, prefix + name)
        f.argtypes = [_vp, _i, _vp]
        f.restype = None
    f = getattr(lib, prefix + "sph_apply_cooling")
    f.argtypes = [_vp, _i, _d]
    f.restype = None
    f = getattr(lib, prefix + "integrator_step")
    f.argtypes = [_vp, _i, _d, _d, _d, _d, _vp, _i]
    f.restype = None
    f = getattr(lib, prefix + "integrator_init_accelerations")
    f.argtypes = [_vp, _i, _d, _d, _d, _vp]
    f.restype = None
    f = getattr(lib, prefix + "quasar_step")
    f.argtypes = [_vp, _c_int_p, _i, _vp, _d]
    f.restype = None


class CpuPhysics:
    """The reference's free-function API over numpy Body/OctreeNode arrays."""

    def __init__(self, lib, prefix):
        self.lib = lib
        self.p = prefix
        _bind(lib, prefix)

    def _f(self, name):
        return getattr(self.lib, self.p + name)

    def octree_build(self, bodies, pool=None):
        n = len(bodies)
        if pool is None:
            pool = np.zeros(max(8 * n, 8), dtype=NODE_DTYPE)
        ps = ctypes.c_int(0)
        self._f("octree_build")(ptr(pool), ctypes.byref(ps), ptr(bodies), n)
        return pool, ps.value

    def octree_compute_forces(self, pool, bodies, G, eps, theta, root=0):
        self._f("octree_compute_forces")(ptr(pool), root, ptr(bodies), len(bodies), G, eps, theta)

    def octree_find_neighbors(self, pool, bodies, c, radius, cap, root=0):
        buf = np.full(max(cap, 1), -1, dtype=np.int32)
        k = self._f("octree_find_neighbors")(ptr(pool), root, ptr(bodies), len(bodies),
                                              c[0], c[1], c[2], radius, ptr(buf), cap)
        return buf[:k].copy()

    def sph_compute_density(self, bodies, pool):
        self._f("sph_compute_density")(ptr(bodies), len(bodies), ptr(pool))

    def sph_compute_forces(self, bodies, pool):
        self._f("sph_compute_forces")(ptr(bodies), len(bodies), ptr(pool))

    def sph_apply_cooling(self, bodies, dt):
        self._f("sph_apply_cooling")(ptr(bodies), len(bodies), dt)

    def integrator_step(self, bodies, dt, G, eps, theta, pool, sph):
        self._f("integrator_step")(ptr(bodies), len(bodies), dt, G, eps, theta, ptr(pool), sph)

    def integrator_init_accelerations(self, bodies, G, eps, theta, pool):
        self._f("integrator_init_accelerations")(ptr(bodies), len(bodies), G, eps, theta,
                                                 ptr(pool))

    def quasar_step(self, bodies, n, cfg, dt):
        """Quasar step on bodies[:n] with room for len(bodies); returns the new
        count (cfg, a QuasarConfig, is updated in place)."""
        nn = ctypes.c_int(n)
        self._f("quasar_step")(ptr(bodies), ctypes.byref(nn), len(bodies), ctypes.byref(cfg), dt)
        return nn.value


class Oracle(CpuPhysics):
    """The C restatement (orc.c) plus its check helpers."""

    def __init__(self):
        if not os.path.exists(ORC_SO):
            build()
        lib = ctypes.CDLL(ORC_SO)
        super().__init__(lib, "orc_")
        lib.orc_octree_count_interactions.argtypes = [_vp, _i, _vp, _i, _d, _vp]
        lib.orc_octree_count_interactions.restype = ctypes.c_int64
        lib.orc_direct_forces.argtypes = [_vp, _i, _vp, _i, _d, _d, _vp]
        lib.orc_direct_forces.restype = None
        lib.orc_total_energy.argtypes = [_vp, _i, _d, _d]
        lib.orc_total_energy.restype = _d
        lib.orc_set_threads.argtypes = [_i]
        lib.orc_set_threads.restype = _i
        lib.orc_quasar_seed.argtypes = [ctypes.c_uint64, _i]
        lib.orc_quasar_seed.restype = None
        lib.orc_generate_ics.argtypes = [_i, _i, ctypes.c_uint64, _vp]
        lib.orc_generate_ics.restype = _i

    def generate_ics(self, kind, n, seed):
        """The library's csg_generate_ics(kind, n, seed) restated on the CPU
        (byte-identical Body[]), so CPU-only runs need not load the library."""
        out = np.zeros(n, dtype=BODY_DTYPE)
        if self.lib.orc_generate_ics(kind, n, seed, ptr(out) if n else None) != n:
            raise ValueError(f"orc_generate_ics: bad kind {kind} or count {n}")
        return out

    def quasar_seed(self, rng_state=1, knot_phase=0):
        self.lib.orc_quasar_seed(rng_state, knot_phase)

    def set_threads(self, n):
        return self.lib.orc_set_threads(n)

    def count_interactions(self, pool, bodies, theta, root=0):
        per = np.zeros(len(bodies), dtype=np.int32)
        tot = self.lib.orc_octree_count_interactions(ptr(pool), root, ptr(bodies), len(bodies),
                                                     theta, ptr(per))
        return tot, per

    def direct_forces(self, bodies, G, eps, idx=None):
        if idx is None:
            m = len(bodies)
            acc = np.zeros((m, 3))
            self.lib.orc_direct_forces(ptr(bodies), len(bodies), None, 0, G, eps, ptr(acc))
        else:
            idx = np.ascontiguousarray(idx, dtype=np.int32)
            acc = np.zeros((len(idx), 3))
            self.lib.orc_direct_forces(ptr(bodies), len(bodies), ptr(idx), len(idx), G, eps,
                                       ptr(acc))
        return acc

    def total_energy(self, bodies, G, eps):
        return self.lib.orc_total_energy(ptr(bodies), len(bodies), G, eps)


def reference():
    """cosmosim's own compiled sources, or None where they were not built here."""
    if not os.path.exists(REF_SO):
        return None
    return CpuPhysics(ctypes.CDLL(REF_SO), "")


__all__ = ["Oracle", "reference", "build", "BODY_DTYPE", "NODE_DTYPE"]
