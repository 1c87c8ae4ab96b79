"""ctypes binding of libcosmosim_gb300.so — the reference API over numpy arrays.

The names and argument meanings follow cosmosim's C API (octree.h,
integrator.h, sph.h, cosmosim_api.h); Body and OctreeNode arrays are numpy
arrays of the ABI dtypes in ``cosmosim_gb300.abi``. There is no fallback: if
the library is missing, loading raises.
"""
import ctypes
import os

import numpy as np

from .abi import BODY_DTYPE, NODE_DTYPE, CosmosimConfig, QuasarConfig, ptr

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcosmosim_gb300.so")

PREC_FP64 = 0
PREC_FP32_MIXED = 1
ADJ_TREE = 0
ADJ_DIRECT = 1

_vp = ctypes.c_void_p
_d = ctypes.c_double
_i = ctypes.c_int
_ip = ctypes.POINTER(ctypes.c_int)


class CsgSimParams(ctypes.Structure):
    _fields_ = [("G", _d), ("softening", _d), ("theta", _d), ("dt", _d),
                ("substeps", _i), ("sph", _i), ("precision", _i)]


class CsgWalkShape(ctypes.Structure):
    _fields_ = [("warps_per_block", _i), ("task_group", _i), ("blocks_per_sm", _i),
                ("ms", ctypes.c_float)]

    def as_dict(self):
        return {"warps_per_block": self.warps_per_block, "task_group": self.task_group,
                "blocks_per_sm": self.blocks_per_sm, "ms": round(float(self.ms), 4)}


class CsgPhaseTimes(ctypes.Structure):
    _fields_ = [(f, _d) for f in ("kick_drift_ms", "build_ms", "gravity_ms", "sph_ms", "kick_ms",
                                  "cooling_ms", "substep_ms")] + [("substeps", ctypes.c_longlong)] + [
        (f, _d) for f in ("build_keys_ms", "build_sort_ms", "build_cells_ms", "build_moments_ms",
                          "build_rest_ms")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class CudaError(RuntimeError):
    pass


_SIGS = {
    "octree_build": ([_vp, _ip, _vp, _i], None),
    "octree_compute_forces": ([_vp, _i, _vp, _i, _d, _d, _d], None),
    "csg_octree_compute_forces_exact": ([_vp, _i, _vp, _i, _d, _d, _d], None),
    "octree_find_neighbors": ([_vp, _i, _vp, _i, _d, _d, _d, _d, _vp, _i], _i),
    "integrator_step": ([_vp, _i, _d, _d, _d, _d, _vp, _i], None),
    "integrator_init_accelerations": ([_vp, _i, _d, _d, _d, _vp], None),
    "sph_compute_density": ([_vp, _i, _vp], None),
    "sph_compute_forces": ([_vp, _i, _vp], None),
    "sph_apply_cooling": ([_vp, _i, _d], None),
    "cosmosim_default_config": ([], CosmosimConfig),
    "cosmosim_create": ([CosmosimConfig], _vp),
    "cosmosim_create_ex": ([CosmosimConfig, _d, _d, _i], _vp),
    "cosmosim_create_from_bodies": ([_vp, _i, ctypes.POINTER(CsgSimParams)], _vp),
    "cosmosim_step": ([_vp], None),
    "cosmosim_get_bodies": ([_vp], _vp),
    "cosmosim_get_count": ([_vp], _i),
    "cosmosim_get_active_count": ([_vp], _i),
    "cosmosim_get_sim_time": ([_vp], _d),
    "cosmosim_destroy": ([_vp], None),
    "cosmosim_last_error": ([_vp], _i),
    "cosmosim_substeps_async": ([_vp, _i], _i),
    "cosmosim_sync": ([_vp], _i),
    "cosmosim_set_stream": ([_vp, _vp], _i),
    "cosmosim_copy_bodies": ([_vp, _vp, _i], _i),
    "cosmosim_set_bodies": ([_vp, _vp, _i], _i),
    "cosmosim_snapshot_f32": ([_vp, _i, _vp, _i, _i], _i),
    "cosmosim_compact": ([_vp], _i),
    "csg_generate_ics_device": ([_i, _i, ctypes.c_uint64, _vp, _vp], _i),
    "cosmosim_create_ensemble_ics": ([_i, _i, _ip, ctypes.c_uint64, ctypes.POINTER(CsgSimParams)],
                                     _vp),
    "csg_quasar_step": ([_vp, _ip, _i, _vp, _d], None),
    "csg_quasar_seed": ([ctypes.c_uint64, _i], None),
    "csg_quasar_default_config": ([], QuasarConfig),
    "cosmosim_build_tree_async": ([_vp], _i),
    "cosmosim_gravity_async": ([_vp], _i),
    "cosmosim_enable_stats": ([_vp, _i], _i),
    "cosmosim_interactions": ([_vp, ctypes.POINTER(ctypes.c_int64)], _i),
    "cosmosim_node_count": ([_vp, _ip], _i),
    "cosmosim_walk_stats": ([_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                             ctypes.POINTER(ctypes.c_int64)], _i),
    "cosmosim_set_precision": ([_vp, _i], _i),
    "csg_last_error": ([], _i),
    "csg_error_string": ([_i], ctypes.c_char_p),
    "csg_set_precision": ([_i], None),
    "csg_release_thread_state": ([], None),
    "cosmosim_enable_phase_timing": ([_vp, _i], _i),
    "cosmosim_phase_times": ([_vp, ctypes.POINTER(CsgPhaseTimes)], _i),
    "csg_enable_phase_timing": ([_i], _i),
    "csg_phase_times": ([ctypes.POINTER(CsgPhaseTimes)], _i),
    "cosmosim_set_wait_limit": ([_vp, _i], _i),
    "csg_set_wait_limit": ([_i], None),
    "csg_check_device_wait": ([_i, _ip], _i),
    "csg_inject_alloc_failure": ([ctypes.c_longlong], None),
    "csg_generate_ics": ([_i, _i, ctypes.c_uint64, _vp], _i),
    "cosmosim_direct_forces": ([_vp, _vp, _i, _vp], _i),
    "cosmosim_energy": ([_vp, ctypes.POINTER(_d), ctypes.POINTER(_d)], _i),
    "cosmosim_launch_count": ([_vp], ctypes.c_int64),
    "csg_measure_fp_peaks": ([ctypes.POINTER(_d), ctypes.POINTER(_d)], _i),
    "csg_check_div_sqrt": ([ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int64),
                            ctypes.POINTER(ctypes.c_int64)], _i),
    "csg_sort_keys": ([_vp, _i, _i, _vp, _vp], _i),
    "cosmosim_enable_graphs": ([_vp, _i], _i),
    "csg_direct_forces_noalloc": ([_vp, _vp, _vp, _vp, _vp, _i, _vp, _i, _d, _d, _vp, _vp], _i),
    "cosmosim_create_ensemble": ([_vp, _i, _i, _ip, ctypes.POINTER(CsgSimParams)], _vp),
    "cosmosim_system_count": ([_vp], _i),
    "cosmosim_set_walk_shape": ([_vp, ctypes.POINTER(CsgWalkShape)], _i),
    "cosmosim_get_walk_shape": ([_vp, ctypes.POINTER(CsgWalkShape)], _i),
    "cosmosim_autotune_walk": ([_vp, _i, ctypes.POINTER(CsgWalkShape),
                                ctypes.POINTER(CsgWalkShape), _i, _ip], _i),
    "csg_adjoint_create": ([_i, ctypes.POINTER(CsgSimParams), _i, _i], _vp),
    "csg_adjoint_destroy": ([_vp], None),
    "csg_adjoint_forward": ([_vp, _vp, _vp, _i, ctypes.POINTER(_d), _vp], _i),
    "csg_adjoint_backward": ([_vp, _vp, _vp], _i),
    "csg_adjoint_forward_frozen": ([_vp, _vp, _vp, ctypes.POINTER(_d)], _i),
    "csg_adjoint_stats": ([_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                           ctypes.POINTER(ctypes.c_int64)], _i),
}

_lib = None


def load(path=None):
    """Loads (once) and returns the ctypes library; raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(
            f"{p} not built: run `python -m cosmosim_gb300.build` (there is no CPU fallback)")
    lib = ctypes.CDLL(p)
    for name, (args, res) in _SIGS.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    if path is None:
        _lib = lib
    return lib


def exported_symbols():
    return sorted(_SIGS)


def _check(lib, what):
    rc = lib.csg_last_error()
    if rc:
        raise CudaError(f"{what}: {lib.csg_error_string(rc).decode()} (code {rc})")


def last_error():
    return load().csg_last_error()


def set_precision(p):
    load().csg_set_precision(p)


# ---- free functions (reference octree.h / integrator.h / sph.h) ----

def octree_build(bodies, pool=None):
    lib = load()
    n = len(bodies)
    if pool is None:
        pool = np.zeros(max(8 * n, 8), dtype=NODE_DTYPE)
    ps = ctypes.c_int(0)
    lib.octree_build(ptr(pool), ctypes.byref(ps), ptr(bodies), n)
    _check(lib, "octree_build")
    return pool, ps.value


def octree_compute_forces(pool, bodies, G, softening, theta, root=0, exact=False):
    lib = load()
    f = lib.csg_octree_compute_forces_exact if exact else lib.octree_compute_forces
    f(ptr(pool), root, ptr(bodies), len(bodies), G, softening, theta)
    _check(lib, "octree_compute_forces")


def octree_find_neighbors(pool, bodies, center, radius, cap, root=0):
    lib = load()
    buf = np.full(max(cap, 1), -1, dtype=np.int32)
    k = lib.octree_find_neighbors(ptr(pool), root, ptr(bodies), len(bodies), center[0],
                                  center[1], center[2], radius, ptr(buf), cap)
    _check(lib, "octree_find_neighbors")
    return buf[:k].copy()


def integrator_step(bodies, dt, G, softening, theta, pool, sph_enabled):
    lib = load()
    lib.integrator_step(ptr(bodies), len(bodies), dt, G, softening, theta, ptr(pool),
                        int(sph_enabled))
    _check(lib, "integrator_step")


def integrator_init_accelerations(bodies, G, softening, theta, pool):
    lib = load()
    lib.integrator_init_accelerations(ptr(bodies), len(bodies), G, softening, theta, ptr(pool))
    _check(lib, "integrator_init_accelerations")


def sph_compute_density(bodies, pool):
    lib = load()
    lib.sph_compute_density(ptr(bodies), len(bodies), ptr(pool))
    _check(lib, "sph_compute_density")


def sph_compute_forces(bodies, pool):
    lib = load()
    lib.sph_compute_forces(ptr(bodies), len(bodies), ptr(pool))
    _check(lib, "sph_compute_forces")


def sph_apply_cooling(bodies, dt):
    lib = load()
    lib.sph_apply_cooling(ptr(bodies), len(bodies), dt)
    _check(lib, "sph_apply_cooling")


def quasar_step(bodies, n, cfg, dt):
    """The GPU quasar step (csg_quasar_step) on bodies[:n] with room for
    len(bodies); returns the new count (cfg.jet_count is updated in place)."""
    lib = load()
    nn = ctypes.c_int(n)
    lib.csg_quasar_step(ptr(bodies), ctypes.byref(nn), len(bodies), ctypes.byref(cfg), dt)
    _check(lib, "csg_quasar_step")
    return nn.value


def quasar_seed(rng_state=1, knot_phase=0):
    lib = load()
    lib.csg_quasar_seed(rng_state, knot_phase)
    _check(lib, "csg_quasar_seed")


def measure_fp_peaks():
    """(FP32, FP64) FMA throughput of the current GPU in TFLOP/s."""
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    rc = load().csg_measure_fp_peaks(ctypes.byref(a), ctypes.byref(b))
    if rc:
        raise CudaError(f"peak probe failed ({rc})")
    return a.value, b.value


def check_div_sqrt(n, seed=1):
    """(division, square root) mismatches of the integer-pipe operators against
    the compiler's correctly rounded ones over n seeded cases (csg_check_div_sqrt)."""
    a, b = ctypes.c_int64(0), ctypes.c_int64(0)
    rc = load().csg_check_div_sqrt(n, seed, ctypes.byref(a), ctypes.byref(b))
    if rc:
        raise CudaError(f"csg_check_div_sqrt failed ({rc})")
    return a.value, b.value


def generate_ics(kind, n, seed):
    """Seeded initial conditions of benchmark configuration `kind` (0-6)."""
    lib = load()
    out = np.zeros(n, dtype=BODY_DTYPE)
    if lib.csg_generate_ics(kind, n, seed, ptr(out)) != n:
        raise ValueError(f"bad ICs request kind={kind} n={n}")
    return out


def sort_keys(keys, bits=64):
    """The tree build's radix sort (csg_sort_keys) on uint64 keys: returns
    (sorted keys, input position of each sorted key); stable."""
    lib = load()
    k = np.ascontiguousarray(keys, dtype=np.uint64)
    out = np.empty_like(k)
    idx = np.empty(len(k), dtype=np.int32)
    rc = lib.csg_sort_keys(ptr(k), len(k), bits, ptr(out), ptr(idx))
    if rc:
        raise CudaError(f"csg_sort_keys: {lib.csg_error_string(rc).decode()} (code {rc})")
    return out, idx


# ---- handle API (reference cosmosim_api.h) ----

class Sim:
    """A device-resident simulation handle (cosmosim_create / _create_from_bodies)."""

    def __init__(self, handle):
        if not handle:
            lib = load()
            raise CudaError(f"create failed: {lib.csg_error_string(lib.csg_last_error()).decode()}")
        self.h = ctypes.c_void_p(handle)
        self.lib = load()

    @classmethod
    def from_config(cls, config=None):
        lib = load()
        return cls(lib.cosmosim_create(config or lib.cosmosim_default_config()))

    @classmethod
    def from_bodies(cls, bodies, G=1.0, softening=0.01, theta=0.5, dt=1e-3, substeps=1,
                    sph=False, precision=PREC_FP64):
        lib = load()
        p = CsgSimParams(G, softening, theta, dt, substeps, int(sph), precision)
        return cls(lib.cosmosim_create_from_bodies(ptr(bodies), len(bodies), ctypes.byref(p)))

    @classmethod
    def ensemble(cls, bodies, counts, G=1.0, softening=0.01, theta=0.5, dt=1e-3, substeps=1,
                 precision=PREC_FP64):
        """One handle over len(counts) independent systems (cosmosim_create_ensemble):
        system g is the counts[g] bodies after those of systems 0..g-1."""
        lib = load()
        c = np.ascontiguousarray(counts, dtype=np.int32)
        p = CsgSimParams(G, softening, theta, dt, substeps, 0, precision)
        return cls(lib.cosmosim_create_ensemble(ptr(bodies), len(bodies), len(c),
                                                c.ctypes.data_as(_ip), ctypes.byref(p)))

    @classmethod
    def ensemble_ics(cls, kind, counts, seed0, G=1.0, softening=0.01, theta=0.5, dt=1e-3,
                     substeps=1, precision=PREC_FP64):
        """Ensemble whose systems are generated on the GPU
        (cosmosim_create_ensemble_ics): system g = csg_generate_ics(kind,
        counts[g], seed0 + g)."""
        lib = load()
        c = np.ascontiguousarray(counts, dtype=np.int32)
        p = CsgSimParams(G, softening, theta, dt, substeps, 0, precision)
        return cls(lib.cosmosim_create_ensemble_ics(kind, len(c), c.ctypes.data_as(_ip), seed0,
                                                    ctypes.byref(p)))

    @property
    def system_count(self):
        return self.lib.cosmosim_system_count(self.h)

    def set_walk_shape(self, warps_per_block=8, task_group=0, blocks_per_sm=0):
        w = CsgWalkShape(warps_per_block, task_group, blocks_per_sm, 0.0)
        self._rc(self.lib.cosmosim_set_walk_shape(self.h, ctypes.byref(w)), "set_walk_shape")

    def walk_shape(self):
        w = CsgWalkShape()
        self._rc(self.lib.cosmosim_get_walk_shape(self.h, ctypes.byref(w)), "walk_shape")
        return w.as_dict()

    def autotune_walk(self, reps=3):
        """Times every candidate walk shape, keeps the fastest; returns
        (best, [all candidates]) as dicts."""
        best = CsgWalkShape()
        cand = (CsgWalkShape * 64)()
        n = ctypes.c_int(0)
        self._rc(self.lib.cosmosim_autotune_walk(self.h, reps, ctypes.byref(best), cand, 64,
                                                 ctypes.byref(n)), "autotune_walk")
        return best.as_dict(), [cand[i].as_dict() for i in range(min(n.value, 64))]

    def _rc(self, rc, what):
        if rc:
            raise CudaError(f"{what}: {self.lib.csg_error_string(rc).decode()} (code {rc})")

    def step(self):
        self.lib.cosmosim_step(self.h)
        self._rc(self.lib.cosmosim_last_error(self.h), "cosmosim_step")

    def substeps_async(self, k):
        self._rc(self.lib.cosmosim_substeps_async(self.h, k), "substeps")

    def sync(self):
        self._rc(self.lib.cosmosim_sync(self.h), "sync")

    def enable_phase_timing(self, on=True):
        """Substeps run as direct launches with CUDA events between phases
        (cosmosim_enable_phase_timing); enabling resets the sums."""
        self._rc(self.lib.cosmosim_enable_phase_timing(self.h, int(on)), "phase_timing")

    def phase_times(self):
        """Summed phase times (ms) and the substeps timed (cosmosim_phase_times)."""
        t = CsgPhaseTimes()
        self._rc(self.lib.cosmosim_phase_times(self.h, ctypes.byref(t)), "phase_times")
        return t.as_dict()

    def set_stream(self, stream_ptr):
        self._rc(self.lib.cosmosim_set_stream(self.h, ctypes.c_void_p(stream_ptr)), "set_stream")

    def build_tree_async(self):
        self._rc(self.lib.cosmosim_build_tree_async(self.h), "build")

    def gravity_async(self):
        self._rc(self.lib.cosmosim_gravity_async(self.h), "gravity")

    def set_precision(self, p):
        self._rc(self.lib.cosmosim_set_precision(self.h, p), "precision")

    def enable_graphs(self, on=True):
        self._rc(self.lib.cosmosim_enable_graphs(self.h, int(on)), "graphs")

    def enable_stats(self, on=True):
        self._rc(self.lib.cosmosim_enable_stats(self.h, int(on)), "stats")

    def interactions(self):
        v = ctypes.c_int64(0)
        self._rc(self.lib.cosmosim_interactions(self.h, ctypes.byref(v)), "interactions")
        return v.value

    def walk_stats(self):
        """(interactions, warp steps, active lane-steps) since enable_stats."""
        v = [ctypes.c_int64(0) for _ in range(3)]
        self._rc(self.lib.cosmosim_walk_stats(self.h, *[ctypes.byref(x) for x in v]), "walk_stats")
        return tuple(x.value for x in v)

    def node_count(self):
        v = ctypes.c_int(0)
        self._rc(self.lib.cosmosim_node_count(self.h, ctypes.byref(v)), "node_count")
        return v.value

    @property
    def count(self):
        return self.lib.cosmosim_get_count(self.h)

    @property
    def active_count(self):
        return self.lib.cosmosim_get_active_count(self.h)

    @property
    def sim_time(self):
        return self.lib.cosmosim_get_sim_time(self.h)

    def bodies(self):
        """Copy of the current bodies (cosmosim_copy_bodies)."""
        out = np.zeros(self.count, dtype=BODY_DTYPE)
        self._rc(self.lib.cosmosim_copy_bodies(self.h, ptr(out), len(out)), "copy_bodies")
        return out

    def set_bodies(self, bodies):
        """Uploads bodies into the handle (cosmosim_set_bodies; asynchronous:
        keep `bodies` alive and unchanged until the next sync)."""
        self._rc(self.lib.cosmosim_set_bodies(self.h, ptr(bodies), len(bodies)), "set_bodies")

    def snapshot(self, fmt=0, max_bodies=None, device_out=None):
        """Alive bodies as float records (cosmosim_snapshot_f32): fmt 0 = 16
        floats (FCosmosimBodyGPU), 1 = 10 floats (renderer). Into a new numpy
        array, or into device_out (a device pointer) when given."""
        stride = 16 if fmt == 0 else 10
        cap = self.count if max_bodies is None else max_bodies
        if device_out is not None:
            k = self.lib.cosmosim_snapshot_f32(self.h, fmt, ctypes.c_void_p(device_out), 1, cap)
            self._rc(0 if k >= 0 else self.lib.cosmosim_last_error(self.h), "snapshot")
            return k
        out = np.zeros((max(cap, 1), stride), dtype=np.float32)
        k = self.lib.cosmosim_snapshot_f32(self.h, fmt, ptr(out), 0, cap)
        self._rc(0 if k >= 0 else self.lib.cosmosim_last_error(self.h), "snapshot")
        return out[:k].copy()

    def compact(self):
        k = self.lib.cosmosim_compact(self.h)
        self._rc(0 if k >= 0 else self.lib.cosmosim_last_error(self.h), "compact")
        return k

    def get_bodies_view(self):
        """The borrowed array cosmosim_get_bodies returns, copied into numpy."""
        p = self.lib.cosmosim_get_bodies(self.h)
        n = self.count
        buf = (ctypes.c_char * (n * BODY_DTYPE.itemsize)).from_address(p)
        return np.frombuffer(buf, dtype=BODY_DTYPE, count=n).copy()

    def direct_forces(self, idx):
        """FP64 direct-sum accelerations of bodies idx (m x 3)."""
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        out = np.zeros((len(idx), 3))
        self._rc(self.lib.cosmosim_direct_forces(self.h, ptr(idx), len(idx), ptr(out)), "direct")
        return out

    def energy(self):
        ke, pe = ctypes.c_double(0), ctypes.c_double(0)
        self._rc(self.lib.cosmosim_energy(self.h, ctypes.byref(ke), ctypes.byref(pe)), "energy")
        return ke.value, pe.value

    def launch_count(self):
        return self.lib.cosmosim_launch_count(self.h)

    def close(self):
        if self.h:
            self.lib.cosmosim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- adjoint of the leapfrog (csg_adjoint_*) ----

class Adjoint:
    """Reverse-mode gradient of a T-substep FP64 leapfrog run w.r.t. the
    initial positions and velocities, loss = mean |x_T - target|^2 over alive
    bodies. mode ADJ_TREE: Barnes-Hut with frozen interaction lists;
    ADJ_DIRECT: FP64 direct sum."""

    def __init__(self, n, G=1.0, softening=0.01, theta=0.5, dt=2e-3, substeps=200,
                 checkpoint_every=20, mode=ADJ_TREE):
        self.lib = load()
        p = CsgSimParams(G, softening, theta, dt, substeps, 0, PREC_FP64)
        h = self.lib.csg_adjoint_create(n, ctypes.byref(p), checkpoint_every, mode)
        if not h:
            rc = self.lib.csg_last_error()
            raise CudaError(f"csg_adjoint_create: {self.lib.csg_error_string(rc).decode()}")
        self.h = ctypes.c_void_p(h)
        self.n = n

    def _rc(self, rc, what):
        if rc:
            raise CudaError(f"{what}: {self.lib.csg_error_string(rc).decode()} (code {rc})")

    @staticmethod
    def _target(target):
        t = np.ascontiguousarray(target, dtype=np.float64).reshape(-1, 3)
        return t

    def forward(self, bodies, target, record=False, final=False):
        t = self._target(target)
        loss = ctypes.c_double(0)
        out = np.zeros(len(bodies), dtype=BODY_DTYPE) if final else None
        self._rc(self.lib.csg_adjoint_forward(self.h, ptr(bodies), ptr(t), int(record),
                                              ctypes.byref(loss),
                                              ptr(out) if final else None), "adjoint forward")
        return (loss.value, out) if final else loss.value

    def forward_frozen(self, bodies, target):
        t = self._target(target)
        loss = ctypes.c_double(0)
        self._rc(self.lib.csg_adjoint_forward_frozen(self.h, ptr(bodies), ptr(t),
                                                     ctypes.byref(loss)), "adjoint frozen")
        return loss.value

    def backward(self):
        gx = np.zeros((self.n, 3))
        gv = np.zeros((self.n, 3))
        self._rc(self.lib.csg_adjoint_backward(self.h, ptr(gx), ptr(gv)), "adjoint backward")
        return gx, gv

    def stats(self):
        b, i, k = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
        self._rc(self.lib.csg_adjoint_stats(self.h, ctypes.byref(b), ctypes.byref(i),
                                            ctypes.byref(k)), "stats")
        return {"device_bytes": b.value, "interactions": i.value, "launches": k.value}

    def close(self):
        if self.h:
            self.lib.csg_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
