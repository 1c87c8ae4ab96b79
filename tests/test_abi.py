"""The C-ABI library: layout, exports, and failure without a device (CPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, has_gpu, same_bytes
from cosmosim_gb300.abi import BODY_DTYPE, NODE_DTYPE, CosmosimConfig


def declared_symbols():
    """Every function declared CSG_EXPORT in include/*.h."""
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"CSG_EXPORT\s+[\w\s\*]+?\b(\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_struct_layouts():
    assert BODY_DTYPE.itemsize == 168
    assert NODE_DTYPE.itemsize == 104
    assert ctypes.sizeof(CosmosimConfig) == 72
    assert BODY_DTYPE.fields["type"][1] == 80
    assert NODE_DTYPE.fields["body_index"][1] == 64
    assert NODE_DTYPE.fields["children"][1] == 68


def test_library_exports_every_declared_symbol(lib):
    so = ctypes.CDLL(lib.LIB_PATH)
    decl = declared_symbols()
    # the reference API and the additive one
    for must in ("octree_build", "octree_compute_forces", "octree_find_neighbors",
                 "integrator_step", "integrator_init_accelerations", "sph_compute_density",
                 "sph_compute_forces", "sph_apply_cooling", "cosmosim_default_config",
                 "cosmosim_create", "cosmosim_step", "cosmosim_get_bodies", "cosmosim_get_count",
                 "cosmosim_get_active_count", "cosmosim_get_sim_time", "cosmosim_destroy"):
        assert must in decl
    missing = [s for s in sorted(decl) if not hasattr(so, s)]
    assert not missing, missing
    # and the Python binding covers them
    assert set(lib.exported_symbols()) <= decl


def test_default_config_matches_reference(lib):
    c = lib.load().cosmosim_default_config()  # src/cosmosim_api.c:30-45
    assert (c.n_bodies, c.merger, c.quasar, c.substeps) == (20000, 0, 0, 2)
    assert (c.dt, c.theta, c.smbh_mass_frac) == (0.005, 0.5, 0.05)
    assert (c.accretion_radius, c.jet_speed, c.feedback_strength) == (6.0, 15.0, 0.3)


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_device_fails_loudly(lib):
    """Without a GPU every call reports CSG_ERR_NO_DEVICE; nothing computes on CPU."""
    L = lib.load()
    b = np.zeros(4, dtype=BODY_DTYPE)
    b["x"] = [0, 1, 2, 3]
    b["mass"] = 1.0
    before = b.copy()
    pool = np.zeros(32, dtype=NODE_DTYPE)
    ps = ctypes.c_int(-1)
    L.octree_build(pool.ctypes.data, ctypes.byref(ps), b.ctypes.data, 4)
    assert L.csg_last_error() == 7
    L.integrator_step(b.ctypes.data, 4, 1e-3, 1.0, 0.01, 0.5, pool.ctypes.data, 0)
    assert L.csg_last_error() == 7
    assert same_bytes(b, before)
    assert not L.cosmosim_create(L.cosmosim_default_config())
    with pytest.raises(lib.CudaError):
        lib.octree_build(b)


def test_ensemble_arguments_are_checked_before_any_device_work(lib):
    """cosmosim_create_ensemble: SPH is refused (CSG_ERR_UNSUPPORTED), counts
    that do not sum to n or are negative are CSG_ERR_BAD_ARG."""
    L = lib.load()
    b = np.zeros(10, dtype=BODY_DTYPE)
    b["mass"] = 1.0
    b["x"] = np.arange(10)

    def create(counts, sph=0):
        c = np.asarray(counts, dtype=np.int32)
        p = lib.CsgSimParams(1.0, 0.01, 0.5, 1e-3, 1, sph, 0)
        return L.cosmosim_create_ensemble(b.ctypes.data, len(b), len(c),
                                          c.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                          ctypes.byref(p))

    assert not create([5, 5], sph=1)
    assert L.csg_last_error() == 8
    assert not create([5, 4])
    assert L.csg_last_error() == 4
    assert not create([11, -1])
    assert L.csg_last_error() == 4
    assert not create([])
    assert L.csg_last_error() == 4


def test_adjoint_arguments_are_checked_before_any_device_work(lib):
    L = lib.load()
    p = lib.CsgSimParams(1.0, 0.01, 0.5, 2e-3, 10, 0, 0)
    assert not L.csg_adjoint_create(0, ctypes.byref(p), 5, 0)
    assert L.csg_last_error() == 4
    assert not L.csg_adjoint_create(100, ctypes.byref(p), 0, 0)
    assert L.csg_last_error() == 4
    assert not L.csg_adjoint_create(100, ctypes.byref(p), 5, 7)
    assert L.csg_last_error() == 4
    p.sph = 1
    assert not L.csg_adjoint_create(100, ctypes.byref(p), 5, 0)
    assert L.csg_last_error() == 4


def test_missing_library_raises(tmp_path):
    from cosmosim_gb300 import lib as libmod

    with pytest.raises(FileNotFoundError):
        libmod.load(str(tmp_path / "nope.so"))


def test_ics_are_seeded_and_shaped(lib):
    a = lib.generate_ics(0, 2000, 42)
    b = lib.generate_ics(0, 2000, 42)
    c = lib.generate_ics(0, 2000, 43)
    assert same_bytes(a, b)
    assert not same_bytes(a, c)
    # cfg0: disk mass 1 shared equally, SMBH 0.01 at the centre
    assert a["mass"][0] == 0.01 and a["type"][0] == 2
    np.testing.assert_allclose(a["mass"][1:].sum(), 1.0, rtol=1e-12)
    assert np.allclose(a["mass"][1:], a["mass"][1])
    m = lib.generate_ics(1, 4000, 5)  # merger with 10% gas
    gas = (m["type"] == 1)
    assert 0.06 < gas.mean() < 0.14
    assert np.all(m["smoothing_h"][gas] > 0) and np.all(m["internal_energy"][gas] > 0)
    p = lib.generate_ics(2, 10000, 9)  # bulge + disk, equal masses summing to 1
    np.testing.assert_allclose(p["mass"].sum(), 1.0, rtol=1e-12)
    assert np.allclose(p["mass"], 1e-4)
    r = np.sqrt(p["x"][:3000] ** 2 + p["y"][:3000] ** 2 + p["z"][:3000] ** 2)
    assert 0.3 < np.median(r) < 1.2  # Plummer half-mass radius 1.305 a = 0.65
    s = lib.generate_ics(4, 1000, 1)
    assert not np.any(s["type"] == 1)
