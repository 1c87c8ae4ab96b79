"""cosmosim's own test program links against this library unchanged.

The drop-in claim: cosmosim's callers (src/main.c, tests/test_physics.c, the
Unreal plugin) keep their sources and only link libcosmosim_gb300.so in
place of the four physics units it replaces (src/octree.c, integrator.c,
sph.c, cosmosim_api.c). `make -C oracle droplink REF=<checkout>` compiles
tests/test_physics.c with the two units the library does not replace
(src/quasar.c, src/initial_conditions.c) as cosmosim's CMakeLists builds it
(CMakeLists.txt:40-52, 79-82) and links it against this library with
--no-undefined.

Needs a cosmosim checkout named by CSG_REFERENCE_DIR (skipped otherwise).
The link check is host work; running the program needs a GPU and the
reference sources on the same machine (the gpu-marked test).
"""
import os
import subprocess

import pytest

from oracle import orc as orc_mod

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "oracle", "_ref", "test_physics_gb300")
LIB = os.path.join(ROOT, "cosmosim_gb300", "libcosmosim_gb300.so")

# The reference's exported hot-path API (src/octree.h:16-36,
# src/integrator.h:7-17, src/sph.h:12-19, src/cosmosim_api.h:35-42) that the
# test program calls.
REPLACED = {
    "octree_build", "octree_compute_forces", "octree_find_neighbors",
    "integrator_step", "integrator_init_accelerations",
    "sph_compute_density", "sph_compute_forces", "sph_apply_cooling",
    "cosmosim_default_config", "cosmosim_create", "cosmosim_step", "cosmosim_get_bodies",
    "cosmosim_get_count", "cosmosim_get_active_count", "cosmosim_get_sim_time",
    "cosmosim_destroy",
}


def _ref():
    ref = orc_mod.reference_dir()
    if not ref or not os.path.exists(os.path.join(ref, "tests", "test_physics.c")):
        pytest.skip("CSG_REFERENCE_DIR does not name a cosmosim checkout")
    return ref


def _nm(args, path):
    out = subprocess.run(["nm"] + args + [path], check=True, capture_output=True, text=True).stdout
    syms = {}
    for line in out.splitlines():
        parts = line.split()
        if len(parts) >= 2:
            syms[parts[-1].split("@")[0]] = parts[-2]
    return syms


def _link(lib):
    ref = _ref()
    if not os.path.exists(lib.LIB_PATH):
        from cosmosim_gb300 import build

        build.build()
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "droplink", f"REF={ref}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return ref


def test_reference_test_program_links_unchanged(lib):
    _link(lib)
    assert os.path.exists(BIN)
    undef = {s for s, t in _nm(["-u"], BIN).items() if t in ("U",)}
    # every replaced entry point the program calls is imported, none defined by it
    calls = undef & REPLACED
    assert calls == REPLACED
    exported = {s for s, t in _nm(["-D", "--defined-only"], LIB).items() if t in ("T", "W", "B", "D")}
    missing = calls - exported
    assert not missing, f"not exported by libcosmosim_gb300.so: {sorted(missing)}"
    # the reference's CPU-only units stay in the program; the library defines
    # none of their symbols, so nothing is duplicated
    prog = {s for s, t in _nm(["-D", "--defined-only"], BIN).items() if t == "T"}
    assert {"quasar_default_config", "generate_spiral_galaxy", "generate_merger"} <= prog
    assert not (prog & exported), f"defined twice: {sorted(prog & exported)}"
    # the library is what the loader resolves those calls to
    ldd = subprocess.run(["ldd", BIN], check=True, capture_output=True, text=True).stdout
    assert "libcosmosim_gb300.so => " + LIB in ldd


@pytest.mark.gpu
def test_reference_test_program_passes_on_the_gpu(lib):
    """All 34 RUN_TESTs of tests/test_physics.c (:1141-1207) pass with the
    GPU library (only where the reference checkout is on the GPU machine)."""
    _link(lib)
    r = subprocess.run([BIN], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "34/34 tests passed" in r.stdout, r.stdout[-3000:]
