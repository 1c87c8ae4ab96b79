"""Programmatic dependent launches (CPU, source check).

A kernel queued by csgd_launch may start while the kernel before it in the
stream still runs; it is correct only if its first statement waits for that
kernel (pdl_enter: griddepcontrol.wait, then launch_dependents). Nothing at
run time would catch a missing wait (the kernel would read data still being
written), so every such kernel is checked here.
"""
import glob
import os
import re

from conftest import ROOT

DEV = os.path.join(ROOT, "cosmosim_gb300", "csrc", "device")


def _sources():
    return {os.path.basename(f): open(f).read() for f in sorted(glob.glob(os.path.join(DEV, "*.cu")))}


def _launched(src):
    names = set()
    for text in src.values():
        for m in re.finditer(r"csgd_launch\(d,\s*(\w+)", text):
            names.add(m.group(1))
    return names


def _missing_waits(src):
    """Kernels queued by csgd_launch whose body does not begin with pdl_enter()."""
    every = "\n".join(src.values())
    names = _launched(src)
    # the walk macro passes its kernel as K
    macro = re.search(r"#define CSG_LAUNCH_WALK\(K,.*?\n(.*?)while \(0\)", every, re.S)
    if macro and "csgd_launch(d, K" in macro.group(1):
        names.discard("K")
        for m in re.finditer(r"CSG_LAUNCH_WALK\((\w+),", every):
            names.add(m.group(1))
    missing = []
    for k in sorted(names):
        m = re.search(r"__global__ void[^\n]*?\b%s\(" % k, every)
        assert m, f"no kernel definition for {k}"
        body = every.index("\n{\n", m.end())
        if not every[body + 3:body + 80].lstrip().startswith("pdl_enter();"):
            missing.append(k)
    return names, missing


def test_every_programmatic_launch_waits_first():
    names, missing = _missing_waits(_sources())
    assert "k_radix_onesweep" in names and "k_moments" in names
    assert not missing, f"kernels queued by csgd_launch without pdl_enter() first: {missing}"


def test_the_check_sees_a_missing_wait():
    src = _sources()
    text = src["dev_tree.cu"]
    at = text.index("__global__ void k_bbox(")
    cut = text.index("    pdl_enter();\n", at)
    src["dev_tree.cu"] = text[:cut] + text[cut + len("    pdl_enter();\n"):]
    assert _missing_waits(src)[1] == ["k_bbox"]


def test_launch_helper_sets_the_attribute():
    hdr = open(os.path.join(DEV, "dev_internal.cuh")).read()
    fn = hdr[hdr.index("inline void csgd_launch("):]
    fn = fn[:fn.index("\n}\n")]
    assert "cudaLaunchAttributeProgrammaticStreamSerialization" in fn
    assert "programmaticStreamSerializationAllowed = 1" in fn
    assert "d->launches++" in fn
    wait = hdr[hdr.index("void pdl_enter()"):]
    wait = wait[:wait.index("}")]
    assert wait.index("pdl_wait()") < wait.index("pdl_release()")
