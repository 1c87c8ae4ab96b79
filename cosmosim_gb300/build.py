"""Builds libcosmosim_gb300.so in-tree for sm_103a.

    python -m cosmosim_gb300.build         # incremental
    python -m cosmosim_gb300.build --clean

CUDA sources are compiled by nvcc for sm_103a only; the C11 host layer by the
system C compiler; everything is linked into one shared library
(cosmosim_gb300/libcosmosim_gb300.so) with the CUDA runtime linked statically.
Objects go to cosmosim_gb300/_build/.
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcosmosim_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr"]
# Kernels that must round exactly like the reference's C (no fused multiply-add).
NO_FMA = {"dev_state.cu", "dev_sph.cu", "dev_quasar.cu", "dev_ics.cu"}
# -ffp-contract=off: the host layer (initial conditions) rounds the same on
# x86_64 and aarch64, and as the device generators do.
CC_FLAGS = ["-std=c11", "-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall",
            "-Wextra", "-Wno-unused-parameter"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers():
    hs = []
    for d in (os.path.join(CSRC, "device"), os.path.join(CSRC, "host"), os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                hs.append(os.path.join(d, f))
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def _jobs():
    nvcc = _nvcc()
    cc = os.environ.get("CC", "gcc")
    jobs = []
    inc = ["-I", os.path.join(ROOT, "include")]
    for f in sorted(os.listdir(os.path.join(CSRC, "device"))):
        if f.endswith(".cu"):
            src = os.path.join(CSRC, "device", f)
            obj = os.path.join(BUILD, f + ".o")
            flags = NVCC_FLAGS + (["-fmad=false"] if f in NO_FMA else [])
            jobs.append((src, obj, [nvcc] + flags + inc + ["-c", src, "-o", obj]))
    for f in sorted(os.listdir(os.path.join(CSRC, "host"))):
        if f.endswith(".c"):
            src = os.path.join(CSRC, "host", f)
            obj = os.path.join(BUILD, f + ".o")
            jobs.append((src, obj, [cc] + CC_FLAGS + inc + ["-c", src, "-o", obj]))
    return nvcc, jobs


def build(verbose=False, force=False):
    """Compiles what changed and links the library. Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc, jobs = _jobs()
    headers = _headers()
    todo = [j for j in jobs if force or _stale(j[1], j[0], headers)]

    def run(job):
        src, obj, cmd = job
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {os.path.basename(src)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(run, todo))
    objs = [j[1] for j in jobs]
    if todo or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lm"]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--clean", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    if a.clean:
        shutil.rmtree(BUILD, ignore_errors=True)
        if os.path.exists(LIB):
            os.remove(LIB)
    print(build(verbose=a.verbose, force=a.clean))


if __name__ == "__main__":
    sys.exit(main())
