"""The repository's host code under AddressSanitizer and UndefinedBehaviorSanitizer.

Builds tests/sanitize/host_check.c with the oracle (oracle/orc.c,
oracle/orc_ics.c) and the library's host files that run without a device
(csrc/host/ics.c: seeded initial conditions; csrc/host/capi_context.c: the
pool scan that guards caller trees, the thread context) and runs it: every
heap access, integer overflow, misaligned or out-of-range access and leak
aborts the run. CPU only (the device layer is stubbed).
"""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_host_code_is_clean_under_asan_and_ubsan(tmp_path):
    cc = shutil.which(os.environ.get("CC", "gcc"))
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "host_check")
    src = [os.path.join(ROOT, p) for p in (
        "tests/sanitize/host_check.c", "oracle/orc.c", "oracle/orc_ics.c",
        "cosmosim_gb300/csrc/host/ics.c", "cosmosim_gb300/csrc/host/capi_context.c")]
    flags = ["-std=gnu11", "-O1", "-g", "-fsanitize=address,undefined",
             "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-fopenmp",
             "-ffp-contract=off", "-I", os.path.join(ROOT, "include")]
    r = subprocess.run([cc] + flags + src + ["-lm", "-o", exe], capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("the compiler has no sanitizer runtime: " + r.stderr[-300:])
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1")
    run = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=env)
    assert run.returncode == 0, run.stderr[-4000:]
    assert "clean under ASan/UBSan" in run.stdout
