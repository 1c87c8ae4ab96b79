"""The allocation-free direct sum (csg_direct_forces_noalloc) matches the
allocating one (cosmosim_direct_forces).

Who needs it: callers that cannot allocate device memory — an engine or
renderer that owns a fixed GPU budget behind its own allocator, or a
real-time thread that must not block on cudaMalloc/cudaFree. They pass
device buffers they already hold; the library's scratch is a fixed array.

This file is collected last on purpose (tests run in file-name order) and
must pass both alone in a fresh process and after the other tests.
Tolerance: per-body |da|/|a| <= 1e-12 (the two entry points split the j sum
into different chunks, so only the last bits may differ).
"""
import ctypes

import numpy as np
import pytest

from cosmosim_gb300.abi import BODY_DTYPE

pytestmark = pytest.mark.gpu

MAX_SAMPLE = 4096


def _device_soa(torch, bodies):
    cols = [torch.tensor(np.ascontiguousarray(bodies[f]), dtype=torch.float64, device="cuda")
            for f in ("x", "y", "z", "mass")]
    return cols


def _noalloc(lib, torch, cols, idx, G, eps):
    L = lib.load()
    d_idx = torch.tensor(idx.astype(np.int32), device="cuda")
    out = torch.zeros(3 * len(idx), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    rc = L.csg_direct_forces_noalloc(
        *[ctypes.c_void_p(c.data_ptr()) for c in cols], len(cols[0]),
        ctypes.c_void_p(d_idx.data_ptr()), len(idx), G, eps,
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, rc
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(-1, 3)


def _rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def test_noalloc_direct_sum_matches_allocating_entry_point(lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(17)
    # two calls in a row: different bodies, softening and sample sizes (the
    # second at the largest sample the fixed scratch holds)
    cases = [(lib.generate_ics(0, 20000, 5), 0.01, 1000),
             (lib.generate_ics(1, 30000, 6), 0.005, MAX_SAMPLE)]
    for bodies, eps, m in cases:
        bodies["mass"][rng.random(len(bodies)) < 0.01] = 0.0  # dead bodies are skipped
        idx = rng.choice(len(bodies), size=m, replace=False)
        sim = lib.Sim.from_bodies(bodies, softening=eps)
        want = sim.direct_forces(idx)
        sim.close()
        got = _noalloc(lib, torch, _device_soa(torch, bodies), idx, 1.0, eps)
        assert _rel(got, want).max() <= 1e-12


def test_noalloc_rejects_samples_beyond_its_scratch(lib):
    L = lib.load()
    rc = L.csg_direct_forces_noalloc(None, None, None, None, 10, None, MAX_SAMPLE + 1, 1.0, 0.01,
                                     None, None)
    assert rc == 4  # CSG_ERR_BAD_ARG, nothing launched
