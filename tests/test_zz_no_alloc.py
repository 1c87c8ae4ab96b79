"""The allocation-free direct sum (csg_direct_forces_noalloc) against the
allocating one (cosmosim_direct_forces) and against the CPU oracle's direct
sum (orc_direct_forces, the reference test helper tests/test_physics.c:54-71).

Who needs it: callers that cannot allocate device memory — an engine or
renderer that owns a fixed GPU budget behind its own allocator, or a
real-time thread that must not block on cudaMalloc/cudaFree. They pass
device buffers they already hold; the library's scratch is a fixed array.

This file is collected last on purpose (tests run in file-name order) and
must pass both alone in a fresh process and after the other tests.
Tolerance: per-body |da|/|a| <= 1e-12 (the entry points and the oracle split
the j sum differently, so only the last bits may differ).
"""
import ctypes

import numpy as np
import pytest

from cosmosim_gb300.abi import BODY_DTYPE

pytestmark = pytest.mark.gpu

MAX_SAMPLE = 4096
TOL = 1e-12


def _device_soa(torch, bodies):
    cols = [torch.tensor(np.ascontiguousarray(bodies[f]), dtype=torch.float64, device="cuda")
            for f in ("x", "y", "z", "mass")]
    return cols


def _noalloc(lib, torch, cols, idx, G, eps, sys=None):
    L = lib.load()
    d_idx = torch.tensor(np.asarray(idx).astype(np.int32), device="cuda")
    d_sys = None if sys is None else torch.tensor(np.asarray(sys, dtype=np.int32), device="cuda")
    out = torch.zeros(3 * len(idx), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    rc = L.csg_direct_forces_noalloc(
        *[ctypes.c_void_p(c.data_ptr()) for c in cols],
        None if d_sys is None else ctypes.c_void_p(d_sys.data_ptr()), len(cols[0]),
        ctypes.c_void_p(d_idx.data_ptr()), len(idx), G, eps,
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, rc
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(-1, 3)


def _rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def test_noalloc_direct_sum_matches_allocating_entry_point_and_oracle(lib, orc):
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
        assert _rel(got, want).max() <= TOL
        assert _rel(got, orc.direct_forces(bodies, 1.0, eps, idx)).max() <= TOL


def test_noalloc_two_systems_attract_only_within_their_system(lib, orc):
    """Two galaxies in one buffer with system ids: each sampled body feels only
    its own galaxy, as the ensemble handle's direct sum and the oracle run on
    each galaxy alone say; without ids both galaxies attract."""
    torch = pytest.importorskip("torch")
    a = lib.generate_ics(5, 3000, 11)
    b = lib.generate_ics(6, 2000, 12)
    b["x"] += 0.5  # overlapping, so the cross-system pull is large
    allb = np.concatenate([a.astype(BODY_DTYPE), b.astype(BODY_DTYPE)]).astype(BODY_DTYPE)
    sys = np.r_[np.zeros(len(a), np.int32), np.ones(len(b), np.int32)]
    rng = np.random.default_rng(3)
    idx = np.sort(rng.choice(len(allb), size=600, replace=False))
    cols = _device_soa(torch, allb)
    got = _noalloc(lib, torch, cols, idx, 1.0, 0.01, sys)
    ens = lib.Sim.ensemble(allb, [len(a), len(b)], softening=0.01)
    want_ens = ens.direct_forces(idx)
    ens.close()
    assert _rel(got, want_ens).max() <= TOL
    ia, ib = idx[idx < len(a)], idx[idx >= len(a)] - len(a)
    want = np.concatenate([orc.direct_forces(a, 1.0, 0.01, ia), orc.direct_forces(b, 1.0, 0.01, ib)])
    assert _rel(got, want).max() <= TOL
    # one system (sys NULL): every body attracts, as the oracle over the whole buffer
    whole = _noalloc(lib, torch, cols, idx, 1.0, 0.01)
    assert _rel(whole, orc.direct_forces(allb, 1.0, 0.01, idx)).max() <= TOL
    assert _rel(whole, want).max() > 1e-3


def test_noalloc_out_of_range_index_gives_nan_row(lib, orc):
    """A sample index outside [0, n) reads no body and yields a NaN row; the
    other rows are unaffected."""
    torch = pytest.importorskip("torch")
    bodies = lib.generate_ics(0, 1000, 9)
    n = len(bodies)
    idx = np.array([0, n, 5, -1, n - 1, 2**31 - 1, -(2**31)], dtype=np.int64)
    got = _noalloc(lib, torch, _device_soa(torch, bodies), idx, 1.0, 0.01)
    bad = (idx < 0) | (idx >= n)
    assert np.isnan(got[bad]).all()
    ok = idx[~bad].astype(np.int32)
    assert _rel(got[~bad], orc.direct_forces(bodies, 1.0, 0.01, ok)).max() <= TOL


def test_noalloc_rejects_samples_beyond_its_scratch(lib):
    L = lib.load()
    rc = L.csg_direct_forces_noalloc(None, None, None, None, None, 10, None, MAX_SAMPLE + 1, 1.0,
                                     0.01, None, None)
    assert rc == 4  # CSG_ERR_BAD_ARG, nothing launched
