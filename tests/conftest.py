"""Shared test set-up.

Markers: `gpu` — needs a CUDA device (parity tests through the C-ABI).
Everything else runs on CPU: the oracle against the golden fixtures, the
library's exports and host logic, multi-process (gloo) logic.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path)")


def has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


@pytest.fixture(scope="session")
def orc():
    from oracle import orc as orc_mod

    orc_mod.build()
    return orc_mod.Oracle()


@pytest.fixture(scope="session")
def lib():
    """The CUDA library (built in-tree if missing). No fallback."""
    from cosmosim_gb300 import build, lib as libmod

    if not os.path.exists(libmod.LIB_PATH):
        build.build()
    return libmod


def same_bytes(a, b):
    """Field-wise bit equality of two structured arrays (padding ignored)."""
    return all(np.ascontiguousarray(a[f]).tobytes() == np.ascontiguousarray(b[f]).tobytes()
               for f in a.dtype.names)


def fields(b, names=("ax", "ay", "az")):
    return np.stack([b[f] for f in names], axis=1)


def rel_err(a, b):
    """Per-row |a-b| / |b| (rows are 3-vectors)."""
    num = np.linalg.norm(a - b, axis=1)
    den = np.linalg.norm(b, axis=1)
    return num / np.where(den > 0, den, 1.0)


def assert_same_topology(pool, ref_pool):
    """Index work: structure and geometry of two pools are identical."""
    assert len(pool) == len(ref_pool)
    np.testing.assert_array_equal(pool["body_index"], ref_pool["body_index"])
    np.testing.assert_array_equal(pool["children"], ref_pool["children"])
    for f in ("center_x", "center_y", "center_z", "half_size"):
        np.testing.assert_array_equal(pool[f], ref_pool[f], err_msg=f)


def assert_moments_close(pool, ref_pool, rel=1e-13):
    """Cell mass and centre of mass agree to rounding (the reference sums them
    in insertion order, this library bottom-up)."""
    np.testing.assert_allclose(pool["total_mass"], ref_pool["total_mass"], rtol=rel, atol=0)
    scale = ref_pool["half_size"][0] + np.abs(ref_pool[["center_x"]][0][0])
    for f in ("cx", "cy", "cz"):
        np.testing.assert_allclose(pool[f], ref_pool[f], rtol=0, atol=rel * 8 * scale + 1e-300,
                                   err_msg=f)
