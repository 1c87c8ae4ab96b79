"""Initial conditions generated on the GPU (csg_generate_ics_device,
cosmosim_create_ensemble_ics) against the host generator csg_generate_ics.

Every body draws the same random numbers (the xorshift64 stream is jumped
ahead on the device), so types, masses and the SMBH are exact; positions and
velocities agree to 1e-13 of each field's largest magnitude (CUDA's log, exp,
sin, cos are within 2 ulp of the C library's).
"""
import ctypes

import numpy as np
import pytest

from conftest import fields
from cosmosim_gb300.abi import BODY_DTYPE

pytestmark = pytest.mark.gpu

F = ["x", "y", "z", "vx", "vy", "vz", "mass", "internal_energy", "smoothing_h"]


def device_ics(lib, kind, n, seed):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(max(n, 1) * BODY_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    rc = lib.load().csg_generate_ics_device(kind, n, seed, ctypes.c_void_p(buf.data_ptr()),
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == n
    return buf.cpu().numpy()[:n * BODY_DTYPE.itemsize].view(BODY_DTYPE).copy()


def close(a, b, rtol=1e-13):
    fa, fb = fields(a, F), fields(b, F)
    scale = np.maximum(np.abs(fb).max(axis=0), 1e-300)
    assert (np.abs(fa - fb) / scale).max() <= rtol


@pytest.mark.parametrize("kind", [0, 3, 5, 6])
@pytest.mark.parametrize("n", [1, 17, 5000])
def test_device_ics_equal_host_ics(lib, kind, n):
    host = lib.generate_ics(kind, n, 1234 + kind)
    dev = device_ics(lib, kind, n, 1234 + kind)
    np.testing.assert_array_equal(dev["type"], host["type"])
    np.testing.assert_array_equal(dev["mass"], host["mass"])
    close(dev, host)


def test_ensemble_generated_on_the_device(lib):
    counts = [3000, 17, 1, 4500]
    seed0 = 777
    ens = lib.Sim.ensemble_ics(3, counts, seed0, softening=0.01, precision=1)
    host = np.concatenate([lib.generate_ics(3, c, seed0 + g) for g, c in enumerate(counts)])
    host = host.astype(BODY_DTYPE)
    ref = lib.Sim.ensemble(host, counts, softening=0.01, precision=1)
    close(ens.bodies(), ref.bodies())
    for s in (ens, ref):
        s.substeps_async(3)
        s.sync()
    close(ens.bodies(), ref.bodies(), 1e-10)
    ens.close()
    ref.close()
