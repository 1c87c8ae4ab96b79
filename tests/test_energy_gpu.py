"""Energy drift over 1000 substeps, the bound the spec asks to state.

Kick-drift-kick at dt = 1e-3, theta = 0.5, FP64 energy (kinetic + softened
potential, all pairs, cosmosim_energy, itself checked against the oracle in
test_diagnostics_gpu.py). Stated bound: |E(1000) - E(0)| / |E(0)| <= 5e-3
(measured on a GB300: 2.5e-3 for the 100k bulge + disk, 2.8e-3 for the 20k
merger); the drift is the integrator's and the softening's, not the
precision's: FP32-mixed and FP64 plain drift alike to within 1e-5 (measured
8e-7 and 4e-7).
"""
import pytest

pytestmark = pytest.mark.gpu

BOUND = 5e-3
PRECISION_GAP = 1e-5


@pytest.mark.parametrize("kind,n,eps", [(2, 100_000, 0.005), (1, 20_000, 0.01)])
def test_energy_drift_over_1000_substeps(lib, kind, n, eps):
    b = lib.generate_ics(kind, n, 0x5EED0000)
    drift = {}
    for prec in (lib.PREC_FP64, lib.PREC_FP32_MIXED):
        s = lib.Sim.from_bodies(b, softening=eps, theta=0.5, dt=1e-3, precision=prec)
        ke, pe = s.energy()
        e0 = ke + pe
        s.substeps_async(1000)
        s.sync()
        ke, pe = s.energy()
        s.close()
        drift[prec] = abs(ke + pe - e0) / abs(e0)
    assert max(drift.values()) <= BOUND, drift
    assert abs(drift[lib.PREC_FP64] - drift[lib.PREC_FP32_MIXED]) <= PRECISION_GAP, drift
