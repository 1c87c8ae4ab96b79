"""The FP64 GPU diagnostics against the CPU oracle.

Every "error against a direct sum" and every energy drift this library
reports rests on two device kernels: the sampled direct sum
(cosmosim_direct_forces) and the O(n^2) energy (cosmosim_energy). Both
restate the reference test helpers (tests/test_physics.c:54-71 and :34-52);
here they are compared with the oracle's restatement of those helpers
(orc_direct_forces, orc_total_energy), which runs the pair sum in the
reference's order on the CPU.

Tolerances: direct sum per body |da|/|a| <= 1e-12; energy (KE + PE) and the
potential alone <= 1e-12 relative. The oracle's sequential PE sum at 20k
bodies is itself within ~4e-13 of an extended-precision sum, and the GPU
splits both sums differently, so only the last bits may differ.
"""
import numpy as np
import pytest

from conftest import golden
from cosmosim_gb300.abi import BODY_DTYPE

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def _pe_only(bodies):
    b = bodies.copy()
    b["vx"] = 0.0
    b["vy"] = 0.0
    b["vz"] = 0.0
    return b


@pytest.mark.parametrize("case", ["merger100k", "disk_3000"])
def test_direct_forces_match_oracle(lib, orc, case):
    rng = np.random.default_rng(4096)
    if case == "merger100k":
        bodies, eps = lib.generate_ics(1, 100_000, 1), 0.01
        idx = np.sort(rng.choice(len(bodies), size=4096, replace=False))
    else:
        bodies, eps = golden("disk_3000.npz")["bodies"].copy(), 0.01
        idx = np.arange(len(bodies))
    sim = lib.Sim.from_bodies(bodies, softening=eps)
    got = sim.direct_forces(idx)
    sim.close()
    want = orc.direct_forces(bodies, 1.0, eps, idx)
    assert _rel(got, want).max() <= TOL


@pytest.mark.parametrize("kind,n,eps", [(0, 20000, 0.01), (1, 20000, 0.01), (2, 20000, 0.005)])
def test_energy_matches_oracle(lib, orc, kind, n, eps):
    bodies = lib.generate_ics(kind, n, 3)
    bodies["mass"][::97] = 0.0  # dead bodies count as massless
    sim = lib.Sim.from_bodies(bodies, softening=eps)
    ke, pe = sim.energy()
    sim.close()
    want_total = orc.total_energy(bodies, 1.0, eps)
    want_pe = orc.total_energy(_pe_only(bodies), 1.0, eps)
    assert abs(pe - want_pe) <= TOL * abs(want_pe)
    assert abs((ke + pe) - want_total) <= TOL * abs(want_total)


def test_ensemble_diagnostics_stay_within_each_system(lib, orc):
    """In an ensemble only bodies of the same system attract: each system's
    direct sum and energy equal the oracle's on that system alone."""
    parts = [lib.generate_ics(3, n, 40 + g) for g, n in enumerate((3000, 1500, 700))]
    allb = np.concatenate([p.astype(BODY_DTYPE) for p in parts]).astype(BODY_DTYPE)
    ens = lib.Sim.ensemble(allb, [len(p) for p in parts], softening=0.01)
    idx = np.arange(len(allb))
    got = ens.direct_forces(idx)
    ke, pe = ens.energy()
    ens.close()
    want = np.concatenate([orc.direct_forces(p, 1.0, 0.01) for p in parts])
    assert _rel(got, want).max() <= TOL
    want_pe = sum(orc.total_energy(_pe_only(p), 1.0, 0.01) for p in parts)
    want_total = sum(orc.total_energy(p, 1.0, 0.01) for p in parts)
    assert abs(pe - want_pe) <= TOL * abs(want_pe)
    assert abs((ke + pe) - want_total) <= TOL * abs(want_total)


def test_direct_forces_rejects_out_of_range_indices(lib):
    bodies = lib.generate_ics(0, 500, 2)
    sim = lib.Sim.from_bodies(bodies, softening=0.01)
    for bad in ([0, 500], [-1], [3, 2**31 - 1]):
        with pytest.raises(lib.CudaError, match="code 4"):
            sim.direct_forces(np.array(bad))
    assert np.isfinite(sim.direct_forces(np.array([0, 499]))).all()  # the handle still works
    sim.close()
