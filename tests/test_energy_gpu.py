"""The energy gate: the mixed-precision iteration reaches the plain FP64
iteration's converged energy.

Both start from the same seeded orbitals (32 on 48^3, h = 0.35, 8 wells)
and stop on DFTsolver's energy test (src/DFTsolver.cc:138-167) at 1e-8 Ha,
a hundred times below the 1e-6 Ha the comparison asserts; the mixed path's
test reads energies evaluated by energy_accurate (FP64 stencils, FP32
products summed to double-float), and its final energy is checked
against a full FP64 evaluation of the same block as well.
"""
import pytest

from mgmol_gb300 import convergence

pytestmark = pytest.mark.gpu


def test_mixed_iteration_reaches_the_fp64_energy():
    r = convergence.run((48, 48, 48), 0.35, 32, 8, 1001, tol_ha=1e-8, max_plain=2000,
                        max_mixed=2000, every=10)
    assert r["plain"]["converged"]
    assert r["mixed"]["converged"]
    assert r["mixed"]["abs_dE_vs_plain_ha"] <= 1e-6
    # the accurate evaluation stands in for the FP64 one
    assert r["accurate_vs_fp64_ha"] <= 5e-8
    # the mixed orbitals follow the FP64 trajectory sweep by sweep
    assert r["mixed"]["max_abs_dE_same_sweep_ha"] <= 1e-6
