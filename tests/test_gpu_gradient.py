"""Analytic RHF nuclear gradient (hf_rhf_gradient) through the C ABI.

The reference has no analytic gradient; its only gradient-like quantity is a
finite difference of energies, so the gradient is pinned against central
finite differences (step 1e-4 bohr) of FP64 SCF energies -- the engine's own
and the oracle's -- and checked for translational and rotational invariance.
Tolerance: 1e-6 Eh/bohr against finite differences of energies converged to
1e-11 Eh (the finite-difference error itself is ~1e-8).
"""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from oracle import oracle as O

pytestmark = pytest.mark.gpu

STEP = 1e-4
CONV = {"convergence_threshold": 1e-11, "max_iter": 200}


def _energy(atoms, gbs):
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    eng = gg.Engine(mol, 1e-14)
    r = eng.rhf_scf(mol.num_electrons, CONV)
    assert r["converged"] == 1
    return r["total_energy"]


def _analytic(atoms, gbs):
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    eng = gg.Engine(mol, 1e-14)
    r = eng.energy_and_gradient(mol.num_electrons, CONV)
    assert r["converged"] == 1
    return r["gradient"], r


def _fd(atoms, energy):
    g = np.zeros((len(atoms), 3))
    for a in range(len(atoms)):
        for k in range(3):
            plus = [list(x) for x in atoms]
            minus = [list(x) for x in atoms]
            plus[a][1 + k] += STEP
            minus[a][1 + k] -= STEP
            g[a, k] = (energy([tuple(x) for x in plus]) - energy([tuple(x) for x in minus])) / (2 * STEP)
    return g


@pytest.mark.parametrize("gbs", ["sto-3g", "6-31g_st", "cc-pvdz"])
def test_gradient_matches_finite_differences(built_library, cuda, gbs):
    atoms = [(z, x + 0.01 * i, y - 0.02 * i, w + 0.015) for i, (z, x, y, w) in enumerate(geometry.water())]
    g, _ = _analytic(atoms, gbs)
    fd = _fd(atoms, lambda a: _energy(a, gbs))
    np.testing.assert_allclose(g, fd, atol=1e-6, rtol=0)


def test_gradient_matches_oracle_finite_differences(built_library, cuda):
    atoms = [(z, x, y + 0.03 * i, w) for i, (z, x, y, w) in enumerate(geometry.water())]
    g, _ = _analytic(atoms, "sto-3g")

    def oracle_energy(a):
        b = O.make_basis(a, gg.basis_path("sto-3g"))
        return O.rhf_from_basis(b, thr_schwarz=1e-14, thr=1e-11, maxiter=200)["total_energy"]

    fd = _fd(atoms, oracle_energy)
    np.testing.assert_allclose(g, fd, atol=1e-6, rtol=0)


def test_gradient_with_p_functions_on_hydrogen(built_library, cuda):
    # cc-pVDZ puts p shells on H and d shells on C: the (dp|pp)-type derivative classes
    atoms = geometry.alkane(1, jitter=0.03, seed=4)  # methane
    g, _ = _analytic(atoms, "cc-pvdz")
    fd = _fd(atoms[:2], lambda a: _energy(a + atoms[2:], "cc-pvdz"))  # carbon and one hydrogen
    np.testing.assert_allclose(g[:2], fd, atol=1e-6, rtol=0)


def test_gradient_invariances_decane(built_library, cuda):
    atoms = geometry.alkane(10, jitter=0.02, seed=0)
    mol = gg.Molecular(atoms, gg.basis_path("6-31g_st"))
    eng = gg.Engine(mol, 1e-12)
    r = eng.energy_and_gradient(mol.num_electrons, {"convergence_threshold": 1e-10})
    g = r["gradient"]
    R = np.array([a[1:] for a in atoms])
    # no net force and no net torque on an isolated molecule
    assert np.abs(g.sum(axis=0)).max() < 1e-7
    assert np.abs(np.cross(R, g).sum(axis=0)).max() < 1e-6
    assert np.abs(g).max() > 1e-4  # a jittered geometry is not a stationary point


@pytest.mark.parametrize("gbs", ["6-31g_st", "cc-pvdz"])
def test_mixed_gradient_matches_fp64(built_library, cuda, gbs):
    # FP32 derivative integrals for the small-bound quartets: within 1e-5 Eh/bohr of FP64
    atoms = geometry.alkane(4, jitter=0.02, seed=3)
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    eng = gg.Engine(mol, 1e-12)
    r = eng.rhf_scf(mol.num_electrons, {"convergence_threshold": 1e-10}, want_matrices=True)
    W = eng.energy_weighted_density(r["coefficients"], r["orbital_energies"], mol.num_electrons // 2)
    g64, _ = eng.gradient(r["density"], W)
    g32, _ = eng.gradient(r["density"], W, mixed_threshold=1e-3)
    assert np.abs(g32 - g64).max() < 1e-5
    assert np.abs(g32.sum(axis=0)).max() < 1e-6
