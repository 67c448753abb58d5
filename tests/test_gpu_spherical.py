"""SCF over the pure (spherical-harmonic) functions through the orthogonaliser
option (no reference counterpart: GANSU is Cartesian), against the oracle's
pure-basis SCF; the Cartesian gradient code applied to the pure-function
densities against finite differences of pure-function energies."""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry, spherical
from oracle import oracle as O

pytestmark = pytest.mark.gpu
CONV = {"convergence_threshold": 1e-11, "max_iter": 200}


def _oracle_pure(atoms, gbs):
    b = O.make_basis(atoms, gg.basis_path(gbs))
    S, T, V = O.one_electron(b)
    H = T + V
    eri = O.eri_tensor(b)
    fock = lambda D: H + np.einsum("ijkl,kl->ij", eri, D) - 0.5 * np.einsum("ikjl,kl->ij", eri, D)
    X = O.spherical_orthogonalizer(S, O.spherical_transform(b))
    return O.rhf(S, H, fock, b.num_electrons // 2, O.nuclear_repulsion(atoms), thr=1e-11, X=X)


@pytest.mark.parametrize("gbs", ["sto-3g", "6-31g_st", "cc-pvdz"])
def test_spherical_scf_matches_oracle(built_library, cuda, gbs):
    atoms = geometry.water()
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    eng = gg.Engine(mol, 1e-12)
    r = eng.rhf_scf(10, dict(CONV, spherical=True))
    ro = _oracle_pure(atoms, gbs)
    assert r["converged"] == 1 and ro["converged"]
    assert abs(r["total_energy"] - ro["total_energy"]) < 1e-9
    rc = eng.rhf_scf(10, CONV)
    if gbs == "sto-3g":  # no d shells: the pure basis is the Cartesian one
        assert abs(r["total_energy"] - rc["total_energy"]) < 1e-10
    else:  # fewer functions: variationally above the Cartesian energy
        assert r["total_energy"] > rc["total_energy"] + 1e-5


def test_spherical_mixed_tier_and_open_shells(built_library, cuda):
    atoms = geometry.alkane(3, jitter=0.02, seed=4)
    mol = gg.Molecular(atoms, gg.basis_path("6-31g_st"))
    eng = gg.Engine(mol, 1e-12)
    ne = mol.num_electrons
    r64 = eng.rhf_scf(ne, dict(CONV, spherical=True))
    rmx = eng.rhf_scf(ne, dict(CONV, spherical=True, precision=gg.HF_PRECISION_MIXED, mixed_threshold=0.1,
                               incremental=1, anchor_threshold=1e-2))
    assert r64["converged"] == 1 and rmx["converged"] == 1
    assert abs(r64["total_energy"] - rmx["total_energy"]) < 1e-6
    # closed shell: UHF and ROHF over the same functions give the RHF energy
    ru = eng.uhf_scf(ne // 2, ne // 2, dict(CONV, spherical=True))
    ro = eng.rohf_scf(ne // 2, ne // 2, dict(CONV, spherical=True))
    assert abs(ru["total_energy"] - r64["total_energy"]) < 5e-8
    assert abs(ro["total_energy"] - r64["total_energy"]) < 1e-9


def test_spherical_gradient_matches_finite_differences(built_library, cuda):
    atoms = geometry.water()
    gbs = gg.basis_path("6-31g_st")

    def energy(at):
        m = gg.Molecular(at, gbs)
        e = gg.Engine(m, 1e-12)
        r = e.rhf_scf(m.num_electrons, dict(CONV, spherical=True))
        e.close()
        return r["total_energy"]

    mol = gg.Molecular(atoms, gbs)
    eng = gg.Engine(mol, 1e-12)
    r = eng.rhf_scf(10, dict(CONV, spherical=True), want_matrices=True)
    W = eng.energy_weighted_density(r["coefficients"], r["orbital_energies"], 5)
    g, _ = eng.gradient(r["density"], W)
    h = 1e-4
    for a in range(3):
        for k in range(3):
            moved = [list(x) for x in atoms]
            moved[a][1 + k] += h
            ep = energy([tuple(x) for x in moved])
            moved[a][1 + k] -= 2 * h
            em = energy([tuple(x) for x in moved])
            assert abs((ep - em) / (2 * h) - g[a, k]) < 2e-6
    assert spherical.num_pure(mol) == 18
