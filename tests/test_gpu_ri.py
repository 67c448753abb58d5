"""RI (density fitting) path through the C ABI against the reference's own RI
kernels (golden fixtures from src/int2c2e.cu / src/int3c2e.cu run on the CPU)
and the oracle's restatement of B, J, K and the RI-SCF.

Tolerances: integrals 1e-12 (absolute, relative to the largest element for
the metric), B 1e-9 relative to its largest element (the triangular solve
carries the metric's conditioning), J / K 1e-10, RI-SCF energy 1e-8 Eh.
"""
from pathlib import Path

import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"
RI_CASES = ["ri_water_sto-3g", "ri_water_cc-pvdz", "ri_methane_cc-pvdz"]


def _setup(case):
    g = np.load(GOLD / f"{case}.npz")
    gbs = case.split("_", 2)[2]
    atoms = [(int(a[0]), float(a[1]), float(a[2]), float(a[3])) for a in g["atoms"]]
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    aux = gg.Molecular(atoms, gg.basis_path("cc-pvdz-rifit"))
    eng = gg.Engine(mol, 1e-12)
    eng.set_auxiliary_basis(aux)
    b = O.make_basis(atoms, gg.basis_path(gbs))
    ax = O.make_basis(atoms, gg.basis_path("cc-pvdz-rifit"))
    return g, eng, b, ax


@pytest.mark.parametrize("case", RI_CASES)
def test_metric_and_three_center_match_reference(built_library, cuda, case):
    g, eng, _, _ = _setup(case)
    V = eng.two_center_eris().cpu().numpy()
    assert np.abs(V - g["V"]).max() < 1e-12 * np.abs(g["V"]).max()
    T = eng.three_center_eris().cpu().numpy()
    if "T" in g:
        assert np.abs(T - g["T"]).max() < 1e-12
    else:
        idx = g["T_idx"]
        assert np.abs(T[idx[:, 0], idx[:, 1], idx[:, 2]] - g["T_val"]).max() < 1e-12
    assert abs(T.sum() - float(g["T_sum"])) < 1e-10 * max(1.0, abs(float(g["T_sum"])))
    assert abs((T * T).sum() - float(g["T_sq_sum"])) < 1e-10 * float(g["T_sq_sum"])


@pytest.mark.parametrize("case", RI_CASES[1:])
def test_b_tensor_and_jk_match_oracle(built_library, cuda, case):
    import torch
    g, eng, b, ax = _setup(case)
    B = eng.ri_intermediate_b().cpu().numpy()
    V, T, _ = O.ri_integrals(b, ax, 1e-12)
    Bo = O.ri_factor(V, T)
    # B = L^-1 T carries the metric's conditioning: compare relative to its largest element
    assert np.abs(B - Bo).max() < 1e-9 * max(1.0, np.abs(Bo).max())
    rng = np.random.default_rng(3)
    N = b.nbf
    # an SCF-like density (PSD) and an indefinite symmetric one (a density difference)
    Cm = rng.normal(size=(N, N)) * 0.3
    D1 = 2.0 * Cm[:, : N // 3] @ Cm[:, : N // 3].T
    A = rng.normal(size=(N, N)) * 0.1
    D2 = A + A.T
    for D in (D1, D2):
        J, K = eng.jk_ri(torch.tensor(D, device="cuda"))
        Jo, Ko = O.ri_jk(Bo, D)
        assert np.abs(J.cpu().numpy() - Jo).max() < 1e-10 * max(1.0, np.abs(Jo).max())
        assert np.abs(K.cpu().numpy() - Ko).max() < 1e-10 * max(1.0, np.abs(Ko).max())
    H = rng.normal(size=(N, N))
    H = H + H.T
    F = eng.fock_ri(torch.tensor(D1, device="cuda"), torch.tensor(H, device="cuda")).cpu().numpy()
    Jo, Ko = O.ri_jk(Bo, D1)
    assert np.abs(F - (H + Jo - 0.5 * Ko)).max() < 1e-10 * max(1.0, np.abs(Jo).max())


@pytest.mark.parametrize("case", RI_CASES)
def test_ri_scf_energy_matches_reference_integrals(built_library, cuda, case):
    g, eng, _, _ = _setup(case)
    r = eng.rhf_scf(eng.mol.num_electrons, {"convergence_threshold": 1e-10, "eri_method": gg.HF_ERI_RI})
    assert r["converged"] == 1
    assert abs(r["total_energy"] - float(g["energy_total"])) < 1e-8


def test_ri_scf_propane_matches_oracle(built_library, cuda):
    atoms = geometry.alkane(3, jitter=0.02, seed=11)
    mol = gg.Molecular(atoms, gg.basis_path("6-31g_st"))
    eng = gg.Engine(mol, 1e-12)
    eng.set_auxiliary_basis(gg.Molecular(atoms, gg.basis_path("cc-pvdz-rifit")))
    r = eng.rhf_scf(mol.num_electrons, {"convergence_threshold": 1e-10, "eri_method": gg.HF_ERI_RI})
    b = O.make_basis(atoms, gg.basis_path("6-31g_st"))
    ax = O.make_basis(atoms, gg.basis_path("cc-pvdz-rifit"))
    ro = O.rhf_ri_from_basis(b, ax, thr_schwarz=1e-12, thr=1e-10)
    assert r["converged"] == 1 and ro["converged"]
    assert abs(r["total_energy"] - ro["total_energy"]) < 1e-8
    # RI error against the exact (direct) energy is small but not zero
    rd = eng.rhf_scf(mol.num_electrons, {"convergence_threshold": 1e-10})
    assert 0 < abs(r["total_energy"] - rd["total_energy"]) < 5e-3


def test_rhf_mirror_ri_method(built_library, cuda, tmp_path):
    xyz = tmp_path / "w.xyz"
    geometry.write_xyz(xyz, geometry.water())
    pm = gg.ParameterManager()
    pm["xyzfilename"] = str(xyz)
    pm["gbsfilename"] = str(gg.basis_path("cc-pvdz"))
    pm["eri_method"] = "ri"
    pm["auxiliary_gbsfilename"] = str(gg.basis_path("cc-pvdz-rifit"))
    pm["convergence_energy_threshold"] = "1e-10"
    hf = gg.HFBuilder.buildHF(pm)
    e = hf.solve()
    g = np.load(GOLD / "ri_water_cc-pvdz.npz")
    assert abs(e - float(g["energy_total"])) < 1e-8


def test_ri_without_auxiliary_basis_is_an_error(built_library, cuda):
    mol = gg.Molecular(geometry.water(), gg.basis_path("sto-3g"))
    eng = gg.Engine(mol, 1e-12)
    with pytest.raises(gg.HFError):
        eng.rhf_scf(mol.num_electrons, {"eri_method": gg.HF_ERI_RI})


@pytest.mark.parametrize("case", RI_CASES[1:])
def test_mixed_ri_scf_matches_fp64_ri(built_library, cuda, case):
    # split-BF16 tensor-core K until max|dD| < 1e-2, one FP64 anchor, then aligned K(dD) increments
    g, eng, _, _ = _setup(case)
    r64 = eng.rhf_scf(eng.mol.num_electrons, {"convergence_threshold": 1e-10, "eri_method": gg.HF_ERI_RI})
    rmx = eng.rhf_scf(eng.mol.num_electrons, {"convergence_threshold": 1e-10, "eri_method": gg.HF_ERI_RI,
                                              "precision": gg.HF_PRECISION_MIXED, "anchor_threshold": 1e-2})
    assert r64["converged"] == 1 and rmx["converged"] == 1
    assert abs(rmx["total_energy"] - r64["total_energy"]) < 1e-6
    assert abs(rmx["total_energy"] - float(g["energy_total"])) < 1e-6


def test_mixed_ri_scf_propane(built_library, cuda):
    atoms = geometry.alkane(3, jitter=0.02, seed=11)
    mol = gg.Molecular(atoms, gg.basis_path("cc-pvdz"))
    eng = gg.Engine(mol, 1e-12)
    eng.set_auxiliary_basis(gg.Molecular(atoms, gg.basis_path("cc-pvdz-rifit")))
    base = {"convergence_threshold": 1e-9, "eri_method": gg.HF_ERI_RI}
    r64 = eng.rhf_scf(mol.num_electrons, base)
    for tau in (1e-1, 1e-2, 1e-3):
        rmx = eng.rhf_scf(mol.num_electrons, dict(base, precision=gg.HF_PRECISION_MIXED, anchor_threshold=tau))
        assert rmx["converged"] == 1
        assert abs(rmx["total_energy"] - r64["total_energy"]) < 1e-6, tau


def test_ri_scf_with_purification(built_library, cuda):
    """RI with the purification eigensolver: the K build takes an orthonormal basis of
    the occupied space from the projector (CholeskyQR2 of P Q_prev), FP64 and mixed."""
    atoms = geometry.alkane(3, jitter=0.02, seed=11)
    mol = gg.Molecular(atoms, gg.basis_path("cc-pvdz"))
    eng = gg.Engine(mol, 1e-12)
    eng.set_auxiliary_basis(gg.Molecular(atoms, gg.basis_path("cc-pvdz-rifit")))
    base = {"convergence_threshold": 1e-10, "eri_method": gg.HF_ERI_RI}
    r64 = eng.rhf_scf(mol.num_electrons, base, want_matrices=True)
    rp = eng.rhf_scf(mol.num_electrons, dict(base, eigensolver=gg.HF_EIGEN_PURIFICATION), want_matrices=True)
    assert rp["converged"] == 1 and abs(rp["total_energy"] - r64["total_energy"]) < 1e-9
    assert abs(rp["iterations"] - r64["iterations"]) <= 1
    np.testing.assert_allclose(rp["orbital_energies"].cpu().numpy(), r64["orbital_energies"].cpu().numpy(),
                               atol=1e-5)
    rm = eng.rhf_scf(mol.num_electrons, dict(base, eigensolver=gg.HF_EIGEN_PURIFICATION,
                                             precision=gg.HF_PRECISION_MIXED, anchor_threshold=1e-2))
    assert rm["converged"] == 1 and abs(rm["total_energy"] - r64["total_energy"]) < 1e-6


RI_CONV = {"convergence_threshold": 1e-11, "max_iter": 200, "eri_method": gg.HF_ERI_RI}
FD_STEP = 1e-4  # bohr


def _ri_energy(atoms, gbs):
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    eng = gg.Engine(mol, 1e-14)
    eng.set_auxiliary_basis(gg.Molecular(atoms, gg.basis_path("cc-pvdz-rifit")))
    r = eng.rhf_scf(mol.num_electrons, RI_CONV)
    eng.close()
    assert r["converged"] == 1
    return r["total_energy"]


@pytest.mark.parametrize("name,atoms,atom_subset", [
    ("water", [(z, x + 0.01 * i, y - 0.02 * i, w + 0.015) for i, (z, x, y, w) in enumerate(geometry.water())],
     None),
    ("methane", geometry.alkane(1, jitter=0.03, seed=4), [0, 1]),
])
def test_ri_gradient_matches_finite_differences(built_library, cuda, name, atoms, atom_subset):
    """Analytic gradient of the RI energy (derivative three-centre and metric
    integrals, hf_rhf_gradient_ri) against central finite differences (h = 1e-4
    bohr) of RI-SCF energies converged to 1e-11 Eh: 1e-6 Eh/bohr; cc-pVDZ with
    cc-pVDZ-RIFIT (p shells on H, d on C/O in the AO basis, up to f in the
    auxiliary basis)."""
    gbs = "cc-pvdz"
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    eng = gg.Engine(mol, 1e-14)
    eng.set_auxiliary_basis(gg.Molecular(atoms, gg.basis_path("cc-pvdz-rifit")))
    r = eng.energy_and_gradient(mol.num_electrons, RI_CONV)
    assert r["converged"] == 1
    g = r["gradient"]
    eng.close()
    # no net force on an isolated molecule
    assert np.abs(g.sum(axis=0)).max() < 1e-8
    for a in (atom_subset if atom_subset is not None else range(len(atoms))):
        for k in range(3):
            plus = [list(x) for x in atoms]
            minus = [list(x) for x in atoms]
            plus[a][1 + k] += FD_STEP
            minus[a][1 + k] -= FD_STEP
            fd = (_ri_energy([tuple(x) for x in plus], gbs) - _ri_energy([tuple(x) for x in minus], gbs)) / (2 * FD_STEP)
            assert abs(g[a, k] - fd) < 1e-6, (name, a, k, g[a, k], fd)


def test_ri_gradient_differs_from_four_centre_gradient_by_the_fitting_error(built_library, cuda):
    """The RI and the four-centre gradients of the same molecule agree to the
    density-fitting error (~1e-4 Eh/bohr), not exactly: the RI one is the gradient
    of the RI energy."""
    atoms = geometry.water()
    mol = gg.Molecular(atoms, gg.basis_path("cc-pvdz"))
    eng = gg.Engine(mol, 1e-14)
    eng.set_auxiliary_basis(gg.Molecular(atoms, gg.basis_path("cc-pvdz-rifit")))
    g_ri = eng.energy_and_gradient(mol.num_electrons, RI_CONV)["gradient"]
    g_4c = eng.energy_and_gradient(mol.num_electrons, {"convergence_threshold": 1e-11})["gradient"]
    eng.close()
    d = np.abs(g_ri - g_4c).max()
    assert 1e-9 < d < 1e-3
