"""Damping and optimal damping (Convergence_RHF/UHF/ROHF_Damping, include/rhf.hpp:182-262,
include/uhf.hpp:196-250, include/rohf.hpp:216-290) against the oracle's restatement
(RHF: energies and iteration counts) and against the DIIS energies (UHF, ROHF)."""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from oracle import oracle as O

pytestmark = pytest.mark.gpu
CONV = {"convergence_threshold": 1e-10, "max_iter": 300}


@pytest.mark.parametrize("method,factor", [(gg.HF_CONV_DAMPING, 0.5), (gg.HF_CONV_OPTIMAL_DAMPING, 0.0)])
def test_rhf_damping_matches_oracle(built_library, cuda, method, factor):
    atoms, gbs = geometry.water(), "6-31g"
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    eng = gg.Engine(mol, 1e-12)
    r = eng.rhf_scf(10, dict(CONV, convergence_method=method, damping_factor=factor))
    b = O.make_basis(atoms, gg.basis_path(gbs))
    S, T, V = O.one_electron(b)
    eri = O.eri_tensor(b)
    fock = lambda D: T + V + np.einsum("ijkl,kl->ij", eri, D) - 0.5 * np.einsum("ikjl,kl->ij", eri, D)
    name = "damping" if method == gg.HF_CONV_DAMPING else "optimaldamping"
    ro = O.rhf(S, T + V, fock, 5, O.nuclear_repulsion(atoms), thr=1e-10, maxiter=300, convergence=name,
               damping=factor)
    assert r["converged"] == 1 and ro["converged"]
    assert abs(r["total_energy"] - ro["total_energy"]) < 1e-9
    assert abs(r["iterations"] - ro["iterations"]) <= 1
    rd = eng.rhf_scf(10, CONV)
    assert abs(r["total_energy"] - rd["total_energy"]) < 1e-8


def test_open_shell_damping_reaches_diis_energies(built_library, cuda):
    half = np.radians(103.4) / 2
    rr = 1.024 * gg.ANGSTROM_TO_BOHR
    atoms = [(7, 0.0, 0.0, 0.0), (1, rr * np.sin(half), 0.0, rr * np.cos(half)),
             (1, -rr * np.sin(half), 0.0, rr * np.cos(half))]
    mol = gg.Molecular(atoms, gg.basis_path("6-31g"))
    eng = gg.Engine(mol, 1e-12)
    conv = dict(CONV, convergence_threshold=1e-11)
    ud = eng.uhf_scf(5, 4, conv)
    uh = eng.uhf_scf(5, 4, dict(conv, convergence_method=gg.HF_CONV_DAMPING, damping_factor=0.5))
    assert uh["converged"] == 1 and abs(uh["total_energy"] - ud["total_energy"]) < 1e-7
    od = eng.rohf_scf(5, 4, conv)
    for method, factor in ((gg.HF_CONV_DAMPING, 0.5), (gg.HF_CONV_OPTIMAL_DAMPING, 0.0)):
        oh = eng.rohf_scf(5, 4, dict(conv, convergence_method=method, damping_factor=factor))
        assert oh["converged"] == 1 and abs(oh["total_energy"] - od["total_energy"]) < 1e-8


def test_mirror_recipe_with_damping(built_library, cuda, tmp_path):
    xyz = tmp_path / "w.xyz"
    geometry.write_xyz(xyz, geometry.water())
    pm = gg.ParameterManager()
    pm["xyzfilename"] = str(xyz)
    pm["gbsfilename"] = str(gg.basis_path("sto-3g"))
    pm["convergence_method"] = "optimaldamping"
    pm["convergence_energy_threshold"] = "1e-10"
    pm["maxiter"] = "300"
    e = gg.HFBuilder.buildHF(pm).solve()
    pm["convergence_method"] = "diis"
    assert abs(e - gg.HFBuilder.buildHF(pm).solve()) < 1e-8
