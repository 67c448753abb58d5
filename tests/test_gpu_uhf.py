"""UHF (hf_uhf_scf) against the oracle's restatement of the reference UHF loop
on open-shell molecules (1e-7 Eh: the reference's per-spin DIIS converges
slowly on open shells, so two runs stopped by the same |dE| test sit a few
1e-8 Eh apart), and against RHF for a closed shell (1e-8 Eh)."""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from oracle import oracle as O

pytestmark = pytest.mark.gpu
CONV = {"convergence_threshold": 1e-12, "max_iter": 300}
ANG = gg.ANGSTROM_TO_BOHR


def _nh2():
    # bent NH2 radical (doublet, no orbital degeneracy): N-H 1.024 A, H-N-H 103.4 deg
    half = np.radians(103.4) / 2
    r = 1.024 * ANG
    return [(7, 0.0, 0.0, 0.0), (1, r * np.sin(half), 0.0, r * np.cos(half)),
            (1, -r * np.sin(half), 0.0, r * np.cos(half))]


def _ch2():
    return [(6, 0.0, 0.0, 0.0), (1, 0.0, 0.86 * ANG, 0.60 * ANG), (1, 0.0, -0.86 * ANG, 0.60 * ANG)]


@pytest.mark.parametrize("atoms,na,nb,gbs", [
    (_nh2(), 5, 4, "sto-3g"),       # NH2 radical, doublet
    (_nh2(), 5, 4, "6-31g_st"),
    (_ch2(), 5, 3, "6-31g"),         # CH2 triplet
    (geometry.water(), 5, 4, "6-31g"),  # H2O+ doublet
])
def test_uhf_matches_oracle(built_library, cuda, atoms, na, nb, gbs):
    mol = gg.Molecular(atoms, gg.basis_path(gbs), charge=sum(a[0] for a in atoms) - na - nb)
    eng = gg.Engine(mol, 1e-12)
    r = eng.uhf_scf(na, nb, CONV)
    b = O.make_basis(atoms, gg.basis_path(gbs))
    ro = O.uhf_from_basis(b, na, nb, thr=1e-12, maxiter=300)
    assert r["converged"] == 1 and ro["converged"]
    assert abs(r["total_energy"] - ro["total_energy"]) < 1e-7


def test_uhf_closed_shell_equals_rhf(built_library, cuda):
    mol = gg.Molecular(geometry.water(), gg.basis_path("6-31g_st"))
    eng = gg.Engine(mol, 1e-12)
    ru = eng.uhf_scf(5, 5, CONV, want_matrices=True)
    rr = eng.rhf_scf(10, CONV, want_matrices=True)
    # the beta symmetry break of the guess decays slowly: both stop at |dE| < 1e-12 within 5e-8 Eh
    assert abs(ru["total_energy"] - rr["total_energy"]) < 5e-8
    # the guess's beta symmetry break decays slowly, along a direction of almost no energy
    # curvature: at |dE| < 1e-12 the densities agree to ~sqrt(5e-8 Eh), i.e. 1e-4
    np.testing.assert_allclose((ru["density_alpha"] + ru["density_beta"]).cpu().numpy(),
                               rr["density"].cpu().numpy(), atol=1e-4)


def test_builder_uhf_recipe(built_library, cuda, tmp_path):
    xyz = tmp_path / "nh2.xyz"
    geometry.write_xyz(xyz, _nh2())
    pm = gg.ParameterManager()
    pm["xyzfilename"] = str(xyz)
    pm["gbsfilename"] = str(gg.basis_path("sto-3g"))
    pm["method"] = "uhf"
    pm["convergence_energy_threshold"] = "1e-12"
    pm["maxiter"] = "300"
    hf = gg.HFBuilder.buildHF(pm)
    ro = O.uhf_from_basis(O.make_basis(_nh2(), gg.basis_path("sto-3g")), 5, 4, thr=1e-12, maxiter=300)
    assert abs(hf.solve() - ro["total_energy"]) < 1e-7
