"""UHF (hf_uhf_scf) against the oracle's restatement of the reference UHF loop
on open-shell molecules, and against RHF for a closed shell (1e-8 Eh)."""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from oracle import oracle as O

pytestmark = pytest.mark.gpu
CONV = {"convergence_threshold": 1e-10}
ANG = gg.ANGSTROM_TO_BOHR


def _oh():
    return [(8, 0.0, 0.0, 0.0), (1, 0.0, 0.0, 0.97 * ANG)]


def _ch2():
    return [(6, 0.0, 0.0, 0.0), (1, 0.0, 0.86 * ANG, 0.60 * ANG), (1, 0.0, -0.86 * ANG, 0.60 * ANG)]


@pytest.mark.parametrize("atoms,na,nb,gbs", [
    (_oh(), 5, 4, "sto-3g"),        # OH radical, doublet
    (_oh(), 5, 4, "6-31g_st"),
    (_ch2(), 5, 3, "6-31g"),         # CH2 triplet
    (geometry.water(), 5, 4, "6-31g"),  # H2O+ doublet
])
def test_uhf_matches_oracle(built_library, cuda, atoms, na, nb, gbs):
    mol = gg.Molecular(atoms, gg.basis_path(gbs), charge=sum(a[0] for a in atoms) - na - nb)
    eng = gg.Engine(mol, 1e-12)
    r = eng.uhf_scf(na, nb, CONV)
    b = O.make_basis(atoms, gg.basis_path(gbs))
    ro = O.uhf_from_basis(b, na, nb, thr=1e-10, maxiter=200)
    assert r["converged"] == 1 and ro["converged"]
    assert abs(r["total_energy"] - ro["total_energy"]) < 1e-8


def test_uhf_closed_shell_equals_rhf(built_library, cuda):
    mol = gg.Molecular(geometry.water(), gg.basis_path("6-31g_st"))
    eng = gg.Engine(mol, 1e-12)
    ru = eng.uhf_scf(5, 5, CONV, want_matrices=True)
    rr = eng.rhf_scf(10, CONV, want_matrices=True)
    assert abs(ru["total_energy"] - rr["total_energy"]) < 1e-8
    np.testing.assert_allclose((ru["density_alpha"] + ru["density_beta"]).cpu().numpy(),
                               rr["density"].cpu().numpy(), atol=1e-6)
