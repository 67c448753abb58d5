"""eri_method = stored (ERI_Stored_RHF, the reference's default method): the
N^4 ERI tensor is computed once per engine and the Fock matrix is built from it
every iteration, all through the C ABI.  Tolerances: SCF total energy within
1e-8 Eh of the energy on the reference's own integrals (golden fixtures) and
within 1e-9 Eh of the direct build's SCF; orbital energies within 1e-6 Eh."""
from pathlib import Path

import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"


@pytest.mark.parametrize("case", ["water_sto-3g", "water_6-31g_st", "propane_6-31g_st"])
def test_stored_scf_matches_reference_and_direct(built_library, cuda, case):
    g = np.load(GOLD / f"{case}.npz")
    atoms = [(int(a[0]), float(a[1]), float(a[2]), float(a[3])) for a in g["atoms"]]
    mol = gg.Molecular(atoms, gg.basis_path(case.split("_", 1)[1]))
    eng = gg.Engine(mol, 1e-12)
    nel = mol.num_electrons
    opts = {"convergence_threshold": 1e-10}
    rs = eng.rhf_scf(nel, dict(opts, eri_method=gg.HF_ERI_STORED), want_matrices=True)
    rd = eng.rhf_scf(nel, opts)
    assert rs["converged"] == 1
    assert abs(rs["total_energy"] - float(g["energy_total"])) < 1e-8
    assert abs(rs["total_energy"] - rd["total_energy"]) < 1e-9
    np.testing.assert_allclose(rs["orbital_energies"].cpu().numpy(), g["orbital_energies"], atol=1e-6)
    # the tensor stays with the engine: a second solve reuses it
    rs2 = eng.rhf_scf(nel, dict(opts, eri_method=gg.HF_ERI_STORED))
    assert abs(rs2["total_energy"] - rs["total_energy"]) < 1e-12
    eng.close()


def test_stored_is_the_recipe_default(built_library, cuda, tmp_path):
    xyz = tmp_path / "w.xyz"
    geometry.write_xyz(xyz, geometry.water())
    pm = gg.ParameterManager()
    pm.parse_command_line_args(["-x", str(xyz), "-g", gg.basis_path("6-31g_st"),
                                "--convergence_energy_threshold", "1e-10"])
    assert pm["eri_method"] == "stored"
    hf = gg.HFBuilder.buildHF(pm)
    assert hf.eri_method == gg.HF_ERI_STORED
    e_stored = hf.solve()
    pm["eri_method"] = "direct"
    assert abs(gg.HFBuilder.buildHF(pm).solve() - e_stored) < 1e-9


def test_stored_rejects_the_mixed_tier(built_library, cuda):
    mol = gg.Molecular(geometry.water(), gg.basis_path("sto-3g"))
    eng = gg.Engine(mol, 1e-12)
    with pytest.raises(gg.HFError) as err:
        eng.rhf_scf(mol.num_electrons, {"eri_method": gg.HF_ERI_STORED, "precision": gg.HF_PRECISION_MIXED})
    assert err.value.status == 1  # HF_ERR_INVALID_ARGUMENT
    eng.close()
