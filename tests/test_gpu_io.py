"""Molden export and Mulliken charges of solved RHF / UHF / ROHF runs
(export_molden_file, src/rhf.cu:363-425, src/uhf.cu:379-440, src/rohf.cu:348-410;
analyze_mulliken_population, src/rhf.cu:427-460)."""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry, molden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _params(tmp_path, atoms, gbs, method, charge=0):
    xyz = tmp_path / "m.xyz"
    geometry.write_xyz(xyz, atoms)
    pm = gg.ParameterManager()
    pm["xyzfilename"] = str(xyz)
    pm["gbsfilename"] = str(gg.basis_path(gbs))
    pm["method"] = method
    pm["charge"] = str(charge)
    pm["convergence_energy_threshold"] = "1e-11"
    pm["maxiter"] = "300"
    return pm


def test_rhf_molden_and_mulliken(built_library, cuda, tmp_path):
    atoms = geometry.water()
    hf = gg.HFBuilder.buildHF(_params(tmp_path, atoms, "6-31g_st", "rhf"))
    hf.solve()
    path = tmp_path / "out.molden"
    hf.export_molden_file(str(path))
    text = path.read_text()
    assert text.startswith("[Molden Format]\ngenerated by GANSU\n[Atoms] (AU)\nO 1 8 ")
    b = O.make_basis(atoms, gg.basis_path("6-31g_st"))
    gto = text.split("[GTO]")[1].split("[MO]")[0]
    shells = [ln for ln in gto.splitlines() if ln.startswith(" ") and ln.split()[0] in "spdfg"]
    assert len(shells) == len(b.l)
    spins, eps, occ, Cm = molden.read_molden_mos(str(path))
    n = hf.mol.num_basis
    assert Cm.shape == (n, n) and spins == ["Alpha"] * n and occ.sum() == 10
    D = (Cm * occ) @ Cm.T
    np.testing.assert_allclose(D, hf.result["density"].cpu().numpy(), atol=1e-12)
    np.testing.assert_allclose(eps[1:], hf.result["orbital_energies"].cpu().numpy()[1:], rtol=1e-15)
    q = hf.analyze_mulliken_population()
    assert abs(q.sum()) < 1e-10 and q[0] < -0.3 and q[1] > 0.15
    ro = O.rhf_from_basis(b, thr=1e-11)
    S = O.one_electron(b)[0]
    pop = np.einsum("ij,ij->i", ro["density"], S)
    ranges = O.atom_ranges(b)
    q_ref = np.array([z - pop[lo:lo + c].sum() for (z, *_), (lo, c) in zip(atoms, ranges)])
    np.testing.assert_allclose(q, q_ref, atol=1e-6)


def test_uhf_and_rohf_molden(built_library, cuda, tmp_path):
    half = np.radians(103.4) / 2
    r = 1.024 * gg.ANGSTROM_TO_BOHR
    atoms = [(7, 0.0, 0.0, 0.0), (1, r * np.sin(half), 0.0, r * np.cos(half)),
             (1, -r * np.sin(half), 0.0, r * np.cos(half))]
    for method in ("uhf", "rohf"):
        pm = _params(tmp_path, atoms, "6-31g", method)
        pm["beta_to_alpha"] = "0"
        hf = gg.HFBuilder.buildHF(pm)
        hf.solve()
        path = tmp_path / f"{method}.molden"
        hf.export_molden_file(str(path))
        spins, eps, occ, Cm = molden.read_molden_mos(str(path))
        n = hf.mol.num_basis
        Da, Db = hf.export_density_matrix()
        if method == "uhf":
            assert spins == ["Alpha"] * n + ["Beta"] * n
            Ca, Cb = Cm[:, :n], Cm[:, n:]
            # the exported orbitals are the ones behind the returned densities
            np.testing.assert_allclose((Ca * occ[:n]) @ Ca.T, Da, atol=1e-12)
            np.testing.assert_allclose((Cb * occ[n:]) @ Cb.T, Db, atol=1e-12)
        else:
            assert spins == ["Alpha"] * n and occ.sum() == 9 and list(occ[:5]) == [2, 2, 2, 2, 1]
            np.testing.assert_allclose((Cm * occ) @ Cm.T, Da + Db, atol=1e-9)
        q = hf.analyze_mulliken_population()
        assert abs(q.sum()) < 1e-9
