"""ROHF (hf_rohf_scf), the density / SAD initial guesses of RHF, UHF, ROHF and
the batch, and the .sad file path, against the oracle's restatements of the
reference loops (src/rohf.cu, include/rhf.hpp:378-588, include/uhf.hpp:484-620,
include/rohf.hpp:416-600)."""
import shutil

import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry, sad
from oracle import oracle as O

pytestmark = pytest.mark.gpu
CONV = {"convergence_threshold": 1e-12, "max_iter": 300}
ANG = gg.ANGSTROM_TO_BOHR


def _nh2():
    half = np.radians(103.4) / 2
    r = 1.024 * ANG
    return [(7, 0.0, 0.0, 0.0), (1, r * np.sin(half), 0.0, r * np.cos(half)),
            (1, -r * np.sin(half), 0.0, r * np.cos(half))]


def _ch2():
    return [(6, 0.0, 0.0, 0.0), (1, 0.0, 0.86 * ANG, 0.60 * ANG), (1, 0.0, -0.86 * ANG, 0.60 * ANG)]


def _engine(atoms, gbs, charge=0):
    mol = gg.Molecular(atoms, gg.basis_path(gbs), charge=charge)
    return mol, gg.Engine(mol, 1e-12)


@pytest.mark.parametrize("atoms,na,nb,gbs", [
    (_nh2(), 5, 4, "sto-3g"),         # NH2 doublet
    (_nh2(), 5, 4, "6-31g_st"),
    (_ch2(), 5, 3, "6-31g"),           # CH2 triplet
    ([(8, 0.0, 0.0, 0.0)], 5, 3, "6-31g"),  # O atom triplet
])
def test_rohf_matches_oracle(built_library, cuda, atoms, na, nb, gbs):
    mol, eng = _engine(atoms, gbs, charge=sum(a[0] for a in atoms) - na - nb)
    r = eng.rohf_scf(na, nb, CONV, want_matrices=True)
    ro = O.rohf_from_basis(O.make_basis(atoms, gg.basis_path(gbs)), na, nb, thr=1e-12, maxiter=300)
    assert r["converged"] == 1 and ro["converged"]
    assert abs(r["total_energy"] - ro["total_energy"]) < 1e-8
    # export_density_matrix: alpha - beta is the open-shell density (trace na - nb in S)
    S = O.one_electron(O.make_basis(atoms, gg.basis_path(gbs)))[0]
    Da, Db = r["density_alpha"].cpu().numpy(), r["density_beta"].cpu().numpy()
    assert abs(np.vdot(Da, S) - na) < 1e-8 and abs(np.vdot(Db, S) - nb) < 1e-8


@pytest.mark.parametrize("name", ["guest-saunders", "mcweeny-diercksen", "binkley-pople-dobosh"])
def test_rohf_coupling_sets_match_oracle(built_library, cuda, name):
    mol, eng = _engine(_nh2(), "sto-3g", charge=0)
    r = eng.rohf_scf(5, 4, CONV, coupling=name)
    ro = O.rohf_from_basis(O.make_basis(_nh2(), gg.basis_path("sto-3g")), 5, 4, thr=1e-12, maxiter=300,
                           coupling=name)
    assert r["converged"] == ro["converged"]
    if ro["converged"]:
        assert abs(r["total_energy"] - ro["total_energy"]) < 1e-8


def test_rohf_closed_shell_equals_rhf(built_library, cuda):
    mol, eng = _engine(geometry.water(), "6-31g_st")
    ro = eng.rohf_scf(5, 5, CONV)
    rr = eng.rhf_scf(10, CONV)
    assert abs(ro["total_energy"] - rr["total_energy"]) < 1e-9


def test_device_atomic_densities_match_oracle(built_library, cuda):
    """The atoms' densities the product computes for the SAD guess (RHF for even Z,
    ROHF doublet for odd Z) against the oracle's (energies; H elementwise)."""
    for gbs in ("sto-3g", "6-31g"):
        for z in (1, 6, 7, 8):
            Da, Db = sad.atomic_density(z, gg.basis_path(gbs), source="compute")
            b = O.make_basis([(z, 0.0, 0.0, 0.0)], gg.basis_path(gbs))
            S, T, V = O.one_electron(b)
            eri = O.eri_tensor(b)
            jk = lambda D: (np.einsum("ijkl,kl->ij", eri, D), np.einsum("ikjl,kl->ij", eri, D))
            Oa, Ob = O.atom_sad_density(z, gg.basis_path(gbs))
            assert abs(O.uhf_energy_of(S, T + V, jk, Da, Db) - O.uhf_energy_of(S, T + V, jk, Oa, Ob)) < 1e-9
            assert abs(np.vdot(Da + Db, S) - z) < 1e-9
            if z == 1:
                np.testing.assert_allclose(Da, Oa, atol=1e-10)


@pytest.mark.parametrize("guess", ["sad", "density"])
def test_rhf_density_guesses_match_oracle(built_library, cuda, guess):
    atoms, gbs = geometry.water(), "6-31g"
    mol, eng = _engine(atoms, gbs)
    Da, Db = eng.sad_density()
    r = eng.rhf_scf(10, dict(CONV, initial_guess=gg._GUESSES[guess], guess_density_a=Da, guess_density_b=Db))
    b = O.make_basis(atoms, gg.basis_path(gbs))
    S, T, V = O.one_electron(b)
    eri = O.eri_tensor(b)
    fock = lambda D: T + V + np.einsum("ijkl,kl->ij", eri, D) - 0.5 * np.einsum("ikjl,kl->ij", eri, D)
    ro = O.rhf(S, T + V, fock, 5, O.nuclear_repulsion(atoms), thr=1e-12, maxiter=300, guess=guess,
               guess_density=(Da + Db).cpu().numpy())
    assert r["converged"] == 1 and ro["converged"]
    assert abs(r["total_energy"] - ro["total_energy"]) < 1e-9
    assert abs(r["iterations"] - ro["iterations"]) <= 1


def test_uhf_and_rohf_sad_guess_match_oracle(built_library, cuda):
    atoms, gbs = _nh2(), "6-31g"
    mol, eng = _engine(atoms, gbs)
    Da, Db = eng.sad_density()
    opts = dict(CONV, initial_guess=gg.HF_GUESS_SAD, guess_density_a=Da, guess_density_b=Db)
    b = O.make_basis(atoms, gg.basis_path(gbs))
    S, T, V = O.one_electron(b)
    eri = O.eri_tensor(b)
    jk = lambda D: (np.einsum("ijkl,kl->ij", eri, D), np.einsum("ikjl,kl->ij", eri, D))
    g = (Da.cpu().numpy(), Db.cpu().numpy())
    enuc = O.nuclear_repulsion(atoms)
    ru = eng.uhf_scf(5, 4, opts)
    ou = O.uhf(S, T + V, jk, 5, 4, enuc, thr=1e-12, maxiter=300, guess="sad", guess_density=g)
    assert ru["converged"] == 1 and ou["converged"] and abs(ru["total_energy"] - ou["total_energy"]) < 1e-7
    rr = eng.rohf_scf(5, 4, opts)
    orr = O.rohf(S, T + V, jk, 5, 4, enuc, thr=1e-12, maxiter=300, guess="sad", guess_density=g)
    assert rr["converged"] == 1 and orr["converged"] and abs(rr["total_energy"] - orr["total_energy"]) < 1e-8


def test_sad_file_is_read_as_the_reference_does(built_library, cuda, tmp_path):
    """A <basis>.sad next to the basis file is used as it is (read_density_from_sad)."""
    gbs = tmp_path / "6-31g.gbs"
    shutil.copy(gg.basis_path("6-31g"), gbs)
    dens = {sad.SYMBOLS[z - 1]: sad.atomic_density(z, gg.basis_path("6-31g"), source="compute") for z in (1, 8)}
    # perturb the file's O density so that reading it is observable
    a, b = dens["O"]
    dens["O"] = (a * 1.01, b * 1.01)
    sad.write_sad(tmp_path / "6-31g.sad", dens)
    back = sad.read_sad(tmp_path / "6-31g.sad")
    np.testing.assert_allclose(back["O"][0], a * 1.01, rtol=1e-9)
    mol = gg.Molecular(geometry.water(), str(gbs))
    Fa, Fb = sad.sad_guess(mol, str(gbs), source="file")
    lo, cnt = sad.atom_basis_ranges(mol)[0]
    np.testing.assert_allclose(Fa[lo:lo + cnt, lo:lo + cnt], a * 1.01, rtol=1e-9)
    eng = gg.Engine(mol, 1e-12)
    r = eng.rhf_scf(10, dict(CONV, initial_guess=gg.HF_GUESS_SAD))
    rc = eng.rhf_scf(10, CONV)
    assert r["converged"] == 1 and abs(r["total_energy"] - rc["total_energy"]) < 1e-9


def test_builder_rohf_recipe_with_sad(built_library, cuda, tmp_path):
    xyz = tmp_path / "nh2.xyz"
    geometry.write_xyz(xyz, _nh2())
    pm = gg.ParameterManager()
    pm["xyzfilename"] = str(xyz)
    pm["gbsfilename"] = str(gg.basis_path("sto-3g"))
    pm["method"] = "rohf"
    pm["initial_guess"] = "sad"
    pm["convergence_energy_threshold"] = "1e-12"
    pm["maxiter"] = "300"
    hf = gg.HFBuilder.buildHF(pm)
    e = hf.solve()
    # the oracle from the same superposition: from SAD, NH2/STO-3G reaches a lower ROHF
    # state (-54.8345 Eh) than from the core guess (-54.7393 Eh)
    Da, Db = hf.engine.sad_density()
    b = O.make_basis(_nh2(), gg.basis_path("sto-3g"))
    S, T, V = O.one_electron(b)
    eri = O.eri_tensor(b)
    jk = lambda D: (np.einsum("ijkl,kl->ij", eri, D), np.einsum("ikjl,kl->ij", eri, D))
    ro = O.rohf(S, T + V, jk, 5, 4, O.nuclear_repulsion(b.atoms), thr=1e-12, maxiter=300, guess="sad",
                guess_density=(Da.cpu().numpy(), Db.cpu().numpy()))
    assert ro["converged"] and abs(e - ro["total_energy"]) < 1e-8
    assert abs(hf.get_total_spin() - 0.75) < 1e-15
    hf.export_sad_cache(str(tmp_path / "cache.dat"))
    assert (tmp_path / "cache.dat").read_text().split()[0] == str(hf.mol.num_basis)


def test_rhf_sad_guess_ri_and_mixed(built_library, cuda):
    """SAD with the RI backend (first K from the guess density itself) and with the
    anchored mixed tier reach the core-guess energies."""
    atoms = geometry.alkane(3, jitter=0.02, seed=3)
    mol, eng = _engine(atoms, "cc-pvdz")
    aux = gg.Molecular(atoms, gg.basis_path("cc-pvdz-rifit"))
    eng.set_auxiliary_basis(aux)
    ne = mol.num_electrons
    base = dict(CONV, convergence_threshold=1e-10)
    for extra in ({"eri_method": gg.HF_ERI_RI}, {"eri_method": gg.HF_ERI_RI, "precision": gg.HF_PRECISION_MIXED,
                                                  "anchor_threshold": 1e-2},
                  {"precision": gg.HF_PRECISION_MIXED, "anchor_threshold": 1e-2, "incremental": 1,
                   "mixed_threshold": 0.1}):
        rc = eng.rhf_scf(ne, dict(base, **extra))
        rs = eng.rhf_scf(ne, dict(base, initial_guess=gg.HF_GUESS_SAD, **extra))
        assert rc["converged"] == 1 and rs["converged"] == 1
        assert abs(rc["total_energy"] - rs["total_energy"]) < 1e-7


def test_batch_sad_guess_matches_single_molecules(built_library, cuda):
    clusters = geometry.water_cluster_set(6, nmax=4, seed=5)
    mols = [gg.Molecular(c, gg.basis_path("6-31g")) for c in clusters]
    batch = gg.Batch(mols)
    opts = {"convergence_threshold": 1e-10, "max_iter": 200, "initial_guess": gg.HF_GUESS_SAD}
    res, _, _ = batch.rhf_scf(opts)
    for m, r in zip(mols, res):
        eng = gg.Engine(m, 1e-12)
        ri = eng.rhf_scf(m.num_electrons, opts)
        assert r["converged"] == 1 and ri["converged"] == 1
        assert abs(r["total_energy"] - ri["total_energy"]) < 1e-8
        assert abs(r["iterations"] - ri["iterations"]) <= 1
    res_g, _, _ = batch.rhf_scf(dict(opts, initial_guess=gg.HF_GUESS_GWH))
    for r, rs in zip(res_g, res):
        assert r["converged"] == 1 and abs(r["total_energy"] - rs["total_energy"]) < 1e-8
