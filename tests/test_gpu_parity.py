"""Parity of the CUDA path (through the C ABI) with the oracle and with the
reference's own integrals (golden fixtures from its kernels).

Tolerances (FP64 tier): integrals and Fock elements 1e-11 absolute (the
reference's own summation is order-nondeterministic at ~1e-15 relative);
SCF total energy 1e-8 Eh.  Mixed tier: Fock elements within 10x the mixed
threshold, SCF energy within 1e-6 Eh, orbital energies within 1e-5 Eh.
"""
from pathlib import Path

import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).parent / "golden"
CASES = ["water_sto-3g", "water_6-31g_st", "water_cc-pvdz", "propane_6-31g_st"]


def _case(case):
    g = np.load(GOLD / f"{case}.npz")
    gbs = case.split("_", 1)[1]
    atoms = [(int(a[0]), float(a[1]), float(a[2]), float(a[3])) for a in g["atoms"]]
    return g, atoms, gbs


def _engine(atoms, gbs, thr=1e-12):
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    return mol, gg.Engine(mol, thr)


def _np(t):
    return t.detach().cpu().numpy()


def _reference_bounds_dense(flat, shell_types):
    """Expand the reference's pair-class layout (src/gpu_manager.cu:413-432,
    index1to2 of include/utils_cuda.hpp:35-44) into a dense matrix."""
    st = np.asarray(shell_types)
    T = st.max() + 1
    start = [int(np.searchsorted(st, t)) for t in range(T)]
    count = [int((st == t).sum()) for t in range(T)]
    n = len(st)
    dense = np.full((n, n), np.nan)
    head = 0
    for s0 in range(T):
        for s1 in range(s0, T):
            if s0 == s1:
                m = count[s0] * (count[s0] + 1) // 2
                for i in range(m):
                    r2 = int((np.sqrt(8 * i + 1) - 1) // 2)
                    r1 = i - r2 * (r2 + 1) // 2
                    a, b = r1 + start[s0], r2 + start[s1]
                    dense[a, b] = dense[b, a] = flat[head + i]
            else:
                m = count[s0] * count[s1]
                for i in range(m):
                    a, b = i // count[s1] + start[s0], i % count[s1] + start[s1]
                    dense[a, b] = dense[b, a] = flat[head + i]
            head += m
    return dense


@pytest.mark.parametrize("case", CASES)
def test_core_hamiltonian_matches_reference(built_library, cuda, case):
    g, atoms, gbs = _case(case)
    _, eng = _engine(atoms, gbs)
    S, H = eng.core_hamiltonian()
    np.testing.assert_allclose(_np(S), g["S"], atol=1e-12, rtol=0)
    np.testing.assert_allclose(_np(H), g["H"], atol=1e-11, rtol=0)


@pytest.mark.parametrize("case", CASES)
def test_primitive_schwarz_bounds_match_reference(built_library, cuda, case):
    g, atoms, gbs = _case(case)
    mol, eng = _engine(atoms, gbs)
    got = eng.primitive_pair_bounds()
    ref = _reference_bounds_dense(g["bounds"], mol.primitive_table()["shell_type"])
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-300)


@pytest.mark.parametrize("case", CASES)
def test_eri_tensor_matches_reference(built_library, cuda, case):
    g, atoms, gbs = _case(case)
    _, eng = _engine(atoms, gbs)
    eri = _np(eng.eri_matrix())
    if "eri" in g:
        np.testing.assert_allclose(eri, g["eri"], atol=1e-12, rtol=0)
    else:
        idx = g["eri_idx"]
        np.testing.assert_allclose(eri[idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3]], g["eri_val"], atol=1e-12, rtol=0)
    assert abs(eri.sum() - float(g["eri_sum"])) < 1e-9 * max(1.0, abs(float(g["eri_sum"])))
    assert abs((eri * eri).sum() - float(g["eri_sq_sum"])) < 1e-9 * float(g["eri_sq_sum"])


def _random_density(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(n, n)) / np.sqrt(n)
    return A + A.T


@pytest.mark.parametrize("case", CASES)
def test_direct_fock_fp64_matches_oracle(built_library, cuda, case):
    g, atoms, gbs = _case(case)
    _, eng = _engine(atoms, gbs)
    b = O.make_basis(atoms, gg.basis_path(gbs))
    eri = O.eri_tensor(b, 1e-12)
    D = _random_density(b.nbf, 1)
    Jr = np.einsum("ijkl,kl->ij", eri, D)
    Kr = np.einsum("ikjl,kl->ij", eri, D)
    Dt = cuda.tensor(D, device="cuda")
    Ht = cuda.tensor(g["H"], device="cuda")
    J, K = eng.jk(Dt)
    np.testing.assert_allclose(_np(J), Jr, atol=1e-11, rtol=0)
    np.testing.assert_allclose(_np(K), Kr, atol=1e-11, rtol=0)
    F = eng.fock_direct(Dt, Ht)
    np.testing.assert_allclose(_np(F), g["H"] + Jr - 0.5 * Kr, atol=1e-11, rtol=0)
    # stored path through the C ABI gives the same Fock matrix
    Fs = eng.fock_stored(Dt, Ht, eng.eri_matrix())
    np.testing.assert_allclose(_np(Fs), _np(F), atol=1e-11, rtol=0)


@pytest.mark.parametrize("case", CASES)
def test_direct_fock_mixed_close_to_fp64(built_library, cuda, case):
    g, atoms, gbs = _case(case)
    _, eng = _engine(atoms, gbs)
    D = cuda.tensor(_random_density(g["S"].shape[0], 2), device="cuda")
    H = cuda.tensor(g["H"], device="cuda")
    F64 = _np(eng.fock_direct(D, H))
    thr = 1e-7
    Fmx = _np(eng.fock_direct(D, H, precision=gg.HF_PRECISION_MIXED, mixed_threshold=thr))
    err = np.abs(Fmx - F64).max()
    # every FP32 quartet contributes at most ~thr * 1e-6 relative error; bound generously
    assert err < 1e-6, err
    # threshold 0 keeps every quartet in FP64: identical up to summation order
    F0 = _np(eng.fock_direct(D, H, precision=gg.HF_PRECISION_MIXED, mixed_threshold=0.0))
    np.testing.assert_allclose(F0, F64, atol=1e-11, rtol=0)


def test_direct_fock_decane_matches_oracle(built_library, cuda):
    atoms = geometry.alkane(10, jitter=0.02, seed=0)
    mol, eng = _engine(atoms, "6-31g_st")
    b = O.make_basis(atoms, gg.basis_path("6-31g_st"))
    S, T, V = O.one_electron(b)
    X = O.transform_matrix(S)
    _, Cm = O.coefficients(T + V, X)
    D = O.density(Cm, b.num_electrons // 2)  # core-guess density: a physical D
    J, K, _ = O.direct_jk(b, D, 1e-12)
    Jg, Kg = eng.jk(cuda.tensor(D, device="cuda"))
    np.testing.assert_allclose(_np(Jg), J, atol=1e-10, rtol=0)
    np.testing.assert_allclose(_np(Kg), K, atol=1e-10, rtol=0)


@pytest.mark.parametrize("case", ["water_sto-3g", "water_6-31g_st", "propane_6-31g_st"])
def test_scf_energy_matches_reference(built_library, cuda, case):
    g, atoms, gbs = _case(case)
    _, eng = _engine(atoms, gbs)
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    r = eng.rhf_scf(mol.num_electrons, {"convergence_threshold": 1e-10}, want_matrices=True)
    assert r["converged"] == 1
    assert abs(r["total_energy"] - float(g["energy_total"])) < 1e-8
    np.testing.assert_allclose(_np(r["orbital_energies"]), g["orbital_energies"], atol=1e-6)


@pytest.mark.parametrize("incremental", [0, 1])
def test_scf_mixed_within_tolerance(built_library, cuda, incremental):
    g, atoms, gbs = _case("propane_6-31g_st")
    mol, eng = _engine(atoms, gbs)
    r64 = eng.rhf_scf(mol.num_electrons, {"convergence_threshold": 1e-10}, want_matrices=True)
    # incremental: FP64 first build, then dD builds under the mixed rule; otherwise
    # every (full) build under the mixed rule
    rmx = eng.rhf_scf(mol.num_electrons, {"convergence_threshold": 1e-10, "precision": gg.HF_PRECISION_MIXED,
                                          "mixed_threshold": 1e-7 if not incremental else 1e-2,
                                          "incremental": incremental,
                                          "full_build_precision": gg.HF_PRECISION_MIXED if not incremental
                                          else gg.HF_PRECISION_FP64},
                      want_matrices=True)
    assert rmx["converged"] == 1
    assert abs(rmx["total_energy"] - r64["total_energy"]) < 1e-6
    np.testing.assert_allclose(_np(rmx["orbital_energies"]), _np(r64["orbital_energies"]), atol=1e-5)
    assert rmx["fp32_quartets"] > 0


def test_diis_entry_points_match_numpy(built_library, cuda):
    g, atoms, gbs = _case("water_6-31g_st")
    _, eng = _engine(atoms, gbs)
    n = g["S"].shape[0]
    rng = np.random.default_rng(5)
    sym = lambda: (lambda a: a + a.T)(rng.normal(size=(n, n)))
    S, F, D = g["S"], sym(), sym()
    X = O.transform_matrix(S)
    t = lambda a: cuda.tensor(np.ascontiguousarray(a), device="cuda")
    E = _np(eng.diis_error(t(S), t(X), t(F), t(D)))
    np.testing.assert_allclose(E, F @ D @ S - S @ D @ F, atol=1e-10)
    Ex = _np(eng.diis_error(t(S), t(X), t(F), t(D), include_transform=True))
    np.testing.assert_allclose(Ex, X @ (F @ D @ S - S @ D @ F) @ X.T, atol=1e-10)
    errs = np.stack([rng.normal(size=(n, n)) for _ in range(5)])
    focks = np.stack([sym() for _ in range(5)])
    Fn = _np(eng.fock_diis(t(errs), t(focks)))
    np.testing.assert_allclose(Fn, O.diis_extrapolate(list(errs), list(focks)), atol=1e-9)


def test_diis_dependent_error_vectors(built_library, cuda):
    """Error vectors that repeat others: the reference's LU (src/gpu_manager.cu:1078-1194)
    has no answer for a singular B; here the repeated vector gets weight 0 and the
    extrapolation is the one over the distinct vectors (never the zero matrix)."""
    g, atoms, gbs = _case("water_6-31g_st")
    _, eng = _engine(atoms, gbs)
    n = g["S"].shape[0]
    rng = np.random.default_rng(9)
    sym = lambda: (lambda a: a + a.T)(rng.normal(size=(n, n)))
    t = lambda a: cuda.tensor(np.ascontiguousarray(a), device="cuda")
    e = [rng.normal(size=(n, n)) for _ in range(3)]
    f = [sym() for _ in range(4)]
    # e0 twice (slots 0 and 2): the later copy is left out
    errs = np.stack([e[0], e[1], e[0], e[2]])
    Fn = _np(eng.fock_diis(t(errs), t(np.stack(f))))
    np.testing.assert_allclose(Fn, O.diis_extrapolate([e[0], e[1], e[2]], [f[0], f[1], f[3]]), atol=1e-9)
    # two equal vectors only: the first one's Fock matrix
    Fn = _np(eng.fock_diis(t(np.stack([e[1], e[1]])), t(np.stack(f[:2]))))
    np.testing.assert_allclose(Fn, f[0], atol=1e-12)
    # a zero error vector: that Fock matrix is self-consistent and is returned
    Fn = _np(eng.fock_diis(t(np.stack([e[1], 0.0 * e[1], e[2]])), t(np.stack(f[:3]))))
    np.testing.assert_allclose(Fn, f[1], atol=1e-12)


def test_builder_recipe_end_to_end(built_library, cuda, tmp_path):
    xyz = tmp_path / "h2o.xyz"
    geometry.write_xyz(xyz, geometry.water())
    rec = tmp_path / "RHF_direct.txt"
    rec.write_text(f"xyzfilename = {xyz}\ngbsfilename = {gg.basis_path('sto-3g')}\nmethod = RHF\n"
                   "eri_method = direct\nconvergence_method = DIIS\ndiis_size = 8\nconvergence_energy_threshold = 1e-10\n")
    pm = gg.ParameterManager()
    pm.parse_command_line_args(["-p", str(rec)])
    hf = gg.HFBuilder.buildHF(pm)
    e = hf.solve()
    g = np.load(GOLD / "water_sto-3g.npz")
    assert abs(e - float(g["energy_total"])) < 1e-8


def test_edge_cases(built_library, cuda):
    # H2: s shells only, 2 basis functions
    mol, eng = _engine([(1, 0.0, 0.0, 0.0), (1, 0.0, 0.0, 1.4)], "sto-3g")
    r = eng.rhf_scf(2, {"convergence_threshold": 1e-10})
    b = O.make_basis([(1, 0.0, 0.0, 0.0), (1, 0.0, 0.0, 1.4)], gg.basis_path("sto-3g"))
    ref = O.rhf_from_basis(b, thr=1e-10)
    assert abs(r["total_energy"] - ref["total_energy"]) < 1e-9
    assert abs(r["total_energy"] - (-1.1167)) < 1e-3  # textbook STO-3G H2 at 1.4 bohr
    # odd electron count is rejected for RHF with an error status, not a crash
    _, eng1 = _engine([(1, 0.0, 0.0, 0.0)], "sto-3g")
    with pytest.raises(gg.HFError):
        eng1.rhf_scf(1)
    # two far-apart waters: inter-fragment quartets screened; Fock still exact
    far = geometry.water() + [(z, x + 60.0, y, w) for z, x, y, w in geometry.water()]
    _, engf = _engine(far, "sto-3g")
    bf = O.make_basis(far, gg.basis_path("sto-3g"))
    D = _random_density(bf.nbf, 9)
    eri = O.eri_tensor(bf, 1e-12)
    J, K = engf.jk(cuda.tensor(D, device="cuda"))
    np.testing.assert_allclose(_np(J), np.einsum("ijkl,kl->ij", eri, D), atol=1e-11)
    np.testing.assert_allclose(_np(K), np.einsum("ikjl,kl->ij", eri, D), atol=1e-11)
    assert engf.stats()["num_quartets"] < eng.stats()["num_quartets"] * 10 ** 6


@pytest.mark.parametrize("anchor,tau", [(1e-2, 0.1), (1e-1, 1.0)])
def test_scf_mixed_anchored_decane(built_library, cuda, anchor, tau):
    # all-FP32 full builds while max|dD| >= anchor, one FP64 build, then FP32-tier dD builds.
    # Converged to |dE| < 1e-10: at 1e-8 the virtual orbital energies of two SCFs that stop
    # at different iterations already differ by ~1e-5 in FP64 alone.
    atoms = geometry.alkane(10, jitter=0.02, seed=0)
    mol, eng = _engine(atoms, "6-31g_st")
    r64 = eng.rhf_scf(mol.num_electrons, {"convergence_threshold": 1e-10}, want_matrices=True)
    rmx = eng.rhf_scf(mol.num_electrons, {"convergence_threshold": 1e-10, "precision": gg.HF_PRECISION_MIXED,
                                          "mixed_threshold": tau, "incremental": 1, "anchor_threshold": anchor},
                      want_matrices=True)
    assert rmx["converged"] == 1
    assert abs(rmx["total_energy"] - r64["total_energy"]) < 1e-6
    np.testing.assert_allclose(_np(rmx["orbital_energies"]), _np(r64["orbital_energies"]), atol=1e-5)
    # exactly one full FP64 build's worth of FP64 quartets: the anchor
    assert rmx["fp64_quartets"] <= r64["fp64_quartets"] / (r64["iterations"] + 1) * 1.5


def test_gwh_guess_matches_oracle(built_library, cuda):
    g, atoms, gbs = _case("water_6-31g_st")
    mol, eng = _engine(atoms, gbs)
    r = eng.rhf_scf(mol.num_electrons, {"convergence_threshold": 1e-10, "initial_guess": gg.HF_GUESS_GWH})
    b = O.make_basis(atoms, gg.basis_path(gbs))
    ro = O.rhf_from_basis(b, thr=1e-10, guess="gwh")
    assert r["converged"] == 1 and ro["converged"]
    assert abs(r["total_energy"] - ro["total_energy"]) < 1e-8
    assert r["iterations"] == ro["iterations"]
    assert abs(r["total_energy"] - float(g["energy_total"])) < 1e-8


def test_purification_density_matches_diagonalisation(built_library, cuda):
    # FP32 SP2 + FP64 McWeeny inside the loop: same energies and iterations as syevd
    atoms = geometry.alkane(10, jitter=0.02, seed=0)
    mol, eng = _engine(atoms, "6-31g_st")
    base = {"convergence_threshold": 1e-9}
    rd = eng.rhf_scf(mol.num_electrons, base, want_matrices=True)
    rp = eng.rhf_scf(mol.num_electrons, dict(base, eigensolver=gg.HF_EIGEN_PURIFICATION), want_matrices=True)
    assert rp["converged"] == 1
    assert abs(rp["total_energy"] - rd["total_energy"]) < 1e-9
    assert abs(rp["iterations"] - rd["iterations"]) <= 1
    # two runs stopped by |dE| < 1e-9 at different points: densities agree to ~sqrt(1e-9)
    np.testing.assert_allclose(_np(rp["density"]), _np(rd["density"]), atol=1e-5)
    np.testing.assert_allclose(_np(rp["orbital_energies"]), _np(rd["orbital_energies"]), atol=1e-5)
    rm = eng.rhf_scf(mol.num_electrons, dict(base, eigensolver=gg.HF_EIGEN_PURIFICATION, precision=gg.HF_PRECISION_MIXED,
                                             mixed_threshold=0.1, incremental=1, anchor_threshold=1e-2))
    assert rm["converged"] == 1 and abs(rm["total_energy"] - rd["total_energy"]) < 1e-6
