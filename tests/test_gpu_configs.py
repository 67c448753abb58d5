"""Parity at the configurations the headline metric is quoted on, through the C ABI.

  config 2  RHF/6-31G* n-decane (N = 194): the engine's FP64 SCF against the
            reference-integral golden energy (tests/golden/decane_6-31g_st.npz:
            the reference's own integral kernels on the CPU, the restated
            reference SCF loop, |dE| < 1e-10), to 1e-8 Eh and orbital energies to
            1e-6 Eh; the mixed tier (bench settings) to 1e-6 Eh and 1e-5 Eh; the
            engine's ERI tensor against the reference's on 4000 sampled elements
            and three checksums.
  config 3  RHF/cc-pVDZ n-decane (N = 260): analytic gradient, FP64 and mixed,
            against central finite differences (h = 1e-4 bohr) of FP64 energies on
            six coordinates (two carbons, two hydrogens), to 1e-5 Eh/bohr.
  config 4  RI-JK RHF/cc-pVDZ + cc-pVDZ-RIFIT C60 (N = 900, naux = 3960): mixed
            RI SCF within 1e-6 Eh of the FP64 RI SCF; B = L^-1 (mu nu|P) on
            sampled columns against the oracle (metric and three-centre
            integrals restated in oracle/md_oracle.c): the fitted integrals
            B_mu nu . B_la si = T V^-1 T to 1e-10 of |B_mu nu| |B_la si|, B
            itself to 1e-6 of its largest element (the metric's conditioning).
  config 5  batched RHF/6-31G on water clusters (H2O)n: a stratified 32 of the
            seeded 256 (two clusters for each n = 1..16), every mixed-batch
            energy within 1e-6 Eh of its own FP64 single-molecule SCF.
"""
from pathlib import Path

import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).parent / "golden"

# the bench's mixed-tier options (bench.py: MIXED_THRESHOLD, ANCHOR_THRESHOLD, ANCHOR_MIXED_THRESHOLD,
# INCREMENTAL_DROP)
MIXED = {"precision": gg.HF_PRECISION_MIXED, "mixed_threshold": 0.1, "incremental": 1, "rebuild_every": 0,
         "full_build_precision": gg.HF_PRECISION_FP64, "anchor_threshold": 1e-2, "anchor_mixed_threshold": 3e-2,
         "incremental_drop": 3e-10}


def _np(t):
    return t.cpu().numpy()


def test_config2_decane_631gs_against_reference_integrals(built_library, cuda):
    torch = cuda
    g = np.load(GOLDEN / "decane_6-31g_st.npz")
    atoms = geometry.alkane(10, jitter=0.02, seed=0)
    np.testing.assert_allclose(np.array(atoms), g["atoms"], atol=1e-12)
    mol = gg.Molecular(atoms, gg.basis_path("6-31g_st"))
    eng = gg.Engine(mol, 1e-12)
    assert mol.num_basis == 194
    # the ERI tensor (11.3 GB on the device) against the reference's own kernels
    eri = eng.eri_matrix()
    idx = torch.tensor(g["eri_idx"], device="cuda")
    vals = _np(eri[idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3]])
    np.testing.assert_allclose(vals, g["eri_val"], atol=1e-12, rtol=0)
    assert abs(float(eri.sum()) - float(g["eri_sum"])) < 1e-8 * abs(float(g["eri_sum"]))
    assert abs(float(eri.abs().sum()) - float(g["eri_abs_sum"])) < 1e-8 * float(g["eri_abs_sum"])
    assert abs(float((eri * eri).sum()) - float(g["eri_sq_sum"])) < 1e-8 * float(g["eri_sq_sum"])
    del eri
    torch.cuda.empty_cache()
    eps_ref = g["orbital_energies"]
    base = {"convergence_threshold": 1e-10}
    for eig in (gg.HF_EIGEN_SYEVD, gg.HF_EIGEN_PURIFICATION):
        r = eng.rhf_scf(mol.num_electrons, dict(base, eigensolver=eig), want_matrices=True)
        assert r["converged"] == 1
        assert abs(r["total_energy"] - float(g["energy_total"])) < 1e-8
        np.testing.assert_allclose(_np(r["orbital_energies"]), eps_ref, atol=1e-6)
        rm = eng.rhf_scf(mol.num_electrons, dict(base, eigensolver=eig, **MIXED), want_matrices=True)
        assert rm["converged"] == 1
        assert abs(rm["total_energy"] - float(g["energy_total"])) < 1e-6
        np.testing.assert_allclose(_np(rm["orbital_energies"]), eps_ref, atol=1e-5)
        assert rm["fp32_quartets"] > rm["fp64_quartets"]
    eng.close()


STEP = 1e-4  # bohr


def test_config3_decane_ccpvdz_gradient_finite_differences(built_library, cuda):
    atoms = geometry.alkane(10, jitter=0.02, seed=0)
    gbs = gg.basis_path("cc-pvdz")
    mol = gg.Molecular(atoms, gbs)
    eng = gg.Engine(mol, 1e-12)
    assert mol.num_basis == 260
    conv = {"convergence_threshold": 1e-11, "max_iter": 200}
    r = eng.rhf_scf(mol.num_electrons, conv, want_matrices=True)
    assert r["converged"] == 1
    W = eng.energy_weighted_density(r["coefficients"], r["orbital_energies"], mol.num_electrons // 2)
    g64, _ = eng.gradient(r["density"], W)
    g32, _ = eng.gradient(r["density"], W, mixed_threshold=1.0)  # the bench's gradient FP32 cut
    eng.close()
    carbons = [i for i, a in enumerate(atoms) if a[0] == 6]
    hydrogens = [i for i, a in enumerate(atoms) if a[0] == 1]
    coords = [(carbons[0], 0), (carbons[4], 2), (carbons[9], 1), (hydrogens[0], 1), (hydrogens[7], 0),
              (hydrogens[15], 2)]

    def energy(a):
        m = gg.Molecular(a, gbs)
        e = gg.Engine(m, 1e-12)
        res = e.rhf_scf(m.num_electrons, dict(conv, initial_guess=gg.HF_GUESS_DENSITY, guess_density_a=r["density"]))
        e.close()
        assert res["converged"] == 1
        return res["total_energy"]

    for atom, k in coords:
        plus = [list(x) for x in atoms]
        minus = [list(x) for x in atoms]
        plus[atom][1 + k] += STEP
        minus[atom][1 + k] -= STEP
        fd = (energy([tuple(x) for x in plus]) - energy([tuple(x) for x in minus])) / (2 * STEP)
        assert abs(g64[atom, k] - fd) < 1e-5, (atom, k, g64[atom, k], fd)
        assert abs(g32[atom, k] - fd) < 1e-5, (atom, k, g32[atom, k], fd)
    assert np.abs(g32 - g64).max() < 1e-5


def test_config4_c60_ri_mixed_vs_fp64_and_b_columns(built_library, cuda):
    torch = cuda
    atoms = geometry.c60(jitter=0.01, seed=0)
    mol = gg.Molecular(atoms, gg.basis_path("cc-pvdz"))
    aux = gg.Molecular(atoms, gg.basis_path("cc-pvdz-rifit"))
    assert mol.num_basis == 900 and aux.num_basis == 3960
    eng = gg.Engine(mol, 1e-12)
    eng.set_auxiliary_basis(aux)
    # B columns against the oracle: B_P,(mu nu) = (L^-1 T)_P for sampled (mu nu)
    B = eng.ri_intermediate_b()
    b = O.make_basis(atoms, gg.basis_path("cc-pvdz"))
    ax = O.make_basis(atoms, gg.basis_path("cc-pvdz-rifit"))
    L = np.linalg.cholesky(O.ri_metric(b, ax))
    rng = np.random.default_rng(4)
    pairs = [tuple(int(s) for s in rng.integers(0, b.nshell, 2)) for _ in range(6)] + [(0, 0), (3, 1)]
    cols = O.ri_three_center_pairs(b, ax, pairs)
    import scipy.linalg
    got, ref = {}, {}
    for (mu, nu), t in cols.items():
        ref[mu, nu] = scipy.linalg.solve_triangular(L, t, lower=True)
        got[mu, nu] = _np(B[:, mu, nu])
        if not np.any(t):  # a pair the Schwarz screen removes entirely: B column zero too
            assert not np.any(got[mu, nu]), (mu, nu)
            continue
        # forward error of B itself: two Cholesky factors of the same ill-conditioned metric
        # (cc-pVDZ-RIFIT on C60) differ along its small-eigenvalue directions
        assert np.abs(got[mu, nu] - ref[mu, nu]).max() <= 1e-6 * np.abs(ref[mu, nu]).max(), (mu, nu)
    # what J and K use: the fitted integrals (mu nu|la si)_RI = B_mu nu . B_la si = T V^-1 T
    keys = [k for k in cols if np.any(cols[k])]
    for k1 in keys:
        for k2 in keys:
            g_ = got[k1] @ got[k2]
            r_ = ref[k1] @ ref[k2]
            assert abs(g_ - r_) <= 1e-10 * np.linalg.norm(ref[k1]) * np.linalg.norm(ref[k2]), (k1, k2, g_, r_)
    del B
    torch.cuda.empty_cache()
    base = {"convergence_threshold": 1e-8, "eri_method": gg.HF_ERI_RI}
    rm = eng.rhf_scf(mol.num_electrons, dict(base, precision=gg.HF_PRECISION_MIXED, anchor_threshold=1e-2),
                     want_matrices=True)
    assert rm["converged"] == 1
    # FP64 RI SCF started from the mixed density: the same fixed point, fewer iterations
    r64 = eng.rhf_scf(mol.num_electrons, dict(base, initial_guess=gg.HF_GUESS_DENSITY,
                                              guess_density_a=rm["density"]), want_matrices=True)
    assert r64["converged"] == 1
    assert abs(rm["total_energy"] - r64["total_energy"]) < 1e-6
    np.testing.assert_allclose(_np(rm["orbital_energies"]), _np(r64["orbital_energies"]), atol=1e-5)
    eng.close()


def test_config5_water_cluster_batch_vs_single_fp64(built_library, cuda):
    clusters = geometry.water_cluster_set(256, 16, seed=0)
    by_n = {}
    for atoms in clusters:
        by_n.setdefault(len(atoms) // 3, []).append(atoms)
    picked = [c for n in sorted(by_n) for c in by_n[n][:2]]
    assert {len(c) // 3 for c in picked} == set(range(1, 17)) and len(picked) == 32
    gbs = gg.basis_path("6-31g")
    mols = [gg.Molecular(a, gbs) for a in picked]
    batch = gg.Batch(mols, 1e-12)
    # the bench's batch settings: SAD guess, purification, the mixed tier
    res, _, _ = batch.rhf_scf(dict(MIXED, convergence_threshold=1e-8, eigensolver=gg.HF_EIGEN_PURIFICATION,
                                   initial_guess=gg.HF_GUESS_SAD))
    batch.close()
    for m, rb in zip(mols, res):
        assert rb["converged"] == 1
        e = gg.Engine(m, 1e-12)
        r = e.rhf_scf(m.num_electrons, {"convergence_threshold": 1e-8, "initial_guess": gg.HF_GUESS_SAD})
        e.close()
        assert r["converged"] == 1
        assert abs(rb["total_energy"] - r["total_energy"]) < 1e-6, (m.num_basis, rb["total_energy"], r["total_energy"])
