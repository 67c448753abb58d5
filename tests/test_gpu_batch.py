"""Batched RHF (hf_engine_create_batch + hf_batch_rhf_scf) against one engine
and one SCF per molecule: every molecule's energy within 1e-8 Eh (the same FP64
arithmetic; only atomic summation orders differ) and the batch converges."""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry

pytestmark = pytest.mark.gpu
CONV = {"convergence_threshold": 1e-9}


def _individual(atoms, gbs):
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    eng = gg.Engine(mol, 1e-12)
    r = eng.rhf_scf(mol.num_electrons, CONV)
    assert r["converged"] == 1
    return r["total_energy"]


def test_batch_matches_individual_runs(built_library, cuda):
    clusters = geometry.water_cluster_set(10, nmax=4, seed=5)
    mols = [gg.Molecular(c, gg.basis_path("6-31g")) for c in clusters]
    batch = gg.Batch(mols)
    res, ms, it = batch.rhf_scf(CONV)
    assert ms > 0 and it > 0
    for c, r in zip(clusters, res):
        assert r["converged"] == 1
        assert abs(r["total_energy"] - _individual(c, "6-31g")) < 1e-8


def test_batch_of_one_and_mixed_basis(built_library, cuda):
    atoms = geometry.water()
    res, _, _ = gg.Batch([gg.Molecular(atoms, gg.basis_path("sto-3g"))]).rhf_scf(CONV)
    assert abs(res[0]["total_energy"] - _individual(atoms, "sto-3g")) < 1e-9
    # different basis sets and sizes in one batch, given out of order
    mols = [gg.Molecular(geometry.alkane(3, seed=2), gg.basis_path("6-31g_st")),
            gg.Molecular(atoms, gg.basis_path("sto-3g")),
            gg.Molecular(atoms, gg.basis_path("6-31g_st"))]
    res, _, _ = gg.Batch(mols).rhf_scf(CONV)
    assert abs(res[0]["total_energy"] - _individual(geometry.alkane(3, seed=2), "6-31g_st")) < 1e-8
    assert abs(res[1]["total_energy"] - _individual(atoms, "sto-3g")) < 1e-8
    assert abs(res[2]["total_energy"] - _individual(atoms, "6-31g_st")) < 1e-8


def test_batch_engine_rejects_single_molecule_entry_points(built_library, cuda):
    mols = [gg.Molecular(geometry.water(), gg.basis_path("sto-3g")) for _ in range(2)]
    b = gg.Batch(mols)
    import ctypes as C
    from dft_gansu_gb300._capi import ScfResult, lib
    r = ScfResult()
    assert lib().hf_rhf_scf(b._h, 10, None, C.byref(r), None, None, None, None) == 1


def test_batch_purification_matches_diagonalisation(built_library, cuda):
    clusters = geometry.water_cluster_set(8, nmax=4, seed=9)
    mols = [gg.Molecular(c, gg.basis_path("6-31g")) for c in clusters]
    batch = gg.Batch(mols)
    rd, _, _ = batch.rhf_scf(CONV)
    rp, _, _ = batch.rhf_scf(dict(CONV, eigensolver=gg.HF_EIGEN_PURIFICATION))
    for a, b in zip(rd, rp):
        assert a["converged"] == 1 and b["converged"] == 1
        assert abs(a["total_energy"] - b["total_energy"]) < 1e-8


def test_batch_mixed_tier_matches_single_molecule_rule(built_library, cuda):
    """The batch's mixed tier (per molecule: FP32 full builds until max|dD| < anchor,
    one FP64 anchor, then incremental builds with the FP32 cut) against the
    single-molecule mixed SCF with the same options (1e-7 Eh) and FP64 (1e-6 Eh)."""
    clusters = geometry.water_cluster_set(12, nmax=8, seed=3)
    mols = [gg.Molecular(c, gg.basis_path("6-31g")) for c in clusters]
    batch = gg.Batch(mols)
    mixed = {"convergence_threshold": 1e-9, "max_iter": 200, "precision": gg.HF_PRECISION_MIXED,
             "mixed_threshold": 0.1, "incremental": 1, "anchor_threshold": 1e-2,
             "initial_guess": gg.HF_GUESS_SAD}
    rm, _, _ = batch.rhf_scf(mixed)
    r64, _, _ = batch.rhf_scf({k: v for k, v in mixed.items() if k not in ("precision",)})
    for m, a, b in zip(mols, rm, r64):
        assert a["converged"] == 1 and b["converged"] == 1
        assert abs(a["total_energy"] - b["total_energy"]) < 1e-6
        eng = gg.Engine(m, 1e-12)
        single = eng.rhf_scf(m.num_electrons, mixed)
        assert single["converged"] == 1 and abs(a["total_energy"] - single["total_energy"]) < 1e-7
        eng.close()


@pytest.mark.parametrize("precision", [gg.HF_PRECISION_FP64, gg.HF_PRECISION_MIXED])
def test_batch_steps_replayed_from_graphs(built_library, cuda, precision):
    """Under use_graph the batch iteration's purified density step and its Fock build
    are captured once and replayed every later iteration; the energies equal those
    of ordinary launches (only atomic summation orders differ)."""
    clusters = geometry.water_cluster_set(8, nmax=4, seed=11)
    mols = [gg.Molecular(c, gg.basis_path("6-31g")) for c in clusters]
    batch = gg.Batch(mols)
    opts = dict(CONV, eigensolver=gg.HF_EIGEN_PURIFICATION, initial_guess=gg.HF_GUESS_SAD, precision=precision)
    if precision == gg.HF_PRECISION_MIXED:
        opts.update(mixed_threshold=0.1, incremental=1, anchor_threshold=1e-2)
    ref, _, _ = batch.rhf_scf(opts)
    batch.set_fock_schedule(2, use_graph=True)
    before = batch.graph_stats()["replays"]
    res, _, iters = batch.rhf_scf(opts)
    replays = batch.graph_stats()["replays"] - before
    # iterations + 1 passes: the first runs ordinary launches, the second captures and replays
    assert iters >= 3 and replays >= 2 * (iters - 1)
    for a, b in zip(ref, res):
        assert a["converged"] == 1 and b["converged"] == 1
        assert abs(a["total_energy"] - b["total_energy"]) < 1e-8
