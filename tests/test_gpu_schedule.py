"""Launch schedule of the direct Fock build: quartet-class launches on
concurrent branches, builds replayed from CUDA graphs, and the autotuner that
chooses grid caps and the branch count (hf_engine_set_fock_schedule,
hf_engine_autotune, hf_engine_fock_schedule), all through the C ABI.

A schedule reorders the same launches, so its results equal the default
schedule's up to the order of the atomic sums: Fock and J/K elements within
1e-11 absolute in FP64, 1e-9 in the mixed tier (FP32 accumulators), SCF
energies within 1e-8 Eh (convergence threshold 1e-10).
"""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry

pytestmark = pytest.mark.gpu


def _setup(torch, seed=3):
    mol = gg.Molecular(geometry.alkane(3, jitter=0.02, seed=1), gg.basis_path("6-31g_st"))
    eng = gg.Engine(mol, 1e-12)
    n = mol.num_basis
    a = np.random.default_rng(seed).standard_normal((n, n)) * 0.1
    D = torch.tensor(a + a.T, dtype=torch.float64, device="cuda")
    H = torch.zeros(n, n, dtype=torch.float64, device="cuda")
    return mol, eng, D, H


def _maxdiff(a, b):
    return float((a - b).abs().max())


def test_branches_and_graph_replay_match_default(built_library, cuda):
    torch = cuda
    mol, eng, D, H = _setup(torch)
    F_ref = eng.fock_direct(D, H).clone()
    J_ref, K_ref = eng.jk(D)
    Fm_ref = eng.fock_direct(D, H, precision=gg.HF_PRECISION_MIXED, mixed_threshold=1e-7).clone()

    # branches without graphs
    eng.set_fock_schedule(3, use_graph=False)
    F = torch.empty_like(D)
    l0 = gg.kernel_launch_count()
    eng.fock_direct(D, H, out=F)
    eager_launches = gg.kernel_launch_count() - l0
    torch.cuda.synchronize()
    assert _maxdiff(F, F_ref) < 1e-11

    # graphs: the first call runs eagerly, the second captures and replays, later ones replay
    eng.set_fock_schedule(3, use_graph=True)
    for _ in range(4):
        F.zero_()
        l0 = gg.kernel_launch_count()
        eng.fock_direct(D, H, out=F)
        last = gg.kernel_launch_count() - l0
        torch.cuda.synchronize()
        assert _maxdiff(F, F_ref) < 1e-11
    assert last == eager_launches  # a replay counts the kernels of its graph

    # the graph reads the density at replay: G is linear in D (H = 0)
    D.mul_(0.5)
    eng.fock_direct(D, H, out=F)
    torch.cuda.synchronize()
    assert _maxdiff(F, 0.5 * F_ref) < 1e-11
    D.mul_(2.0)

    J, K = eng.jk(D)
    assert _maxdiff(J, J_ref) < 1e-11 and _maxdiff(K, K_ref) < 1e-11
    Fm = torch.empty_like(D)
    for _ in range(3):
        eng.fock_direct(D, H, precision=gg.HF_PRECISION_MIXED, mixed_threshold=1e-7, out=Fm)
        torch.cuda.synchronize()
        assert _maxdiff(Fm, Fm_ref) < 1e-9
    eng.close()


def test_schedule_rejects_bad_branch_count(built_library, cuda):
    mol, eng, D, H = _setup(cuda)
    for nb in (0, 9):
        with pytest.raises(gg.HFError):
            eng.set_fock_schedule(nb)
    eng.close()


def test_autotune_then_scf(built_library, cuda):
    torch = cuda
    mol, eng, D, H = _setup(torch, seed=5)
    nel = mol.num_electrons
    F_ref = eng.fock_direct(D, H).clone()
    opts = {"convergence_threshold": 1e-10, "precision": gg.HF_PRECISION_MIXED, "mixed_threshold": 0.1,
            "incremental": 1, "rebuild_every": 0, "full_build_precision": gg.HF_PRECISION_FP64,
            "anchor_threshold": 1e-2}
    e_mixed = eng.rhf_scf(nel, opts)["total_energy"]
    e_fp64 = eng.rhf_scf(nel, {"convergence_threshold": 1e-10})["total_energy"]

    rep = eng.autotune(D)
    assert rep["build_ms_default"] > 0 and rep["build_ms_tuned"] > 0
    assert rep["num_branches"] in (1, 2, 4, 8)
    k = len(rep["cap_fp64"])
    assert 0 < rep["num_class_pairs"] <= k
    assert all(c in (2, 4, 8, 16, 32) for c in rep["cap_fp64"] + rep["cap_fp32"])
    assert all(0 <= b < rep["num_branches"] for b in rep["branch"])
    assert all(c["prim_fp64"] == 0 and c["prim_fp32"] == 0 for c in eng.class_stats())  # reset by the tuning
    F = eng.fock_direct(D, H)
    torch.cuda.synchronize()
    assert _maxdiff(F, F_ref) < 1e-11

    eng.set_fock_schedule(rep["num_branches"], use_graph=True)
    assert eng.fock_schedule()["cap_fp64"] == rep["cap_fp64"]  # the caps stay with the engine
    for _ in range(2):
        r_mixed = eng.rhf_scf(nel, opts)
        r_fp64 = eng.rhf_scf(nel, {"convergence_threshold": 1e-10})
        assert r_mixed["converged"] and r_fp64["converged"]
        assert abs(r_mixed["total_energy"] - e_mixed) < 1e-8
        assert abs(r_fp64["total_energy"] - e_fp64) < 1e-8
    eng.close()


def test_grid_caps_transfer_and_gradient_branches(built_library, cuda):
    torch = cuda
    mol, eng, D, H = _setup(torch, seed=7)
    nel = mol.num_electrons
    r = eng.rhf_scf(nel, {"convergence_threshold": 1e-10}, want_matrices=True)
    W = eng.energy_weighted_density(r["coefficients"], r["orbital_energies"], nel // 2)
    g_ref, _ = eng.gradient(r["density"], W)
    F_ref = eng.fock_direct(D, H).clone()
    tune = eng.autotune(r["density"])

    # another engine over the same molecule takes the tuned schedule without timing
    eng2 = gg.Engine(mol, 1e-12)
    eng2.set_fock_schedule(tune["num_branches"], use_graph=True, grid_caps=tune)
    assert eng2.fock_schedule() == {k: tune[k] for k in ("cap_fp64", "cap_fp32", "branch")}
    for _ in range(3):
        F2 = eng2.fock_direct(D, H)
        torch.cuda.synchronize()
        assert _maxdiff(F2, F_ref) < 1e-11
    eng2.close()

    # the gradient's class launches on the branches of the schedule
    for nb in (tune["num_branches"], 4):
        eng.set_fock_schedule(nb)
        g, _ = eng.gradient(r["density"], W)
        assert np.abs(g - g_ref).max() < 1e-10

    eng.set_fock_schedule(1, grid_caps="default")
    assert set(eng.fock_schedule()["cap_fp64"]) == {16} and set(eng.fock_schedule()["cap_fp32"]) == {16}
    with pytest.raises(gg.HFError):  # a schedule of another class-pair count
        eng.set_fock_schedule(1, grid_caps={"cap_fp64": [16], "cap_fp32": [16], "branch": [0]})
    with pytest.raises(gg.HFError):  # caps outside 1..64
        k = len(tune["cap_fp64"])
        eng.set_fock_schedule(1, grid_caps={"cap_fp64": [0] * k, "cap_fp32": [16] * k, "branch": [0] * k})
    eng.close()


def test_batch_schedule_matches_default(built_library, cuda):
    clusters = geometry.water_cluster_set(6, nmax=3, seed=2)
    b = gg.Batch([gg.Molecular(c, gg.basis_path("6-31g")) for c in clusters])
    opts = {"convergence_threshold": 1e-10}
    ref, _, _ = b.rhf_scf(opts)
    tune = b.autotune()
    assert tune["num_branches"] in (1, 2, 4, 8)
    b.set_fock_schedule(max(2, tune["num_branches"]), grid_caps=tune)
    res, _, _ = b.rhf_scf(opts)
    assert all(r["converged"] for r in res)
    for a, c in zip(ref, res):
        assert abs(a["total_energy"] - c["total_energy"]) < 1e-8
    b.close()


def test_purification_under_graph_schedule(built_library, cuda):
    """The RHF loop's purification density (HF_EIGEN_PURIFICATION) under the graph
    schedule: at this size (N <= 512) the purification is one cooperative launch and
    needs no graph; the Fock builds are captured once and replayed; same energies.
    (The library-call purification above N = 512 and its graph: test_gpu_purify.py.)"""
    torch = cuda
    mol, eng, D, H = _setup(torch, seed=11)
    nel = mol.num_electrons
    opts = {"convergence_threshold": 1e-10, "eigensolver": gg.HF_EIGEN_PURIFICATION}
    mixed = dict(opts, precision=gg.HF_PRECISION_MIXED, mixed_threshold=0.1, incremental=1, rebuild_every=0,
                 full_build_precision=gg.HF_PRECISION_FP64, anchor_threshold=1e-2)
    ref = [eng.rhf_scf(nel, o) for o in (opts, mixed)]
    assert eng.graph_stats() == {"fock_graphs": 0, "purification_graphs": 0, "replays": 0}
    eng.set_fock_schedule(2, use_graph=True)
    for _ in range(2):
        got = [eng.rhf_scf(nel, o) for o in (opts, mixed)]
        for a, b in zip(ref, got):
            assert b["converged"] and abs(a["total_energy"] - b["total_energy"]) < 1e-8
    st = eng.graph_stats()
    assert st["purification_graphs"] == 0 and st["fock_graphs"] >= 1
    assert st["replays"] > 2 * ref[0]["iterations"]
    eng.close()
