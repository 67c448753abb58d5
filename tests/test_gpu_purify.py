"""RHF density by purification (HF_EIGEN_PURIFICATION), through the C ABI.

The reference diagonalises F' every iteration (computeCoefficientMatrix,
src/gpu_manager.cu:529-599); purification must give the same aufbau density
whenever the HOMO-LUMO gap is open.  Tolerances: SCF energies within 1e-9 Eh of
the syevd SCF (convergence threshold 1e-10 on |dE|), orbital energies within
1e-5 Eh (the energy is stationary, so |dE| < 1e-10 leaves the density, and the
orbital energies of two SCFs that stop at different iterations, ~1e-5 apart).
Sizes: N <= 512 runs the fused single-launch purification (csrc/purify.cu),
larger N the SP2/McWeeny library calls; both check the purified projector
(trace = nocc to 1e-6, idempotency to 1e-8) and a failed check reruns the SCF
with syevd (hf_scf_result.eigensolver_used).
"""
import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry

pytestmark = pytest.mark.gpu

BASE = {"convergence_threshold": 1e-10}


def _pair(atoms, gbs, **extra):
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    eng = gg.Engine(mol, 1e-12)
    rd = eng.rhf_scf(mol.num_electrons, dict(BASE, **extra), want_matrices=True)
    rp = eng.rhf_scf(mol.num_electrons, dict(BASE, eigensolver=gg.HF_EIGEN_PURIFICATION, **extra),
                     want_matrices=True)
    return mol, eng, rd, rp


@pytest.mark.parametrize("name,atoms,gbs", [
    ("water sto-3g (N=7)", geometry.water(), "sto-3g"),
    ("water 6-31G* (N=19)", geometry.water(), "6-31g_st"),
    ("propane 6-31G* (N=61)", geometry.alkane(3, jitter=0.02, seed=7), "6-31g_st"),
    ("pentane cc-pVDZ (N=130)", geometry.alkane(5, jitter=0.02, seed=2), "cc-pvdz"),
])
def test_fused_purification_matches_diagonalisation(built_library, cuda, name, atoms, gbs):
    mol, eng, rd, rp = _pair(atoms, gbs)
    assert rd["converged"] == 1 and rp["converged"] == 1
    assert rp["eigensolver_used"] == gg.HF_EIGEN_PURIFICATION
    assert abs(rp["total_energy"] - rd["total_energy"]) < 1e-9
    np.testing.assert_allclose(rp["orbital_energies"].cpu().numpy(), rd["orbital_energies"].cpu().numpy(), atol=1e-5)
    eng.close()


def test_unconverged_projector_reruns_with_diagonalisation(built_library, cuda):
    """Two SP2 steps cannot reach the projector: the trace/idempotency check rejects
    it and the SCF reruns with syevd, so the result is the syevd SCF's."""
    mol, eng, rd, rp = _pair(geometry.water(), "6-31g_st", purification_max_steps=2)
    assert rd["eigensolver_used"] == gg.HF_EIGEN_SYEVD
    assert rp["eigensolver_used"] == gg.HF_EIGEN_SYEVD
    assert rp["converged"] == 1
    assert abs(rp["total_energy"] - rd["total_energy"]) < 1e-10
    eng.close()


def test_degenerate_homo(built_library, cuda):
    """Closed-shell carbon atom: three degenerate 2p levels hold one electron pair
    (HOMO = LUMO in the core guess).  Whichever way the degeneracy is broken (FP32
    rounding in SP2, or a rejected projector and syevd), the SCF reaches the energy
    of the syevd SCF: every choice of the occupied p direction is equivalent."""
    mol, eng, rd, rp = _pair([(6, 0.0, 0.0, 0.0)], "6-31g")
    assert rp["converged"] == rd["converged"] == 1
    assert abs(rp["total_energy"] - rd["total_energy"]) < 1e-8
    eng.close()


def _h2_lattice(count=52, spacing=6.0, bond=0.74):
    atoms = []
    for k in range(count):
        x, y, z = k % 4, (k // 4) % 4, k // 16
        atoms.append((1, x * spacing, y * spacing, z * spacing))
        atoms.append((1, x * spacing, y * spacing, z * spacing + bond))
    return atoms


def test_library_purification_above_fused_size(built_library, cuda):
    """N = 520 (52 H2 in cc-pVDZ): SP2 as cuBLAS SGEMMs and McWeeny as DGEMMs, checked
    the same way; under the graph schedule the purification is captured and replayed.
    SAD guess: the core Hamiltonian of the lattice (no electron screening) mixes the
    bonding and antibonding bands and leaves no gap for the fixed 50 SP2 steps."""
    mol, eng, rd, rp = _pair(_h2_lattice(), "cc-pvdz", initial_guess=gg.HF_GUESS_SAD)
    assert mol.num_basis == 520
    assert rd["converged"] == 1 and rp["converged"] == 1
    assert rp["eigensolver_used"] == gg.HF_EIGEN_PURIFICATION
    assert abs(rp["total_energy"] - rd["total_energy"]) < 1e-9
    eng.set_fock_schedule(2, use_graph=True)
    for _ in range(2):
        rg = eng.rhf_scf(mol.num_electrons, dict(BASE, eigensolver=gg.HF_EIGEN_PURIFICATION,
                                                 initial_guess=gg.HF_GUESS_SAD))
        assert rg["converged"] == 1 and abs(rg["total_energy"] - rd["total_energy"]) < 1e-9
    assert eng.graph_stats()["purification_graphs"] >= 1
    eng.close()
