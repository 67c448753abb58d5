"""Generates the golden fixtures in tests/golden/ from the reference's own
integral kernels (oracle/refcpu: src/int2e.cu and src/int1e.cu of the
reference compiled for the CPU) on the inputs below.  Needs the reference
tree (GANSU_REFERENCE, default /root/reference); the fixtures themselves are
committed so that the tests need neither the reference nor this script.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from dft_gansu_gb300 import geometry  # noqa: E402
from oracle import oracle as O  # noqa: E402

BASIS = ROOT / "dft_gansu_gb300" / "basis"
CASES = {
    "water_sto-3g": (geometry.water(), "sto-3g", True),
    "water_6-31g_st": (geometry.water(), "6-31g_st", False),
    "water_cc-pvdz": (geometry.water(), "cc-pvdz", False),
    "propane_6-31g_st": (geometry.alkane(3, jitter=0.02, seed=7), "6-31g_st", False),
}


def main():
    O.build_refcpu()
    rng = np.random.default_rng(0)
    for name, (atoms, gbs, full) in CASES.items():
        b = O.make_basis(atoms, BASIS / f"{gbs}.gbs")
        r = O.refcpu_integrals(b, thr=1e-12)
        eri = r["eri"]
        N = b.nbf
        # SCF on the reference's own integrals with the restated reference loop
        H = r["H"]
        fock = lambda D: H + np.einsum("ijkl,kl->ij", eri, D) - 0.5 * np.einsum("ikjl,kl->ij", eri, D)
        scf = O.rhf(r["S"], H, fock, b.num_electrons // 2, O.nuclear_repulsion(atoms), thr=1e-10)
        out = {"atoms": np.array(atoms), "S": r["S"], "H": H, "bounds": r["bounds"],
               "energy_total": scf["total_energy"], "iterations": scf["iterations"],
               "orbital_energies": scf["orbital_energies"], "eri_sum": eri.sum(), "eri_abs_sum": np.abs(eri).sum(),
               "eri_sq_sum": (eri * eri).sum()}
        if full:
            out["eri"] = eri
        else:
            idx = rng.integers(0, N, size=(4000, 4))
            out["eri_idx"] = idx
            out["eri_val"] = eri[idx[:, 0], idx[:, 1], idx[:, 2], idx[:, 3]]
        np.savez_compressed(Path(__file__).parent / f"{name}.npz", **out)
        print(f"{name}: N={N} E={scf['total_energy']:.10f} iters={scf['iterations']}")


if __name__ == "__main__":
    main()
