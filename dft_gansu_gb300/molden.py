"""Molden export and Mulliken populations of a solved SCF.

``write_molden`` produces the file of RHF/UHF/ROHF::export_molden_file
(src/rhf.cu:363-425, src/uhf.cu:379-440, src/rohf.cu:348-410): an [Atoms]
section in bohr, a [GTO] section with, per atom and per shell, the shell's
primitives (exponent, coefficient) in the order of the primitive list, and an
[MO] section with energies, spins, occupations and coefficients.  Numbers are
formatted as the reference's output stream does: six significant digits until
the first coefficient line switches the stream to seventeen (so the first
orbital's energy and occupation keep six).
"""
from __future__ import annotations

import numpy as np

SHELL_NAMES = "spdfghi"


class _Stream:
    """%g with the stream's sticky precision (6, then 17)."""

    def __init__(self):
        self.prec = 6

    def num(self, v) -> str:
        return f"{float(v):.{self.prec}g}"


def write_molden(filename: str, mol, orbital_sets) -> None:
    """orbital_sets: list of (spin "Alpha"/"Beta", energies (N), coefficients
    (N x N, orbitals as columns), occupations (N))."""
    from .sad import SYMBOLS, atom_basis_ranges

    st = _Stream()
    t = mol.primitive_table()
    n = mol.num_basis
    nprim = np.zeros(n, dtype=int)
    stype = np.zeros(n, dtype=int)
    for bi, ty in zip(t["basis_index"], t["shell_type"]):
        nprim[bi] += 1
        stype[bi] = ty
    lines = ["[Molden Format]", "generated by GANSU", "[Atoms] (AU)"]
    atoms = mol.get_atoms()
    for i, (z, x, y, w) in enumerate(atoms):
        lines.append(f"{SYMBOLS[z - 1]} {i + 1} {z} {st.num(x)} {st.num(y)} {st.num(w)}")
    lines.append("[GTO]")
    for i, (lo, cnt) in enumerate(atom_basis_ranges(mol)):
        lines.append(f"{i + 1} 0")
        for j in range(lo, lo + cnt):
            if nprim[j] == 0:  # only the first function of a shell carries its primitives
                continue
            lines.append(f" {SHELL_NAMES[stype[j]]} {nprim[j]} 1.00")
            for k in np.nonzero(t["basis_index"] == j)[0]:
                lines.append(f"\t{st.num(t['exponent'][k])} {st.num(t['coefficient'][k])}")
        lines.append("")
    lines.append("")
    lines.append("[MO]")
    for spin, eps, Cm, occ in orbital_sets:
        eps, Cm, occ = np.asarray(eps), np.asarray(Cm), np.asarray(occ)
        for i in range(n):
            lines.append("Sym= A")
            lines.append(f"Ene= {st.num(eps[i])}")
            lines.append(f"Spin= {spin}")
            lines.append(f"Occup= {st.num(occ[i])}")
            st.prec = 17
            for j in range(n):
                lines.append(f" {j + 1} {st.num(Cm[j, i])}")
    with open(filename, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_molden_mos(filename: str):
    """(spins, energies, occupations, coefficients N x M) of a Molden [MO] section."""
    spins, eps, occ, cols = [], [], [], []
    cur = None
    with open(filename) as f:
        in_mo = False
        for line in f:
            s = line.strip()
            if s.startswith("["):
                in_mo = s == "[MO]"
                continue
            if not in_mo or not s:
                continue
            if s.startswith("Sym="):
                cur = []
                cols.append(cur)
            elif s.startswith("Ene="):
                eps.append(float(s.split()[1]))
            elif s.startswith("Spin="):
                spins.append(s.split()[1])
            elif s.startswith("Occup="):
                occ.append(float(s.split()[1]))
            else:
                cur.append(float(s.split()[1]))
    return spins, np.array(eps), np.array(occ), np.array(cols).T


def mulliken_charges(mol, density, overlap) -> np.ndarray:
    """Atomic charges Z_A - sum_{i in A} (D S)_ii (analyze_mulliken_population,
    src/rhf.cu:427-460); density is the total (alpha + beta) density."""
    from .sad import atom_basis_ranges

    D, S = np.asarray(density), np.asarray(overlap)
    pop = np.einsum("ij,ij->i", D, S)
    return np.array([z - pop[lo:lo + cnt].sum()
                     for (z, *_), (lo, cnt) in zip(mol.get_atoms(), atom_basis_ranges(mol))])
