"""Superposition-of-atomic-densities (SAD) guess and the .sad file format.

The reference's SAD guess (InitialGuess_RHF_SAD / _UHF_SAD / _ROHF_SAD,
include/rhf.hpp:464-588, include/uhf.hpp:580-620, include/rohf.hpp:513-600)
pastes per-element alpha and beta atomic densities into the diagonal blocks of
the molecule's density (atom_to_basis_range) and hands that to the SCF.  The
atomic densities come from ``<basis>.sad`` next to the basis file
(read_density_from_sad, src/utils.cpp:21-56): blocks of ``<element> <n>``
followed by n rows of the alpha and n rows of the beta density, row-major.

Here the same file is read when it exists (values used as they are, as the
reference does).  Otherwise an element's densities are computed on the GPU the
way the reference's generator makes the files (script/generate_sad_cache.py:
the isolated atom at the origin, even Z by RHF, odd Z by ROHF with one unpaired
electron, core guess) and cached for the process.  ``write_sad`` writes the
same format, ``export_sad_cache`` the single-atom cache file of
HF::generate_sad_cache (include/hf.hpp:372-405).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

SYMBOLS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar",
           "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr",
           "Rb", "Sr", "Y", "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te", "I", "Xe"]

_CACHE: dict = {}


def read_sad(path) -> dict:
    """{element symbol: (D_alpha, D_beta)} of a .sad file."""
    toks = Path(path).read_text().split()
    out, i = {}, 0
    while i + 1 < len(toks):
        el, n = toks[i], int(toks[i + 1])
        i += 2
        vals = np.array(toks[i:i + 2 * n * n], dtype=float)
        if vals.size != 2 * n * n:
            raise ValueError(f"{path}: truncated block for {el}")
        i += 2 * n * n
        out[el] = (vals[:n * n].reshape(n, n), vals[n * n:].reshape(n, n))
    return out


def _rows(f, M):
    for row in M:
        f.write(" ".join(f"{v:.10e}" for v in row) + " \n")


def write_sad(path, densities: dict) -> None:
    """Write {element symbol: (D_alpha, D_beta)} in the .sad format."""
    with open(path, "w") as f:
        for el, (a, b) in densities.items():
            n = a.shape[0]
            f.write(f"{el} {n}\n")
            _rows(f, a)
            _rows(f, b)


def export_sad_cache(path, density_alpha, density_beta) -> None:
    """The single-molecule cache file of HF::generate_sad_cache: N, then the
    alpha and beta densities row-major (%.10e)."""
    a, b = np.asarray(density_alpha), np.asarray(density_beta)
    with open(path, "w") as f:
        f.write(f"{a.shape[0]}\n")
        _rows(f, a)
        _rows(f, b)


def atom_basis_ranges(mol) -> list:
    """(first function, count) of every atom (HF::get_atom_to_basis_range)."""
    t = mol.primitive_table()
    ncart = (t["shell_type"] + 1) * (t["shell_type"] + 2) // 2
    last = t["basis_index"] + ncart
    out = []
    for ia in range(mol.num_atoms):
        sel = t["atom_index"] == ia
        lo, hi = int(t["basis_index"][sel].min()), int(last[sel].max())
        out.append((lo, hi - lo))
    return out


def _compute_atom(z: int, gbs_filename: str):
    """(D_alpha, D_beta) of the isolated atom: RHF for even Z, ROHF doublet for odd Z."""
    from . import Engine, Molecular  # the GPU path

    mol = Molecular([(z, 0.0, 0.0, 0.0)], gbs_filename)
    eng = Engine(mol)
    try:
        opts = {"convergence_threshold": 1e-10, "max_iter": 300}
        if z % 2 == 0:
            r = eng.rhf_scf(z, opts, want_matrices=True)
            if not r["converged"]:
                raise RuntimeError(f"SAD: the RHF of {SYMBOLS[z - 1]} did not converge")
            D = r["density"].double().cpu().numpy()
            return 0.5 * D, 0.5 * D
        r = eng.rohf_scf((z + 1) // 2, (z - 1) // 2, opts, want_matrices=True)
        if not r["converged"]:
            raise RuntimeError(f"SAD: the ROHF of {SYMBOLS[z - 1]} did not converge")
        return r["density_alpha"].double().cpu().numpy(), r["density_beta"].double().cpu().numpy()
    finally:
        eng.close()


def atomic_density(z: int, gbs_filename: str, source: str = "auto"):
    """(D_alpha, D_beta) of element z in the basis gbs_filename.  source:
    "file" (``<basis>.sad`` only), "compute" (atomic SCF only) or "auto"
    (the file when it has the element, else the atomic SCF)."""
    key = (str(Path(gbs_filename).resolve()), int(z), source)
    if key in _CACHE:
        return _CACHE[key]
    el = SYMBOLS[z - 1]
    dens = None
    if source in ("auto", "file"):
        sad_path = Path(gbs_filename).with_suffix(".sad")
        if sad_path.exists():
            table = read_sad(sad_path)
            dens = table.get(el)
        if dens is None and source == "file":
            raise FileNotFoundError(f"no density for {el} in {sad_path}")
    if dens is None:
        dens = _compute_atom(z, gbs_filename)
    _CACHE[key] = dens
    return dens


def sad_guess(mol, gbs_filename: str, source: str = "auto"):
    """Block-diagonal (D_alpha, D_beta) of a Molecular (numpy, N x N)."""
    n = mol.num_basis
    Da, Db = np.zeros((n, n)), np.zeros((n, n))
    for (z, *_), (lo, cnt) in zip(mol.get_atoms(), atom_basis_ranges(mol)):
        a, b = atomic_density(z, gbs_filename, source)
        if a.shape != (cnt, cnt):
            raise ValueError(f"SAD density of {SYMBOLS[z - 1]} is {a.shape[0]}x{a.shape[0]}, the atom has {cnt} functions")
        Da[lo:lo + cnt, lo:lo + cnt] = a
        Db[lo:lo + cnt, lo:lo + cnt] = b
    return Da, Db
