"""Spherical-harmonic (pure) functions on top of the Cartesian basis.

The reference is Cartesian only (six d components per shell).  A d shell's
Cartesian space is the five real solid harmonics times the radial part plus
the contaminant r^2 = x^2 + y^2 + z^2, which has s symmetry and is
S-orthogonal to them.  With the Cartesian order of a d shell
(xx, yy, zz, xy, xz, yz) and equal normalisation of xx, yy, zz (and of xy, xz,
yz), the pure functions in the order m = -2..2 are

    xy,  yz,  2zz - xx - yy,  xz,  xx - yy

as combinations of the basis functions themselves; s and p shells are kept as
they are.  The SCF then runs in the span of these combinations through an
orthogonaliser X = T U s^{-1/2} of S' = T^T S T (eigenvalues below 1e-6
dropped, as for the Cartesian X), padded with zero columns to N x N.  The
integral engine, the Fock build and the gradient stay Cartesian: a pure
function is a fixed combination of Cartesian functions on the same centre, so
the same AO densities give the spherical energy and its gradient.
"""
from __future__ import annotations

import numpy as np

# pure d combinations over (xx, yy, zz, xy, xz, yz), m = -2..2
D_PURE = np.array([
    [0.0, 0.0, 0.0, 1.0, 0.0, 0.0],
    [0.0, 0.0, 0.0, 0.0, 0.0, 1.0],
    [-1.0, -1.0, 2.0, 0.0, 0.0, 0.0],
    [0.0, 0.0, 0.0, 0.0, 1.0, 0.0],
    [1.0, -1.0, 0.0, 0.0, 0.0, 0.0],
]).T


def shells(mol) -> list:
    """(first basis function, shell type) of every contracted shell, in basis order."""
    t = mol.primitive_table()
    seen = {}
    for bi, ty in zip(t["basis_index"], t["shell_type"]):
        seen[int(bi)] = int(ty)
    return sorted(seen.items())


def transform(mol) -> np.ndarray:
    """T (N_cart x N_pure): columns are the pure functions over the Cartesian basis."""
    sh = shells(mol)
    n = mol.num_basis
    npure = sum(2 * l + 1 for _, l in sh)
    T = np.zeros((n, npure))
    col = 0
    for bf, l in sh:
        if l <= 1:
            for i in range((l + 1) * (l + 2) // 2):
                T[bf + i, col + i] = 1.0
        elif l == 2:
            T[bf:bf + 6, col:col + 5] = D_PURE
        else:
            raise ValueError("spherical functions are provided for s, p and d shells")
        col += 2 * l + 1
    return T


def num_pure(mol) -> int:
    return sum(2 * l + 1 for _, l in shells(mol))


def orthogonalizer(S, T, tol: float = 1e-6) -> np.ndarray:
    """X (N x N, zero columns beyond the orbital space) with X^T S X = 1 on the span of T."""
    Sp = T.T @ S @ T
    w, U = np.linalg.eigh(Sp)
    keep = w >= tol
    Xp = U[:, keep] / np.sqrt(w[keep])
    X = np.zeros((S.shape[0], S.shape[0]))
    X[:, :Xp.shape[1]] = T @ Xp
    return X
