"""CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported only by tests/, by __graft_entry__.smoke() as the checker and by
bench.py's CPU legs.  The product never imports it.

Contents, each a restatement of the reference (file:line in the reference):
  - .gbs / .xyz parsing and primitive expansion    src/basis_set.cpp:32-124,
                                                   src/parseXYZ.cpp:43-119,
                                                   include/molecular.hpp:117-186
  - CGTO factors with the L/2 integer quirk        include/basis_set.hpp:106-137
  - MD integrals, Schwarz, J/K, S/T/V             oracle/md_oracle.c (C, OpenMP)
  - RHF SCF with DIIS                              src/hf.cu:171-314,
                                                   include/rhf.hpp:272-396,
                                                   src/gpu_manager.cu:529-599,1020-1194
Pins:
  - refcpu_*: the reference's own int2e.cu / int1e.cu kernels compiled for the
    CPU (oracle/refcpu, built into oracle/_ref; needs the reference tree, so
    only available where it is mounted);
  - known answers of the reference's linear-algebra tests
    (test/test_gpu_manager.cu) in tests/test_oracle_pins.py.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import scipy.linalg

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
# root of the reference source tree, from GANSU_REFERENCE only (unset: the
# reference-backed checks are skipped and the committed golden fixtures stand in)
REFERENCE_ROOT = Path(os.environ["GANSU_REFERENCE"]) if os.environ.get("GANSU_REFERENCE") else None
ANG2BOHR = 1.8897259886

ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar"]
CART = {
    0: [(0, 0, 0)],
    1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
    2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)],
}
L_OF = {"S": 0, "P": 1, "D": 2, "F": 3, "G": 4}


# ------------------------------------------------------------------ build
def build_oracle(force: bool = False) -> Path:
    """Compile oracle/md_oracle.c into oracle/_build/libmdoracle.so."""
    BUILD.mkdir(exist_ok=True)
    so = BUILD / "libmdoracle.so"
    src = HERE / "md_oracle.c"
    if force or not so.exists() or so.stat().st_mtime < src.stat().st_mtime:
        tmp = so.with_suffix(".tmp.so")
        subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(src), "-o", str(tmp), "-lm"],
                       check=True)
        os.replace(tmp, so)
    return so


def build_refcpu() -> Path | None:
    """Compile the reference's integral kernels for the CPU (needs the reference tree)."""
    if REFERENCE_ROOT is None or not (REFERENCE_ROOT / "src" / "int2e.cu").exists():
        return None
    subprocess.run(["make", "-s", "-C", str(HERE / "refcpu"), f"REF={REFERENCE_ROOT}", f"OUT={REF_OUT}"], check=True)
    return REF_OUT / "librefcpu.so"


_oracle = None
_refcpu = None


def _lib():
    global _oracle
    if _oracle is None:
        L = C.CDLL(str(build_oracle()))
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        basis = [C.c_int, ip, ip, ip, ip, dp, dp, dp, dp, C.c_int]
        L.oracle_boys.argtypes = [C.c_int, C.c_double, dp]
        L.oracle_cgto_factor.argtypes = [C.c_int, C.c_int, dp, dp]
        L.oracle_cgto_factor.restype = C.c_double
        L.oracle_eri_tensor.argtypes = basis + [C.c_double, dp]
        L.oracle_direct_jk.argtypes = basis + [C.c_double, dp, dp, dp, C.c_int]
        L.oracle_direct_jk.restype = C.c_long
        L.oracle_direct_jk_sample.argtypes = basis + [C.c_double, dp, dp, dp, C.c_int, C.c_int]
        L.oracle_direct_jk_sample.restype = C.c_long
        L.oracle_one_electron.argtypes = basis + [C.c_int, dp, dp, dp, dp, dp]
        L.oracle_prim_pair_bounds.argtypes = basis + [C.c_int, dp]
        L.oracle_ri_three_center_pairs.argtypes = basis + basis + [C.c_double, C.c_int, ip, ip, dp]
        _oracle = L
    return _oracle


def refcpu_available() -> bool:
    return (REF_OUT / "librefcpu.so").exists()


def _ref():
    global _refcpu
    if _refcpu is None:
        L = C.CDLL(str(REF_OUT / "librefcpu.so"))
        dp, ip, lp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_longlong)
        L.refcpu_integrals.argtypes = [C.c_int, dp, dp, dp, ip, lp, ip, dp, C.c_int, C.c_int, ip, dp, C.c_double,
                                       dp, dp, dp, dp, lp]
        _refcpu = L
    return _refcpu


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


# ---------------------------------------------------------- input model
def parse_gbs(path) -> dict:
    """{element: [(l, [exps], [coefs]), ...]} in file order."""
    lines = Path(path).read_text().splitlines()
    i = 0
    while i < len(lines) and not (lines[i][:1].isalpha()):
        i += 1
    out: dict = {}
    while i < len(lines):
        toks = lines[i].split()
        i += 1
        if not toks:
            continue
        shells = out.setdefault(toks[0], [])
        while i < len(lines):
            hdr = lines[i].strip()
            i += 1
            if hdr.startswith("****"):
                break
            t = hdr.split()
            if not t:
                continue
            typ, nprim = t[0], int(t[1])
            rows = [lines[i + k].replace("D", "E").split() for k in range(nprim)]
            i += nprim
            for col, letter in enumerate(typ):
                shells.append((L_OF[letter.upper()], [float(r[0]) for r in rows], [float(r[1 + col]) for r in rows]))
    return out


def parse_xyz(path):
    lines = Path(path).read_text().splitlines()
    n = int(lines[0])
    atoms = []
    for ln in lines[2:]:
        t = ln.split()
        if not t:
            continue
        atoms.append((ELEMENTS.index(t[0]) + 1, float(t[1]) * ANG2BOHR, float(t[2]) * ANG2BOHR,
                      float(t[3]) * ANG2BOHR))
    assert len(atoms) == n
    return atoms


def cgto_factor(L, exps, coefs):
    """include/basis_set.hpp:106-137 (second primitive uses L//2)."""
    s = 0.0
    for a, ca in zip(exps, coefs):
        na = (2 * math.pi) ** -0.75 * (4 * a) ** (L / 2.0 + 0.75)
        for b, cb in zip(exps, coefs):
            nb = (2 * math.pi) ** -0.75 * (4 * b) ** (L // 2 + 0.75)
            s += ca * na * cb * nb / (2 * (a + b)) ** (L + 1.5)
    return (s * (2 * math.pi) ** 1.5) ** -0.5


@dataclass
class Basis:
    atoms: list
    l: np.ndarray
    nprim: np.ndarray
    prim_off: np.ndarray
    bf_off: np.ndarray
    xyz: np.ndarray
    alpha: np.ndarray
    coef: np.ndarray
    cgto: np.ndarray
    nbf: int
    shell_atom: np.ndarray
    num_electrons: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def nshell(self):
        return len(self.l)

    def cargs(self):
        return (C.c_int(self.nshell), _ip(self.l), _ip(self.nprim), _ip(self.prim_off), _ip(self.bf_off),
                _dp(self.xyz), _dp(self.alpha), _dp(self.coef), _dp(self.cgto), C.c_int(self.nbf))

    def reference_primitives(self):
        """Primitive list as the reference's Molecular builds it: per atom, per
        shell in file order, then stably sorted by shell type."""
        rows = []
        for s in range(self.nshell):
            for k in range(self.nprim[s]):
                p = self.prim_off[s] + k
                rows.append((int(self.l[s]), float(self.alpha[p]), float(self.coef[p]), tuple(self.xyz[s]),
                             int(self.bf_off[s]), int(self.shell_atom[s])))
        rows.sort(key=lambda r: r[0])
        return rows


def make_basis(atoms, gbs_path, charge=0) -> Basis:
    table = parse_gbs(gbs_path)
    l, nprim, prim_off, bf_off, xyz, alpha, coef, cgto, shell_atom = [], [], [], [], [], [], [], [], []
    bf = 0
    for ia, (z, x, y, w) in enumerate(atoms):
        for (L, exps, cfs) in table[ELEMENTS[z - 1]]:
            l.append(L)
            nprim.append(len(exps))
            prim_off.append(len(alpha))
            bf_off.append(bf)
            xyz.append((x, y, w))
            alpha.extend(exps)
            coef.extend(cfs)
            shell_atom.append(ia)
            nc = (L + 1) * (L + 2) // 2
            cgto.extend([cgto_factor(L, exps, cfs)] * nc)
            bf += nc
    ne = sum(a[0] for a in atoms) - charge
    return Basis(atoms=list(atoms), l=np.array(l, np.int32), nprim=np.array(nprim, np.int32),
                 prim_off=np.array(prim_off, np.int32), bf_off=np.array(bf_off, np.int32),
                 xyz=np.ascontiguousarray(np.array(xyz, float)), alpha=np.array(alpha, float),
                 coef=np.array(coef, float), cgto=np.array(cgto, float), nbf=bf,
                 shell_atom=np.array(shell_atom, np.int32), num_electrons=ne)


# ------------------------------------------------------------ integrals
def boys(nmax, x):
    out = np.zeros(nmax + 1)
    _lib().oracle_boys(nmax, float(x), _dp(out))
    return out


def one_electron(b: Basis):
    N = b.nbf
    S, T, V = np.zeros((N, N)), np.zeros((N, N)), np.zeros((N, N))
    z = np.array([a[0] for a in b.atoms], float)
    xyz = np.ascontiguousarray(np.array([a[1:] for a in b.atoms], float))
    _lib().oracle_one_electron(*b.cargs(), len(b.atoms), _dp(z), _dp(xyz), _dp(S), _dp(T), _dp(V))
    return S, T, V


def eri_tensor(b: Basis, thr=1e-12):
    N = b.nbf
    eri = np.zeros((N, N, N, N))
    _lib().oracle_eri_tensor(*b.cargs(), float(thr), _dp(eri))
    return eri


def direct_jk(b: Basis, D, thr=1e-12, nthreads=0):
    N = b.nbf
    D = np.ascontiguousarray(D, dtype=float)
    J, K = np.zeros((N, N)), np.zeros((N, N))
    kept = _lib().oracle_direct_jk(*b.cargs(), float(thr), _dp(D), _dp(J), _dp(K), int(nthreads))
    return J, K, kept


def direct_jk_sample(b: Basis, D, thr=1e-12, nthreads=0, bra_stride=1):
    """J/K over every bra_stride-th bra shell pair (timing sample); returns the
    primitive quartets evaluated."""
    N = b.nbf
    D = np.ascontiguousarray(D, dtype=float)
    J, K = np.zeros((N, N)), np.zeros((N, N))
    return _lib().oracle_direct_jk_sample(*b.cargs(), float(thr), _dp(D), _dp(J), _dp(K), int(nthreads),
                                          int(bra_stride))


def nuclear_repulsion(atoms):
    e = 0.0
    for i in range(len(atoms)):
        for j in range(i + 1, len(atoms)):
            d = math.dist(atoms[i][1:], atoms[j][1:])
            e += atoms[i][0] * atoms[j][0] / d
    return e


# ------------------------------------------------------------------ SCF
def transform_matrix(S):
    """X = U s^{-1/2}, s < 1e-6 -> 0 (src/hf.cu:171-243, src/gpu_kernels.cu:28-43)."""
    s, U = np.linalg.eigh(S)
    d = np.where(s < 1e-6, 0.0, 1.0 / np.sqrt(np.where(s < 1e-6, 1.0, s)))
    return U * d


def coefficients(F, X):
    e, Cp = np.linalg.eigh(X.T @ F @ X)
    return e, X @ Cp


def density(Cm, nocc):
    Co = Cm[:, :nocc]
    return 2.0 * Co @ Co.T


def diis_extrapolate(errs, focks):
    m = len(errs)
    B = -np.ones((m + 1, m + 1))
    B[m, m] = 0.0
    for i in range(m):
        for j in range(m):
            B[i, j] = np.vdot(errs[i], errs[j])
    rhs = np.zeros(m + 1)
    rhs[m] = -1.0
    try:
        c = np.linalg.solve(B, rhs)
    except np.linalg.LinAlgError:  # exactly dependent error vectors (e.g. all zero): least squares
        c = np.linalg.lstsq(B, rhs, rcond=None)[0]
    return sum(ci * Fi for ci, Fi in zip(c[:m], focks))


def gwh_guess(S, H):
    """GWH guess F_pq = 1.75 S_pq (H_pp + H_qq) / 2, diagonal included (src/gpu_kernels.cu:535-545)."""
    d = np.diag(H)
    return 1.75 * S * (d[:, None] + d[None, :]) * 0.5


def spherical_transform(b: Basis):
    """Pure-function combinations over each shell's Cartesian functions: s, p kept;
    d (xx, yy, zz, xy, xz, yz) -> xy, yz, 2zz - xx - yy, xz, xx - yy.  Restates the
    real solid harmonics of degree 2 (no reference counterpart: GANSU is Cartesian)."""
    cols = []
    for L, off in zip(b.l, b.bf_off):
        L, off = int(L), int(off)
        if L <= 1:
            for i in range((L + 1) * (L + 2) // 2):
                v = np.zeros(b.nbf); v[off + i] = 1.0; cols.append(v)
        else:
            xx, yy, zz, xy, xz, yz = (off + i for i in range(6))
            for comb in ({xy: 1.0}, {yz: 1.0}, {zz: 2.0, xx: -1.0, yy: -1.0}, {xz: 1.0}, {xx: 1.0, yy: -1.0}):
                v = np.zeros(b.nbf)
                for k, c in comb.items():
                    v[k] = c
                cols.append(v)
    return np.array(cols).T


def spherical_orthogonalizer(S, T, tol=1e-6):
    """X = T U s^{-1/2} of T^T S T (eigenvalues below tol dropped), zero-padded to N x N."""
    w, U = np.linalg.eigh(T.T @ S @ T)
    keep = w >= tol
    X = np.zeros((S.shape[0], S.shape[0]))
    X[:, :keep.sum()] = T @ (U[:, keep] / np.sqrt(w[keep]))
    return X


def damp(old, new, a):
    """damping (src/gpu_manager.cu:989, the update behind Convergence_RHF_Damping):
    (1 - a) old + a new."""
    return (1.0 - a) * old + a * new


def damping_factor(F, Fp, D, Dp):
    """computeOptimalDampingFactor_RHF (src/gpu_manager.cu:898-963): s = Tr[F_old dD],
    c = Tr[(F - F_old) dD]; 1 if c <= -s/2, else -s/(2c)."""
    dD = D - Dp
    sv, cv = np.trace(Fp @ dD), np.trace((F - Fp) @ dD)
    return 1.0 if cv <= -sv / 2.0 else -0.5 * sv / cv


def rhf(S, H, fock, nocc, enuc, maxiter=100, thr=1e-6, diis_size=8, include_transform=False, guess="core",
        guess_density=None, X=None, convergence="diis", damping=0.9):
    """The reference SCF loop (src/hf.cu:278-307) with DIIS and the core, GWH,
    density (F = F(D)) or SAD (F(D), C, D, F) guess (include/rhf.hpp:378-588);
    guess_density is the total density D_a + D_b.  X: an orthogonaliser over a
    subspace (the DIIS error is then taken in the orthogonal basis)."""
    project = X is not None  # DIIS error X^T e X in the orthonormal basis of the subspace
    if X is None:
        X = transform_matrix(S)
    if guess in ("density", "sad"):
        F = fock(guess_density)
        if guess == "sad":
            _, Cm = coefficients(F, X)
            F = fock(density(Cm, nocc))
    else:
        _, Cm = coefficients(gwh_guess(S, H) if guess == "gwh" else H, X)
        D = density(Cm, nocc)
        F = fock(D)
    prev, energy, it, diis_it = np.finfo(float).max, 0.0, 0, 0
    errs, focks = [None] * diis_size, [None] * diis_size
    eps = None
    converged = False
    history = []
    damp_prev = None
    while it < maxiter:
        eps, Cm = coefficients(F, X)
        D = density(Cm, nocc)
        F = fock(D)
        energy = 0.5 * (np.vdot(D, H) + np.vdot(D, F))
        history.append(energy)
        if abs(energy - prev) < thr:
            converged = True
            break
        it += 1
        prev = energy
        if convergence != "diis":  # Convergence_RHF_Damping (include/rhf.hpp:182-262)
            if damp_prev is None:
                damp_prev = (F.copy(), D.copy())
            else:
                Fp, Dp = damp_prev
                a = damping_factor(F, Fp, D, Dp) if convergence == "optimaldamping" else damping
                F = damp(Fp, F, a)
                if convergence == "optimaldamping":
                    D = damp(Dp, D, a)
                    damp_prev = (F.copy(), D.copy())
                else:
                    damp_prev = (F.copy(), Dp)
            diis_it += 1
            continue
        e = F @ D @ S - S @ D @ F
        if project:
            e = X.T @ e @ X
        elif include_transform:
            e = X @ e @ X.T
        slot = diis_it % diis_size
        errs[slot], focks[slot] = e, F.copy()
        nprev = min(diis_it + 1, diis_size)
        if nprev > 1:
            F = diis_extrapolate(errs[:nprev], focks[:nprev])
        diis_it += 1
    return {"electronic_energy": energy, "total_energy": energy + enuc, "iterations": it, "converged": converged,
            "orbital_energies": eps, "density": D, "fock": F, "history": history}


def break_symmetry(Cb):
    """InitialGuess_UHF::break_symmetry (include/uhf.hpp:429-436): the last basis
    function's row and the last orbital's column of the beta coefficients zeroed."""
    Cb = Cb.copy()
    Cb[-1, :] = 0.0
    Cb[:, -1] = 0.0
    return Cb


def uhf(S, H, jk, na, nb, enuc, maxiter=100, thr=1e-6, diis_size=8, include_transform=False, guess="core",
        guess_density=None):
    """The reference UHF loop (src/uhf.cu, Convergence_UHF_DIIS include/uhf.hpp:291-380):
    F_s = H + J(Da + Db) - K(D_s), one DIIS ring per spin.  Guesses
    (include/uhf.hpp:484-620): core / GWH orbitals for both spins with the beta
    symmetry break; density / SAD: F(Da, Db), C, break, D, F."""
    X = transform_matrix(S)

    def fock(Da, Db):
        Ja, Ka = jk(Da)
        Jb, Kb = jk(Db)
        return H + Ja + Jb - Ka, H + Ja + Jb - Kb

    if guess in ("density", "sad"):
        Da, Db = guess_density
        Fa, Fb = fock(Da, Db)
        _, Ca = coefficients(Fa, X)
        _, Cb = coefficients(Fb, X)
    else:
        _, Ca = coefficients(gwh_guess(S, H) if guess == "gwh" else H, X)
        Cb = Ca
    Cb = break_symmetry(Cb)
    Da, Db = Ca[:, :na] @ Ca[:, :na].T, Cb[:, :nb] @ Cb[:, :nb].T
    Fa, Fb = fock(Da, Db)
    prev, energy, it, diis_it = np.finfo(float).max, 0.0, 0, 0
    ring = {"a": ([None] * diis_size, [None] * diis_size), "b": ([None] * diis_size, [None] * diis_size)}
    converged = False
    while it < maxiter:
        _, Ca = coefficients(Fa, X)
        _, Cb = coefficients(Fb, X)
        Da, Db = Ca[:, :na] @ Ca[:, :na].T, Cb[:, :nb] @ Cb[:, :nb].T
        Fa, Fb = fock(Da, Db)
        energy = 0.5 * (np.vdot(Da + Db, H) + np.vdot(Da, Fa) + np.vdot(Db, Fb))
        if abs(energy - prev) < thr:
            converged = True
            break
        it += 1
        prev = energy
        slot = diis_it % diis_size
        nprev = min(diis_it + 1, diis_size)
        out = []
        for key, F, D in (("a", Fa, Da), ("b", Fb, Db)):
            e = F @ D @ S - S @ D @ F
            if include_transform:
                e = X @ e @ X.T
            errs, focks = ring[key]
            errs[slot], focks[slot] = e, F.copy()
            out.append(diis_extrapolate(errs[:nprev], focks[:nprev]) if nprev > 1 else F)
        Fa, Fb = out
        diis_it += 1
    return {"electronic_energy": energy, "total_energy": energy + enuc, "iterations": it, "converged": converged,
            "density_alpha": Da, "density_beta": Db}


# ROHF coupling constants (A_cc, B_cc, A_oo, B_oo, A_vv, B_vv), src/rohf.cu:30-39
ROHF_COUPLINGS = {
    "roothaan": (-0.5, 1.5, 0.5, 0.5, 1.5, -0.5),
    "mcweeny-diercksen": (1 / 3, 2 / 3, 1 / 3, 1 / 3, 2 / 3, 1 / 3),
    "davidson": (0.5, 1.0, 0.0, 1.0, 1.0, 0.0),
    "guest-saunders": (0.5, 0.5, 0.5, 0.5, 0.5, 0.5),
    "binkley-pople-dobosh": (0.5, 0.5, 1.0, 0.0, 0.0, 1.0),
    "faegri-manne": (0.5, 0.5, 1.0, 0.0, 0.5, 0.5),
    "goddard": (0.5, 0.5, 0.5, 0.0, 1.0, 0.0),
    "plakhutin-gorelik-breslavskaya": (0.0, 1.0, 1.0, 0.0, 1.0, 0.0),
}


def rohf_unified(Fc_mo, Fo_mo, nc, no, coupling):
    """computeUnifiedFockMatrix_ROHF_kernel (src/gpu_kernels.cu:421-498): the MO-basis
    unified Fock matrix by orbital classes, element (i, j) read at (min, max)."""
    acc, bcc, aoo, boo, avv, bvv = coupling
    n = Fc_mo.shape[0]
    cls = np.where(np.arange(n) < nc, 0, np.where(np.arange(n) < nc + no, 1, 2))
    R = np.zeros((n, n))
    for i in range(n):
        for j in range(i, n):
            fc, fo = Fc_mo[i, j], Fo_mo[i, j]
            a, b = cls[i], cls[j]
            if a == 0 and b == 0:
                d = 2.0 * (acc * fo + bcc * (fc - fo))
            elif a == 0 and b == 1:
                d = 2.0 * (fc - fo)
            elif a == 0:
                d = fc
            elif a == 1 and b == 1:
                d = 2.0 * (aoo * fo + boo * (fc - fo))
            elif a == 1:
                d = 2.0 * fo
            else:
                d = 2.0 * (avv * fo + bvv * (fc - fo))
            R[i, j] = R[j, i] = d
    return R


def rohf(S, H, jk, na, nb, enuc, maxiter=100, thr=1e-6, diis_size=8, include_transform=False, guess="core",
         guess_density=None, coupling="roothaan"):
    """The reference ROHF (src/rohf.cu; computeFockMatrix_ROHF, src/gpu_manager.cu:733-817;
    energy :871-884; Convergence_ROHF_DIIS include/rohf.hpp:307-360):
    D_c = 2 C_c C_c^T, D_o = C_o C_o^T; F_c = H + J(D) - K(D_c)/2 - K(D_o)/2,
    F_o = (H + J(D) - K(D_c)/2 - K(D_o))/2; unified R from C^T F_c C, C^T F_o C;
    F = S C R C^T S; DIIS on F with D = D_c + D_o.  Density / SAD guess: D_c = 2 D_b,
    D_o = D_a - D_b, first unified F with the core-guess orbitals, then C, D, F."""
    cp = ROHF_COUPLINGS[coupling] if isinstance(coupling, str) else tuple(coupling)
    nc, no = nb, na - nb
    X = transform_matrix(S)

    def dens(Cm):
        Dc = 2.0 * Cm[:, :nc] @ Cm[:, :nc].T
        Do = Cm[:, nc:nc + no] @ Cm[:, nc:nc + no].T
        return Dc, Do

    def fock(Dc, Do, Cm):
        Jc, Kc = jk(Dc)
        Jo, Ko = jk(Do) if no > 0 else (np.zeros_like(Dc), np.zeros_like(Dc))
        h = H + Jc + Jo - 0.5 * Kc
        Fc, Fo = h - 0.5 * Ko, 0.5 * (h - Ko)
        R = rohf_unified(Cm.T @ Fc @ Cm, Cm.T @ Fo @ Cm, nc, no, cp)
        SC = S @ Cm
        return Fc, Fo, SC @ R @ SC.T

    if guess in ("density", "sad"):
        Da, Db = guess_density
        _, Cm = coefficients(H, X)
        _, _, F = fock(2.0 * Db, Da - Db, Cm)
        _, Cm = coefficients(F, X)
    else:
        _, Cm = coefficients(gwh_guess(S, H) if guess == "gwh" else H, X)
    Dc, Do = dens(Cm)
    Fc, Fo, F = fock(Dc, Do, Cm)
    prev, energy, it, diis_it = np.finfo(float).max, 0.0, 0, 0
    errs, focks = [None] * diis_size, [None] * diis_size
    converged = False
    eps = None
    while it < maxiter:
        eps, Cm = coefficients(F, X)
        Dc, Do = dens(Cm)
        Fc, Fo, F = fock(Dc, Do, Cm)
        energy = 0.5 * (np.vdot(Dc, H + Fc) + np.vdot(Do, H) + 2.0 * np.vdot(Do, Fo))
        if abs(energy - prev) < thr:
            converged = True
            break
        it += 1
        prev = energy
        D = Dc + Do
        e = F @ D @ S - S @ D @ F
        if include_transform:
            e = X @ e @ X.T
        slot = diis_it % diis_size
        errs[slot], focks[slot] = e, F.copy()
        nprev = min(diis_it + 1, diis_size)
        if nprev > 1:
            F = diis_extrapolate(errs[:nprev], focks[:nprev])
        diis_it += 1
    return {"electronic_energy": energy, "total_energy": energy + enuc, "iterations": it, "converged": converged,
            "density_alpha": 0.5 * Dc + Do, "density_beta": 0.5 * Dc, "orbital_energies": eps}


def rohf_from_basis(b: Basis, na: int, nb: int, thr_schwarz=1e-12, **kw):
    S, T, V = one_electron(b)
    eri = eri_tensor(b, thr_schwarz)
    jk = lambda D: (np.einsum("ijkl,kl->ij", eri, D), np.einsum("ikjl,kl->ij", eri, D))
    return rohf(S, T + V, jk, na, nb, nuclear_repulsion(b.atoms), **kw)


# ------------------------------------------------------------ SAD
def read_sad(path):
    """Parse a .sad file (read_density_from_sad, src/utils.cpp:21-56): blocks of
    "<element> <n>" followed by n rows of the alpha density and n rows of the beta
    density (row-major).  Returns {element: (Da, Db)}."""
    out = {}
    toks = open(path).read().split()
    i = 0
    while i < len(toks):
        el, n = toks[i], int(toks[i + 1])
        i += 2
        vals = np.array(toks[i:i + 2 * n * n], float)
        i += 2 * n * n
        out[el] = (vals[:n * n].reshape(n, n), vals[n * n:].reshape(n, n))
    return out


def atom_ranges(b: Basis):
    """(start, count) of every atom's basis functions (get_atom_to_basis_range)."""
    ranges = []
    for ia in range(len(b.atoms)):
        sh = np.nonzero(b.shell_atom == ia)[0]
        start = int(b.bf_off[sh[0]])
        count = int(sum((int(b.l[k]) + 1) * (int(b.l[k]) + 2) // 2 for k in sh))
        ranges.append((start, count))
    return ranges


def sad_density(b: Basis, atom_densities):
    """Block-diagonal alpha and beta densities (InitialGuess_RHF_SAD::guess,
    include/rhf.hpp:551-584); atom_densities maps an atomic number to (Da, Db)."""
    Da = np.zeros((b.nbf, b.nbf))
    Db = np.zeros((b.nbf, b.nbf))
    for (z, *_), (st, cnt) in zip(b.atoms, atom_ranges(b)):
        a, bb = atom_densities[z]
        assert a.shape == (cnt, cnt)
        Da[st:st + cnt, st:st + cnt] = a
        Db[st:st + cnt, st:st + cnt] = bb
    return Da, Db


def atom_sad_density(z, gbs_path, thr=1e-10, maxiter=200):
    """The atomic density of a .sad file as the reference's generator makes it
    (script/generate_sad_cache.py: even Z -> RHF, odd Z -> ROHF doublet; core
    guess, stored ERIs): returns (Da, Db)."""
    b = make_basis([(z, 0.0, 0.0, 0.0)], gbs_path)
    ne = z
    if ne % 2 == 0:
        r = rhf_from_basis(b, thr=thr, maxiter=maxiter)
        D = r["density"]
        return 0.5 * D, 0.5 * D
    r = rohf_from_basis(b, (ne + 1) // 2, (ne - 1) // 2, thr=thr, maxiter=maxiter)
    return r["density_alpha"], r["density_beta"]


def uhf_energy_of(S, H, jk, Da, Db):
    """1/2 [<Da + Db, H> + <Da, Fa> + <Db, Fb>] of given spin densities (equals the
    ROHF energy when Da = D_c/2 + D_o, Db = D_c/2, and the RHF one when Da = Db)."""
    Ja, Ka = jk(Da)
    Jb, Kb = jk(Db)
    Fa, Fb = H + Ja + Jb - Ka, H + Ja + Jb - Kb
    return 0.5 * (np.vdot(Da + Db, H) + np.vdot(Da, Fa) + np.vdot(Db, Fb))


def uhf_from_basis(b: Basis, na: int, nb: int, thr_schwarz=1e-12, **kw):
    S, T, V = one_electron(b)
    eri = eri_tensor(b, thr_schwarz)
    jk = lambda D: (np.einsum("ijkl,kl->ij", eri, D), np.einsum("ikjl,kl->ij", eri, D))
    return uhf(S, T + V, jk, na, nb, nuclear_repulsion(b.atoms), **kw)


def rhf_from_basis(b: Basis, thr_schwarz=1e-12, stored=True, **kw):
    S, T, V = one_electron(b)
    H = T + V
    if stored:
        eri = eri_tensor(b, thr_schwarz)
        fock = lambda D: H + np.einsum("ijkl,kl->ij", eri, D) - 0.5 * np.einsum("ikjl,kl->ij", eri, D)
    else:
        def fock(D):
            J, K, _ = direct_jk(b, D, thr_schwarz)
            return H + J - 0.5 * K
    return rhf(S, H, fock, b.num_electrons // 2, nuclear_repulsion(b.atoms), **kw)


# ------------------------------------------------------------ RI
def ri_integrals(b: Basis, aux: Basis, thr=1e-12):
    """Metric V (naux x naux), three-centre T (naux x N x N) and the auxiliary
    primitive bounds, restated from src/int2c2e.cu, src/int3c2e.cu and
    src/schwarz.txt:480-682 (md_oracle.c: oracle_ri_integrals)."""
    M, N = aux.nbf, b.nbf
    V, T = np.zeros((M, M)), np.zeros((M, N, N))
    qp = np.zeros(len(aux.alpha))
    _lib().oracle_ri_integrals(*b.cargs(), *aux.cargs(), C.c_double(thr), _dp(V), _dp(T), _dp(qp))
    return V, T, qp


def ri_metric(b: Basis, aux: Basis, thr=1e-12):
    """The metric V = (P|Q) alone (oracle_ri_integrals without the three-centre tensor)."""
    M = aux.nbf
    V = np.zeros((M, M))
    _lib().oracle_ri_integrals(*b.cargs(), *aux.cargs(), C.c_double(thr), _dp(V), None, None)
    return V


def ri_three_center_pairs(b: Basis, aux: Basis, shell_pairs, thr=1e-12):
    """(mu nu|P) for the AO shell pairs listed (A, B): {(mu, nu): vector over P}."""
    pa = np.array([p[0] for p in shell_pairs], np.int32)
    pb = np.array([p[1] for p in shell_pairs], np.int32)
    M = aux.nbf
    T = np.zeros((len(shell_pairs), 225, M))
    _lib().oracle_ri_three_center_pairs(*b.cargs(), *aux.cargs(), C.c_double(thr), len(shell_pairs), _ip(pa),
                                        _ip(pb), _dp(T))
    out = {}
    for k, (A, B) in enumerate(shell_pairs):
        na, nb = (b.l[A] + 1) * (b.l[A] + 2) // 2, (b.l[B] + 1) * (b.l[B] + 2) // 2
        for ia in range(na):
            for ib in range(nb):
                out[(int(b.bf_off[A]) + ia, int(b.bf_off[B]) + ib)] = T[k, ia * nb + ib].copy()
    return out


def ri_factor(V, T):
    """B = L^-1 T with V = L L^T (src/gpu_manager.cu:1448-1526: potrf, then a
    lower-triangular solve on the naux x N^2 matrix)."""
    L = np.linalg.cholesky(V)
    M = T.shape[0]
    return scipy.linalg.solve_triangular(L, T.reshape(M, -1), lower=True).reshape(T.shape)


def ri_jk(B, D):
    """J = sum_P B_P (B_P . D), K = sum_P B_P D B_P^T (src/gpu_manager.cu:1543-1632)."""
    W = np.einsum("pij,ij->p", B, D)
    J = np.einsum("p,pij->ij", W, B)
    K = np.einsum("pik,kl,pjl->ij", B, D, B, optimize=True)
    return J, K


def rhf_ri_from_basis(b: Basis, aux: Basis, thr_schwarz=1e-12, **kw):
    """RI-RHF with the reference's SCF loop (ERI_RI_RHF, include/rhf.hpp:644-691)."""
    S, T1, V1 = one_electron(b)
    H = T1 + V1
    V, T, _ = ri_integrals(b, aux, thr_schwarz)
    B = ri_factor(V, T)

    def fock(D):
        J, K = ri_jk(B, D)
        return H + J - 0.5 * K
    return rhf(S, H, fock, b.num_electrons // 2, nuclear_repulsion(b.atoms), **kw)


# -------------------------------------------------- reference on the CPU
def refcpu_integrals(b: Basis, thr=1e-12, want_eri=True):
    """S, H, primitive Schwarz bounds (reference layout) and the ERI tensor as
    computed by the reference's own kernels run on the CPU."""
    rows = b.reference_primitives()
    n = len(rows)
    exps = np.array([r[1] for r in rows])
    coefs = np.array([r[2] for r in rows])
    xyz = np.ascontiguousarray(np.array([r[3] for r in rows]))
    stype = np.array([r[0] for r in rows], np.int32)
    bidx = np.array([r[4] for r in rows], np.int64)
    aidx = np.array([r[5] for r in rows], np.int32)
    N = b.nbf
    S, H = np.zeros((N, N)), np.zeros((N, N))
    eri = np.zeros((N, N, N, N)) if want_eri else None
    bounds = np.zeros(n * (n + 1) // 2 + n * n)
    nb = C.c_longlong(0)
    z = np.array([a[0] for a in b.atoms], np.int32)
    axyz = np.ascontiguousarray(np.array([a[1:] for a in b.atoms], float))
    _ref().refcpu_integrals(n, _dp(exps), _dp(coefs), _dp(xyz), _ip(stype),
                            bidx.ctypes.data_as(C.POINTER(C.c_longlong)), _ip(aidx), _dp(b.cgto), N, len(b.atoms),
                            _ip(z), _dp(axyz), float(thr), _dp(S), _dp(H), _dp(eri) if want_eri else None,
                            _dp(bounds), C.byref(nb))
    return {"S": S, "H": H, "eri": eri, "bounds": bounds[: nb.value], "primitives": rows}


def refcpu_ri_integrals(b: Basis, aux: Basis, thr=1e-12):
    """(P|Q), (mu nu|P) and the auxiliary primitive bounds from the reference's
    own RI kernels run on the CPU (bounds in the reference's primitive order)."""
    def cols(bb):
        rows = bb.reference_primitives()
        return (len(rows), np.array([r[1] for r in rows]), np.array([r[2] for r in rows]),
                np.ascontiguousarray(np.array([r[3] for r in rows])), np.array([r[0] for r in rows], np.int32),
                np.array([r[4] for r in rows], np.int64), np.array([r[5] for r in rows], np.int32))
    n, e, c, x, st, bi, ai = cols(b)
    an, ae, ac, ax, ast, abi, aai = cols(aux)
    M, N = aux.nbf, b.nbf
    V, T, qp = np.zeros((M, M)), np.zeros((M, N, N)), np.zeros(an)
    ll = lambda a: a.ctypes.data_as(C.POINTER(C.c_longlong))
    _ref().refcpu_ri_integrals(n, _dp(e), _dp(c), _dp(x), _ip(st), ll(bi), _ip(ai), _dp(b.cgto), N,
                               an, _dp(ae), _dp(ac), _dp(ax), _ip(ast), ll(abi), _ip(aai), _dp(aux.cgto), M,
                               C.c_double(thr), _dp(V), _dp(T), _dp(qp))
    return V, T, qp
