"""GB300-native Hartree-Fock hot path with the reference's API surface.

Python mirror of the reference's host classes (Molecular, ParameterManager,
HFBuilder, RHF) over the C ABI of libgansu_gb300.so.  Device buffers are torch
CUDA tensors; every compute call goes through the CUDA library, and there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from ._capi import (HF_CONV_DAMPING, HF_CONV_DIIS, HF_CONV_OPTIMAL_DAMPING, HF_EIGEN_PURIFICATION, HF_EIGEN_SYEVD, HF_GUESS_CORE, HF_GUESS_DENSITY, HF_GUESS_GWH,
                    HF_GUESS_SAD, HF_ERR_NOT_CONVERGED,
                    HF_ERI_DIRECT, HF_ERI_RI, HF_ERI_STORED, HF_PRECISION_FP64, HF_PRECISION_MIXED, Atom, HFError, PrimitiveShell, ScfOptions, ScfResult,
                    check, lib)

BASIS_DIR = Path(__file__).resolve().parent / "basis"
ANGSTROM_TO_BOHR = 1.8897259886

__all__ = [
    "Molecular", "Engine", "ParameterManager", "HFBuilder", "RHF", "HFError", "BASIS_DIR",
    "HF_PRECISION_FP64", "HF_PRECISION_MIXED", "HF_ERI_DIRECT", "HF_ERI_RI", "HF_ERI_STORED", "basis_path",
    "optimize_geometry", "energy_and_gradient_at", "Batch", "UHF", "HF_EIGEN_PURIFICATION", "HF_EIGEN_SYEVD",
    "HF_GUESS_CORE", "HF_GUESS_GWH", "HF_GUESS_DENSITY", "HF_GUESS_SAD", "HF_CONV_DIIS", "HF_CONV_DAMPING",
    "HF_CONV_OPTIMAL_DAMPING", "ROHF", "ROHF_COUPLINGS",
]


def basis_path(name: str) -> str:
    """Path of a bundled Gaussian basis file, e.g. basis_path('sto-3g')."""
    p = Path(name)
    if p.exists():
        return str(p)
    cand = BASIS_DIR / (name if name.endswith(".gbs") else name + ".gbs")
    if not cand.exists():
        raise FileNotFoundError(f"basis set {name!r} not found in {BASIS_DIR}")
    return str(cand)


class Molecular:
    """Mirror of gansu::Molecular (include/molecular.hpp:53-294)."""

    def __init__(self, atoms, gbs_filename: str, charge: int = 0, beta_to_alpha: int = 0):
        """atoms: iterable of (atomic_number, x, y, z) in bohr."""
        atoms = list(atoms)
        arr = (Atom * len(atoms))(*[Atom(int(z), float(x), float(y), float(w)) for z, x, y, w in atoms])
        h = C.c_void_p()
        check(lib().hf_molecule_from_atoms(arr, len(atoms), str(gbs_filename).encode(), charge, beta_to_alpha,
                                           C.byref(h)), "hf_molecule_from_atoms")
        self._init_from_handle(h)
        self.gbs_filename = str(gbs_filename)

    @classmethod
    def from_files(cls, xyz_filename: str, gbs_filename: str, charge: int = 0, beta_to_alpha: int = 0):
        h = C.c_void_p()
        check(lib().hf_molecule_from_files(str(xyz_filename).encode(), str(gbs_filename).encode(), charge,
                                           beta_to_alpha, C.byref(h)), "hf_molecule_from_files")
        obj = cls.__new__(cls)
        obj._init_from_handle(h)
        obj.gbs_filename = str(gbs_filename)
        return obj

    def _init_from_handle(self, h):
        L = lib()
        vals = [C.c_int() for _ in range(6)]
        check(L.hf_molecule_sizes(h, *[C.byref(v) for v in vals]), "hf_molecule_sizes")
        (self.num_basis, self.num_primitives, self.num_atoms, self.num_electrons, self.num_alpha_spins,
         self.num_beta_spins) = [v.value for v in vals]
        self._prims = (PrimitiveShell * self.num_primitives)()
        self._cgto = (C.c_double * self.num_basis)()
        self._atoms = (Atom * self.num_atoms)()
        check(L.hf_molecule_get(h, self._prims, self._cgto, self._atoms), "hf_molecule_get")
        L.hf_molecule_destroy(h)

    # getters named as in the reference
    def get_num_basis(self) -> int:
        return self.num_basis

    def get_num_electrons(self) -> int:
        return self.num_electrons

    def get_primitive_shells(self):
        return self._prims

    def get_cgto_normalization_factors(self) -> np.ndarray:
        return np.ctypeslib.as_array(self._cgto).copy()

    def get_atoms(self):
        return [(a.atomic_number, a.x, a.y, a.z) for a in self._atoms]

    def primitive_table(self) -> dict:
        """Primitive shells as numpy columns (exponent, coefficient, xyz, shell_type, basis_index, atom_index)."""
        p = self._prims
        return {
            "exponent": np.array([q.exponent for q in p]),
            "coefficient": np.array([q.coefficient for q in p]),
            "xyz": np.array([[q.x, q.y, q.z] for q in p]),
            "shell_type": np.array([q.shell_type for q in p], dtype=np.int32),
            "basis_index": np.array([q.basis_index for q in p], dtype=np.int64),
            "atom_index": np.array([q.atom_index for q in p], dtype=np.int32),
        }


def kernel_launch_count() -> int:
    """Kernels launched by libgansu_gb300 in this process."""
    return int(lib().hf_kernel_launch_count())


def measure_fma_peak(precision: int) -> float:
    """Sustained FMA TFLOP/s of the current GPU (0: FP64, 1: FP32)."""
    v = C.c_double()
    check(lib().hf_measure_fma_peak(precision, C.byref(v)), "hf_measure_fma_peak")
    return v.value


def _ptr(t) -> int:
    return 0 if t is None else int(t.data_ptr())


def _stream(stream) -> C.c_void_p:
    if stream is None:
        return C.c_void_p(0)
    return C.c_void_p(int(getattr(stream, "cuda_stream", stream)))


def _scf_options(options: dict | None):
    """hf_scf_options from a dict; guess_density_a/_b may be CUDA tensors (kept
    alive by the returned list for the duration of the call)."""
    opt = ScfOptions()
    lib().hf_scf_options_default(C.byref(opt))
    keep = []
    for k, v in (options or {}).items():
        if k in ("guess_density_a", "guess_density_b", "orthogonalizer"):
            if v is not None and not isinstance(v, int):
                v = v.contiguous().double()
                keep.append(v)
                v = int(v.data_ptr())
            setattr(opt, k, v)
        else:
            setattr(opt, k, v)
    return opt, keep


# ROHF coupling constants (A_cc, B_cc, A_oo, B_oo, A_vv, B_vv) by rohf_parameter_name (src/rohf.cu:30-39)
ROHF_COUPLINGS = {
    "roothaan": (-0.5, 1.5, 0.5, 0.5, 1.5, -0.5),
    "mcweeny-diercksen": (1.0 / 3.0, 2.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 2.0 / 3.0, 1.0 / 3.0),
    "davidson": (0.5, 1.0, 0.0, 1.0, 1.0, 0.0),
    "guest-saunders": (0.5, 0.5, 0.5, 0.5, 0.5, 0.5),
    "binkley-pople-dobosh": (0.5, 0.5, 1.0, 0.0, 0.0, 1.0),
    "faegri-manne": (0.5, 0.5, 1.0, 0.0, 0.5, 0.5),
    "goddard": (0.5, 0.5, 0.5, 0.0, 1.0, 0.0),
    "plakhutin-gorelik-breslavskaya": (0.0, 1.0, 1.0, 0.0, 1.0, 0.0),
}


class _FockScheduleMixin:
    """Launch schedule of the direct Fock build (hf_engine_set_fock_schedule,
    hf_engine_set_fock_grid_caps, hf_engine_autotune, hf_engine_fock_schedule);
    the analytic gradient's class launches use the same branches."""

    def set_fock_schedule(self, num_branches: int = 1, use_graph: bool = False, grid_caps=None):
        """Class launches on num_branches concurrent streams; use_graph replays each
        distinct build from a CUDA graph (single-molecule engines; for a batch, the
        SCF iteration's purified density step and Fock build).  grid_caps: a
        schedule from autotune() or fock_schedule() of an engine over the same
        molecules (cap_fp64, cap_fp32, branch lists), applied without timing, or
        "default" for 16 blocks per SM everywhere; None keeps the caps in force."""
        check(lib().hf_engine_set_fock_schedule(self._h, int(num_branches), 1 if use_graph else 0),
              "hf_engine_set_fock_schedule")
        if isinstance(grid_caps, str):
            if grid_caps != "default":
                raise ValueError(f"unknown grid_caps {grid_caps!r}")
            n = len(self.fock_schedule()["cap_fp64"])
            check(lib().hf_engine_set_fock_grid_caps(self._h, n, None, None, None), "hf_engine_set_fock_grid_caps")
        elif grid_caps is not None:
            k = len(grid_caps["cap_fp64"])
            arr = [(C.c_int * max(k, 1))(*grid_caps[key]) for key in ("cap_fp64", "cap_fp32", "branch")]
            check(lib().hf_engine_set_fock_grid_caps(self._h, k, *arr), "hf_engine_set_fock_grid_caps")

    def _schedule_density(self):
        raise NotImplementedError

    def autotune(self, D=None, stream=None) -> dict:
        """Chooses grid caps and the branch count by timing Fock builds on density D
        (the timed class lists do not depend on its values; default: zeros)."""
        from ._capi import AutotuneReport
        if D is None:
            D = self._schedule_density()
        rep = AutotuneReport()
        check(lib().hf_engine_autotune(self._h, _ptr(D), C.byref(rep), _stream(stream)), "hf_engine_autotune")
        out = {f: getattr(rep, f) for f, _ in AutotuneReport._fields_}
        out.update(self.fock_schedule())
        return out

    def purification_status(self) -> dict:
        """Diagnostics of the last RHF purification (hf_engine_purification_status)."""
        out = (C.c_double * 16)()
        check(lib().hf_engine_purification_status(self._h, out, 16), "hf_engine_purification_status")
        v = list(out)
        return {"sp2_steps": int(v[0]), "trace_error": v[1], "idempotency_error": v[2], "sp2_error": v[3],
                "sp2_converged": bool(v[4]), "mcweeny_steps": int(v[5]), "barrier_timeout": bool(v[6]),
                "barriers": int(v[7]),
                "phase_end_us": dict(zip(("fprime", "p0", "sp2", "mcweeny", "xp", "density"), v[8:14]))}

    def graph_stats(self) -> dict:
        """Graphs captured under use_graph (Fock builds, RHF purifications) and replays so far."""
        nf, npur, rep = C.c_int(), C.c_int(), C.c_longlong()
        check(lib().hf_engine_graph_stats(self._h, C.byref(nf), C.byref(npur), C.byref(rep)),
              "hf_engine_graph_stats")
        return {"fock_graphs": nf.value, "purification_graphs": npur.value, "replays": rep.value}

    def fock_schedule(self) -> dict:
        n = C.c_int()
        check(lib().hf_engine_fock_schedule(self._h, 0, C.byref(n), None, None, None), "hf_engine_fock_schedule")
        k = n.value
        c64, c32, br = (C.c_int * max(k, 1))(), (C.c_int * max(k, 1))(), (C.c_int * max(k, 1))()
        check(lib().hf_engine_fock_schedule(self._h, k, C.byref(n), c64, c32, br), "hf_engine_fock_schedule")
        return {"cap_fp64": list(c64)[:k], "cap_fp32": list(c32)[:k], "branch": list(br)[:k]}


class Engine(_FockScheduleMixin):
    """Device-resident integral engine (the ERI plugin's precomputation)."""

    def __init__(self, mol: Molecular, schwarz_screening_threshold: float = 1e-12):
        import torch  # device memory and streams

        self.torch = torch
        self.mol = mol
        self.N = mol.num_basis
        h = C.c_void_p()
        check(lib().hf_engine_create(mol._prims, mol.num_primitives, mol._cgto, mol.num_basis, mol._atoms,
                                     mol.num_atoms, float(schwarz_screening_threshold), C.byref(h)),
              "hf_engine_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().hf_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _empty(self, *shape):
        return self.torch.zeros(*shape, dtype=self.torch.float64, device="cuda")

    def stats(self) -> dict:
        ns, npair, nq = C.c_int(), C.c_longlong(), C.c_longlong()
        check(lib().hf_engine_stats(self._h, C.byref(ns), C.byref(npair), C.byref(nq)), "hf_engine_stats")
        return {"num_shells": ns.value, "num_shell_pairs": npair.value, "num_quartets": nq.value}

    def class_stats(self) -> list:
        n = C.c_int()
        check(lib().hf_engine_class_stats(self._h, 0, C.byref(n), None, None, None, None, None), "hf_engine_class_stats")
        k = n.value
        cl = (C.c_int * (4 * k))()
        arrs = [(C.c_longlong * k)() for _ in range(4)]
        check(lib().hf_engine_class_stats(self._h, k, C.byref(n), cl, *arrs), "hf_engine_class_stats")
        return [{"class": tuple(cl[4 * i:4 * i + 4]), "prim_fp64": arrs[0][i], "prim_fp32": arrs[1][i],
                 "contracted_fp64": arrs[2][i], "contracted_fp32": arrs[3][i]} for i in range(k)]

    def reset_stats(self):
        check(lib().hf_engine_reset_stats(self._h), "hf_engine_reset_stats")

    def h2d_bytes(self) -> int:
        v = C.c_longlong()
        check(lib().hf_engine_transfer_bytes(self._h, C.byref(v)), "hf_engine_transfer_bytes")
        return v.value

    def core_hamiltonian(self, stream=None):
        S, H = self._empty(self.N, self.N), self._empty(self.N, self.N)
        check(lib().hf_compute_core_hamiltonian(self._h, _ptr(S), _ptr(H), _stream(stream)),
              "hf_compute_core_hamiltonian")
        return S, H

    def primitive_pair_bounds(self) -> np.ndarray:
        n = self.mol.num_primitives
        out = np.zeros((n, n))
        check(lib().hf_primitive_pair_bounds(self._h, out.ctypes.data_as(C.POINTER(C.c_double))),
              "hf_primitive_pair_bounds")
        return out

    def eri_matrix(self, stream=None):
        eri = self._empty(self.N, self.N, self.N, self.N)
        check(lib().hf_compute_eri_matrix(self._h, _ptr(eri), _stream(stream)), "hf_compute_eri_matrix")
        return eri

    def fock_stored(self, D, H, eri, stream=None):
        F = self._empty(self.N, self.N)
        check(lib().hf_compute_fock_stored_rhf(_ptr(D), _ptr(H), _ptr(eri), _ptr(F), self.N, _stream(stream)),
              "hf_compute_fock_stored_rhf")
        return F

    def fock_direct(self, D, H, precision=HF_PRECISION_FP64, mixed_threshold=1e-7, out=None, stream=None):
        F = out if out is not None else self._empty(self.N, self.N)
        check(lib().hf_compute_fock_direct_rhf(self._h, _ptr(D), _ptr(H), _ptr(F), precision, mixed_threshold,
                                               _stream(stream)), "hf_compute_fock_direct_rhf")
        return F

    def jk(self, D, precision=HF_PRECISION_FP64, mixed_threshold=1e-7, stream=None):
        J, K = self._empty(self.N, self.N), self._empty(self.N, self.N)
        check(lib().hf_compute_jk_direct(self._h, _ptr(D), _ptr(J), _ptr(K), precision, mixed_threshold,
                                         _stream(stream)), "hf_compute_jk_direct")
        return J, K

    def _schedule_density(self):
        return self._empty(self.N, self.N).zero_()

    def diis_error(self, S, X, F, D, include_transform=False, stream=None):
        E = self._empty(self.N, self.N)
        check(lib().hf_compute_diis_error(self._h, _ptr(S), _ptr(X), _ptr(F), _ptr(D), _ptr(E),
                                          int(include_transform), _stream(stream)), "hf_compute_diis_error")
        return E

    def fock_diis(self, errors, focks, stream=None):
        m = errors.shape[0]
        F = self._empty(self.N, self.N)
        check(lib().hf_compute_fock_diis(self._h, _ptr(errors), _ptr(focks), _ptr(F), m, _stream(stream)),
              "hf_compute_fock_diis")
        return F

    def energy_weighted_density(self, coefficients, orbital_energies, num_occupied: int, stream=None):
        W = self._empty(self.N, self.N)
        check(lib().hf_energy_weighted_density(self._h, _ptr(coefficients), _ptr(orbital_energies), int(num_occupied),
                                               _ptr(W), _stream(stream)), "hf_energy_weighted_density")
        return W

    def gradient(self, density, energy_weighted_density, stream=None, mixed_threshold=None):
        """Analytic nuclear gradient (natom, 3) in Eh/bohr and its device time in ms.
        mixed_threshold: None for FP64, else the FP64/FP32 quartet cut."""
        g = np.zeros(3 * self.mol.num_atoms)
        ms = C.c_double()
        gp = g.ctypes.data_as(C.POINTER(C.c_double))
        if mixed_threshold is None:
            check(lib().hf_rhf_gradient(self._h, _ptr(density), _ptr(energy_weighted_density), gp, C.byref(ms),
                                        _stream(stream)), "hf_rhf_gradient")
        else:
            check(lib().hf_rhf_gradient_mixed(self._h, _ptr(density), _ptr(energy_weighted_density),
                                              float(mixed_threshold), gp, C.byref(ms), _stream(stream)),
                  "hf_rhf_gradient_mixed")
        return g.reshape(-1, 3), ms.value

    def gradient_ri(self, density, energy_weighted_density, coefficients, num_occupied: int, stream=None):
        """Analytic gradient of the RI energy (eri_method ri; hf_rhf_gradient_ri): (natom, 3) Eh/bohr, ms."""
        g = np.zeros(3 * self.mol.num_atoms)
        ms = C.c_double()
        check(lib().hf_rhf_gradient_ri(self._h, _ptr(density), _ptr(energy_weighted_density), _ptr(coefficients),
                                       int(num_occupied), g.ctypes.data_as(C.POINTER(C.c_double)), C.byref(ms),
                                       _stream(stream)), "hf_rhf_gradient_ri")
        return g.reshape(-1, 3), ms.value

    def uhf_scf(self, num_alpha: int, num_beta: int, options: dict | None = None, want_matrices: bool = False):
        """Unrestricted HF (hf_uhf_scf)."""
        opt, _keep = _scf_options(self._with_guess(options))
        res = ScfResult()
        outs = [self._empty(self.N, self.N), self._empty(self.N, self.N), self._empty(self.N),
                self._empty(self.N), self._empty(self.N, self.N),
                self._empty(self.N, self.N)] if want_matrices else [None] * 6
        st = lib().hf_uhf_scf(self._h, int(num_alpha), int(num_beta), C.byref(opt), C.byref(res),
                              *[_ptr(t) for t in outs])
        out = {f: getattr(res, f) for f, _ in ScfResult._fields_}
        out["status"] = st
        if st not in (0, 4):
            check(st, "hf_uhf_scf")
        if want_matrices:
            (out["density_alpha"], out["density_beta"], out["orbital_energies_alpha"], out["orbital_energies_beta"],
             out["coefficients_alpha"], out["coefficients_beta"]) = outs
        return out

    def sad_density(self, source: str = "auto"):
        """SAD alpha and beta densities of the molecule (CUDA tensors, N x N)."""
        from . import sad

        a, b = sad.sad_guess(self.mol, self.mol.gbs_filename, source)
        t = self.torch
        return t.from_numpy(a).to("cuda"), t.from_numpy(b).to("cuda")

    def spherical_orthogonalizer(self):
        """X over the pure (spherical-harmonic) functions (dft_gansu_gb300/spherical.py), CUDA N x N."""
        if getattr(self, "_x_pure", None) is None:
            from . import spherical

            S = self.core_hamiltonian()[0].double().cpu().numpy()
            X = spherical.orthogonalizer(S, spherical.transform(self.mol))
            self._x_pure = self.torch.from_numpy(X).to("cuda")
        return self._x_pure

    def _with_guess(self, options: dict | None) -> dict:
        """initial_guess SAD without densities: assemble them from the atoms;
        spherical=True: the pure-function orthogonaliser."""
        options = dict(options or {})
        if options.pop("spherical", False):
            options["orthogonalizer"] = self.spherical_orthogonalizer()
        if options.get("initial_guess") == HF_GUESS_SAD and options.get("guess_density_a") is None:
            options["guess_density_a"], options["guess_density_b"] = self.sad_density()
        return options

    def rohf_scf(self, num_alpha: int, num_beta: int, options: dict | None = None, want_matrices: bool = False,
                 coupling="roothaan"):
        """Restricted open-shell HF (hf_rohf_scf); coupling: a rohf_parameter_name or six constants."""
        opt, _keep = _scf_options(self._with_guess(options))
        cp = ROHF_COUPLINGS[coupling] if isinstance(coupling, str) else tuple(float(c) for c in coupling)
        cparr = (C.c_double * 6)(*cp)
        res = ScfResult()
        outs = [self._empty(self.N, self.N), self._empty(self.N, self.N), self._empty(self.N),
                self._empty(self.N, self.N)] if want_matrices else [None] * 4
        st = lib().hf_rohf_scf(self._h, int(num_alpha), int(num_beta), C.cast(cparr, C.c_void_p), C.byref(opt),
                               C.byref(res), *[_ptr(t) for t in outs])
        out = {f: getattr(res, f) for f, _ in ScfResult._fields_}
        out["status"] = st
        if st not in (0, 4):
            check(st, "hf_rohf_scf")
        if want_matrices:
            out["density_alpha"], out["density_beta"], out["orbital_energies"], out["coefficients"] = outs
        return out

    # ------------------------------------------------------------ RI
    def set_auxiliary_basis(self, aux: "Molecular"):
        """Attach the auxiliary basis (Molecular(atoms, auxiliary_gbsfilename))."""
        check(lib().hf_engine_set_auxiliary_basis(self._h, aux._prims, aux.num_primitives, aux._cgto, aux.num_basis),
              "hf_engine_set_auxiliary_basis")
        self.aux = aux
        self.naux = aux.num_basis

    def two_center_eris(self, stream=None):
        V = self._empty(self.naux, self.naux)
        check(lib().hf_compute_two_center_eris(self._h, _ptr(V), _stream(stream)), "hf_compute_two_center_eris")
        return V

    def three_center_eris(self, stream=None):
        T = self._empty(self.naux, self.N, self.N)
        check(lib().hf_compute_three_center_eris(self._h, _ptr(T), _stream(stream)), "hf_compute_three_center_eris")
        return T

    def ri_intermediate_b(self, want: bool = True, stream=None):
        B = self._empty(self.naux, self.N, self.N) if want else None
        check(lib().hf_compute_ri_intermediate_b(self._h, _ptr(B), _stream(stream)), "hf_compute_ri_intermediate_b")
        return B

    def jk_ri(self, density, stream=None):
        J, K = self._empty(self.N, self.N), self._empty(self.N, self.N)
        check(lib().hf_compute_jk_ri(self._h, _ptr(density), _ptr(J), _ptr(K), _stream(stream)), "hf_compute_jk_ri")
        return J, K

    def fock_ri(self, density, core_hamiltonian, stream=None):
        F = self._empty(self.N, self.N)
        check(lib().hf_compute_fock_ri_rhf(self._h, _ptr(density), _ptr(core_hamiltonian), _ptr(F), _stream(stream)),
              "hf_compute_fock_ri_rhf")
        return F

    def energy_and_gradient(self, num_electrons: int, options: dict | None = None):
        """Forward (SCF energy) and backward (analytic gradient) pair."""
        r = self.rhf_scf(num_electrons, options, want_matrices=True)
        W = self.energy_weighted_density(r["coefficients"], r["orbital_energies"], num_electrons // 2)
        if (options or {}).get("eri_method") == HF_ERI_RI:
            # the gradient of the RI energy (derivative three-centre and metric integrals)
            g, ms = self.gradient_ri(r["density"], W, r["coefficients"], num_electrons // 2)
        else:
            g, ms = self.gradient(r["density"], W)
        r["gradient"], r["gradient_ms"] = g, ms
        return r

    def rhf_scf(self, num_electrons: int, options: dict | None = None, want_matrices: bool = False):
        opt, _keep = _scf_options(self._with_guess(options))
        res = ScfResult()
        outs = [self._empty(self.N, self.N), self._empty(self.N, self.N), self._empty(self.N),
                self._empty(self.N, self.N)] if want_matrices else [None] * 4
        st = lib().hf_rhf_scf(self._h, int(num_electrons), C.byref(opt), C.byref(res), *[_ptr(t) for t in outs])
        out = {f: getattr(res, f) for f, _ in ScfResult._fields_}
        out["status"] = st
        if st not in (0, 4):
            check(st, "hf_rhf_scf")
        if want_matrices:
            out["density"], out["fock"], out["orbital_energies"], out["coefficients"] = outs
        return out


# ------------------------------------------------------------ parameters
_DEFAULTS = {
    "parameter_file": "", "xyzfilename": "", "gbsfilename": "", "verbose": "0", "method": "rhf", "charge": "0",
    "beta_to_alpha": "0", "eri_method": "stored", "auxiliary_gbsfilename": "", "maxiter": "100",
    "convergence_energy_threshold": "1e-6", "schwarz_screening_threshold": "1e-12", "initial_guess": "core",
    "convergence_method": "diis", "damping_factor": "0.9", "diis_size": "8", "diis_include_transform": "0",
    "rohf_parameter_name": "roothaan", "geometry_optimization": "0", "geometry_optimization_method": "powell",
    "export_sad_cache": "0",
    # added by this engine, same parsing rules
    "precision": "fp64", "mixed_threshold": "1e-7", "incremental_fock": "0", "spherical": "0",
    "eigensolver": "syevd",
}
_EIGENSOLVERS = {"syevd": HF_EIGEN_SYEVD, "syevj": 1, "purification": HF_EIGEN_PURIFICATION}
_SHORT = {"-m": "method", "-v": "verbose", "-p": "parameter_file", "-x": "xyzfilename", "-g": "gbsfilename",
          "-ag": "auxiliary_gbsfilename", "-c": "charge"}
_KEEP_CASE = {"xyzfilename", "gbsfilename", "parameter_file", "auxiliary_gbsfilename"}


class Batch(_FockScheduleMixin):
    """Many independent molecules in one engine (hf_engine_create_batch) and
    their RHF in lockstep (hf_batch_rhf_scf).  Molecules are ordered by
    (N, electrons) inside, so that equal sizes form batched linear-algebra
    groups; results come back in the caller's order."""

    def __init__(self, molecules, schwarz_screening_threshold: float = 1e-12):
        self.molecules = list(molecules)
        n = len(self.molecules)
        self.order = sorted(range(n), key=lambda i: (self.molecules[i].num_basis, self.molecules[i].num_electrons))
        ms = [self.molecules[i] for i in self.order]
        P = C.c_void_p * n
        I = C.c_int * n
        h = C.c_void_p()
        check(lib().hf_engine_create_batch(
            n, P(*[C.cast(m._prims, C.c_void_p) for m in ms]), I(*[m.num_primitives for m in ms]),
            P(*[C.cast(m._cgto, C.c_void_p) for m in ms]), I(*[m.num_basis for m in ms]),
            P(*[C.cast(m._atoms, C.c_void_p) for m in ms]), I(*[m.num_atoms for m in ms]),
            float(schwarz_screening_threshold), C.byref(h)), "hf_engine_create_batch")
        self._h = h
        self._sorted = ms

    def close(self):
        if getattr(self, "_h", None):
            lib().hf_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _schedule_density(self):
        import torch
        return torch.zeros(sum(m.num_basis ** 2 for m in self._sorted), dtype=torch.float64, device="cuda")

    def sad_density(self, source: str = "auto"):
        """SAD alpha and beta densities of every molecule in the block layout (CUDA tensors)."""
        import torch

        from . import sad

        pa, pb = [], []
        for m in self._sorted:
            a, b = sad.sad_guess(m, m.gbs_filename, source)
            pa.append(a.ravel())
            pb.append(b.ravel())
        return torch.from_numpy(np.concatenate(pa)).to("cuda"), torch.from_numpy(np.concatenate(pb)).to("cuda")

    def rhf_scf(self, options: dict | None = None):
        """Returns (per-molecule result dicts in the caller's order, batch ms, batch iterations).
        initial_guess HF_GUESS_SAD without guess densities assembles them (sad_density)."""
        options = dict(options or {})
        if options.get("initial_guess") == HF_GUESS_SAD and options.get("guess_density_a") is None:
            options["guess_density_a"], options["guess_density_b"] = self.sad_density()
        opt, _keep = _scf_options(options)
        n = len(self._sorted)
        res = (ScfResult * n)()
        ne = (C.c_int * n)(*[m.num_electrons for m in self._sorted])
        ms, it = C.c_double(), C.c_int()
        st = lib().hf_batch_rhf_scf(self._h, ne, C.byref(opt), res, C.byref(ms), C.byref(it))
        if st not in (0, 4):
            check(st, "hf_batch_rhf_scf")
        out = [None] * n
        for k, i in enumerate(self.order):
            out[i] = {f: getattr(res[k], f) for f, _ in ScfResult._fields_}
            out[i]["status"] = st
        return out, ms.value, it.value


class ParameterManager:
    """Mirror of gansu::ParameterManager (src/parameter_manager.cpp:40-224):
    string values with defaults, short options, ``key = value`` recipes,
    values lower-cased except file names, unknown keys rejected."""

    def __init__(self, set_default_values: bool = True):
        self._p: dict[str, str] = dict(_DEFAULTS) if set_default_values else {}

    def __setitem__(self, key, value):
        if key not in _DEFAULTS:
            raise KeyError(f"Unknown parameter: {key}")
        v = str(value)
        self._p[key] = v if key in _KEEP_CASE else v.lower()

    def __getitem__(self, key):
        return self._p[key]

    def get(self, key, typ=str):
        v = self._p[key]
        if typ is bool:
            return v not in ("0", "false", "")
        return typ(v)

    def parse_command_line_args(self, argv):
        i = 0
        while i < len(argv):
            k = argv[i]
            key = _SHORT.get(k, k[2:] if k.startswith("--") else None)
            if key is None or i + 1 >= len(argv):
                raise KeyError(f"Invalid option: {k}")
            self[key] = argv[i + 1]
            i += 2
        if self._p.get("parameter_file"):
            self.load_from_file(self._p["parameter_file"], override=False)

    def load_from_file(self, path, override=True):
        for line in Path(path).read_text().splitlines():
            line = line.split("#", 1)[0].strip()
            if not line or "=" not in line:
                continue
            k, v = (s.strip() for s in line.split("=", 1))
            if k not in _DEFAULTS:
                raise KeyError(f"Unknown parameter: {k}")
            if override or self._p.get(k, _DEFAULTS[k]) == _DEFAULTS[k]:
                self[k] = v


_GUESSES = {"core": HF_GUESS_CORE, "gwh": HF_GUESS_GWH, "density": HF_GUESS_DENSITY, "sad": HF_GUESS_SAD}
_CONVERGENCE = {"diis": HF_CONV_DIIS, "damping": HF_CONV_DAMPING, "optimaldamping": HF_CONV_OPTIMAL_DAMPING}


class _HFBase:
    """The parts of gansu::HF (include/hf.hpp, src/hf.cu) shared by the RHF, UHF
    and ROHF mirrors: parameter checks, the engine (and the auxiliary basis for
    eri_method ri, src/rhf.cu:76-79), the SCF options and the guess densities."""

    _stored_tensor = False  # eri_method stored keeps an N^4 tensor (RHF)

    def __init__(self, molecular: Molecular, parameters: ParameterManager):
        self.mol = molecular
        self.params = parameters
        method = parameters["eri_method"]
        if method not in ("stored", "direct", "ri"):
            raise ValueError(f"Invalid ERI method name: {method}")
        if parameters["convergence_method"] not in _CONVERGENCE:
            raise ValueError(f"Invalid convergence_method: {parameters['convergence_method']}")
        if parameters["initial_guess"] not in _GUESSES:
            raise ValueError(f"Invalid initial guess method: {parameters['initial_guess']}")
        if parameters["initial_guess"] == "sad" and not parameters["gbsfilename"] and \
                not getattr(molecular, "gbs_filename", ""):
            raise ValueError("The basis set file is not specified for SAD initial guess method.")
        self.engine = Engine(molecular, parameters.get("schwarz_screening_threshold", float))
        # stored: the conventional RHF build from the N^4 tensor (ERI_Stored_RHF), FP64; the
        # UHF and ROHF mirrors and the mixed tier build the same Fock matrices directly
        stored = self._stored_tensor and parameters["precision"] != "mixed"
        self.eri_method = {"ri": HF_ERI_RI, "direct": HF_ERI_DIRECT}.get(
            method, HF_ERI_STORED if stored else HF_ERI_DIRECT)
        if method == "ri":
            atoms = [(a.atomic_number, a.x, a.y, a.z) for a in molecular._atoms]
            self.auxiliary = Molecular(atoms, parameters["auxiliary_gbsfilename"])
            self.engine.set_auxiliary_basis(self.auxiliary)
        self.result = None

    def _options(self, density_alpha=None, density_beta=None, force_density=False) -> dict:
        p = self.params
        guess = p["initial_guess"]
        if force_density:
            guess = "density"
        opts = {
            "max_iter": p.get("maxiter", int),
            "convergence_threshold": p.get("convergence_energy_threshold", float),
            "diis_size": p.get("diis_size", int),
            "diis_include_transform": int(p.get("diis_include_transform", bool)),
            "precision": HF_PRECISION_MIXED if p["precision"] == "mixed" else HF_PRECISION_FP64,
            "mixed_threshold": p.get("mixed_threshold", float),
            "verbose": p.get("verbose", int),
            "eri_method": self.eri_method,
            "initial_guess": _GUESSES[guess],
            "spherical": bool(p.get("spherical", bool)),
            "convergence_method": _CONVERGENCE[p["convergence_method"]],
            "damping_factor": p.get("damping_factor", float),
            "eigensolver": _EIGENSOLVERS[p["eigensolver"]],
        }
        if guess == "density":
            if density_alpha is None or density_beta is None:
                # guess_initial_fock_matrix falls back to the core guess (src/rhf.cu:129-132)
                opts["initial_guess"] = HF_GUESS_CORE
            else:
                t = self.engine.torch
                opts["guess_density_a"] = t.as_tensor(np.asarray(density_alpha, float).reshape(self.mol.num_basis, -1)).to("cuda")
                opts["guess_density_b"] = t.as_tensor(np.asarray(density_beta, float).reshape(self.mol.num_basis, -1)).to("cuda")
        return opts

    def get_total_energy(self) -> float:
        return self.result["total_energy"]

    def get_energy(self) -> float:
        return self.result["electronic_energy"]

    def get_nuclear_repulsion_energy(self) -> float:
        return self.result["nuclear_repulsion"]

    def report(self) -> str:
        r = self.result
        return (f"Total energy: {r['total_energy']:.12f}\nIterations: {r['iterations']}\n"
                f"Converged: {bool(r['converged'])}\n")

    def export_sad_cache(self, filename: str = "temp_sad_cache.dat") -> None:
        """HF::generate_sad_cache (include/hf.hpp:372-405) of the solved molecule."""
        from . import sad

        Da, Db = self.export_density_matrix()
        sad.export_sad_cache(filename, Da, Db)

    def export_molden_file(self, filename: str = "output.molden") -> None:
        """export_molden_file (src/rhf.cu:363-425 and the UHF/ROHF variants)."""
        from . import molden

        molden.write_molden(filename, self.mol, self._orbital_sets())

    def analyze_mulliken_population(self) -> np.ndarray:
        """Mulliken atomic charges (analyze_mulliken_population, src/rhf.cu:427-460)."""
        from . import molden

        Da, Db = self.export_density_matrix()
        S = self.engine.core_hamiltonian()[0].double().cpu().numpy()
        return molden.mulliken_charges(self.mol, Da + Db, S)

    @staticmethod
    def _np(t):
        return t.double().cpu().numpy()


class RHF(_HFBase):
    """Mirror of gansu::RHF (include/rhf.hpp, src/rhf.cu): ``solve()`` runs the
    SCF on the GPU.  ``stored`` (the default) computes the N^4 ERI tensor once
    and builds F from it every iteration (ERI_Stored_RHF; FP64), ``direct`` runs
    the fused direct build (no tensor), ``ri`` uses Molecular(atoms,
    auxiliary_gbsfilename).
    Guesses core / gwh / density / sad (include/rhf.hpp:378-588)."""

    _stored_tensor = True

    def __init__(self, molecular: Molecular, parameters: ParameterManager):
        if molecular.num_alpha_spins != molecular.num_beta_spins:
            raise ValueError("In restricted Hartree Fock method, the number of alpha and beta electrons should be equal.")
        super().__init__(molecular, parameters)

    def solve(self, density_matrix_alpha=None, density_matrix_beta=None, force_density: bool = False) -> float:
        opts = self._options(density_matrix_alpha, density_matrix_beta, force_density)
        opts["incremental"] = int(self.params.get("incremental_fock", bool))
        self.result = self.engine.rhf_scf(self.mol.num_electrons, opts, want_matrices=True)
        return self.result["total_energy"]

    def export_density_matrix(self):
        """alpha = beta = D/2 (RHF::export_density_matrix)."""
        D = self.result["density"].double().cpu().numpy()
        return 0.5 * D, 0.5 * D

    def _orbital_sets(self):
        n, nocc = self.mol.num_basis, self.mol.num_electrons // 2
        occ = np.where(np.arange(n) < nocc, 2.0, 0.0)
        return [("Alpha", self._np(self.result["orbital_energies"]), self._np(self.result["coefficients"]), occ)]


class UHF(_HFBase):
    """Mirror of gansu::UHF (include/uhf.hpp, src/uhf.cu): ``solve()`` runs
    hf_uhf_scf for the molecule's alpha/beta counts (direct or RI)."""

    def solve(self, density_matrix_alpha=None, density_matrix_beta=None, force_density: bool = False) -> float:
        opts = self._options(density_matrix_alpha, density_matrix_beta, force_density)
        self.result = self.engine.uhf_scf(self.mol.num_alpha_spins, self.mol.num_beta_spins, opts,
                                          want_matrices=True)
        return self.result["total_energy"]

    def export_density_matrix(self):
        return (self.result["density_alpha"].double().cpu().numpy(),
                self.result["density_beta"].double().cpu().numpy())

    def _orbital_sets(self):
        n, r = self.mol.num_basis, self.result
        idx = np.arange(n)
        return [("Alpha", self._np(r["orbital_energies_alpha"]), self._np(r["coefficients_alpha"]),
                 np.where(idx < self.mol.num_alpha_spins, 1.0, 0.0)),
                ("Beta", self._np(r["orbital_energies_beta"]), self._np(r["coefficients_beta"]),
                 np.where(idx < self.mol.num_beta_spins, 1.0, 0.0))]


class ROHF(_HFBase):
    """Mirror of gansu::ROHF (include/rohf.hpp, src/rohf.cu): ``solve()`` runs
    hf_rohf_scf with the coupling constants of rohf_parameter_name."""

    def __init__(self, molecular: Molecular, parameters: ParameterManager):
        name = parameters["rohf_parameter_name"]
        if name not in ROHF_COUPLINGS:
            raise ValueError(f"Invalid ROHF parameter name: {name}")
        if molecular.num_alpha_spins > molecular.num_basis or molecular.num_beta_spins > molecular.num_basis:
            raise ValueError("The number of alpha or beta electrons should be less than or equal to the number of "
                             "basis functions.")
        super().__init__(molecular, parameters)
        self.coupling = ROHF_COUPLINGS[name]

    def solve(self, density_matrix_alpha=None, density_matrix_beta=None, force_density: bool = False) -> float:
        opts = self._options(density_matrix_alpha, density_matrix_beta, force_density)
        self.result = self.engine.rohf_scf(self.mol.num_alpha_spins, self.mol.num_beta_spins, opts,
                                           want_matrices=True, coupling=self.coupling)
        return self.result["total_energy"]

    def export_density_matrix(self):
        return (self.result["density_alpha"].double().cpu().numpy(),
                self.result["density_beta"].double().cpu().numpy())

    def _orbital_sets(self):
        n, r = self.mol.num_basis, self.result
        idx = np.arange(n)
        occ = np.where(idx < self.mol.num_beta_spins, 2.0, np.where(idx < self.mol.num_alpha_spins, 1.0, 0.0))
        return [("Alpha", self._np(r["orbital_energies"]), self._np(r["coefficients"]), occ)]

    def get_total_spin(self) -> float:
        """S(S+1) with S = (open orbitals)/2 (ROHF::get_total_spin)."""
        no = self.mol.num_alpha_spins - self.mol.num_beta_spins
        return (no / 2.0) * (no / 2.0 + 1.0)


class HFBuilder:
    """Mirror of gansu::HFBuilder::buildHF (include/builder.hpp:43-106)."""

    @staticmethod
    def buildHF(parameters: ParameterManager):
        method = parameters["method"]
        if method not in ("rhf", "uhf", "rohf"):
            raise ValueError(f"Invalid method: {method}")
        mol = Molecular.from_files(parameters["xyzfilename"], parameters["gbsfilename"],
                                   parameters.get("charge", int), parameters.get("beta_to_alpha", int))
        return {"rhf": RHF, "uhf": UHF, "rohf": ROHF}[method](mol, parameters)

    @staticmethod
    def buildOtimizer(parameters: ParameterManager) -> float:
        """Geometry optimisation with the analytic gradient; same entry point and
        return value (the final total energy) as gansu::HFBuilder::buildOtimizer
        (include/builder.hpp:108-275), which instead searches each coordinate of
        atoms 1.. with energy-only step halving.  The first atom stays fixed as
        there.  BFGS on the Cartesian coordinates with a backtracking line search;
        converged when max|gradient| < 1e-4 Eh/bohr and |dE| < 1e-6 Eh."""
        if parameters["method"] != "rhf":
            raise ValueError("geometry optimisation is provided for RHF")
        mol = Molecular.from_files(parameters["xyzfilename"], parameters["gbsfilename"],
                                   parameters.get("charge", int), parameters.get("beta_to_alpha", int))
        atoms = [(a.atomic_number, a.x, a.y, a.z) for a in mol._atoms]
        opts = {"convergence_threshold": min(parameters.get("convergence_energy_threshold", float), 1e-9),
                "max_iter": parameters.get("maxiter", int)}
        energy, _, _ = optimize_geometry(atoms, parameters["gbsfilename"], opts,
                                         charge=parameters.get("charge", int),
                                         schwarz=parameters.get("schwarz_screening_threshold", float))
        return energy


def energy_and_gradient_at(atoms, gbs_filename: str, scf_options: dict | None = None, charge: int = 0,
                           schwarz: float = 1e-12):
    """Total energy (Eh) and analytic gradient (natom x 3, Eh/bohr) of one geometry."""
    mol = Molecular(atoms, gbs_filename, charge)
    eng = Engine(mol, schwarz)
    try:
        r = eng.energy_and_gradient(mol.num_electrons, scf_options)
        if r["converged"] != 1:
            raise HFError(HF_ERR_NOT_CONVERGED, "energy_and_gradient_at", "SCF did not converge")
        return r["total_energy"], np.array(r["gradient"])
    finally:
        eng.close()


def optimize_geometry(atoms, gbs_filename: str, scf_options: dict | None = None, charge: int = 0,
                      schwarz: float = 1e-12, gtol: float = 1e-4, etol: float = 1e-6, max_steps: int = 100,
                      fixed_first_atom: bool = True):
    """BFGS minimisation of the RHF energy over Cartesian coordinates (bohr).
    Returns (energy, atoms, history of (energy, max|g|))."""
    Z = [int(a[0]) for a in atoms]
    x = np.array([a[1:] for a in atoms], dtype=float).ravel()
    mask = np.ones_like(x)
    if fixed_first_atom:
        mask[:3] = 0.0

    def evaluate(xv):
        e, g = energy_and_gradient_at([(z, *xv[3 * i:3 * i + 3]) for i, z in enumerate(Z)], gbs_filename,
                                      scf_options, charge, schwarz)
        return e, g.ravel() * mask

    e, g = evaluate(x)
    Hinv = np.eye(x.size) * 0.5  # initial inverse Hessian (bohr^2/Eh), a stiff-bond guess
    history = [(e, float(np.abs(g).max()))]
    for _ in range(max_steps):
        if np.abs(g).max() < gtol:
            break
        p = -Hinv @ g
        step = np.abs(p).max()
        if step > 0.3:  # trust radius in bohr
            p *= 0.3 / step
        t, e_new, g_new = 1.0, None, None
        for _ls in range(20):
            e_new, g_new = evaluate(x + t * p)
            if e_new <= e + 1e-4 * t * float(g @ p):
                break
            t *= 0.5
        s_vec, y_vec = t * p, g_new - g
        x, de, e, g = x + s_vec, e_new - e, e_new, g_new
        history.append((e, float(np.abs(g).max())))
        sy = float(s_vec @ y_vec)
        if sy > 1e-12:
            rho = 1.0 / sy
            I = np.eye(x.size)
            Hinv = (I - rho * np.outer(s_vec, y_vec)) @ Hinv @ (I - rho * np.outer(y_vec, s_vec)) + \
                rho * np.outer(s_vec, s_vec)
        if np.abs(g).max() < gtol and abs(de) < etol:
            break
    final = [(z, *x[3 * i:3 * i + 3]) for i, z in enumerate(Z)]
    return e, final, history
