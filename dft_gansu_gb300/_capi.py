"""ctypes declarations of the C ABI in include/gansu_gb300.h.

The shared object is the in-tree build (dft_gansu_gb300/libgansu_gb300.so).
There is no fallback: if the library is missing or cannot be loaded,
``lib()`` raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgansu_gb300.so"

HF_OK = 0
HF_ERR_INVALID_ARGUMENT = 1
HF_ERR_CUDA = 2
HF_ERR_OUT_OF_MEMORY = 3
HF_ERR_NOT_CONVERGED = 4
HF_ERR_SOLVER = 5
HF_ERR_IO = 6
HF_ERR_NOT_SPD = 7

HF_PRECISION_FP64 = 0
HF_PRECISION_MIXED = 1
HF_ERI_DIRECT = 0
HF_ERI_RI = 1
HF_ERI_STORED = 2
HF_GUESS_CORE = 0
HF_GUESS_GWH = 1
HF_GUESS_DENSITY = 2
HF_GUESS_SAD = 3
HF_CONV_DIIS = 0
HF_CONV_DAMPING = 1
HF_CONV_OPTIMAL_DAMPING = 2
HF_EIGEN_SYEVD = 0
HF_EIGEN_SYEVJ = 1
HF_EIGEN_PURIFICATION = 2


class PrimitiveShell(C.Structure):
    """Binary layout of gansu::PrimitiveShell (include/types.hpp:116-125)."""

    _fields_ = [
        ("exponent", C.c_double),
        ("coefficient", C.c_double),
        ("x", C.c_double),
        ("y", C.c_double),
        ("z", C.c_double),
        ("shell_type", C.c_int),
        ("basis_index", C.c_size_t),
        ("atom_index", C.c_int),
    ]


class Atom(C.Structure):
    """Binary layout of gansu::Atom (include/types.hpp:131-135), bohr."""

    _fields_ = [("atomic_number", C.c_int), ("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class ScfOptions(C.Structure):
    _fields_ = [
        ("max_iter", C.c_int),
        ("convergence_threshold", C.c_double),
        ("diis_size", C.c_int),
        ("diis_include_transform", C.c_int),
        ("precision", C.c_int),
        ("mixed_threshold", C.c_double),
        ("incremental", C.c_int),
        ("rebuild_every", C.c_int),
        ("full_build_precision", C.c_int),
        ("eigensolver", C.c_int),
        ("verbose", C.c_int),
        ("eri_method", C.c_int),
        ("anchor_threshold", C.c_double),
        ("initial_guess", C.c_int),
        ("guess_density_a", C.c_void_p),
        ("guess_density_b", C.c_void_p),
        ("orthogonalizer", C.c_void_p),
        ("convergence_method", C.c_int),
        ("damping_factor", C.c_double),
        ("purification_max_steps", C.c_int),
        ("anchor_mixed_threshold", C.c_double),
        ("incremental_drop", C.c_double),
        ("pre_anchor_drop", C.c_double),
    ]


class ScfResult(C.Structure):
    _fields_ = [
        ("electronic_energy", C.c_double),
        ("nuclear_repulsion", C.c_double),
        ("total_energy", C.c_double),
        ("iterations", C.c_int),
        ("converged", C.c_int),
        ("fock_ms_total", C.c_double),
        ("scf_ms_total", C.c_double),
        ("setup_ms", C.c_double),
        ("diag_ms_total", C.c_double),
        ("diis_ms_total", C.c_double),
        ("fp64_quartets", C.c_longlong),
        ("fp32_quartets", C.c_longlong),
        ("eigensolver_used", C.c_int),
    ]


class AutotuneReport(C.Structure):
    _fields_ = [
        ("build_ms_default", C.c_double),
        ("build_ms_tuned", C.c_double),
        ("num_branches", C.c_int),
        ("num_class_pairs", C.c_int),
        ("num_caps_changed", C.c_int),
    ]


_P = C.c_void_p
_I = C.c_int
_D = C.c_double

# name -> (restype, argtypes); every symbol declared in include/gansu_gb300.h
SIGNATURES = {
    "hf_last_error": (C.c_char_p, []),
    "hf_version": (C.c_char_p, []),
    "hf_molecule_from_files": (_I, [C.c_char_p, C.c_char_p, _I, _I, C.POINTER(_P)]),
    "hf_molecule_from_atoms": (_I, [C.POINTER(Atom), _I, C.c_char_p, _I, _I, C.POINTER(_P)]),
    "hf_molecule_destroy": (None, [_P]),
    "hf_molecule_sizes": (_I, [_P] + [C.POINTER(_I)] * 6),
    "hf_molecule_get": (_I, [_P, C.POINTER(PrimitiveShell), C.POINTER(_D), C.POINTER(Atom)]),
    "hf_engine_create": (_I, [C.POINTER(PrimitiveShell), _I, C.POINTER(_D), _I, C.POINTER(Atom), _I, _D,
                              C.POINTER(_P)]),
    "hf_engine_destroy": (None, [_P]),
    "hf_engine_stats": (_I, [_P, C.POINTER(_I), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "hf_engine_class_stats": (_I, [_P, _I, C.POINTER(_I), C.POINTER(_I)] + [C.POINTER(C.c_longlong)] * 4),
    "hf_engine_reset_stats": (_I, [_P]),
    "hf_engine_transfer_bytes": (_I, [_P, C.POINTER(C.c_longlong)]),
    "hf_kernel_launch_count": (C.c_longlong, []),
    "hf_measure_fma_peak": (_I, [_I, C.POINTER(_D)]),
    "hf_compute_core_hamiltonian": (_I, [_P, _P, _P, _P]),
    "hf_primitive_pair_bounds": (_I, [_P, C.POINTER(_D)]),
    "hf_compute_eri_matrix": (_I, [_P, _P, _P]),
    "hf_compute_fock_stored_rhf": (_I, [_P, _P, _P, _P, _I, _P]),
    "hf_compute_fock_direct_rhf": (_I, [_P, _P, _P, _P, _I, _D, _P]),
    "hf_compute_jk_direct": (_I, [_P, _P, _P, _P, _I, _D, _P]),
    "hf_engine_set_fock_schedule": (_I, [_P, _I, _I]),
    "hf_engine_set_fock_grid_caps": (_I, [_P, _I, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    "hf_engine_autotune": (_I, [_P, _P, C.POINTER(AutotuneReport), _P]),
    "hf_engine_graph_stats": (_I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_longlong)]),
    "hf_engine_fock_schedule": (_I, [_P, _I, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    "hf_compute_diis_error": (_I, [_P, _P, _P, _P, _P, _P, _I, _P]),
    "hf_compute_fock_diis": (_I, [_P, _P, _P, _P, _I, _P]),
    "hf_compute_fock_diis_noalloc": (_I, [_P, _P, _P, _I, _I, _P]),
    "hf_combine_uhf_fock": (_I, [_P, _P, _P, _P, _P, _P, _P, _I, _P]),
    "hf_engine_purification_status": (_I, [_P, _P, _I]),
    "hf_rhf_gradient_ri": (_I, [_P, _P, _P, _P, _I, _P, _P, _P]),
    "hf_energy_weighted_density": (_I, [_P, _P, _P, _I, _P, _P]),
    "hf_rhf_gradient": (_I, [_P, _P, _P, C.POINTER(_D), C.POINTER(_D), _P]),
    "hf_rhf_gradient_mixed": (_I, [_P, _P, _P, _D, C.POINTER(_D), C.POINTER(_D), _P]),
    "hf_engine_set_auxiliary_basis": (_I, [_P, _P, _I, _P, _I]),
    "hf_compute_two_center_eris": (_I, [_P, _P, _P]),
    "hf_compute_three_center_eris": (_I, [_P, _P, _P]),
    "hf_compute_ri_intermediate_b": (_I, [_P, _P, _P]),
    "hf_compute_fock_ri_rhf": (_I, [_P, _P, _P, _P, _P]),
    "hf_compute_jk_ri": (_I, [_P, _P, _P, _P, _P]),
    "hf_split_bf16_matmul": (_I, [_P, _P, _P, _I, _I, _I, _I, _P]),
    "hf_engine_create_batch": (_I, [_I, _P, _P, _P, _P, _P, _P, _D, _P]),
    "hf_uhf_scf": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "hf_rohf_scf": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "hf_batch_rhf_scf": (_I, [_P, _P, _P, _P, _P, _P]),
    "hf_scf_options_default": (None, [C.POINTER(ScfOptions)]),
    "hf_rhf_scf": (_I, [_P, _I, C.POINTER(ScfOptions), C.POINTER(ScfResult), _P, _P, _P, _P]),
}

_lib = None


class HFError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where} failed with status {status}: {msg}")
        self.status = status


def lib() -> C.CDLL:
    """Load the in-tree library (raises if it is not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built; run dft_gansu_gb300.build.build() first")
        handle = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(status: int, where: str) -> None:
    if status != HF_OK:
        raise HFError(status, where, lib().hf_last_error().decode())
