"""The allocation-free DIIS entry point (hf_compute_fock_diis_noalloc).

It serves callers that cannot allocate device memory during an SCF step (a
CUDA graph being recorded, an application that owns all device memory through
its own pool, a thread that must not synchronise the device).  The test calls
it through the C ABI twice in a row, with different inputs, and compares each
result with the engine-based hf_compute_fock_diis (tolerance 1e-11 absolute),
so a result that leaked from the shared static scratch of the first call would
show in the second.  Collected last (file name) so a failure here comes after
every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from dft_gansu_gb300._capi import HF_ERR_INVALID_ARGUMENT, lib

pytestmark = pytest.mark.gpu


def _call_noalloc(errs, focks, out):
    n = errs.shape[-1]
    return lib().hf_compute_fock_diis_noalloc(errs.data_ptr(), focks.data_ptr(), out.data_ptr(), errs.shape[0], n,
                                              C.c_void_p(0))


def test_noalloc_diis_matches_engine_entry_point(built_library, cuda):
    torch = cuda
    mol = gg.Molecular(geometry.water(), gg.basis_path("6-31g_st"))
    eng = gg.Engine(mol)
    n = mol.num_basis
    rng = np.random.default_rng(11)
    for m in (5, 8):  # two calls in a row, different sizes and data
        errs = torch.tensor(rng.normal(size=(m, n, n)), device="cuda")
        f = rng.normal(size=(m, n, n))
        focks = torch.tensor(f + f.transpose(0, 2, 1), device="cuda")
        out = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        assert _call_noalloc(errs, focks, out) == 0, lib().hf_last_error()
        ref = eng.fock_diis(errs, focks)
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), ref.cpu().numpy(), atol=1e-11, rtol=0)


def test_noalloc_diis_rejects_more_pairs_than_its_scratch(built_library, cuda):
    torch = cuda
    n = 4
    errs = torch.zeros((17, n, n), dtype=torch.float64, device="cuda")
    out = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    assert _call_noalloc(errs, errs, out) == HF_ERR_INVALID_ARGUMENT
    assert b"between 2 and 16" in lib().hf_last_error()


def test_noalloc_diis_dependent_error_vectors(built_library, cuda):
    """A repeated error vector gets weight 0 in both DIIS entry points, so the
    extrapolation is the one over the distinct vectors and never zero."""
    torch = cuda
    mol = gg.Molecular(geometry.water(), gg.basis_path("6-31g_st"))
    eng = gg.Engine(mol)
    n = mol.num_basis
    rng = np.random.default_rng(12)
    e = [rng.normal(size=(n, n)) for _ in range(2)]
    f = rng.normal(size=(3, n, n))
    f = f + f.transpose(0, 2, 1)
    errs = torch.tensor(np.stack([e[0], e[1], e[1]]), device="cuda")
    focks = torch.tensor(f, device="cuda")
    for _ in range(2):  # twice in a row: the shared scratch keeps nothing between calls
        out = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        assert _call_noalloc(errs, focks, out) == 0, lib().hf_last_error()
        ref = eng.fock_diis(errs, focks)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, ref.cpu().numpy(), atol=1e-11, rtol=0)
        assert np.abs(got).max() > 0.1
