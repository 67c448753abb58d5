"""Split-BF16 tcgen05 GEMM (hf_split_bf16_matmul) against an FP64 numpy product.

Three BF16 products (hi*hi + hi*lo + lo*hi) with FP32 accumulation carry
about 16-17 significant bits: the bound used is 5e-5 of the largest element
of the exact product, far inside one BF16 product's error (~4e-3) so that a
missing term or a wrong descriptor fails.
"""
import ctypes as C

import numpy as np
import pytest

from dft_gansu_gb300._capi import lib

pytestmark = pytest.mark.gpu
TOL = 5e-5


def _run(A, B, mode, m, n, k):
    import torch
    a = torch.tensor(A, dtype=torch.float64, device="cuda")
    b = torch.tensor(B, dtype=torch.float64, device="cuda") if B is not None else None
    c = torch.zeros((m, n), dtype=torch.float64, device="cuda")
    st = lib().hf_split_bf16_matmul(a.data_ptr(), 0 if b is None else b.data_ptr(), c.data_ptr(), m, n, k, mode,
                                    C.c_void_p(0))
    assert st == 0, lib().hf_last_error().decode()
    return c.cpu().numpy()


@pytest.mark.parametrize("m,n,k", [(128, 192, 64), (300, 180, 200), (1000, 37, 900)])
def test_split_store_product(built_library, cuda, m, n, k):
    rng = np.random.default_rng(m + n + k)
    A, B = rng.normal(size=(m, k)), rng.normal(size=(n, k))
    ref = A @ B.T
    got = _run(A, B, 0, m, n, k)
    assert np.abs(got - ref).max() < TOL * np.abs(ref).max()


@pytest.mark.parametrize("m,k", [(128, 64), (200, 1000), (333, 4100)])
def test_symmetric_product(built_library, cuda, m, k):
    rng = np.random.default_rng(m * k)
    A = rng.normal(size=(m, k))
    ref = A @ A.T
    got = _run(A, None, 1, m, m, k)
    assert np.abs(got - ref).max() < TOL * np.abs(ref).max()
    assert np.abs(got - got.T).max() <= 1e-12 * np.abs(ref).max()  # split-K atomics may reorder the last bits


@pytest.mark.parametrize("m,k", [(130, 100), (260, 500)])
def test_symmetrized_product(built_library, cuda, m, k):
    rng = np.random.default_rng(7 * m + k)
    A, B = rng.normal(size=(m, k)), rng.normal(size=(m, k))
    ref = A @ B.T + B @ A.T
    got = _run(A, B, 2, m, m, k)
    assert np.abs(got - ref).max() < TOL * np.abs(ref).max()


def test_three_products_beat_one(built_library, cuda):
    # the split must carry far more than one BF16 product's 8 bits
    rng = np.random.default_rng(5)
    A, B = rng.normal(size=(256, 512)), rng.normal(size=(192, 512))
    ref = A @ B.T
    got = _run(A, B, 0, 256, 192, 512)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-5
