"""64-bit indexing past 2^31 elements per matrix.

The reference computes buffer sizes and offsets in `int` (m * k products in
src/cosma/local_multiply.cpp:343-346, scalapack::local_buffer_size returning
int in src/cosma/scalapack.hpp:72), which overflows at the sizes of the
out-of-HBM configuration.  Here op(A) has m * k = 65536 * 32769 > 2^31
elements (17.2 GB of FP64):
* through the Tiled-MM entry from the caller's host array (the streamer's
  tile offsets), and
* through the device-pointer entry on a device-resident A (the kernel's
  element offsets).
Entries are multiples of 2^-9 below 1, so every partial sum of the product is
exact in FP64 whatever the summation order: sampled entries of C must equal
the exact integer computation bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M, K, N = 65536, 32769, 256


def _dyadic(rows, cols, a, b, col0=0):
    """((a*i + b*j) mod 1023 - 511) / 512 for i < rows, j in [col0, col0 + cols)."""
    i = np.arange(rows, dtype=np.int64)[:, None]
    j = np.arange(col0, col0 + cols, dtype=np.int64)[None, :]
    return (((a * i + b * j) % 1023) - 511).astype(np.float64) / 512.0


@pytest.fixture(scope="module")
def operands():
    assert M * K > 2 ** 31
    A = np.empty((M, K), order="F")
    step = 2048
    for l0 in range(0, K, step):
        l1 = min(K, l0 + step)
        A[:, l0:l1] = _dyadic(M, l1 - l0, 7, 13, l0)
    B = np.asfortranarray(_dyadic(K, N, 5, 11))
    rng = np.random.default_rng(11)
    rows = np.concatenate([rng.integers(0, M, 200), [0, M - 1, M - 1, 0, 65535]])
    cols = np.concatenate([rng.integers(0, N, 200), [0, N - 1, 0, N - 1, 255]])
    Ai = np.rint(A[rows, :] * 512).astype(np.int64)          # samples x K
    Bi = np.rint(B[:, cols].T * 512).astype(np.int64)         # samples x K
    exact = (Ai * Bi).sum(axis=1).astype(np.float64) / 2.0 ** 18  # |sum| < 2^34: exact
    return A, B, rows, cols, exact


def test_host_entry_streams_a_matrix_beyond_2_31_elements(native_lib, cuda, operands):
    import cosma_gb300 as cg
    A, B, rows, cols, exact = operands
    Cm = np.zeros((M, N), order="F")
    h = cg.make_context("d", 2, 0, 0, 0)
    try:
        cg.gemm(h, "N", "N", M, N, K, 1.0, A, M, B, K, 0.0, Cm, M)
    finally:
        h.close()
    np.testing.assert_array_equal(Cm[rows, cols], exact)


def test_device_entry_indexes_a_matrix_beyond_2_31_elements(native_lib, cuda, operands):
    import torch

    import cosma_gb300 as cg
    A, B, rows, cols, exact = operands
    dA = torch.from_numpy(A.reshape(-1, order="F")).cuda()
    dB = torch.from_numpy(B.reshape(-1, order="F")).cuda()
    dC = torch.zeros(M * N, dtype=torch.float64, device="cuda")
    cg.gemm_device("N", "N", M, N, K, 1.0, dA, M, dB, K, 0.0, dC, M, method="native")
    torch.cuda.synchronize()
    C = dC.cpu().numpy().reshape(N, M).T
    np.testing.assert_array_equal(C[rows, cols], exact)
    del dA, dB, dC
    torch.cuda.empty_cache()
