"""The Ozaki DGEMM entry point that allocates nothing (cosma_gpu_dgemm_ozaki_noalloc).

It exists for callers that cannot let a library allocate device memory: programs
whose device memory is all owned by their own pool allocator, and programs that
cannot afford the device-wide synchronisation cudaMalloc and cudaFree bring.
Its scratch is one static device array, so these checks call it through the C
ABI twice in a row (the second call finds the first call's leftovers in that
array) and compare each result with the allocating entry point's on the same
inputs.  Both run the same kernels, so the results must agree bit for bit.
This file sorts last so that a stop-at-first-failure run has already run every
other test; it passes on its own in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

import oracle
from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu


def _call(fn, ta, tb, m, n, k, A, lda, B, ldb, C, ldc, slices, alpha=1.0, beta=0.0):
    from cosma_gb300 import _native
    info = _native.OzakiInfo()
    st = fn(ta.encode(), tb.encode(), m, n, k, alpha, A.data_ptr(), lda, B.data_ptr(), ldb, beta, C.data_ptr(), ldc,
            slices, None, ctypes.byref(info))
    return st, info


def test_no_alloc_matches_allocating_entry_point_on_consecutive_calls(native_lib, cuda):
    import torch
    lib = native_lib
    cases = [  # second call is smaller, so it runs on the first call's leftover scratch
        ("N", "N", 700, 500, 1024, 13, 0),
        ("T", "N", 300, 260, 900, 0, 8),
    ]
    for ta, tb, m, n, k, slices, phi in cases:
        A = oracle.exp_spread((m, k) if ta == "N" else (k, m), m + 1, phi)
        B = oracle.exp_spread((k, n) if tb == "N" else (n, k), n + 2, phi)
        C0 = oracle.uniform((m, n), 3)
        dA, dB = to_dev(A), to_dev(B)
        ref = to_dev(C0)
        got = to_dev(C0)
        st, ref_info = _call(lib.cosma_gpu_dgemm_ozaki_device, ta, tb, m, n, k, dA, A.shape[0], dB, B.shape[0],
                             ref, m, slices, alpha=1.5, beta=-0.5)
        assert st == 0, lib.cosma_gpu_last_error_string()
        for _ in range(2):  # two calls in a row on the same output
            got.copy_(to_dev(C0))
            st, info = _call(lib.cosma_gpu_dgemm_ozaki_noalloc, ta, tb, m, n, k, dA, A.shape[0], dB, B.shape[0],
                             got, m, slices, alpha=1.5, beta=-0.5)
            assert st == 0, lib.cosma_gpu_last_error_string()
            torch.cuda.synchronize()
            assert info.slices == ref_info.slices and info.products == ref_info.products
            np.testing.assert_array_equal(from_dev(got, m, n), from_dev(ref, m, n))


def test_no_alloc_multi_pass_k_and_nan_fallback(native_lib, cuda):
    """k beyond one exact pass (65536) runs as two passes accumulated through C
    (beta becomes 1 after the first), and an operand holding NaN falls back to
    the native kernel; both paths differ in code from the allocating twin, so
    both are compared bit for bit against it, twice in a row."""
    lib = native_lib
    # 2 slices keep the 65536-deep pass inside the static array: 2 x (128 + 256) x 65536 bytes
    m, n, k, slices = 72, 40, 65536 + 64, 2
    A = oracle.uniform((m, k), 11)
    B = oracle.uniform((k, n), 12)
    C0 = oracle.uniform((m, n), 13)
    nanA = A[:, :200].copy()
    nanA[5, 17] = np.nan
    cases = [(A, B, k, False), (nanA, B[:200].copy(), 200, True)]
    for a, b, kk, fallback in cases:
        dA, dB = to_dev(a), to_dev(b)
        ref = to_dev(C0)
        st, ref_info = _call(lib.cosma_gpu_dgemm_ozaki_device, "N", "N", m, n, kk, dA, m, dB, kk, ref, m, slices,
                             alpha=0.75, beta=2.0)
        assert st == 0, lib.cosma_gpu_last_error_string()
        assert ref_info.fallback_native == int(fallback)
        want = from_dev(ref, m, n)
        if fallback:
            assert np.isnan(want[5]).all() and not np.isnan(np.delete(want, 5, axis=0)).any()
        for _ in range(2):
            got = to_dev(C0)
            st, info = _call(lib.cosma_gpu_dgemm_ozaki_noalloc, "N", "N", m, n, kk, dA, m, dB, kk, got, m, slices,
                             alpha=0.75, beta=2.0)
            assert st == 0, lib.cosma_gpu_last_error_string()
            assert info.fallback_native == int(fallback)
            assert info.prep_ms == 0.0 and info.gemm_ms == 0.0  # documented: no timing events here
            np.testing.assert_array_equal(from_dev(got, m, n), want)


def test_no_alloc_rejects_problems_beyond_its_scratch(native_lib, cuda):
    import torch
    lib = native_lib
    m = n = k = 4096  # needs ~0.5 GB of scratch; real buffers, so nothing is out of bounds either way
    dA = torch.zeros(m * k, dtype=torch.float64, device="cuda")
    dB = torch.zeros(k * n, dtype=torch.float64, device="cuda")
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    st, _ = _call(lib.cosma_gpu_dgemm_ozaki_noalloc, "N", "N", m, n, k, dA, m, dB, k, dC, m, 13)
    assert st == 1  # COSMA_GPU_ERROR_INVALID_ARGUMENT
    msg = lib.cosma_gpu_last_error_string().decode()
    assert "scratch" in msg and str(64 << 20) in msg
