"""3xBF16 single-precision GEMM on the BF16 tensor cores vs the oracle.

The oracle multiplies the FP32 inputs exactly and accumulates in FP64, rounding
once (oracle_gemm_s); 3xBF16 must stay within single-precision GEMM error
bounds of it and be no less accurate than an FP32 GEMM.
"""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu

U32 = 2.0 ** -24


def _op_shape(op, m, k):
    return (m, k) if op == "N" else (k, m)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (77, 300, 65), (256, 256, 1024), (129, 513, 200)])
def test_bf16x3_within_fp32_bounds(native_lib, cuda, ta, tb, m, n, k):
    from cosma_gb300 import gemm_device
    A = oracle.normal(_op_shape(ta, m, k), m + 3 * k, dtype=np.float32)
    B = oracle.normal(_op_shape(tb, k, n), n + 5 * k, dtype=np.float32)
    C0 = oracle.normal((m, n), 9, dtype=np.float32)
    alpha, beta = 1.25, -0.5
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C0)
    gemm_device(ta, tb, m, n, k, alpha, dA, A.shape[0], dB, B.shape[0], beta, dC, m, method="bf16x3", scalar="s")
    got = from_dev(dC, m, n).astype(np.float64)
    ref = oracle.gemm(ta, tb, np.float32(alpha), A, B, np.float32(beta), C0.copy(order="F")).astype(np.float64)
    opA = (A if ta == "N" else A.T).astype(np.float64)
    opB = (B if tb == "N" else B.T).astype(np.float64)
    bound = 4 * (k + 8) * U32 * (abs(alpha) * np.abs(opA) @ np.abs(opB) + abs(beta) * np.abs(C0)) + 1e-30
    assert np.all(np.abs(got - ref) <= bound)


def test_bf16x3_as_accurate_as_fp32_gemm(native_lib, cuda):
    from cosma_gb300 import gemm_device
    m = n = 512
    k = 4096
    A = oracle.normal((m, k), 1, dtype=np.float32)
    B = oracle.normal((k, n), 2, dtype=np.float32)
    dA, dB = to_dev(A), to_dev(B)
    dC = to_dev(np.zeros((m, n), dtype=np.float32), fill=np.nan)
    gemm_device("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dC, m, method="bf16x3", scalar="s")
    got = from_dev(dC, m, n).astype(np.float64)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    fp32 = np.zeros((m, n), dtype=np.float32)
    for j0 in range(0, k, 256):  # a plain FP32 GEMM: sequential FP32 accumulation over K blocks
        fp32 += (A[:, j0:j0 + 256] @ B[j0:j0 + 256, :]).astype(np.float32)
    err3 = np.abs(got - exact).max()
    err32 = np.abs(fp32.astype(np.float64) - exact).max()
    assert not np.isnan(got).any()
    assert err3 <= 2.0 * err32, (err3, err32)


def test_bf16x3_k_zero_and_alpha_zero(native_lib, cuda):
    from cosma_gb300 import gemm_device
    m, n = 40, 30
    C0 = oracle.normal((m, n), 3, dtype=np.float32)
    dC = to_dev(C0)
    d1 = to_dev(np.ones((m, 1), dtype=np.float32))
    gemm_device("N", "N", m, n, 0, 1.0, d1, m, d1, 1, 2.0, dC, m, method="bf16x3", scalar="s")
    np.testing.assert_array_equal(from_dev(dC, m, n), 2.0 * C0)


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
@pytest.mark.parametrize("ta,tb,beta,shape", [("N", "N", 0.0, (2100, 2300, 300)), ("T", "N", -0.5, (2100, 2300, 300)),
                                              ("N", "T", 1.0, (4500, 4200, 64)), ("T", "T", 0.0, (1000, 4500, 70))])
def test_bf16x3_overlapped_one_step(native_lib, cuda, monkeypatch, ta, tb, beta, shape, pinned):
    """SGEMM (3xBF16, the AUTO method for float) through the Tiled-MM entry on
    host arrays in the overlapped one-step form: panels split as they land,
    block GEMMs, C blocks copied out while later ones compute.  The bits of
    the same call without overlap and of the device call; transfers count
    A, B (and C when read) once."""
    import torch
    from cosma_gb300 import gemm, gemm_device, make_context
    m, n, k = shape
    ldc = m + 1
    A = oracle.normal(_op_shape(ta, m, k), 31, dtype=np.float32)
    B = oracle.normal(_op_shape(tb, k, n), 32, dtype=np.float32)
    C0 = np.zeros((ldc, n), dtype=np.float32)
    C0[:m] = oracle.normal((m, n), 33, dtype=np.float32)

    def host(X):
        if not pinned:
            return np.asfortranarray(X.copy()), None
        t = torch.from_numpy(np.ascontiguousarray(X.T).reshape(-1)).pin_memory()
        return t, t

    outs = {}
    for mode in ("ON", "OFF"):
        monkeypatch.setenv("COSMA_GPU_BF16X3_OVERLAP", mode)
        hA, _ = host(A)
        hB, _ = host(B)
        hC, tC = host(C0)
        h = make_context("s", 3)
        gemm(h, ta, tb, m, n, k, 1.25, hA, A.shape[0], hB, B.shape[0], beta, hC, ldc)
        outs[mode] = (np.array(tC.numpy().reshape(n, ldc).T if tC is not None else hC), h.last_overlapped(),
                      h.transfer_bytes())
        h.close()
    on, ov_on, moved = outs["ON"]
    off, ov_off, _ = outs["OFF"]
    assert ov_on and not ov_off
    assert on.tobytes() == off.tobytes()
    np.testing.assert_array_equal(on[m:], C0[m:])  # rows past m untouched
    assert moved == (4 * (m * k + k * n + (m * n if beta != 0 else 0)), 4 * m * n)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C0, ldc)
    gemm_device(ta, tb, m, n, k, 1.25, dA, A.shape[0], dB, B.shape[0], beta, dC, ldc, method="bf16x3")
    assert on[:m].tobytes() == np.ascontiguousarray(from_dev(dC, m, n, ldc)).tobytes()
