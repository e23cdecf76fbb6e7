"""Parity at the benchmark's full sizes, through size-independent checks.

* precision configuration, m = n = k = 16384, u*2^e entries: the Ozaki
  result is bit-exact against the oracle's restatement on 1000 sampled
  entries (row and column exponents depend on one row / column each, so the
  restatement of a sampled entry is exact), edges included;
* pdgemm configuration, C = 1.5 A^T B + 0.5 C with m = n = 4096, k = 65536,
  128 x 128 blocks: sampled entries against the oracle's pack -> GEMM ->
  unpack within the reference's own tolerance (validate_results, 1e-6) and
  within 2(k+2)u(|alpha||A^T||B| + |beta||C|) for the native arithmetic.
"""
import numpy as np
import pytest

import oracle
from oracle import ozaki as oz

pytestmark = pytest.mark.gpu


def test_precision_config_16384_sampled_bit_exact(native_lib, cuda):
    import torch
    from cosma_gb300 import dgemm_ozaki_device
    n = 16384
    A = oracle.exp_spread((n, n), 1, 0)
    B = oracle.exp_spread((n, n), 2, 0)
    dA = torch.from_numpy(A.reshape(-1, order="F")).cuda()
    dB = torch.from_numpy(B.reshape(-1, order="F")).cuda()
    dC = torch.empty(n * n, dtype=torch.float64, device="cuda")
    info = dgemm_ozaki_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n)
    torch.cuda.synchronize()
    rng = np.random.default_rng(16384)
    rows = np.concatenate([rng.integers(0, n, 1000), [0, n - 1, 0, n - 1]])
    cols = np.concatenate([rng.integers(0, n, 1000), [0, n - 1, n - 1, 0]])
    flat = torch.from_numpy(rows + cols * n).cuda()
    got = dC[flat].cpu().numpy()
    del dA, dB, dC
    torch.cuda.empty_cache()
    ref = oz.ozaki_gemm_sampled("N", "N", A, B, info["slices"], rows, cols)
    np.testing.assert_array_equal(got, ref)


def test_pdgemm_config_full_size_sampled(native_lib, cuda):
    import torch
    from cosma_gb300 import descinit, pxgemm
    m = n = 4096
    k = 65536
    A = oracle.normal((k, m), 21)   # stored k x m, op T
    B = oracle.normal((k, n), 22)
    C0 = oracle.normal((m, n), 23)
    dA = torch.from_numpy(A.reshape(-1, order="F")).cuda()
    dB = torch.from_numpy(B.reshape(-1, order="F")).cuda()
    dC = torch.from_numpy(C0.reshape(-1, order="F").copy()).cuda()
    desca = descinit(k, m, 128, 128, 0, 0, 0, k)
    descb = descinit(k, n, 128, 128, 0, 0, 0, k)
    descc = descinit(m, n, 128, 128, 0, 0, 0, m)
    pxgemm("T", "N", m, n, k, 1.5, dA, 1, 1, desca, dB, 1, 1, descb, 0.5, dC, 1, 1, descc, scalar="d")
    torch.cuda.synchronize()
    rng = np.random.default_rng(65536)
    rows, cols = rng.integers(0, m, 512), rng.integers(0, n, 512)
    got = dC[torch.from_numpy(rows + cols * m).cuda()].cpu().numpy()
    prod = np.einsum("li,li->i", A[:, rows], B[:, cols])        # (A^T B)_ij
    absp = np.einsum("li,li->i", np.abs(A[:, rows]), np.abs(B[:, cols]))
    want = 1.5 * prod + 0.5 * C0[rows, cols]
    bound = 2.0 * (k + 2) * 2.0 ** -53 * (1.5 * absp + 0.5 * np.abs(C0[rows, cols]))
    assert np.all(np.abs(got - want) <= bound)
    assert oracle.validate_results(got.reshape(-1, 1), want.reshape(-1, 1))
