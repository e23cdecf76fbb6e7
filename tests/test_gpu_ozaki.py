"""Ozaki-split FP64-accurate GEMM on the FP8 tensor cores vs the oracle.

* bit-exact against the CPU restatement of the same algorithm (oracle/ozaki.py)
  on small sizes, every op combination;
* exactness of the FP32 accumulation: integer inputs give the exact integer
  product at K = 16384 (sums up to 2^24 inside one accumulator);
* accuracy against the double-double oracle (max elementwise relative error
  <= 1e-15, and <= 2^-52 |A||B| componentwise) for the precision
  configuration's distributions, phi in {0, 8, 32};
* edge cases: ragged sizes, k = 1, k above one exact accumulator pass, alpha
  and beta, beta == 0 with NaN in C, non-finite inputs.
"""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, to_dev
from oracle import ozaki as oz

pytestmark = pytest.mark.gpu


def _op_shape(op, m, k):
    return (m, k) if op == "N" else (k, m)


def _run(ta, tb, m, n, k, A, B, alpha=1.0, beta=0.0, C0=None, slices=0, lda=None, ldb=None, ldc=None):
    from cosma_gb300 import dgemm_ozaki_device
    lda = lda or A.shape[0]
    ldb = ldb or B.shape[0]
    ldc = ldc or m
    dA, dB = to_dev(A, lda), to_dev(B, ldb)
    dC = to_dev(C0 if C0 is not None else np.zeros((m, n)), ldc)
    info = dgemm_ozaki_device(ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, slices=slices)
    return from_dev(dC, m, n, ldc), info


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("m,n,k,S", [(17, 9, 33, 4), (64, 40, 130, 7), (130, 260, 200, 13), (5, 300, 129, 16)])
def test_bit_exact_against_restatement(native_lib, cuda, ta, tb, m, n, k, S):
    A = oracle.exp_spread(_op_shape(ta, m, k), m + k, 6)
    B = oracle.exp_spread(_op_shape(tb, k, n), n + k, 6)
    got, info = _run(ta, tb, m, n, k, A, B, slices=S, lda=A.shape[0] + 1, ldc=m + 3)
    ref = oz.ozaki_gemm(ta, tb, A, B, S)
    assert info["slices"] == S and info["products"] == S * (S + 1) // 2
    np.testing.assert_array_equal(got, ref)


# Both forms of the slice-product GEMM, at sizes with several tiles per CTA
# (persistent loop, partial sums reused across tiles), checked bit for bit on
# sampled entries, edges included.
@pytest.mark.parametrize("ta,tb,m,n,k,S", [
    ("N", "N", 2560, 2304, 256, 5),   # CTA pairs, 90 tiles of 256 x 256
    ("T", "N", 1300, 700, 300, 13),   # CTA pairs, m padded to 1536
    ("N", "T", 1152, 5120, 200, 6),   # single CTAs in clusters of 4 along N, 180 tiles
    ("T", "T", 384, 512, 130, 9),     # single CTAs in clusters of 2
    ("N", "N", 640, 1280, 70, 7),     # single CTAs, no cluster
])
def test_bit_exact_sampled_gemm_forms(native_lib, cuda, ta, tb, m, n, k, S):
    A = oracle.exp_spread(_op_shape(ta, m, k), m + 3, 6)
    B = oracle.exp_spread(_op_shape(tb, k, n), n + 5, 6)
    got, info = _run(ta, tb, m, n, k, A, B, slices=S)
    rng = np.random.default_rng(m + n)
    rows = np.concatenate([rng.integers(0, m, 1500), [0, m - 1, m - 1, 0]])
    cols = np.concatenate([rng.integers(0, n, 1500), [0, n - 1, 0, n - 1]])
    ref = oz.ozaki_gemm_sampled(ta, tb, A, B, S, rows, cols)
    np.testing.assert_array_equal(got[rows, cols], ref)


def test_fp32_accumulation_is_exact_at_k16384(native_lib, cuda):
    rng = np.random.default_rng(1)
    m, n, k = 256, 256, 16384
    A = np.asfortranarray(rng.integers(-15, 16, (m, k)).astype(np.float64))
    B = np.asfortranarray(rng.integers(-15, 16, (k, n)).astype(np.float64))
    # all-maximal digits in a few rows/cols stress the 2^24 bound
    A[:4, :] = 15.0
    B[:, :4] = 15.0
    got, info = _run("N", "N", m, n, k, A, B, slices=4)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    assert info["groups"] < info["products"]  # several products share one accumulator
    np.testing.assert_array_equal(got, exact)


@pytest.mark.parametrize("phi", [0, 8, 32])
def test_accuracy_against_double_double(native_lib, cuda, phi):
    m = n = 384
    k = 2048
    A = oracle.exp_spread((m, k), 10 + phi, phi)
    B = oracle.exp_spread((k, n), 20 + phi, phi)
    got, info = _run("N", "N", m, n, k, A, B)
    rng = np.random.default_rng(phi)
    rows = rng.integers(0, m, 2048)
    cols = rng.integers(0, n, 2048)
    hi, lo, ab = oracle.gemm_dd_sampled("N", "N", A, B, rows, cols)
    st = oracle.error_stats(got[rows, cols], hi, lo, ab)
    assert st["max_rel_err"] <= 1e-15, (st, info)
    assert st["max_err_over_absab"] <= 2.0 ** -52, (st, info)


def test_alpha_beta_and_nan_c(native_lib, cuda):
    m, n, k = 100, 70, 90
    A, B = oracle.uniform((m, k), 1), oracle.uniform((k, n), 2)
    C0 = oracle.uniform((m, n), 3)
    S = 12
    base = oz.ozaki_gemm("N", "N", A, B, S)
    got, _ = _run("N", "N", m, n, k, A, B, alpha=1.5, beta=-0.5, C0=C0, slices=S)
    np.testing.assert_array_equal(got, 1.5 * base + (-0.5) * C0)
    nanc = np.full((m, n), np.nan)
    got, _ = _run("N", "N", m, n, k, A, B, alpha=2.0, beta=0.0, C0=nanc, slices=S)
    np.testing.assert_array_equal(got, 2.0 * base)


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (1, 257, 3), (129, 1, 257), (7, 300, 1)])
def test_ragged_sizes(native_lib, cuda, m, n, k):
    A, B = oracle.uniform((m, k), m), oracle.uniform((k, n), n)
    got, _ = _run("N", "N", m, n, k, A, B, slices=13)
    np.testing.assert_array_equal(got, oz.ozaki_gemm("N", "N", A, B, 13))


def test_k_beyond_one_accumulator_pass(native_lib, cuda):
    # k > 65536 is processed in exact passes accumulated through C
    m, n, k = 8, 8, 70000
    A, B = oracle.uniform((m, k), 5), oracle.uniform((k, n), 6)
    got, info = _run("N", "N", m, n, k, A, B)
    hi, lo, ab = oracle.gemm_dd("N", "N", A, B)
    st = oracle.error_stats(got, hi, lo, ab)
    assert st["max_err_over_absab"] <= 2.0 ** -51


def test_nonfinite_inputs_fall_back_to_native(native_lib, cuda):
    m, n, k = 40, 30, 20
    A, B = oracle.uniform((m, k), 7), oracle.uniform((k, n), 8)
    A[3, 4] = np.inf
    A[5, 6] = np.nan
    got, info = _run("N", "N", m, n, k, A, B)
    assert info["fallback_native"] == 1
    ref = A @ B
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))


def test_auto_slices_follow_spread(native_lib, cuda):
    m = n = 256
    k = 1024
    s = {}
    for phi in (0, 32):
        A = oracle.exp_spread((m, k), 1, phi)
        B = oracle.exp_spread((k, n), 2, phi)
        _, info = _run("N", "N", m, n, k, A, B)
        s[phi] = info["slices"]
    assert s[32] > s[0]


def test_tiled_mm_handle_with_ozaki_method(native_lib, cuda):
    from cosma_gb300 import gemm, make_context
    h = make_context("d", 2, 200, 200, 300)
    h.set_method("ozaki", 13)
    m, n, k = 333, 222, 700
    A, B = oracle.uniform((m, k), 11), oracle.uniform((n, k), 12)
    Cg = np.zeros((m, n), order="F")
    gemm(h, "N", "T", m, n, k, 1.0, A, m, B, n, 0.0, Cg, m)
    hi, lo, ab = oracle.gemm_dd("N", "T", A, B)
    st = oracle.error_stats(Cg, hi, lo, ab)
    assert st["max_err_over_absab"] <= 2.0 ** -51  # K tiles add one rounding each
    assert h.ozaki_info()["slices"] == 13
    h.close()


@pytest.mark.parametrize("direct", ["ON", "OFF"])
def test_handle_host_c_matches_device_path(native_lib, cuda, monkeypatch, direct):
    """A whole-problem Ozaki DGEMM through the handle on host operands
    (pageable numpy and torch-pinned C, beta 0 and beta != 0, op T on A),
    over either host copy route: bit-identical to the same GEMM on device
    pointers, with C's bytes crossing the link once each way."""
    import torch
    from cosma_gb300 import dgemm_ozaki_device, gemm, host_copy_route, make_context
    monkeypatch.setenv("COSMA_GPU_HOST_DIRECT", direct)
    m, n, k = 700, 515, 900
    A, B = oracle.uniform((k, m), 41), oracle.uniform((k, n), 42)   # op(A) = A^T
    C0 = oracle.uniform((m + 3, n), 43)
    dA = torch.from_numpy(A.reshape(-1, order="F").copy()).cuda()
    dB = torch.from_numpy(B.reshape(-1, order="F").copy()).cuda()
    for beta in (0.0, -0.75):
        dC = torch.from_numpy(C0.reshape(-1, order="F").copy()).cuda()
        dgemm_ozaki_device("T", "N", m, n, k, 1.5, dA, k, dB, k, beta, dC, m + 3)
        ref = dC.cpu().numpy().reshape(n, m + 3).T
        h = make_context("d", 2, 0, 0, 0)
        h.set_method("ozaki", 0)
        Cp = C0.copy(order="F")
        gemm(h, "T", "N", m, n, k, 1.5, A, k, B, k, beta, Cp, m + 3)
        assert Cp.tobytes() == np.asfortranarray(ref).tobytes()
        h2d, d2h = h.transfer_bytes()
        assert d2h == m * n * 8
        assert h2d == A.nbytes + B.nbytes + (m * n * 8 if beta != 0 else 0)
        pinned = torch.from_numpy(C0.reshape(-1, order="F").copy()).pin_memory()
        assert host_copy_route(pinned) == ("memcpy" if direct == "OFF" else host_copy_route(pinned))
        gemm(h, "T", "N", m, n, k, 1.5, A, k, B, k, beta, pinned, m + 3)
        assert pinned.numpy().tobytes() == np.asfortranarray(ref).reshape(-1, order="F").tobytes()
        h.close()


def test_memory_limited_handle_streams_in_tiles(native_lib, cuda):
    """A handle under a 256 MiB device budget runs a larger Ozaki DGEMM from
    host memory in tiles: the operands travel several times and the result
    still meets the accuracy bound."""
    from cosma_gb300 import gemm, make_context
    h = make_context("d", 2, 0, 0, 0)
    h.set_method("ozaki", 0)
    h.set_memory_limit(256 << 20)
    tm, tn, tk = h.tiles()
    m, n, k = 3000, 2600, 2800
    assert tm < m and tk < k
    A, B = oracle.uniform((m, k), 31), oracle.uniform((k, n), 32)
    Cg = np.zeros((m, n), order="F")
    gemm(h, "N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cg, m)
    h2d, d2h = h.transfer_bytes()
    assert h2d > (A.nbytes + B.nbytes)  # operand tiles are re-sent across output tiles
    rng = np.random.default_rng(3)
    rows, cols = rng.integers(0, m, 512), rng.integers(0, n, 512)
    hi, lo, ab = oracle.gemm_dd_sampled("N", "N", A, B, rows, cols)
    assert oracle.error_stats(Cg[rows, cols], hi, lo, ab)["max_err_over_absab"] <= 2.0 ** -51
