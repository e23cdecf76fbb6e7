"""Complex Ozaki-split ZGEMM (four real products per complex one) vs the oracle.

* bit-exact against the CPU restatement (oracle/ozaki.py: ozaki_zgemm) for
  every combination of op N / T / C, on both forms of the slice GEMM;
* sampled bit-exact checks at sizes with several tiles per CTA;
* accuracy of each part against the double-double oracle;
* real alpha/beta (applied in the epilogue), complex alpha/beta (applied by
  the alpha*T + beta*C pass), K beyond one exact pass, non-finite inputs,
  and the Tiled-MM handle with the Ozaki method on complex data.
"""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, to_dev
from oracle import ozaki as oz

pytestmark = pytest.mark.gpu


def _cplx(shape, seed, phi=0):
    return oracle.exp_spread(shape, seed, phi) + 1j * oracle.exp_spread(shape, seed + 1000, phi)


def _op_shape(op, m, k):
    return (m, k) if op == "N" else (k, m)


def _run(ta, tb, m, n, k, A, B, alpha=1.0, beta=0.0, C0=None, slices=0, lda=None, ldb=None, ldc=None):
    from cosma_gb300 import zgemm_ozaki_device
    lda = lda or A.shape[0]
    ldb = ldb or B.shape[0]
    ldc = ldc or m
    dA, dB = to_dev(A, lda), to_dev(B, ldb)
    dC = to_dev(C0 if C0 is not None else np.zeros((m, n), dtype=np.complex128), ldc)
    info = zgemm_ozaki_device(ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, slices=slices)
    return from_dev(dC, m, n, ldc), info


@pytest.mark.parametrize("ta", ["N", "T", "C"])
@pytest.mark.parametrize("tb", ["N", "T", "C"])
def test_bit_exact_every_op(native_lib, cuda, ta, tb):
    m, n, k, S = 37, 29, 45, 7
    A = _cplx(_op_shape(ta, m, k), 3, 5)
    B = _cplx(_op_shape(tb, k, n), 4, 5)
    got, info = _run(ta, tb, m, n, k, A, B, slices=S, lda=A.shape[0] + 2, ldc=m + 1)
    assert info["slices"] == S and info["products"] == S * (S + 1) // 2
    np.testing.assert_array_equal(got, oz.ozaki_zgemm(ta, tb, A, B, S))


@pytest.mark.parametrize("ta,tb,m,n,k,S", [
    ("N", "C", 130, 260, 70, 13),    # CTA pairs
    ("C", "N", 100, 300, 129, 10),   # single CTAs, clusters of 2 along the 2n columns
])
def test_bit_exact_both_gemm_forms(native_lib, cuda, ta, tb, m, n, k, S):
    A = _cplx(_op_shape(ta, m, k), 5, 3)
    B = _cplx(_op_shape(tb, k, n), 6, 3)
    got, _ = _run(ta, tb, m, n, k, A, B, slices=S)
    np.testing.assert_array_equal(got, oz.ozaki_zgemm(ta, tb, A, B, S))


@pytest.mark.parametrize("ta,tb,m,n,k,S", [
    ("N", "C", 1300, 900, 200, 13),   # CTA pairs, many tiles
    ("T", "N", 384, 1500, 150, 9),    # single CTAs
])
def test_bit_exact_sampled_large(native_lib, cuda, ta, tb, m, n, k, S):
    A = _cplx(_op_shape(ta, m, k), 7, 4)
    B = _cplx(_op_shape(tb, k, n), 8, 4)
    got, _ = _run(ta, tb, m, n, k, A, B, slices=S)
    rng = np.random.default_rng(9)
    rows = np.concatenate([rng.integers(0, m, 800), [0, m - 1]])
    cols = np.concatenate([rng.integers(0, n, 800), [n - 1, 0]])
    np.testing.assert_array_equal(got[rows, cols], oz.ozaki_zgemm_sampled(ta, tb, A, B, S, rows, cols))


@pytest.mark.parametrize("phi", [0, 8])
def test_accuracy_against_double_double(native_lib, cuda, phi):
    m = n = 320
    k = 1024
    A = _cplx((m, k), 10 + phi, phi)
    B = _cplx((n, k), 20 + phi, phi)
    got, info = _run("N", "C", m, n, k, A, B)
    Acat, Bre, Bim = oz._cplx_operands("N", "C", A, B)
    rng = np.random.default_rng(phi)
    rows = rng.integers(0, m, 1024)
    cols = rng.integers(0, n, 1024)
    for part, Bp in ((got.real, Bre), (got.imag, Bim)):
        hi, lo, ab = oracle.gemm_dd_sampled("N", "N", Acat, Bp, rows, cols)
        st = oracle.error_stats(part[rows, cols], hi, lo, ab)
        assert st["max_err_over_absab"] <= 2.0 ** -52, (st, info)
        assert st["max_rel_err"] <= 1e-15, (st, info)


def test_real_alpha_beta_in_the_epilogue(native_lib, cuda):
    m, n, k, S = 60, 50, 40, 11
    A, B, C0 = _cplx((m, k), 1), _cplx((k, n), 2), _cplx((m, n), 3)
    base = oz.ozaki_zgemm("N", "N", A, B, S)
    got, _ = _run("N", "N", m, n, k, A, B, alpha=2.0, beta=-0.75, C0=C0, slices=S)
    want = (2.0 * base.real + (-0.75) * C0.real) + 1j * (2.0 * base.imag + (-0.75) * C0.imag)
    np.testing.assert_array_equal(got, want)
    nanc = np.full((m, n), np.nan + 1j * np.nan)
    got, _ = _run("N", "N", m, n, k, A, B, alpha=1.0, beta=0.0, C0=nanc, slices=S)
    np.testing.assert_array_equal(got, base)


def test_complex_alpha_beta(native_lib, cuda):
    m, n, k, S = 45, 33, 52, 12
    A, B, C0 = _cplx((k, m), 4), _cplx((n, k), 5), _cplx((m, n), 6)
    alpha, beta = 1.5 - 0.5j, 0.25 + 2.0j
    base = oz.ozaki_zgemm("T", "C", A, B, S)
    got, _ = _run("T", "C", m, n, k, A, B, alpha=alpha, beta=beta, C0=C0, slices=S)
    want = np.asfortranarray(C0.copy())
    oracle.unpack(alpha, np.asfortranarray(base), beta, want)
    np.testing.assert_array_equal(got, want)


def test_k_beyond_one_pass(native_lib, cuda):
    m, n, k = 6, 5, 40000  # 2k real terms > 65536: two exact passes through C
    A, B = _cplx((m, k), 7), _cplx((k, n), 8)
    got, _ = _run("N", "N", m, n, k, A, B)
    Acat, Bre, Bim = oz._cplx_operands("N", "N", A, B)
    for part, Bp in ((got.real, Bre), (got.imag, Bim)):
        hi, lo, ab = oracle.gemm_dd("N", "N", Acat, Bp)
        assert oracle.error_stats(part, hi, lo, ab)["max_err_over_absab"] <= 2.0 ** -51


def test_nonfinite_inputs_fall_back_to_native(native_lib, cuda):
    m, n, k = 20, 16, 12
    A, B = _cplx((m, k), 9), _cplx((k, n), 10)
    A[2, 3] = complex(np.inf, 0.0)
    got, info = _run("N", "N", m, n, k, A, B)
    assert info["fallback_native"] == 1
    assert np.isinf(got[2, :]).any() or np.isnan(got[2, :]).any()


def test_tiled_mm_handle_with_ozaki_method_complex(native_lib, cuda):
    from cosma_gb300 import gemm, make_context
    h = make_context("z", 2, 200, 160, 256)
    h.set_method("ozaki", 13)
    m, n, k = 333, 222, 600
    A, B = _cplx((m, k), 11), _cplx((n, k), 12)
    Cg = np.zeros((m, n), dtype=np.complex128, order="F")
    gemm(h, "N", "C", m, n, k, 1.0, A, m, B, n, 0.0, Cg, m)
    Acat, Bre, Bim = oz._cplx_operands("N", "C", A, B)
    for part, Bp in ((Cg.real, Bre), (Cg.imag, Bim)):
        hi, lo, ab = oracle.gemm_dd("N", "N", Acat, Bp)
        assert oracle.error_stats(part, hi, lo, ab)["max_err_over_absab"] <= 2.0 ** -50
