"""Pins the Ozaki restatement (CPU): digits against the rational fixture,
exact recombination against rational arithmetic, accuracy against the
double-double oracle."""
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

import oracle
from oracle import ozaki

GOLD = Path(__file__).resolve().parent / "golden"


def test_digits_match_rational_fixture():
    f = np.load(GOLD / "ozaki_digits.npz")
    for S in np.unique(f["slices"]):
        sel = f["slices"] == S
        got = ozaki.digits(f["x"][sel], f["e_row"][sel], int(S))
        np.testing.assert_array_equal(got, f["digits"][sel][:, :S])


def test_digits_reconstruct_and_bounds():
    rng = np.random.default_rng(3)
    x = np.ldexp(rng.uniform(-1, 1, 2000), rng.integers(-20, 20, 2000))
    E = np.frexp(np.abs(x))[1] + rng.integers(0, 4, 2000)
    for S in (2, 7, 12, 16):
        d = ozaki.digits(x, E, S)
        assert np.abs(d).max() <= 16
        assert np.all(np.abs(d[:, 1:]) <= 16)
        F = ozaki.error_bound_bits(S)
        for i in range(0, 2000, 97):
            val = sum(Fraction(int(d[i, s])) * Fraction(2) ** (-4 - 5 * s) for s in range(S))
            exact = Fraction(float(x[i])) / Fraction(2) ** int(E[i])
            assert abs(val - exact) <= Fraction(1, 2 ** (F + 1))


def test_exact_recombination_matches_rationals():
    rng = np.random.default_rng(4)
    A = oracle.uniform((5, 9), 1)
    B = oracle.uniform((9, 4), 2)
    S = 3
    C = ozaki.ozaki_gemm("N", "N", A, B, S)
    EA, EB = ozaki.row_exponents(A), ozaki.row_exponents(B.T)
    DA, DB = ozaki.digits(A, EA[:, None], S), ozaki.digits(B.T, EB[:, None], S)
    for i in range(5):
        for j in range(4):
            v = Fraction(0)
            for s in range(S):
                for t in range(S - s):
                    for l in range(9):
                        v += Fraction(int(DA[i, l, s] * DB[j, l, t])) * Fraction(2) ** (-8 - 5 * (s + t))
            v *= Fraction(2) ** int(EA[i] + EB[j])
            assert C[i, j] == float(v)
    del rng


@pytest.mark.parametrize("phi", [0, 8, 32])
def test_accuracy_against_double_double(phi):
    A = oracle.exp_spread((24, 300), 11 + phi, phi)
    B = oracle.exp_spread((300, 20), 12 + phi, phi)
    hi, lo, ab = oracle.gemm_dd("N", "N", A, B)
    S = 16  # short K with a wide exponent spread needs the full slice budget
    C = ozaki.ozaki_gemm("N", "N", A, B, S)
    st = oracle.error_stats(C, hi, lo, ab)
    assert st["max_err_over_absab"] < 2.0 ** -52


def test_integer_inputs_are_exact():
    rng = np.random.default_rng(5)
    A = np.asfortranarray(rng.integers(-15, 16, (6, 40)).astype(np.float64))
    B = np.asfortranarray(rng.integers(-15, 16, (40, 5)).astype(np.float64))
    C = ozaki.ozaki_gemm("N", "N", A, B, 3)
    np.testing.assert_array_equal(C, A @ B)


def test_sampled_restatement_matches_full():
    rng = np.random.default_rng(3)
    for ta, tb in (("N", "N"), ("T", "N"), ("N", "T")):
        m, n, k, S = 23, 17, 41, 6
        A = oracle.exp_spread((m, k) if ta == "N" else (k, m), 4, 5)
        B = oracle.exp_spread((k, n) if tb == "N" else (n, k), 5, 5)
        full = ozaki.ozaki_gemm(ta, tb, A, B, S)
        rows = rng.integers(0, m, 60)
        cols = rng.integers(0, n, 60)
        np.testing.assert_array_equal(ozaki.ozaki_gemm_sampled(ta, tb, A, B, S, rows, cols), full[rows, cols])


def test_complex_restatement_is_the_complex_product():
    rng = np.random.default_rng(4)
    for ta, tb in (("N", "N"), ("T", "C"), ("C", "T")):
        m, n, k = 13, 11, 19
        sa = (m, k) if ta == "N" else (k, m)
        sb = (k, n) if tb == "N" else (n, k)
        A = rng.uniform(-1, 1, sa) + 1j * rng.uniform(-1, 1, sa)
        B = rng.uniform(-1, 1, sb) + 1j * rng.uniform(-1, 1, sb)
        opA = A if ta == "N" else (A.T if ta == "T" else A.conj().T)
        opB = B if tb == "N" else (B.T if tb == "T" else B.conj().T)
        got = ozaki.ozaki_zgemm(ta, tb, A, B, 13)
        np.testing.assert_allclose(got, opA @ opB, rtol=0, atol=1e-14)
        rows, cols = rng.integers(0, m, 30), rng.integers(0, n, 30)
        np.testing.assert_array_equal(ozaki.ozaki_zgemm_sampled(ta, tb, A, B, 13, rows, cols), got[rows, cols])
