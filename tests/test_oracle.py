"""Pins the oracle (CPU, no GPU): against exact rational fixtures, against
numpy/OpenBLAS, and replays the reference's own one-rank test cases with the
reference's own checkers."""
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLD = Path(__file__).resolve().parent / "golden"


def _load(name):
    return np.load(GOLD / name, allow_pickle=True)


@pytest.mark.parametrize("idx", range(8))
def test_gemm_against_exact_fixture(idx):
    c = _load("gemm_exact.npz")["cases"][idx]
    A, B = np.asfortranarray(c["A"]), np.asfortranarray(c["B"])
    Cm = np.asfortranarray(c["C"].copy())
    oracle.gemm(c["ta"], c["tb"], c["alpha"], A, B, c["beta"], Cm)
    k = c["k"]
    # sequential FP64 accumulation: within k*u*(|alpha||A||B| + |beta||C|)
    absA = np.abs(A if c["ta"] == "N" else A.T)
    absB = np.abs(B if c["tb"] == "N" else B.T)
    bound = (k + 2) * 2.0 ** -53 * (abs(c["alpha"]) * absA @ absB + abs(c["beta"]) * np.abs(c["C"])) + 1e-300
    assert np.all(np.abs(Cm - c["expected"]) <= bound)


@pytest.mark.parametrize("idx", range(8))
def test_double_double_is_exactly_rounded(idx):
    c = _load("gemm_exact.npz")["cases"][idx]
    A, B = np.asfortranarray(c["A"]), np.asfortranarray(c["B"])
    hi, lo, ab = oracle.gemm_dd(c["ta"], c["tb"], A, B)
    # hi + lo carries ~106 bits: rounding it to double gives the exact product rounded once
    np.testing.assert_array_equal(hi + lo, c["product"])


def test_local_multiply_cpu_matches_numpy():
    # tests/multiply.cpp:144-145 one-rank cases, alpha = beta = 1 (cosma_utils.hpp:43-44),
    # checked with test_cosma's comparison at epsilon 1e-8 (tests/multiply.cpp:99)
    for (m, n, k) in [(4, 4, 4), (3, 4, 5)]:
        rng = np.random.default_rng(m * 100 + n * 10 + k)
        A = np.asfortranarray(rng.uniform(0, 10, (m, k)))
        B = np.asfortranarray(rng.uniform(0, 10, (k, n)))
        C0 = np.asfortranarray(rng.uniform(0, 10, (m, n)))
        Cm = C0.copy(order="F")
        oracle.local_multiply_cpu(A, B, Cm, 1.0, 1.0)
        assert oracle.cosma_check(Cm, A @ B + C0, 1e-8)


def test_gemm_matches_openblas_all_ops():
    rng = np.random.default_rng(5)
    for ta in "NT":
        for tb in "NT":
            m, n, k = 37, 29, 53
            A = np.asfortranarray(rng.standard_normal((m, k) if ta == "N" else (k, m)))
            B = np.asfortranarray(rng.standard_normal((k, n) if tb == "N" else (n, k)))
            C0 = np.asfortranarray(rng.standard_normal((m, n)))
            Cm = C0.copy(order="F")
            oracle.gemm(ta, tb, 1.5, A, B, 0.5, Cm)
            ref = 1.5 * (A if ta == "N" else A.T) @ (B if tb == "N" else B.T) + 0.5 * C0
            assert oracle.validate_results(Cm, ref, 1e-12)


def test_complex_gemm_with_conjugate():
    rng = np.random.default_rng(6)
    m, n, k = 9, 7, 11
    A = oracle.uniform((k, m), 1, dtype=np.complex128)
    B = oracle.uniform((n, k), 2, dtype=np.complex128)
    C0 = oracle.uniform((m, n), 3, dtype=np.complex128)
    Cm = C0.copy(order="F")
    al, be = 1.0 - 0.5j, 0.25 + 1j
    oracle.gemm("C", "T", al, A, B, be, Cm)
    ref = al * (A.conj().T @ B.T) + be * C0
    assert np.max(np.abs(Cm - ref)) < 1e-12
    del rng


def test_beta_zero_never_reads_c():
    A = oracle.uniform((5, 4), 1)
    B = oracle.uniform((4, 3), 2)
    Cm = np.full((5, 3), np.nan, order="F")
    oracle.gemm("N", "N", 1.0, A, B, 0.0, Cm)
    assert not np.isnan(Cm).any()
    D = np.full((5, 3), np.nan, order="F")
    oracle.unpack(1.5, oracle.uniform((5, 3), 3), 0.0, D)
    assert not np.isnan(D).any()


@pytest.mark.parametrize("idx", range(18))
def test_block_cyclic_map_against_fixture(idx):
    c = _load("block_cyclic.npz")["cases"][idx]
    G = np.asfortranarray(c["G"])
    lr = oracle.numroc(G.shape[0], c["mb"], c["myrow"], c["rsrc"], c["prow"])
    lc = oracle.numroc(G.shape[1], c["nb"], c["mycol"], c["csrc"], c["pcol"])
    assert (lr, lc) == (c["lr"], c["lc"])
    L = oracle.scatter_block_cyclic(G, c["mb"], c["nb"], c["prow"], c["pcol"], c["rsrc"], c["csrc"], c["myrow"],
                                    c["mycol"])
    np.testing.assert_array_equal(L[:lr, :lc], c["L"][:lr, :lc])


def test_one_by_one_grid_is_identity_layout():
    # On a 1x1 grid the block-cyclic local buffer is the global matrix itself:
    # the fact the 1x1 pack kernels rely on.
    G = oracle.uniform((83, 77), 4)
    for mb, nb in [(32, 32), (1, 1), (7, 13), (128, 128)]:
        L = oracle.scatter_block_cyclic(G, mb, nb, 1, 1, 0, 0, 0, 0)
        np.testing.assert_array_equal(L, G)


def test_numroc_partitions_every_dimension():
    for n in [0, 1, 7, 64, 65, 1000]:
        for nb in [1, 3, 32]:
            for p in [1, 2, 3, 5]:
                for src in range(p):
                    assert sum(oracle.numroc(n, nb, i, src, p) for i in range(p)) == n


def test_pack_transpose_and_conjugate_bit_exact():
    Z = oracle.uniform((6, 5), 9, dtype=np.complex128)
    P = oracle.pack("C", Z, 5, 6)
    np.testing.assert_array_equal(P, Z.conj().T)
    X = oracle.uniform((6, 5), 10)
    np.testing.assert_array_equal(oracle.pack("T", X, 5, 6), X.T)
    np.testing.assert_array_equal(oracle.pack("N", X, 6, 5), X)


def test_unpack_rounding_is_two_products_and_a_sum():
    rng = np.random.default_rng(11)
    S = np.asfortranarray(rng.standard_normal((8, 8)))
    D0 = np.asfortranarray(rng.standard_normal((8, 8)))
    D = D0.copy(order="F")
    oracle.unpack(1.5, S, 0.5, D)
    np.testing.assert_array_equal(D, (1.5 * S) + (0.5 * D0))  # numpy never contracts


def test_validate_results_restatement():
    assert oracle.validate_results([1.0, 2.0], [1.0, 2.0 + 1e-7])
    assert not oracle.validate_results([1.0, np.nan], [1.0, np.nan])
    assert not oracle.validate_results([1.0], [1.1])
    assert oracle.validate_results([1e-4], [1e-4 + 5e-10])  # absolute below the 1e-3 floor


def test_error_stats():
    hi = np.array([1.0, 2.0, 4.0])
    lo = np.zeros(3)
    c = hi * (1 + np.array([1e-16, 0.0, -2e-16]))
    s = oracle.error_stats(c, hi, lo, np.abs(hi))
    assert s["max_rel_err"] == pytest.approx(2e-16, rel=0.2)
