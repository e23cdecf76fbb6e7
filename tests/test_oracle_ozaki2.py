"""CPU checks of the Chinese-remainder restatement and of the library's
host-side planning (no GPU needed)."""
import math

import numpy as np
import pytest

import oracle
from oracle import ozaki2 as o2


def test_moduli_pairwise_coprime_and_residues_exact_in_bf16():
    for i, p in enumerate(o2.MODULI):
        assert p <= 255
        for q in o2.MODULI[i + 1:]:
            assert math.gcd(p, q) == 1
    # balanced residues stay within [-127, 127]: exact in BF16, and 1024
    # products of two of them sum below 2^24
    for p in o2.MODULI:
        rs = {o2.residues(v, p) for v in range(-3 * p, 3 * p)}
        assert max(abs(r) for r in rs) <= 127
    assert 1024 * 127 * 127 < 2 ** 24


@pytest.mark.parametrize("nmod", [2, 7, 18, 28])
def test_crt_reconstruction_is_exact(nmod):
    M = math.prod(o2.MODULI[:nmod])
    rng = np.random.default_rng(nmod)
    for _ in range(200):
        v = int(rng.integers(-2 ** 62, 2 ** 62)) * int(rng.integers(1, 2 ** 62)) % (M // 2)
        v = v if rng.integers(2) else -v
        res = [o2.residues(v, p) for p in o2.MODULI[:nmod]]
        assert o2.crt_reconstruct(res, nmod) == v


def test_fraction_bits_keep_products_inside_the_modulus_range():
    for nmod in range(2, o2.MAX_MODULI + 1):
        for k in (1, 2, 3, 1000, 1024, 16384, 65536, 4194240):
            P = o2.max_fraction_bits(nmod, k)
            M = math.prod(o2.MODULI[:nmod])
            if P < 1:
                continue
            assert M > 4 * k * 2 ** (2 * P)          # |V| <= k 2^(2P) < M / 4
            assert M <= 4 * k * 2 ** (2 * P + 2) * 2 ** math.ceil(math.log2(k) - math.log2(k) + 1)


def test_scaled_integers_round_half_away_and_bound():
    X = np.array([[0.75, -0.5, 2.0 ** -60, -(2.0 ** -61), 0.0, 0.999999]])
    E = oracle.ozaki.row_exponents(X)
    got = o2.scaled_integers(X, E, 4)
    # 2^(P - E) = 2^4: 0.75*16 = 12, -8, tiny values round to 0, 0.999999*16 -> 16
    assert list(got[0]) == [12, -8, 0, 0, 0, 16]
    Y = oracle.exp_spread((5, 300), 3, 20)
    EY = oracle.ozaki.row_exponents(Y)
    for P in (10, 40, 90):
        Z = o2.scaled_integers(Y, EY, P)
        assert max(abs(int(z)) for z in Z.ravel()) <= 2 ** P


def test_restatement_converges_to_the_exact_product():
    A = oracle.exp_spread((12, 40), 1, 8)
    B = oracle.exp_spread((40, 9), 2, 8)
    hi, lo, ab = oracle.gemm_dd("N", "N", A, B)
    C = o2.ozaki2_gemm("N", "N", A, B, 110)  # every input bit kept: correctly rounded product
    assert np.all(np.abs(C - (hi + lo)) <= np.spacing(np.abs(hi)) * 0.5 + 1e-300)
    # inputs rounded to P bits below each row's leading bit, then one final
    # rounding: the extra error is ~2^-P relative to the row maxima, so rows
    # spanning 2^8 (phi = 8) need ~8 more bits for the same bound
    for phi, P in ((0, 60), (8, 70)):
        A = oracle.exp_spread((12, 40), 3, phi)
        B = oracle.exp_spread((40, 9), 4, phi)
        hi, lo, ab = oracle.gemm_dd("N", "N", A, B)
        C = o2.ozaki2_gemm("N", "N", A, B, P)
        extra = np.abs(C - (hi + lo)) - 0.5 * np.spacing(np.abs(hi))
        assert np.max(extra / ab) < 2.0 ** -55


def test_host_plan_matches_the_restatement(native_lib):
    """cosma_gpu_ozaki2_choose (host-only) against the oracle's rule."""
    import cosma_gb300 as cg
    for k in (1, 7, 1000, 16384, 65536):
        for nmod in (2, 9, 18, 28):
            P = o2.max_fraction_bits(nmod, k)
            if P < 1:  # two moduli cannot hold a product of depth 1000
                with pytest.raises(cg.CosmaGpuError):
                    cg.ozaki2_choose(k, 0.0, nmod)
                continue
            assert cg.ozaki2_choose(k, 0.0, nmod) == (nmod, min(P, 116))
        for spread in (0.0, 5.2, 12.0, 40.0):
            lk = math.log2(k)
            want = math.ceil(max(60.0, 65.0 + 0.85 * (spread - 3.3) - (lk - 8.0))) + 16
            assert cg.ozaki2_choose(k, spread) == o2.choose_moduli(want, k)
            for exact in (1, 53, 61, 85, 200):
                assert cg.ozaki2_choose(k, spread, exact_bits=exact) == o2.choose_moduli(want, k, exact)


def test_exact_fraction_bits():
    X = np.array([[0.75, -0.5, 0.0], [2.0 ** -60, 1.0, 3.0]])
    # row 0: E = 0, lowest set bits 2^-2 (0.75), 2^-1 -> 2; row 1: E = 2, lowest 2^-60 -> 62
    assert o2.exact_fraction_bits(X) == 62
    assert o2.exact_fraction_bits(np.zeros((3, 4))) == 0
    U = oracle.uniform((50, 200), 3)  # numpy uniforms are multiples of 2^-53
    assert o2.exact_fraction_bits(U) <= 53
    # with P >= the exact bits every scaled integer is exact: no rounding happened
    Y = oracle.exp_spread((6, 40), 5, 8)
    P = o2.exact_fraction_bits(Y)
    E = oracle.ozaki.row_exponents(Y)
    Z = o2.scaled_integers(Y, E, P)
    for i in range(Y.shape[0]):
        for l in range(Y.shape[1]):
            assert math.ldexp(int(Z[i, l]), int(E[i]) - P) == Y[i, l]
