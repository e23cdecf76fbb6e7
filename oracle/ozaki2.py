"""CPU restatement of the Chinese-remainder (Ozaki scheme II) FP64 GEMM.

Test infrastructure only: the product path never imports this module.  The
reference has no counterpart (it runs a native DGEMM); this restates the
published integer-modular form of the Ozaki scheme (Ozaki, Uchino & Imamura,
"Ozaki Scheme II: A GEMM-oriented emulation of floating-point matrix
multiplication using an integer modular technique", 2025) as the GPU kernels
realise it, so that their result can be checked bit for bit:
  * E_i = 1 + floor(log2 max_l |a_il|) per row of op(A) (0 for zero rows),
    F_j likewise per column of op(B) (the same exponents as the slice form);
  * a'_il = sign(a_il) * round_half_away(|a_il| * 2^(P - E_i)), an integer of
    at most P bits (likewise b'_lj with F_j);
  * V_ij = sum_l a'_il b'_lj, exact.  The GPU obtains V from its residues
    modulo N pairwise coprime moduli p_t <= 255 (one BF16 GEMM per modulus)
    and the Chinese remainder theorem; that is exact because the product M of
    the moduli exceeds 4 k 2^(2P) > 2 max |V|;
  * C_ij = V_ij * 2^(E_i + F_j - 2P) rounded once to double, then
    fl(fl(alpha * C) + fl(beta * C_old)).
Since the reconstruction is exact, the restatement needs only the exact
integer product, which Python integers give directly.
"""
from __future__ import annotations

import math

import numpy as np

from .ozaki import row_exponents

# Pairwise coprime moduli, largest first: 255 = 3*5*17, 254 = 2*127,
# 253 = 11*23, 247 = 13*19, the rest primes.  Balanced residues lie in
# [-127, 127], so every residue is exact in BF16 and 1024 products of two
# residues sum below 2^24 (exact in the FP32 accumulator).  The automatic
# count is the fewer of the accuracy rule's and the count that keeps every
# input bit (then the product is exact and C correctly rounded).
MODULI = (255, 254, 253, 251, 247, 241, 239, 233, 229, 227, 223, 211, 199, 197, 193, 191, 181, 179, 173, 167,
          163, 157, 151, 149, 139, 137, 131, 113)
MAX_MODULI = len(MODULI)


def product_bits(nmod):
    """Bit length of M = p_1 * ... * p_nmod."""
    return math.prod(MODULI[:nmod]).bit_length()


def ceil_log2(k):
    return max(0, (int(k) - 1).bit_length())


def max_fraction_bits(nmod, k):
    """The largest P with M >= 2^(2P + ceil(log2 k) + 2), i.e. M > 4 k 2^(2P)."""
    return (product_bits(nmod) - 1 - ceil_log2(k) - 2) // 2


def _fewest(p_req, k):
    for nmod in range(2, MAX_MODULI + 1):
        if max_fraction_bits(nmod, k) >= p_req:
            return nmod
    return MAX_MODULI + 1


def choose_moduli(p_req, k, exact_bits=None):
    """The automatic choice: the fewer moduli of those whose product admits
    P >= p_req (the accuracy rule) and those that keep every input bit
    (P >= exact_bits); returns (N, P) with P the largest N allows (<= 116)."""
    nmod = _fewest(p_req, k)
    if exact_bits is not None:
        nmod = min(nmod, _fewest(max(int(exact_bits), 1), k))
    nmod = min(nmod, MAX_MODULI)
    return nmod, min(max_fraction_bits(nmod, k), 116)


def exact_fraction_bits(X):
    """Max over the rows of X of E_i minus the weight (log2) of the lowest set
    significand bit in the row: the fraction bits that represent every
    element exactly (0 for an all-zero X)."""
    X = np.asarray(X, dtype=np.float64)
    E = row_exponents(X)
    b = X.view(np.uint64)
    ef = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    frac = b & np.uint64(0xFFFFFFFFFFFFF)
    M = np.where(ef == 0, frac, frac | np.uint64(1 << 52))
    eu = np.where(ef == 0, -1074, ef - 1075)
    low = M & (~M + np.uint64(1))                      # lowest set bit of M
    tz = np.log2(np.where(M == 0, 1, low).astype(np.float64)).astype(np.int64)
    lsb = np.where(M == 0, 1 << 30, eu + tz)
    rowmin = lsb.min(axis=1) if X.shape[1] else np.full(X.shape[0], 1 << 30)
    bits = np.where(rowmin < (1 << 30), E - rowmin, 0)
    return int(bits.max()) if bits.size else 0


def scaled_integers(X, E, P):
    """Object array of sign(x) * round_half_away(|x| * 2^(P - E)) for X (rows x k), E per row."""
    X = np.asarray(X, dtype=np.float64)
    out = np.empty(X.shape, dtype=object)
    for i in range(X.shape[0]):
        e = int(E[i])
        for l in range(X.shape[1]):
            x = float(X[i, l])
            if x == 0.0:
                out[i, l] = 0
                continue
            mant, ex = math.frexp(abs(x))          # |x| = mant * 2^ex, mant in [0.5, 1)
            M = int(mant * (1 << 53))              # 53-bit integer, |x| = M * 2^(ex - 53)
            sh = ex - 53 - e + P
            if sh >= 0:
                v = M << sh
            else:
                r = -sh
                v = (M + (1 << (r - 1))) >> r if r <= 64 else 0
            out[i, l] = -v if x < 0 else v
    return out


def _round_scaled(v, e):
    """v * 2^e rounded once to double (v a Python int)."""
    if v == 0:
        return 0.0
    if e >= 0:
        return float(v << e)
    return v / (1 << (-e))  # CPython's int true division rounds correctly (subnormals included)


def _ops(ta, tb, A, B):
    opA = np.asarray(A if ta in "Nn" else A.T, dtype=np.float64)
    opB = np.asarray(B if tb in "Nn" else B.T, dtype=np.float64)
    return opA, opB


def ozaki2_gemm(ta, tb, A, B, P, alpha=1.0, beta=0.0, C0=None):
    """Exact restatement of the GPU result (small sizes: Python integer arithmetic)."""
    opA, opB = _ops(ta, tb, A, B)
    m, n = opA.shape[0], opB.shape[1]
    EA = row_exponents(opA)
    EB = row_exponents(opB.T)
    XA = scaled_integers(opA, EA, P)
    XB = scaled_integers(opB.T, EB, P)
    V = XA.dot(XB.T)
    C = np.zeros((m, n))
    for i in range(m):
        for j in range(n):
            C[i, j] = _round_scaled(int(V[i, j]), int(EA[i] + EB[j] - 2 * P))
    return _alpha_beta(C, alpha, beta, C0)


def ozaki2_gemm_sampled(ta, tb, A, B, P, rows, cols):
    """The same exact result at the sampled entries (rows[i], cols[i]) only
    (alpha = 1, beta = 0): exponents depend on one row / column each."""
    opA, opB = _ops(ta, tb, A, B)
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    Ar = opA[rows]
    Bc = opB[:, cols].T
    EA = row_exponents(opA)[rows]
    EB = row_exponents(opB.T)[cols]
    XA = scaled_integers(Ar, EA, P)
    XB = scaled_integers(Bc, EB, P)
    out = np.zeros(len(rows))
    for i in range(len(rows)):
        v = sum(int(a) * int(b) for a, b in zip(XA[i], XB[i]))
        out[i] = _round_scaled(v, int(EA[i] + EB[i] - 2 * P))
    return out


def _alpha_beta(C, alpha, beta, C0):
    """fl(fl(alpha * C) + fl(beta * C0)) elementwise, no contraction; C0 unread when beta = 0."""
    out = C.copy()
    if alpha != 1.0:
        out = np.float64(alpha) * out
    if beta != 0.0:
        out = out + np.float64(beta) * np.asarray(C0, dtype=np.float64)
    return out


def _cplx_operands(ta, tb, A, B):
    """op(A) as the real m x 2k matrix [Re | Im]; op(B) as [Re ; -Im] (real part
    of C) and [Im ; Re] (imaginary part), conjugation applied."""
    A = np.asarray(A, dtype=np.complex128)
    B = np.asarray(B, dtype=np.complex128)
    opA = A if ta in "Nn" else (A.T if ta in "Tt" else A.conj().T)
    opB = B if tb in "Nn" else (B.T if tb in "Tt" else B.conj().T)
    Acat = np.concatenate([opA.real, opA.imag], axis=1)
    Bre = np.concatenate([opB.real, -opB.imag], axis=0)
    Bim = np.concatenate([opB.imag, opB.real], axis=0)
    # a column's exponent covers both parts of op(B): [Re; -Im] and [Im; Re] share it
    return Acat, Bre, Bim


def ozaki2_zgemm(ta, tb, A, B, P):
    """Exact restatement of the complex GPU result (alpha = 1, beta = 0): one
    real product of depth 2k per part of C, exponents over both parts."""
    Acat, Bre, Bim = _cplx_operands(ta, tb, A, B)
    return ozaki2_gemm("N", "N", Acat, Bre, P) + 1j * ozaki2_gemm("N", "N", Acat, Bim, P)


def ozaki2_zgemm_sampled(ta, tb, A, B, P, rows, cols):
    Acat, Bre, Bim = _cplx_operands(ta, tb, A, B)
    re = ozaki2_gemm_sampled("N", "N", Acat, Bre, P, rows, cols)
    im = ozaki2_gemm_sampled("N", "N", Acat, Bim, P, rows, cols)
    return re + 1j * im


def residues(v, p):
    """Balanced residue of the Python int v modulo p, as the split kernel
    stores it: ((v + h) mod p) - h with h = floor(p / 2), in [-h, p - 1 - h]."""
    h = p // 2
    return (v + h) % p - h


def crt_reconstruct(res, nmod):
    """V from its balanced residues (list over the first nmod moduli), centred in (-M/2, M/2)."""
    M = math.prod(MODULI[:nmod])
    x = 0
    for t in range(nmod):
        p = MODULI[t]
        Mt = M // p
        x += (res[t] % p) * Mt * pow(Mt, -1, p)
    x %= M
    return x - M if x > M // 2 else x
