"""CPU restatement of the Ozaki-split FP64 GEMM (test infrastructure only).

The reference has no counterpart (it runs a native DGEMM); this restates the
published error-free splitting (Ozaki, Ogita, Oishi & Rump 2012; integer
slices as in Ootomo, Ozaki & Yokota 2024) exactly as the GPU kernels realise
it, so their result can be checked bit for bit:
  * E_i = 1 + floor(log2 max_l |a_il|) per row of op(A) (0 for zero rows),
    F_j likewise per column of op(B);
  * |a| / 2^E_i rounded half away from zero to F = 4 + 5(S-1) fraction bits,
    written as balanced base-32 digits (leading digit 4 bits), sign applied;
  * V_ij = sum over s + t <= S + 1 of (A_s B_t)_ij * 2^(5(S+1 - s - t)),
    exact;
  * C_ij = V_ij * 2^(E_i + F_j - 8 - 5(S-1)) rounded once to double.
"""
from __future__ import annotations

from fractions import Fraction

import numpy as np


def row_exponents(X):
    """E per row of X (rows x k): 1 + floor(log2 max |x|), 0 for zero rows."""
    X = np.asarray(X, dtype=np.float64)
    ax = np.abs(X)
    mx = ax.max(axis=1) if X.shape[1] else np.zeros(X.shape[0])
    E = np.zeros(X.shape[0], dtype=np.int64)
    nz = mx > 0
    E[nz] = np.frexp(mx[nz])[1]  # frexp: mx = f * 2^e with f in [0.5, 1) -> floor(log2) = e - 1
    return E


def digits(x, E, S):
    """Digits (..., S) of x / 2^E, most significant first (vectorised)."""
    x = np.asarray(x, dtype=np.float64)
    E = np.asarray(E, dtype=np.int64)
    b = x.view(np.uint64)
    neg = (b >> np.uint64(63)) != 0
    ef = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    M = b & np.uint64(0xFFFFFFFFFFFFF)
    eu = np.where(ef == 0, -1074, ef - 1075)
    M = np.where(ef == 0, M, M | np.uint64(1 << 52))
    F = 4 + 5 * (S - 1)
    sh = eu - E + F
    sh = np.where(M == 0, 0, sh)
    out = np.zeros(x.shape + (S,), dtype=np.int64)
    neg_sh = sh < 0
    r = np.where(neg_sh, -sh, 0)
    # rounded X = (M + 2^(r-1)) >> r for sh < 0 (0 when r > 63)
    Mr = M.copy()
    rr = np.clip(r, 1, 63).astype(np.uint64)
    rounded = (M + (np.uint64(1) << (rr - np.uint64(1)))) >> rr
    Mr = np.where(neg_sh, np.where(r > 63, np.uint64(0), rounded), M)
    sh = np.where(neg_sh, 0, sh)
    carry = np.zeros(x.shape, dtype=np.int64)
    for p in range(S):
        pos = 5 * p - sh
        right = np.clip(pos, 0, 63).astype(np.uint64)
        left = np.clip(-pos, 0, 63).astype(np.uint64)
        v = np.where(pos >= 64, np.uint64(0), np.where(pos >= 0, Mr >> right, Mr << left))
        u = (v & np.uint64(31)).astype(np.int64) if p < S - 1 else v.astype(np.int64)
        u = u + carry
        if p < S - 1:
            carry = (u >= 16).astype(np.int64)
            dd = np.where(carry == 1, u - 32, u)
        else:
            dd = u
        out[..., S - 1 - p] = np.where(neg, -dd, dd)
    return out


def ozaki_gemm(ta, tb, A, B, S):
    """Exact restatement of the GPU result for alpha = 1, beta = 0 (small sizes)."""
    opA = np.asarray(A if ta in "Nn" else A.T, dtype=np.float64)
    opB = np.asarray(B if tb in "Nn" else B.T, dtype=np.float64)
    m, k = opA.shape
    n = opB.shape[1]
    EA = row_exponents(opA)
    EB = row_exponents(opB.T)
    DA = digits(opA, EA[:, None], S)          # m x k x S
    DB = digits(opB.T, EB[:, None], S)        # n x k x S
    L = 8 + 5 * (S - 1)
    V = np.zeros((m, n), dtype=object)
    for s in range(1, S + 1):
        for t in range(1, S + 2 - s):
            P = DA[:, :, s - 1] @ DB[:, :, t - 1].T  # exact in int64 for k <= 2^46
            V = V + P.astype(object) * (1 << (5 * (S + 1 - s - t)))
    C = np.zeros((m, n))
    for i in range(m):
        for j in range(n):
            e = int(EA[i] + EB[j] - L)
            v = Fraction(int(V[i, j])) * (Fraction(2) ** e)
            C[i, j] = float(v)
    return C


def ozaki_gemm_sampled(ta, tb, A, B, S, rows, cols):
    """The same exact result at the sampled entries (rows[i], cols[i]) only.

    Row and column exponents depend on one row of op(A) / one column of
    op(B) each, so restricting to the sampled rows and columns is exact; this
    pins large problems (many tiles per CTA) at a cost linear in the sample.
    """
    opA = np.asarray(A if ta in "Nn" else A.T, dtype=np.float64)
    opB = np.asarray(B if tb in "Nn" else B.T, dtype=np.float64)
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    Ar = opA[rows]                     # samples x k
    Bc = opB[:, cols].T                # samples x k
    EA = row_exponents(opA)[rows]
    EB = row_exponents(opB.T)[cols]
    DA = digits(Ar, EA[:, None], S)    # samples x k x S
    DB = digits(Bc, EB[:, None], S)
    L = 8 + 5 * (S - 1)
    out = np.zeros(len(rows))
    V = [0] * len(rows)
    for s in range(1, S + 1):
        for t in range(1, S + 2 - s):
            P = np.einsum("ik,ik->i", DA[:, :, s - 1], DB[:, :, t - 1])  # exact in int64
            w = 1 << (5 * (S + 1 - s - t))
            for i in range(len(rows)):
                V[i] += int(P[i]) * w
    for i in range(len(rows)):
        e = int(EA[i] + EB[i] - L)
        out[i] = float(Fraction(V[i]) * (Fraction(2) ** e))
    return out


def _cplx_operands(ta, tb, A, B):
    """op(A) as the real m x 2k matrix [Re | Im] and op(B) as the two real
    2k x n matrices [Re ; -Im] (real part of C) and [Im ; Re] (imaginary
    part), conjugation applied: Re c = sum Re a Re b - Im a Im b and
    Im c = sum Re a Im b + Im a Re b."""
    A = np.asarray(A, dtype=np.complex128)
    B = np.asarray(B, dtype=np.complex128)
    opA = A if ta in "Nn" else (A.T if ta in "Tt" else A.conj().T)
    opB = B if tb in "Nn" else (B.T if tb in "Tt" else B.conj().T)
    Acat = np.asfortranarray(np.concatenate([opA.real, opA.imag], axis=1))
    Bre = np.asfortranarray(np.concatenate([opB.real, -opB.imag], axis=0))
    Bim = np.asfortranarray(np.concatenate([opB.imag, opB.real], axis=0))
    return Acat, Bre, Bim


def ozaki_zgemm(ta, tb, A, B, S):
    """Exact restatement of the complex GPU result (alpha = 1, beta = 0).

    Follows the layout of the complex slice-product GEMM: one real Ozaki
    product of depth 2k per part, with the row exponent of op(A) and the
    column exponent of op(B) taken over both parts (the exponents of
    [Re ; -Im] and [Im ; Re] columns coincide)."""
    Acat, Bre, Bim = _cplx_operands(ta, tb, A, B)
    return ozaki_gemm("N", "N", Acat, Bre, S) + 1j * ozaki_gemm("N", "N", Acat, Bim, S)


def ozaki_zgemm_sampled(ta, tb, A, B, S, rows, cols):
    """ozaki_zgemm at the sampled entries (rows[i], cols[i])."""
    Acat, Bre, Bim = _cplx_operands(ta, tb, A, B)
    re = ozaki_gemm_sampled("N", "N", Acat, Bre, S, rows, cols)
    im = ozaki_gemm_sampled("N", "N", Acat, Bim, S, rows, cols)
    return re + 1j * im


def error_bound_bits(S):
    """Fraction bits F = 4 + 5(S-1) carried by S slices."""
    return 4 + 5 * (S - 1)
