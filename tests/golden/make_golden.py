"""Generates the known-answer fixtures in tests/golden/ (run from the repo root:
``python tests/golden/make_golden.py``).

The reference ships no golden vectors (its tests compare two implementations
on random inputs), so these fixtures pin the oracle independently:
* gemm_exact.npz - small GEMMs whose expected result is the exactly rounded
  value of alpha*op(A)*op(B) + beta*C, computed in rational arithmetic
  (fractions.Fraction) from seeded random doubles; also the exact product
  rounded to double for the double-double oracle.
* block_cyclic.npz - ScaLAPACK block-cyclic local buffers of a global matrix
  for several grids, built element by element from the index map of
  utils/pxgemm_utils.hpp:71-87 written out independently in Python, plus the
  local sizes (numroc, src/cosma/scalapack.cpp:49-88).
* ozaki_digits.npz - balanced base-32 digit expansions of seeded doubles,
  computed in exact rational arithmetic (the slicing the Ozaki kernels use).
"""
from __future__ import annotations

from fractions import Fraction
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


def exact_gemm(ta, tb, alpha, A, B, beta, Cin):
    opA = A if ta == "N" else A.T
    opB = B if tb == "N" else B.T
    m, k = opA.shape
    n = opB.shape[1]
    out = np.zeros((m, n))
    prod = np.zeros((m, n))
    for i in range(m):
        for j in range(n):
            s = sum((Fraction(float(opA[i, l])) * Fraction(float(opB[l, j])) for l in range(k)), Fraction(0))
            prod[i, j] = float(s)  # Fraction -> float rounds to nearest
            v = Fraction(alpha) * s
            if beta != 0:
                v += Fraction(beta) * Fraction(float(Cin[i, j]))
            out[i, j] = float(v)
    return out, prod


def gemm_cases():
    rng = np.random.default_rng(20240607)
    cases = []
    for (m, n, k, ta, tb, alpha, beta) in [
        (4, 4, 4, "N", "N", 1.0, 1.0), (3, 4, 5, "N", "N", 1.0, 1.0), (10, 11, 13, "N", "N", 1.0, 0.0),
        (3, 3, 7, "T", "N", 1.0, 0.0), (7, 5, 9, "N", "T", 0.5, 0.5), (6, 8, 3, "T", "T", 1.5, -1.0),
        (1, 1, 1, "N", "N", 1.0, 0.0), (5, 1, 17, "T", "N", -2.0, 0.25),
    ]:
        A = rng.uniform(-1, 1, size=(m, k) if ta == "N" else (k, m))
        B = rng.uniform(-1, 1, size=(k, n) if tb == "N" else (n, k))
        Cin = rng.uniform(-1, 1, size=(m, n))
        exp, prod = exact_gemm(ta, tb, alpha, A, B, beta, Cin)
        cases.append(dict(m=m, n=n, k=k, ta=ta, tb=tb, alpha=alpha, beta=beta, A=A, B=B, C=Cin, expected=exp,
                          product=prod))
    return cases


def bc_local(G, mb, nb, prow, pcol, rsrc, csrc, myrow, mycol):
    """Local buffer of process (myrow, mycol), from the index map written out
    per element: owner row (gi // mb + rsrc) % prow, local row
    (gi // (mb * prow)) * mb + gi % mb (columns alike)."""
    M, N = G.shape
    rows = [gi for gi in range(M) if (gi // mb + rsrc) % prow == myrow]
    cols = [gj for gj in range(N) if (gj // nb + csrc) % pcol == mycol]
    L = np.zeros((max(len(rows), 1), max(len(cols), 1)))
    for gi in rows:
        li = (gi // (mb * prow)) * mb + gi % mb
        for gj in cols:
            lj = (gj // (nb * pcol)) * nb + gj % nb
            L[li, lj] = G[gi, gj]
    return L, len(rows), len(cols)


def block_cyclic_cases():
    rng = np.random.default_rng(7)
    cases = []
    for (M, N, mb, nb, prow, pcol, rsrc, csrc) in [
        (10, 10, 2, 2, 1, 1, 0, 0), (13, 11, 3, 2, 2, 3, 0, 0), (83, 77, 32, 32, 1, 1, 0, 0),
        (17, 9, 4, 5, 3, 2, 1, 1), (64, 48, 8, 8, 2, 2, 1, 0),
    ]:
        G = rng.uniform(-1, 1, size=(M, N))
        for myrow in range(prow):
            for mycol in range(pcol):
                L, lr, lc = bc_local(G, mb, nb, prow, pcol, rsrc, csrc, myrow, mycol)
                cases.append(dict(G=G, mb=mb, nb=nb, prow=prow, pcol=pcol, rsrc=rsrc, csrc=csrc, myrow=myrow,
                                  mycol=mycol, L=L, lr=lr, lc=lc))
    return cases


def balanced_digits(x: float, e_row: int, nslices: int):
    """Digits d_1..d_S of x / 2**e_row with a 4-bit first digit and 5-bit
    digits after it: |x| / 2**e_row is rounded to F = 4 + 5(S-1) fraction
    bits (half away from zero), written in balanced base 32 (every digit in
    [-16, 15] except the leading one, in [0, 16]), and the sign of x applied
    to every digit, so x / 2**e_row ~= sum_s d_s 2**(-4 - 5(s-1))."""
    F = 4 + 5 * (nslices - 1)
    v = Fraction(x) / Fraction(2) ** e_row * Fraction(2) ** F
    sgn = -1 if v < 0 else 1
    a = abs(v)
    X = int(a)
    if a - X >= Fraction(1, 2):
        X += 1
    digits = []
    for _ in range(nslices - 1):
        d = ((X + 16) % 32) - 16
        digits.append(d)
        X = (X - d) // 32
    digits.append(X)
    digits.reverse()
    digits = [sgn * d for d in digits]
    assert all(abs(d) <= 16 for d in digits), digits
    return digits


def ozaki_digit_cases():
    rng = np.random.default_rng(99)
    xs = np.concatenate([rng.uniform(-1, 1, 64), np.ldexp(rng.uniform(-1, 1, 32), rng.integers(-40, 40, 32)),
                         np.array([0.0, 1.0, -1.0, 0.5, -0.5, 2.0 ** -60, 0.99999999999, 5e-324])])
    out = []
    for S in (4, 8, 11, 13):
        for x in xs:
            e_row = int(np.frexp(x)[1]) if x != 0 else 0  # |x| < 2**e_row
            e_row += int(rng.integers(0, 3))              # row maximum may be larger
            out.append((float(x), e_row, S, balanced_digits(float(x), e_row, S)))
    return out


def main():
    g = gemm_cases()
    np.savez_compressed(OUT / "gemm_exact.npz", cases=np.array(g, dtype=object), allow_pickle=True)
    bc = block_cyclic_cases()
    np.savez_compressed(OUT / "block_cyclic.npz", cases=np.array(bc, dtype=object), allow_pickle=True)
    oz = ozaki_digit_cases()
    xs = np.array([c[0] for c in oz])
    er = np.array([c[1] for c in oz], dtype=np.int64)
    ss = np.array([c[2] for c in oz], dtype=np.int64)
    dg = np.zeros((len(oz), 13), dtype=np.int64)
    for i, c in enumerate(oz):
        dg[i, :len(c[3])] = c[3]
    np.savez_compressed(OUT / "ozaki_digits.npz", x=xs, e_row=er, slices=ss, digits=dg)
    print("wrote", len(g), "gemm cases,", len(bc), "block-cyclic cases,", len(oz), "digit cases")


if __name__ == "__main__":
    main()
