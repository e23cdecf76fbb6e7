"""multiply_using_layout on one rank vs the oracle.

Matrices are split into uneven blocks (some empty), each block in host or
device memory with its own leading dimension.  Every op combination, real and
complex, alpha / beta, the corner cases of multiply.cpp:99-109, and the Ozaki
method bit-exact against the oracle's restatement.
"""
import numpy as np
import pytest

import oracle
from gpu_util import gemm_bound
from oracle import ozaki as oz

pytestmark = pytest.mark.gpu


def _split(n, parts, rng):
    cuts = np.sort(rng.integers(0, n + 1, parts - 1))
    return [0] + [int(x) for x in cuts] + [n]


def _blocks(G, rs, cs, rng):
    """Block layout of G; blocks alternate randomly between host and device."""
    import torch
    from cosma_gb300 import BlockLayout
    blocks, keep = {}, {}
    for r in range(len(rs) - 1):
        for c in range(len(cs) - 1):
            sub = G[rs[r]:rs[r + 1], cs[c]:cs[c + 1]]
            ld = max(sub.shape[0], 1) + int(rng.integers(0, 3))
            host = np.zeros((ld, max(sub.shape[1], 1)), dtype=G.dtype, order="F")
            host[:sub.shape[0], :sub.shape[1]] = sub
            buf = host if rng.random() < 0.5 else torch.from_numpy(host.reshape(-1, order="F").copy()).cuda()
            blocks[(r, c)] = (buf, ld)
    return BlockLayout(rs, cs, blocks)


def _gather(lay, rows, cols, dtype):
    out = np.zeros((rows, cols), dtype=dtype)
    rs, cs = list(lay.rowsplit), list(lay.colsplit)
    for (r, c), (buf, ld) in lay._keep.items():
        h = buf if isinstance(buf, np.ndarray) else buf.cpu().numpy().reshape(-1, ld).T
        nr, nc = rs[r + 1] - rs[r], cs[c + 1] - cs[c]
        out[rs[r]:rs[r + 1], cs[c]:cs[c + 1]] = h[:nr, :nc]
    return out


@pytest.mark.parametrize("scalar", ["d", "z"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "C"), ("C", "T")])
def test_blocks_against_oracle(native_lib, cuda, scalar, ta, tb):
    from cosma_gb300 import multiply_using_layout
    rng = np.random.default_rng(hash((scalar, ta, tb)) % 1000)
    m, n, k = 70, 53, 91
    dt = np.float64 if scalar == "d" else np.complex128

    def rand(shape, seed):
        x = oracle.uniform(shape, seed)
        return x if scalar == "d" else x + 1j * oracle.uniform(shape, seed + 500)

    A = rand((m, k) if ta == "N" else (k, m), 1)
    B = rand((k, n) if tb == "N" else (n, k), 2)
    C0 = rand((m, n), 3)
    alpha, beta = (1.5, 0.5) if scalar == "d" else (1.5 - 0.5j, 0.25 + 1j)
    la = _blocks(A, _split(A.shape[0], 3, rng), _split(A.shape[1], 4, rng), rng)
    lb = _blocks(B, _split(B.shape[0], 2, rng), _split(B.shape[1], 3, rng), rng)
    lc = _blocks(C0, _split(m, 3, rng), _split(n, 2, rng), rng)
    multiply_using_layout(ta, tb, alpha, la, lb, beta, lc, scalar=scalar)
    got = _gather(lc, m, n, dt)
    opA = A if ta == "N" else (A.T if ta == "T" else A.conj().T)
    opB = B if tb == "N" else (B.T if tb == "T" else B.conj().T)
    ref = alpha * (opA @ opB) + beta * C0
    bound = 2.0 * (k + 2) * 2.0 ** -53 * (abs(alpha) * (np.abs(opA) @ np.abs(opB)) + abs(beta) * np.abs(C0)) * 4
    assert np.all(np.abs(got - ref) <= bound + 1e-300)


def test_corner_cases(native_lib, cuda):
    from cosma_gb300 import multiply_using_layout
    rng = np.random.default_rng(4)
    m, n, k = 20, 15, 9
    A, B, C0 = oracle.uniform((m, k), 1), oracle.uniform((k, n), 2), oracle.uniform((m, n), 3)
    # alpha == 0: C <- beta * C
    lc = _blocks(C0, _split(m, 2, rng), _split(n, 2, rng), rng)
    multiply_using_layout("N", "N", 0.0, _blocks(A, [0, m], [0, k], rng), _blocks(B, [0, k], [0, n], rng), 2.0, lc)
    np.testing.assert_array_equal(_gather(lc, m, n, np.float64), 2.0 * C0)
    # beta == 0: C is never read (NaN in C does not propagate)
    nan = np.full((m, n), np.nan)
    lc = _blocks(nan, _split(m, 2, rng), _split(n, 3, rng), rng)
    multiply_using_layout("N", "N", 1.0, _blocks(A, [0, m], [0, k], rng), _blocks(B, [0, k], [0, n], rng), 0.0, lc)
    got = _gather(lc, m, n, np.float64)
    assert np.all(np.isfinite(got))
    assert np.all(np.abs(got - A @ B) <= gemm_bound("N", "N", 1.0, A, B, 0.0, None, k))


def test_ozaki_method_bit_exact(native_lib, cuda):
    from cosma_gb300 import multiply_using_layout, pxgemm_set_method
    rng = np.random.default_rng(5)
    m, n, k = 300, 140, 170
    A, B, C0 = oracle.exp_spread((k, m), 6, 3), oracle.exp_spread((k, n), 7, 3), oracle.uniform((m, n), 8)
    la = _blocks(A, _split(k, 3, rng), _split(m, 2, rng), rng)
    lb = _blocks(B, _split(k, 2, rng), _split(n, 2, rng), rng)
    lc = _blocks(C0, _split(m, 2, rng), _split(n, 3, rng), rng)
    pxgemm_set_method("ozaki")
    try:
        multiply_using_layout("T", "N", 1.5, la, lb, 0.5, lc)
    finally:
        pxgemm_set_method("native")
    got = _gather(lc, m, n, np.float64)
    from cosma_gb300 import dgemm_ozaki_device  # noqa: F401  (same slice rule as the device entry)
    import torch
    dA = torch.from_numpy(A.reshape(-1, order="F").copy()).cuda()
    dB = torch.from_numpy(B.reshape(-1, order="F").copy()).cuda()
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    S = dgemm_ozaki_device("T", "N", m, n, k, 1.0, dA, k, dB, k, 0.0, dC, m)["slices"]
    want = 1.5 * oz.ozaki_gemm("T", "N", A, B, S) + 0.5 * C0
    np.testing.assert_array_equal(got, want)
