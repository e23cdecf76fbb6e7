"""COSTA 1x1 pack / unpack kernels: bit-exact against the oracle."""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (7, 3), (64, 64), (65, 63), (83, 77), (130, 257), (1000, 31)]


@pytest.mark.parametrize("rows,cols", SHAPES)
@pytest.mark.parametrize("op", ["N", "T", "C"])
@pytest.mark.parametrize("dtype", [np.float64, np.complex128, np.float32, np.complex64])
def test_pack_bit_exact(native_lib, cuda, rows, cols, op, dtype):
    from cosma_gb300 import pack
    src_shape = (rows, cols) if op == "N" else (cols, rows)
    S = oracle.uniform(src_shape, rows * 31 + cols, dtype=dtype)
    if np.iscomplexobj(S):
        S.flat[0] = complex(-0.0, -0.0)  # signed zeros survive conjugation as IEEE negation
    lds, ldd = src_shape[0] + 5, rows + 3
    dS = to_dev(S, lds)
    dD = to_dev(np.zeros((rows, cols), dtype=dtype), ldd)
    pack(op, rows, cols, dS, lds, dD, ldd, is_complex=np.iscomplexobj(S), elem_bytes=S.itemsize)
    got = from_dev(dD, rows, cols, ldd)
    ref = oracle.pack(op, S, rows, cols)
    assert got.tobytes() == ref.tobytes()


@pytest.mark.parametrize("alpha,beta", [(1.5, 0.5), (1.0, 0.0), (0.5, 1.0), (-2.0, -0.25), (1.0, 0.3), (0.5, 0.0),
                                        (-0.7, 1.0)])
@pytest.mark.parametrize("rows,ldd_extra", [(129, 7), (128, 8)])  # element-wise, and 16-byte pairs
def test_unpack_real_bit_exact(native_lib, cuda, alpha, beta, rows, ldd_extra):
    from cosma_gb300 import unpack
    cols = 77
    S = oracle.normal((rows, cols), 1)
    D0 = oracle.normal((rows, cols), 2)
    ldd = rows + ldd_extra
    dS = to_dev(S)
    dD = to_dev(D0, ldd, fill=np.nan if beta == 0 else None)
    unpack(rows, cols, alpha, dS, rows, beta, dD, ldd, scalar="d")
    got = from_dev(dD, rows, cols, ldd)
    ref = oracle.unpack(alpha, S, beta, D0.copy(order="F"))
    assert got.tobytes() == ref.tobytes()


@pytest.mark.parametrize("alpha,beta", [(2.0, 0.5), (0.25, 4.0), (1.0, 2.0 ** -1000), (2.0 ** 1000, 1.0),
                                        (1.5, 0.5), (-3.0, 0.75), (1.0 + 2.0 ** -10, -2047.0), (1.5 * 2.0 ** 900, 1.0),
                                        (0.75 * 2.0 ** -1000, -1.5)])
def test_unpack_power_of_two_scales_at_the_range_edges(native_lib, cuda, alpha, beta):
    """Power-of-two alpha / beta scale by moving the exponent field, and scales
    with a significand of at most 11 bits (1.5, -3, 0.75, 1 + 2^-10, -2047)
    multiply in integer arithmetic; values whose product leaves the normal
    range (subnormals, overflow to Inf, the smallest normals), zeros of both
    signs and Inf / NaN must still round exactly as the FP64 multiply does."""
    from cosma_gb300 import unpack
    rows, cols = 64, 9
    rng = np.random.default_rng(9)
    S = oracle.normal((rows, cols), 5)
    D0 = oracle.normal((rows, cols), 6)
    edge = np.array([0.0, -0.0, 5e-324, -7e-322, 2.2250738585072014e-308, 4.4e-308, 1.7e308, -1.2e308,
                     np.inf, -np.inf, 3.0e-300, 1e-310, 2.0 ** -1022 * 3, 1.0, 0.75, 2.0 ** 1023])
    for X in (S, D0):
        X[:edge.size, 0] = edge
        X[:edge.size, 1] = -edge[::-1]
        X[:, 2] = rng.choice(edge, rows)
    dS, dD = to_dev(S), to_dev(D0)
    unpack(rows, cols, alpha, dS, rows, beta, dD, rows, scalar="d")
    got = from_dev(dD, rows, cols)
    with np.errstate(all="ignore"):
        ref = oracle.unpack(alpha, S, beta, D0.copy(order="F"))
    # inf + -inf: NaN on both sides (host and device encode NaN differently); every other value bit for bit
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    assert got[~nan].tobytes() == ref[~nan].tobytes()


def test_unpack_complex_bit_exact(native_lib, cuda):
    from cosma_gb300 import unpack
    rows, cols = 65, 33
    S = oracle.uniform((rows, cols), 3, dtype=np.complex128)
    D0 = oracle.uniform((rows, cols), 4, dtype=np.complex128)
    for al, be in [(1.5 - 0.5j, 0.25 + 2j), (1.0, 0.0)]:
        dD = to_dev(D0, fill=np.nan if be == 0 else None)
        unpack(rows, cols, al, to_dev(S), rows, be, dD, rows, scalar="z")
        got = from_dev(dD, rows, cols)
        ref = oracle.unpack(al, S, be, D0.copy(order="F"))
        assert got.tobytes() == ref.tobytes()


def test_pack_transpose_large_roundtrip(native_lib, cuda):
    # size-independent property at a larger size: T(T(X)) == X bit for bit
    import torch
    from cosma_gb300 import pack
    rows, cols = 4096 + 17, 2048 + 3
    X = torch.randn(rows * cols, dtype=torch.float64, device="cuda")
    Y = torch.empty_like(X)
    Z = torch.empty_like(X)
    pack("T", cols, rows, X, rows, Y, cols)
    pack("T", rows, cols, Y, cols, Z, rows)
    torch.cuda.synchronize()
    assert torch.equal(X, Z)
