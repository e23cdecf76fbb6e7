"""Native FP64 / complex / FP32 GEMM on the GPU vs the oracle (device pointers
and the host-pointer Tiled-MM / local_multiply entry points)."""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, gemm_bound, to_dev

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (7, 5, 3), (64, 64, 16), (83, 77, 83), (127, 129, 65), (200, 96, 257), (256, 256, 512)]


def _op_shape(op, m, k):
    return (m, k) if op == "N" else (k, m)


@pytest.mark.parametrize("m,n,k", SHAPES)
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_dgemm_device_all_ops(native_lib, cuda, m, n, k, ta, tb):
    from cosma_gb300 import gemm_device
    A = oracle.uniform(_op_shape(ta, m, k), 1)
    B = oracle.uniform(_op_shape(tb, k, n), 2)
    C0 = oracle.uniform((m, n), 3)
    alpha, beta = 1.5, -0.5
    lda, ldb, ldc = A.shape[0] + 3, B.shape[0] + 1, m + 2
    dA, dB, dC = to_dev(A, lda), to_dev(B, ldb), to_dev(C0, ldc)
    gemm_device(ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, scalar="d")
    got = from_dev(dC, m, n, ldc)
    ref = oracle.gemm(ta, tb, alpha, A, B, beta, C0.copy(order="F"))
    assert np.all(np.abs(got - ref) <= gemm_bound(ta, tb, alpha, A, B, beta, C0, k))
    # padding between columns untouched
    full = dC.cpu().numpy().reshape(n, ldc)
    assert np.all(full[:, m:] == 0)


def test_dgemm_beta_zero_does_not_read_c(native_lib, cuda):
    from cosma_gb300 import gemm_device
    m, n, k = 70, 50, 40
    A, B = oracle.uniform((m, k), 4), oracle.uniform((k, n), 5)
    dA, dB = to_dev(A), to_dev(B)
    dC = to_dev(np.zeros((m, n)), fill=np.nan)
    gemm_device("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dC, m, scalar="d")
    got = from_dev(dC, m, n)
    assert not np.isnan(got).any()
    ref = oracle.gemm("N", "N", 1.0, A, B, 0.0, np.zeros((m, n), order="F"))
    assert np.all(np.abs(got - ref) <= gemm_bound("N", "N", 1.0, A, B, 0.0, None, k))


def test_dgemm_k_zero_and_alpha_zero_scale_c(native_lib, cuda):
    from cosma_gb300 import gemm_device
    m, n = 33, 17
    C0 = oracle.uniform((m, n), 6)
    for k, alpha in [(0, 1.0), (9, 0.0)]:
        dC = to_dev(C0)
        A, B = oracle.uniform((m, max(k, 1)), 7), oracle.uniform((max(k, 1), n), 8)
        gemm_device("N", "N", m, n, k, alpha, to_dev(A), m, to_dev(B), max(k, 1), 0.25, dC, m, scalar="d")
        np.testing.assert_array_equal(from_dev(dC, m, n), 0.25 * C0)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "N"), ("N", "C"), ("T", "C")])
def test_zgemm_device(native_lib, cuda, ta, tb):
    from cosma_gb300 import gemm_device
    m, n, k = 45, 38, 71
    A = oracle.uniform(_op_shape(ta, m, k), 11, dtype=np.complex128)
    B = oracle.uniform(_op_shape(tb, k, n), 12, dtype=np.complex128)
    C0 = oracle.uniform((m, n), 13, dtype=np.complex128)
    al, be = 0.75 - 0.25j, 0.5 + 0.5j
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C0)
    gemm_device(ta, tb, m, n, k, al, dA, A.shape[0], dB, B.shape[0], be, dC, m, scalar="z")
    got = from_dev(dC, m, n)
    ref = oracle.gemm(ta, tb, al, A, B, be, C0.copy(order="F"))
    bound = 4 * gemm_bound(ta, tb, abs(al), np.abs(A), np.abs(B), abs(be), np.abs(C0), 2 * k)
    assert np.all(np.abs(got - ref) <= bound)


def test_sgemm_native_device(native_lib, cuda):
    from cosma_gb300 import gemm_device
    m, n, k = 96, 80, 300
    A = oracle.uniform((m, k), 21, dtype=np.float32)
    B = oracle.uniform((n, k), 22, dtype=np.float32)
    C0 = oracle.uniform((m, n), 23, dtype=np.float32)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C0)
    gemm_device("N", "T", m, n, k, 1.0, dA, m, dB, n, 1.0, dC, m, scalar="s")
    got = from_dev(dC, m, n)
    ref = oracle.gemm("N", "T", np.float32(1.0), A, B, np.float32(1.0), C0.copy(order="F"))
    # FP32 inputs multiplied in FP64: only the final rounding to FP32 differs
    assert np.all(np.abs(got - ref) <= 2 * np.finfo(np.float32).eps * (np.abs(A) @ np.abs(B.T) + np.abs(C0)))


@pytest.mark.parametrize("m,n,k", [(4, 4, 4), (3, 4, 5)])
def test_local_multiply_one_rank_cases(native_lib, cuda, m, n, k):
    # tests/multiply.cpp:144-145 (P = 1), alpha = beta = 1, checked like test_cosma
    # (utils/cosma_utils.hpp:365-377, epsilon 1e-8) against local_multiply_cpu.
    from cosma_gb300 import local_multiply
    rng = np.random.default_rng(m + n + k)
    A = np.asfortranarray(rng.uniform(0, 10, (m, k)))
    B = np.asfortranarray(rng.uniform(0, 10, (k, n)))
    C0 = np.asfortranarray(rng.uniform(0, 10, (m, n)))
    Cg = C0.copy(order="F")
    local_multiply(A, B, Cg, m, n, k, 1.0, 1.0)
    Cr = C0.copy(order="F")
    oracle.local_multiply_cpu(A, B, Cr, 1.0, 1.0)
    assert oracle.cosma_check(Cg, Cr, 1e-8)


def test_tiled_mm_host_pointers_force_tiling(native_lib, cuda):
    # CI forces Tiled-MM tiling with COSMA_GPU_MAX_TILE_{M,N,K}=100 (ci/cscs.yml:47-49);
    # the same here through explicit tile sizes and 3 streams.
    from cosma_gb300 import gemm, make_context
    h = make_context("d", 3, 100, 100, 100)
    for ta, tb in [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")]:
        m, n, k = 257, 131, 333
        A = oracle.uniform(_op_shape(ta, m, k), 31)
        B = oracle.uniform(_op_shape(tb, k, n), 32)
        C0 = oracle.uniform((m, n), 33)
        Cg = C0.copy(order="F")
        gemm(h, ta, tb, m, n, k, 0.5, A, A.shape[0], B, B.shape[0], 2.0, Cg, m)
        ref = oracle.gemm(ta, tb, 0.5, A, B, 2.0, C0.copy(order="F"))
        assert np.all(np.abs(Cg - ref) <= gemm_bound(ta, tb, 0.5, A, B, 2.0, C0, k, c=4))
    h.close()


def test_tiled_mm_copy_c_back_false_keeps_c_on_device(native_lib, cuda):
    import torch
    from cosma_gb300 import gemm, make_context
    h = make_context("d", 2, 64, 64, 64)
    m, n, k = 100, 90, 80
    A, B = oracle.uniform((m, k), 41), oracle.uniform((k, n), 42)
    Cg = np.zeros((m, n), order="F")
    gemm(h, "N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cg, m, copy_c_back=False)
    assert np.all(Cg == 0)  # host C untouched
    ptr = h.device_buffer_c()
    assert ptr
    out = torch.empty(m * n, dtype=torch.float64, device="cuda")
    from cosma_gb300 import pack
    pack("N", m, n, ptr, m, out, m)  # device-to-device copy of the handle's C buffer
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(n, m).T
    ref = oracle.gemm("N", "N", 1.0, A, B, 0.0, np.zeros((m, n), order="F"))
    assert np.all(np.abs(got - ref) <= gemm_bound("N", "N", 1.0, A, B, 0.0, None, k))
    h.close()


def test_zgemm_host_pointers_a_times_b_conj(native_lib, cuda):
    # the out-of-HBM configuration's operation (C = A * B^H) at a small size
    from cosma_gb300 import gemm, make_context
    h = make_context("z", 2, 96, 96, 64)
    m, n, k = 150, 130, 170
    A = oracle.uniform((m, k), 51, dtype=np.complex128)
    B = oracle.uniform((n, k), 52, dtype=np.complex128)
    Cg = np.zeros((m, n), dtype=np.complex128, order="F")
    gemm(h, "N", "C", m, n, k, 1.0, A, m, B, n, 0.0, Cg, m)
    ref = A @ B.conj().T
    assert np.max(np.abs(Cg - ref)) < 1e-12 * k
    h.close()


def test_invalid_arguments_raise(native_lib, cuda):
    from cosma_gb300 import CosmaGpuError, gemm_device
    import torch
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(CosmaGpuError):
        gemm_device("X", "N", 2, 2, 2, 1.0, d, 2, d, 2, 0.0, d, 2, scalar="d")
    with pytest.raises(CosmaGpuError):
        gemm_device("N", "N", 4, 2, 2, 1.0, d, 2, d, 2, 0.0, d, 2, scalar="d")  # lda < m


@pytest.mark.parametrize("scalar", ["d", "s", "z"])
def test_tiled_mm_pageable_tiles_in_place_and_staged(native_lib, cuda, monkeypatch, scalar):
    """Tiles of pageable matrices with odd leading dimensions stream through
    either host route (device copy kernel in place, or the driver's pageable
    copies with the pin flag registering them): both give bit-identical C,
    matching the same tiling on device pointers."""
    import torch
    from cosma_gb300 import gemm, make_context
    dt = {"d": np.float64, "s": np.float32, "z": np.complex128}[scalar]
    m, n, k = 301, 203, 257
    lda, ldb, ldc = m + 3, k + 1, m + 5
    rng = np.random.default_rng(5)

    def mat(r, c):
        x = rng.uniform(-1, 1, (r, c))
        if scalar == "z":
            x = x + 1j * rng.uniform(-1, 1, (r, c))
        return np.asfortranarray(x.astype(dt))
    A, B, C0 = mat(lda, k), mat(ldb, n), mat(ldc, n)
    alpha, beta = (0.75, -0.5) if scalar != "z" else (0.75 - 0.25j, 0.5 + 1j)
    outs = []
    for direct, pin in (("ON", True), ("OFF", True), ("OFF", False)):
        monkeypatch.setenv("COSMA_GPU_HOST_DIRECT", direct)
        h = make_context(scalar, 3, 96, 64, 80)
        Cg = C0.copy(order="F")
        gemm(h, "N", "N", m, n, k, alpha, A, lda, B, ldb, beta, Cg, ldc, pin_host_buffers=pin)
        h.close()
        outs.append(Cg.tobytes())
    assert outs[0] == outs[1] == outs[2]
    h = make_context(scalar, 3, 96, 64, 80)
    dB = torch.from_numpy(B.reshape(-1, order="F").copy()).cuda()
    Ch = C0.copy(order="F")
    gemm(h, "N", "N", m, n, k, alpha, A, lda, dB, ldb, beta, Ch, ldc)   # mixed host / device operands
    h.close()
    assert Ch.tobytes() == outs[0]
