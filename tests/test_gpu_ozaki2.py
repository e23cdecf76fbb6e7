"""Chinese-remainder (Ozaki scheme II) FP64-accurate GEMM vs the oracle.

* bit-exact against the CPU restatement (oracle/ozaki2.py: the exact integer
  product of the rounded operands, rounded once) on small sizes, every op
  combination, explicit and automatic modulus counts;
* K beyond one exact FP32 accumulation (1024) and beyond the 64-chunk
  reduction of the 32-bit running sums;
* several tiles per CTA pair (persistent loop over (modulus, tile) units) on
  sampled entries;
* alpha and beta, beta == 0 with NaN in C, non-finite inputs (native path);
* the complex form (four real products per complex one), ops N/T/C;
* accuracy against the double-double oracle for the precision
  configuration's distributions.
"""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, to_dev
from oracle import ozaki2 as o2

pytestmark = pytest.mark.gpu


def _op_shape(op, m, k):
    return (m, k) if op == "N" else (k, m)


def _run(ta, tb, m, n, k, A, B, alpha=1.0, beta=0.0, C0=None, moduli=0, lda=None, ldb=None, ldc=None):
    from cosma_gb300 import dgemm_ozaki2_device
    lda = lda or A.shape[0]
    ldb = ldb or B.shape[0]
    ldc = ldc or m
    dA, dB = to_dev(A, lda), to_dev(B, ldb)
    dC = to_dev(C0 if C0 is not None else np.zeros((m, n)), ldc)
    info = dgemm_ozaki2_device(ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, moduli=moduli)
    return from_dev(dC, m, n, ldc), info


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("m,n,k,N", [(17, 9, 33, 6), (64, 40, 130, 12), (130, 70, 200, 18), (5, 300, 129, 28)])
def test_bit_exact_against_restatement(native_lib, cuda, ta, tb, m, n, k, N):
    A = oracle.exp_spread(_op_shape(ta, m, k), m + k, 6)
    B = oracle.exp_spread(_op_shape(tb, k, n), n + k, 6)
    got, info = _run(ta, tb, m, n, k, A, B, moduli=N, lda=A.shape[0] + 1, ldc=m + 3)
    P = o2.max_fraction_bits(N, k)
    assert info["slices"] == N and info["fraction_bits"] == P
    np.testing.assert_array_equal(got, o2.ozaki2_gemm(ta, tb, A, B, P))


def test_automatic_modulus_count(native_lib, cuda):
    """The automatic count is the host rule on the measured spread and exact
    bits; where it keeps every input bit the result is the correctly rounded
    product."""
    import cosma_gb300 as cg
    m, n, k = 48, 40, 300
    for phi in (0, 8, 32):
        A = oracle.exp_spread((m, k), 10 + phi, phi)
        B = oracle.exp_spread((k, n), 20 + phi, phi)
        got, info = _run("N", "N", m, n, k, A, B)
        exact = max(o2.exact_fraction_bits(A), o2.exact_fraction_bits(B.T))
        assert (info["slices"], info["fraction_bits"]) == cg.ozaki2_choose(k, info["spread_bits"], exact_bits=exact)
        assert info["exact_product"] == int(info["fraction_bits"] >= exact)
        np.testing.assert_array_equal(got, o2.ozaki2_gemm("N", "N", A, B, info["fraction_bits"]))
        if info["exact_product"]:
            hi, lo, ab = oracle.gemm_dd("N", "N", A, B)
            np.testing.assert_array_equal(got, hi + lo)  # correctly rounded


@pytest.mark.parametrize("k", [1024, 1025, 5000, 70000])
def test_long_k_chunks_and_reductions(native_lib, cuda, k):
    """1024 products per exact accumulation; 64 chunks per running-sum reduction."""
    m, n = 9, 7
    A = oracle.uniform((m, k), k)
    B = oracle.uniform((k, n), k + 1)
    got, info = _run("N", "N", m, n, k, A, B, moduli=18)
    assert info["groups"] == 18 * -(-k // 1024)
    np.testing.assert_array_equal(got, o2.ozaki2_gemm("N", "N", A, B, info["fraction_bits"]))


def test_exact_integer_product_at_maximal_residues(native_lib, cuda):
    """Integer inputs are represented exactly, so C is the exact integer product;
    rows / columns of maximal magnitude stress the 2^24 accumulator bound."""
    rng = np.random.default_rng(3)
    m, n, k = 256, 256, 4096
    A = np.asfortranarray(rng.integers(-2 ** 20, 2 ** 20, (m, k)).astype(np.float64))
    B = np.asfortranarray(rng.integers(-2 ** 20, 2 ** 20, (k, n)).astype(np.float64))
    A[:4, :] = 2.0 ** 20 - 1
    B[:, :4] = -(2.0 ** 20 - 1)
    got, info = _run("N", "N", m, n, k, A, B, moduli=20)
    exact = A.astype(np.int64) @ B.astype(np.int64)  # |sum| < 2^52: exact in int64 and in double
    np.testing.assert_array_equal(got, exact.astype(np.float64))


@pytest.mark.parametrize("ta,tb,m,n,k,N", [
    ("N", "N", 2560, 2304, 256, 8),   # 90 pair tiles x 8 moduli over 76 pairs
    ("T", "N", 1300, 700, 300, 18),   # m padded to 1536
    ("N", "T", 384, 5120, 200, 12),
])
def test_bit_exact_sampled_many_tiles(native_lib, cuda, ta, tb, m, n, k, N):
    A = oracle.exp_spread(_op_shape(ta, m, k), m + 3, 6)
    B = oracle.exp_spread(_op_shape(tb, k, n), n + 5, 6)
    got, info = _run(ta, tb, m, n, k, A, B, moduli=N)
    rng = np.random.default_rng(m + n)
    rows = np.concatenate([rng.integers(0, m, 600), [0, m - 1, m - 1, 0]])
    cols = np.concatenate([rng.integers(0, n, 600), [0, n - 1, 0, n - 1]])
    ref = o2.ozaki2_gemm_sampled(ta, tb, A, B, info["fraction_bits"], rows, cols)
    np.testing.assert_array_equal(got[rows, cols], ref)


def test_alpha_beta_and_nan_safety(native_lib, cuda):
    m, n, k = 70, 50, 90
    A = oracle.uniform((m, k), 1)
    B = oracle.uniform((k, n), 2)
    C0 = oracle.uniform((m, n), 3)
    got, info = _run("N", "N", m, n, k, A, B, alpha=-1.5, beta=0.75, C0=C0, moduli=18)
    np.testing.assert_array_equal(got, o2.ozaki2_gemm("N", "N", A, B, info["fraction_bits"], -1.5, 0.75, C0))
    Cnan = np.full((m, n), np.nan)
    got, info = _run("N", "N", m, n, k, A, B, alpha=2.0, beta=0.0, C0=Cnan, moduli=18)
    assert not np.isnan(got).any()
    np.testing.assert_array_equal(got, o2.ozaki2_gemm("N", "N", A, B, info["fraction_bits"], 2.0))


def test_non_finite_inputs_run_native(native_lib, cuda):
    m, n, k = 20, 10, 30
    A = oracle.uniform((m, k), 4)
    A[3, 7] = np.inf
    B = oracle.uniform((k, n), 5)
    got, info = _run("N", "N", m, n, k, A, B)
    assert info["fallback_native"] == 1
    assert np.all(~np.isfinite(got[3])) and np.all(np.isfinite(np.delete(got, 3, axis=0)))


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "C"), ("T", "N"), ("C", "T")])
def test_complex_bit_exact(native_lib, cuda, ta, tb):
    from cosma_gb300 import zgemm_ozaki2_device
    m, n, k, N = 40, 30, 36, 18
    A = oracle.uniform(_op_shape(ta, m, k), 5, dtype=np.complex128)
    B = oracle.uniform(_op_shape(tb, k, n), 7, dtype=np.complex128)
    dA, dB = to_dev(A), to_dev(B)
    dC = to_dev(np.zeros((m, n), dtype=np.complex128))
    info = zgemm_ozaki2_device(ta, tb, m, n, k, 1.0, dA, A.shape[0], dB, B.shape[0], 0.0, dC, m, moduli=N)
    assert info["fraction_bits"] == o2.max_fraction_bits(N, 2 * k)
    np.testing.assert_array_equal(from_dev(dC, m, n), o2.ozaki2_zgemm(ta, tb, A, B, info["fraction_bits"]))


def test_complex_alpha_beta(native_lib, cuda):
    from cosma_gb300 import zgemm_ozaki2_device
    m, n, k = 33, 17, 40
    A = oracle.uniform((m, k), 8, dtype=np.complex128)
    B = oracle.uniform((k, n), 9, dtype=np.complex128)
    C0 = oracle.uniform((m, n), 10, dtype=np.complex128)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C0)
    al, be = 0.5 - 1.25j, 2.0 + 0.5j
    zgemm_ozaki2_device("N", "N", m, n, k, al, dA, m, dB, k, be, dC, m)
    exact = A.astype(np.complex256) @ B.astype(np.complex256) if hasattr(np, "complex256") else A @ B
    want = al * exact.astype(np.complex128) + be * C0
    np.testing.assert_allclose(from_dev(dC, m, n), want, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("phi", [0, 8, 32])
def test_accuracy_against_double_double(native_lib, cuda, phi):
    m = n = 384
    k = 2048
    A = oracle.exp_spread((m, k), 40 + phi, phi)
    B = oracle.exp_spread((k, n), 50 + phi, phi)
    got, info = _run("N", "N", m, n, k, A, B)
    hi, lo, ab = oracle.gemm_dd("N", "N", A, B)
    st = oracle.error_stats(got.ravel(), hi.ravel(), lo.ravel(), ab.ravel())
    assert st["max_err_over_absab"] <= 2.0 ** -52
    assert st["max_rel_err"] <= 1e-15, st


def test_residual_mode_is_exact(native_lib, cuda):
    """E = op(A) op(B) - Ct exact before one rounding, Rx = the product rounded
    once, against rational arithmetic (every input bit is kept at 28 moduli)."""
    from fractions import Fraction

    import cosma_gb300 as cg
    m, n, k = 40, 24, 300
    A = oracle.uniform((k, m), 61)  # op(A) = A^T
    B = oracle.uniform((k, n), 62)
    Ct = np.asfortranarray(A.T @ B)  # a candidate with ordinary FP64 rounding errors
    Ct[0, 0] = 0.0
    dA, dB, dCt = to_dev(A), to_dev(B), to_dev(Ct)
    dE, dR = to_dev(np.zeros((m, n))), to_dev(np.zeros((m, n)))
    info = cg.dgemm_ozaki2_residual("T", "N", m, n, k, dA, k, dB, k, dCt, m, dE, dR, m, moduli=28)
    assert info["slices"] == 28 and info["fraction_bits"] >= 98
    E, R = from_dev(dE, m, n), from_dev(dR, m, n)
    for i in range(m):
        for j in range(n):
            exact = sum(Fraction(float(A[l, i])) * Fraction(float(B[l, j])) for l in range(k))
            assert R[i, j] == float(exact)
            assert E[i, j] == float(exact - Fraction(float(Ct[i, j])))


def test_full_result_accuracy_at_4096(native_lib, cuda):
    """Every entry of the 4096^3 precision-configuration product (phi = 0)
    against the exact product: max elementwise relative error <= 1e-15, and
    <= 2^-52 of (|A||B|)_ij."""
    import torch

    import cosma_gb300 as cg
    n = 4096
    A = oracle.exp_spread((n, n), 71, 0)
    B = oracle.exp_spread((n, n), 72, 0)
    dA = torch.from_numpy(A.reshape(-1, order="F")).cuda()
    dB = torch.from_numpy(B.reshape(-1, order="F")).cuda()
    dC = torch.empty(n * n, dtype=torch.float64, device="cuda")
    info = cg.dgemm_ozaki2_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n)
    dE, dR = torch.empty_like(dC), torch.empty_like(dC)
    cg.dgemm_ozaki2_residual("N", "N", n, n, n, dA, n, dB, n, dC, n, dE, dR, n, moduli=28)
    absab = torch.empty_like(dC)
    cg.dgemm_ozaki2_device("N", "N", n, n, n, 1.0, dA.abs(), n, dB.abs(), n, 0.0, absab, n, moduli=8)
    torch.cuda.synchronize()
    assert not torch.isnan(dE).any()
    nz = dR != 0
    rel = (dE.abs()[nz] / dR.abs()[nz])
    normwise = dE.abs() / absab
    assert float(normwise.max()) <= 2.0 ** -52, info
    assert float(rel.max()) <= 1e-15, (float(rel.max()), int((rel > 1e-15).sum()), info)


@pytest.mark.parametrize("scalar", ["d", "z"])
def test_tiled_mm_one_step_c_in_place(native_lib, cuda, monkeypatch, scalar):
    """A one-step Tiled-MM call with the Chinese-remainder method: the
    reconstruction kernel reads and writes host C in place (device access to
    host memory) or C is staged through a device slot; both give the bits of
    the device-pointer call, and the D2H count still reports C once."""
    from cosma_gb300 import dgemm_ozaki2_device, gemm, make_context, zgemm_ozaki2_device
    dt = np.float64 if scalar == "d" else np.complex128
    m, n, k = 150, 97, 210
    ldc = m + 3
    A = oracle.uniform((m, k), 61, dtype=dt)
    B = oracle.uniform((n, k), 62, dtype=dt)
    C0 = np.asfortranarray(oracle.uniform((ldc, n), 63, dtype=dt))
    alpha, beta = (0.75, -0.5) if scalar == "d" else (0.75 - 0.25j, 0.5 + 1j)
    tb = "T" if scalar == "d" else "C"
    outs = []
    for direct in ("ON", "OFF"):
        monkeypatch.setenv("COSMA_GPU_HOST_DIRECT", direct)
        h = make_context(scalar, 2)
        h.set_method("ozaki2", 20)
        Cg = C0.copy(order="F")
        gemm(h, "N", tb, m, n, k, alpha, A, m, B, n, beta, Cg, ldc)
        assert h.transfer_bytes()[1] == m * n * Cg.itemsize
        h.close()
        outs.append(Cg)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C0[:m], ldc)
    run = dgemm_ozaki2_device if scalar == "d" else zgemm_ozaki2_device
    run("N", tb, m, n, k, alpha, dA, m, dB, n, beta, dC, ldc, moduli=20)
    want = from_dev(dC, m, n, ldc)
    for got in outs:
        np.testing.assert_array_equal(got[:m], want)
        np.testing.assert_array_equal(got[m:], C0[m:])  # rows past m untouched


def _host_matrix(A, pinned):
    """Column-major host copy of A, pageable numpy or page-locked torch memory."""
    import torch
    if not pinned:
        return np.asfortranarray(A), None
    t = torch.from_numpy(np.ascontiguousarray(A.T).reshape(-1)).pin_memory()  # column-major flat
    return t, t


def _tmm_call(ta, tb, m, n, k, A, B, C0, alpha, beta, ldc, pinned, overlap, monkeypatch, moduli=0, streams=3):
    from cosma_gb300 import gemm, make_context
    monkeypatch.setenv("COSMA_GPU_OZAKI2_OVERLAP", "ON" if overlap else "OFF")
    hA, _ = _host_matrix(A, pinned)
    hB, _ = _host_matrix(B, pinned)
    Cfull = np.zeros((ldc, n))
    Cfull[:m] = C0
    hC, tC = _host_matrix(Cfull, pinned)
    h = make_context("d", streams)
    h.set_method("ozaki2", moduli)
    gemm(h, ta, tb, m, n, k, alpha, hA, A.shape[0], hB, B.shape[0], beta, hC, ldc)
    moved = h.transfer_bytes()
    info = h.ozaki_info()
    h.close()
    out = tC.numpy().reshape(n, ldc).T if tC is not None else hC
    return np.array(out), moved, info


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
@pytest.mark.parametrize("ta,tb,beta,shape", [("N", "N", 0.0, (2100, 2300, 300)), ("T", "N", 0.5, (2100, 2300, 300)),
                                              ("N", "T", -1.0, (2100, 2300, 300)), ("T", "T", 0.0, (2100, 2300, 300)),
                                              ("T", "N", 0.5, (4500, 2300, 96)), ("N", "T", 0.0, (4500, 4200, 40)),
                                              ("N", "N", 0.5, (1000, 4500, 64)), ("T", "T", -1.0, (2100, 2300, 1))])
def test_tiled_mm_overlapped_panels(native_lib, cuda, monkeypatch, ta, tb, beta, shape, pinned):
    """One-step Tiled-MM calls on host arrays (page-locked torch memory or
    pageable numpy arrays, whose copies a worker thread issues) large enough
    for the overlapped form (2 x 2 panels: op(A) rows and op(B) columns arrive
    while earlier blocks compute): the bits of the one-step form without
    overlap and of the device-pointer call; transfers count A and B (and C,
    when it is read) once.  Handles with two streams carry the C blocks on the
    copy stream.  The overlapped form times no phases (gemm_ms stays 0), which
    tells it from the one-step form.  With m >= 4096 the first op(A) panel is
    a shorter lead panel (2048 rows, then 2304 and a ragged 148: 3 x 2
    blocks; 3 x 4 with n = 4200), more blocks than the ring of residue
    buffers holds; one op(A) panel against four op(B) panels; k = 1."""
    m, n, k = shape
    ldc = m + 3
    A = oracle.exp_spread(_op_shape(ta, m, k), 71, 4)
    B = oracle.exp_spread(_op_shape(tb, k, n), 72, 4)
    C0 = oracle.uniform((m, n), 73)
    alpha = 0.75
    on, moved, info = _tmm_call(ta, tb, m, n, k, A, B, C0, alpha, beta, ldc, pinned, True, monkeypatch,
                                streams=2 if beta != 0 else 3)
    off, _, info_off = _tmm_call(ta, tb, m, n, k, A, B, C0, alpha, beta, ldc, pinned, False, monkeypatch)
    np.testing.assert_array_equal(on[:m], off[:m])
    np.testing.assert_array_equal(on[m:], np.zeros((ldc - m, n)))  # rows past m untouched
    assert info["slices"] == info_off["slices"] and info["fraction_bits"] == info_off["fraction_bits"]
    assert info["gemm_ms"] == 0.0 and info_off["gemm_ms"] > 0.0
    assert moved == (8 * (m * k + k * n + (m * n if beta != 0 else 0)), 8 * m * n)
    from cosma_gb300 import dgemm_ozaki2_device
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C0, ldc)
    dgemm_ozaki2_device(ta, tb, m, n, k, alpha, dA, A.shape[0], dB, B.shape[0], beta, dC, ldc)
    np.testing.assert_array_equal(on[:m], from_dev(dC, m, n, ldc))


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
@pytest.mark.parametrize("case", ["wide_spread_late", "nan_late"])
def test_tiled_mm_overlapped_falls_back(native_lib, cuda, monkeypatch, case, pinned):
    """The modulus count is chosen from the first panels: when a later panel
    needs more (a wider exponent spread in op(B)'s last columns) or holds NaN,
    the overlapped form gives way before writing C and the regular one-step
    path runs: the same bits as with the overlap switched off."""
    m, n, k = 2100, 2300, 300
    A = oracle.exp_spread((m, k), 81, 0)
    B = oracle.exp_spread((k, n), 82, 0)
    if case == "wide_spread_late":
        B[:, -500:] = oracle.exp_spread((k, 500), 83, 40)
    else:
        A[-3, 7] = np.nan
    C0 = np.zeros((m, n))
    on, _, info = _tmm_call("N", "N", m, n, k, A, B, C0, 1.0, 0.0, m, pinned, True, monkeypatch)
    off, _, info_off = _tmm_call("N", "N", m, n, k, A, B, C0, 1.0, 0.0, m, pinned, False, monkeypatch)
    np.testing.assert_array_equal(np.isnan(on), np.isnan(off))
    np.testing.assert_array_equal(np.nan_to_num(on), np.nan_to_num(off))
    for key in ("slices", "fraction_bits", "exact_product", "fallback_native"):
        assert info[key] == info_off[key]
    assert info["fallback_native"] == (1 if case == "nan_late" else 0)


def _host_matrix_z(A, pinned):
    """Column-major complex host copy of A: pageable numpy or page-locked torch memory."""
    import torch
    if not pinned:
        return np.asfortranarray(A), None
    t = torch.from_numpy(np.ascontiguousarray(A.T).reshape(-1)).pin_memory()
    return t, t


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
@pytest.mark.parametrize("ta,tb,alpha,beta", [("N", "N", 0.75, 0.0), ("T", "C", 1.0, 0.5), ("C", "N", -1.5, -1.0),
                                              ("N", "T", 1.0, 0.0)])
def test_tiled_mm_overlapped_complex(native_lib, cuda, monkeypatch, ta, tb, alpha, beta, pinned):
    """ZGEMM through the Tiled-MM entry on host arrays in the overlapped
    one-step form (real alpha and beta; op(B) columns become the two stacked
    rows of each block's GEMM): the bits of the same call without overlap and
    of the device call; a complex alpha keeps the regular one-step form."""
    from cosma_gb300 import gemm, make_context, zgemm_ozaki2_device
    m, n, k = 2100, 2300, 70
    shp = lambda op, r, c: (r, c) if op == "N" else (c, r)
    A = oracle.uniform(shp(ta, m, k), 101) + 1j * oracle.uniform(shp(ta, m, k), 102)
    B = oracle.uniform(shp(tb, k, n), 103) + 1j * oracle.uniform(shp(tb, k, n), 104)
    ldc = m + 2
    C0 = np.zeros((ldc, n), dtype=np.complex128)
    C0[:m] = oracle.uniform((m, n), 105) + 1j * oracle.uniform((m, n), 106)
    outs = {}
    for mode in ("ON", "OFF"):
        monkeypatch.setenv("COSMA_GPU_OZAKI2_OVERLAP", mode)
        hA, _ = _host_matrix_z(A, pinned)
        hB, _ = _host_matrix_z(B, pinned)
        hC, tC = _host_matrix_z(C0, pinned)
        h = make_context("z", 3)
        h.set_method("ozaki2", 0)
        gemm(h, ta, tb, m, n, k, alpha, hA, A.shape[0], hB, B.shape[0], beta, hC, ldc)
        info = h.ozaki_info()
        moved = h.transfer_bytes()
        h.close()
        out = tC.numpy().reshape(n, ldc).T if tC is not None else hC
        outs[mode] = (np.array(out), info, moved)
    on, info_on, moved = outs["ON"]
    off, info_off, _ = outs["OFF"]
    assert info_on["gemm_ms"] == 0.0 and info_off["gemm_ms"] > 0.0
    assert info_on["slices"] == info_off["slices"]
    assert on.tobytes() == off.tobytes()
    np.testing.assert_array_equal(on[m:], C0[m:])  # rows past m untouched
    assert moved == (16 * (m * k + k * n + (m * n if beta != 0 else 0)), 16 * m * n)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C0, ldc)
    zgemm_ozaki2_device(ta, tb, m, n, k, alpha, dA, A.shape[0], dB, B.shape[0], beta, dC, ldc)
    assert on[:m].tobytes() == np.ascontiguousarray(from_dev(dC, m, n, ldc)).tobytes()
    # a complex alpha: the regular one-step form
    monkeypatch.setenv("COSMA_GPU_OZAKI2_OVERLAP", "ON")
    hA, _ = _host_matrix_z(A, pinned)
    hB, _ = _host_matrix_z(B, pinned)
    hC, _ = _host_matrix_z(C0, pinned)
    h = make_context("z", 3)
    h.set_method("ozaki2", 0)
    gemm(h, ta, tb, m, n, k, 0.5 + 0.25j, hA, A.shape[0], hB, B.shape[0], beta, hC, ldc)
    assert h.ozaki_info()["gemm_ms"] > 0.0
    h.close()


def test_tiled_mm_overlapped_concurrent_handles(native_lib, cuda, monkeypatch):
    """Two host threads, each with its own handle, run the overlapped form at
    the same time on pageable arrays (two copy threads sharing the staging
    buffers and the host copy pool): each gets the bits of the same call made
    alone."""
    import threading
    from cosma_gb300 import gemm, make_context
    monkeypatch.setenv("COSMA_GPU_OZAKI2_OVERLAP", "ON")
    m, n, k = 2100, 2300, 64
    cases = [(oracle.exp_spread((m, k), 111 + 2 * s, 3), oracle.exp_spread((k, n), 112 + 2 * s, 3)) for s in range(2)]

    def run(A, B, out, idx):
        h = make_context("d", 3)
        h.set_method("ozaki2", 0)
        C = np.zeros((m, n), order="F")
        for _ in range(3):
            gemm(h, "N", "N", m, n, k, 1.0, np.asfortranarray(A), m, np.asfortranarray(B), k, 0.0, C, m)
        out[idx] = (C.copy(), h.ozaki_info()["gemm_ms"])
        h.close()

    alone = [None, None]
    for i, (A, B) in enumerate(cases):
        run(A, B, alone, i)
    together = [None, None]
    threads = [threading.Thread(target=run, args=(A, B, together, i)) for i, (A, B) in enumerate(cases)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for i in range(2):
        assert together[i] is not None and together[i][1] == 0.0  # the overlapped form ran
        assert together[i][0].tobytes() == alone[i][0].tobytes()
