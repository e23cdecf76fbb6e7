"""ScaLAPACK p?gemm on a 1x1 grid vs the oracle: the reference's 1x1 test
cases (tests/pdgemm.cpp:382-383,415,419-456,796-907) and its edge cases,
checked with its validate_results (utils/pxgemm_utils.hpp:415-449, 1e-6)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _run_case(ma, na, mb_, nb_, mc, nc, bma, bna, bmb, bnb, bmc, bnc, ia, ja, ib, jb, ic, jc, m, n, k, ta, tb,
              alpha, beta, lld_a, lld_b, lld_c, seed=0, dtype=np.float64, prefix="p", suffix="_", method=None):
    from cosma_gb300 import descinit, pxgemm, pxgemm_set_method
    ta_lib, tb_lib = ta, tb          # flags as the caller passes them (any case)
    ta, tb = ta.upper(), tb.upper()  # the reference upper-cases them (cosma_pxgemm.cpp:57-58)
    rng_seed = seed * 7919 + m * 31 + n * 17 + k
    A = oracle.uniform((lld_a, na), rng_seed + 1, 0.0, 1.0, dtype=dtype)  # random_generator: U[0, 1)
    B = oracle.uniform((lld_b, nb_), rng_seed + 2, 0.0, 1.0, dtype=dtype)
    C = oracle.uniform((lld_c, nc), rng_seed + 3, 0.0, 1.0, dtype=dtype)
    if beta == 0:  # pdgemm must not read C when beta == 0 (pxgemm_utils.hpp:604-614)
        C[ic - 1:ic - 1 + m, jc - 1:jc - 1 + n] = np.nan
    desca = descinit(ma, na, bma, bna, 0, 0, 0, lld_a)
    descb = descinit(mb_, nb_, bmb, bnb, 0, 0, 0, lld_b)
    descc = descinit(mc, nc, bmc, bnc, 0, 0, 0, lld_c)
    # oracle: COSTA pack -> gemm NN (alpha 1, beta 0) -> unpack alpha/beta
    Asub = A[ia - 1:ia - 1 + (m if ta == "N" else k), ja - 1:ja - 1 + (k if ta == "N" else m)]
    Bsub = B[ib - 1:ib - 1 + (k if tb == "N" else n), jb - 1:jb - 1 + (n if tb == "N" else k)]
    Ap = oracle.pack(ta, np.asfortranarray(Asub), m, k)
    Bp = oracle.pack(tb, np.asfortranarray(Bsub), k, n)
    Cc = oracle.gemm("N", "N", 1.0, Ap, Bp, 0.0, np.zeros((m, n), dtype=dtype, order="F"))
    ref = C.copy(order="F")
    sub = np.asfortranarray(ref[ic - 1:ic - 1 + m, jc - 1:jc - 1 + n])
    if k == 0 or alpha == 0:
        sub = oracle.scale(beta, sub) if beta != 0 else np.zeros_like(sub)
    else:
        oracle.unpack(alpha, Cc, beta, sub)
    ref[ic - 1:ic - 1 + m, jc - 1:jc - 1 + n] = sub
    if method:
        pxgemm_set_method(method)
    try:
        pxgemm(ta_lib, tb_lib, m, n, k, alpha, A, ia, ja, desca, B, ib, jb, descb, beta, C, ic, jc, descc,
               prefix=prefix, suffix=suffix)
    finally:
        if method:
            pxgemm_set_method("native")
    got = C
    assert oracle.validate_results(got[ic - 1:ic - 1 + m, jc - 1:jc - 1 + n], ref[ic - 1:ic - 1 + m, jc - 1:jc - 1 + n])
    # everything outside the C sub-matrix is untouched (bit for bit)
    mask = np.ones(got.shape, bool)
    mask[ic - 1:ic - 1 + m, jc - 1:jc - 1 + n] = False
    assert got[mask].tobytes() == ref[mask].tobytes()


def _short(m, n, k, bm, bn, bk, ta, tb, alpha, beta, **kw):
    """pxgemm_params short constructor (src/cosma/pxgemm_params.hpp:177-200) on a 1x1 grid."""
    bma, bna = (bk, bm) if ta != "N" else (bm, bk)
    bmb, bnb = (bn, bk) if tb != "N" else (bk, bn)
    ma, na = (k, m) if ta != "N" else (m, k)
    mb_, nb_ = (n, k) if tb != "N" else (k, n)
    _run_case(ma, na, mb_, nb_, m, n, bma, bna, bmb, bnb, bm, bn, 1, 1, 1, 1, 1, 1, m, n, k, ta, tb, alpha, beta,
              max(1, ma), max(1, mb_), max(1, m), **kw)


@pytest.mark.parametrize("case", [
    (10, 10, 10, 2, 2, 2, "N", "N", 1.0, 0.0),   # tests/pdgemm.cpp:382
    (10, 11, 13, 2, 2, 2, "N", "N", 1.0, 0.0),   # tests/pdgemm.cpp:383
    (3, 3, 7, 3, 3, 3, "T", "N", 1.0, 0.0),      # tests/pdgemm.cpp:415
    (10, 11, 12, 3, 2, 3, "T", "N", 1.0, 1.0),   # alpha/beta variants (tests/pdgemm.cpp:392-404)
    (10, 11, 12, 3, 2, 3, "T", "N", 0.0, 0.0),
    (10, 11, 12, 3, 2, 3, "T", "N", 0.0, 1.0),
    (10, 11, 12, 3, 2, 3, "T", "N", 0.5, 0.5),
    (5, 5, 5, 2, 2, 2, "T", "N", 0.5, 0.0),
    (8, 4, 8, 2, 2, 2, "N", "N", 0.5, 0.0),
    (13, 13, 448, 13, 13, 13, "N", "N", 1.0, 0.5),
    (26, 13, 448, 13, 13, 13, "T", "N", 1.0, 0.5),
])
def test_reference_one_by_one_cases(native_lib, cuda, case):
    _short(*case)


def test_adapt_strategy_case(native_lib, cuda):
    # tests/pdgemm.cpp:419-456: A 1280x128 'T', bs 32, m = n = 128, k = 1280, 1x1 'C'
    _run_case(1280, 128, 1280, 128, 128, 128, 32, 32, 32, 32, 32, 32, 1, 1, 1, 1, 1, 1, 128, 128, 1280, "T", "N",
              1.0, 0.0, 1280, 1280, 128)


@pytest.mark.parametrize("ta,tb,nn", [("N", "T", 83), ("T", "N", 77)])
def test_83_cases(native_lib, cuda, ta, tb, nn):
    # tests/pdgemm.cpp:796-907 (problem sizes :813, :850, :887)
    _run_case(83, 83, 83, nn, 83, nn, 32, 32, 32, 32, 32, 32, 1, 1, 1, 1, 1, 1, 83, nn, 83, ta, tb, 1.0, 0.0, 83, 83, 83)


def test_submatrix_offsets_and_padding(native_lib, cuda):
    # sub-matrices ia, ja, ib, jb, ic, jc != 1 with LLD > M on a 1x1 grid
    _run_case(40, 50, 60, 45, 30, 35, 8, 8, 8, 8, 8, 8, 3, 5, 7, 2, 4, 6, 20, 25, 30, "N", "N", 1.5, 0.5, 47, 61, 33)
    _run_case(50, 40, 45, 60, 30, 35, 8, 8, 8, 8, 8, 8, 5, 3, 2, 7, 4, 6, 20, 25, 30, "T", "T", -1.0, 2.0, 50, 45, 30)


@pytest.mark.parametrize("m,n,k", [(0, 5, 5), (5, 0, 5), (5, 5, 0)])
def test_zero_sizes(native_lib, cuda, m, n, k):
    # m or n == 0: no-op; k == 0: C <- beta*C (cosma_pxgemm.cpp:39-46)
    _run_case(max(m, 1), max(k, 1), max(k, 1), max(n, 1), max(m, 1), max(n, 1), 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1,
              m, n, k, "N", "N", 1.0, 0.5, max(m, 1), max(k, 1), max(m, 1))


def test_lowercase_flags_and_all_spellings(native_lib, cuda):
    for prefix, suffix in [("p", ""), ("p", "_"), ("P", ""), ("P", "_"), ("cosma_p", ""), ("cosma_p", "_"),
                           ("COSMA_P", ""), ("COSMA_P", "_")]:
        _run_case(9, 7, 7, 8, 9, 8, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 9, 8, 7, "n", "n", 1.0, 0.0, 9, 7, 9,
                  prefix=prefix, suffix=suffix)


def test_pzgemm_conjugate(native_lib, cuda):
    _run_case(12, 10, 12, 11, 10, 11, 4, 4, 4, 4, 4, 4, 1, 1, 1, 1, 1, 1, 10, 11, 12, "C", "N", 1.0 - 1.0j,
              0.5 + 0.5j, 12, 12, 10, dtype=np.complex128)


def test_psgemm(native_lib, cuda):
    # FP32: validate_results 1e-6 relative to max(1e-3, |v|) at k = 40
    _run_case(30, 40, 40, 20, 30, 20, 8, 8, 8, 8, 8, 8, 1, 1, 1, 1, 1, 1, 30, 20, 40, "N", "N", 1.0, 0.0, 30, 40, 30,
              dtype=np.float32)


@pytest.mark.parametrize("direct", ["ON", "OFF"])
def test_large_host_arrays_through_staged_copies(native_lib, cuda, monkeypatch, direct):
    """Host (pageable) operands larger than one pinned staging buffer
    (128 MiB): with COSMA_GPU_HOST_DIRECT=OFF they travel in several staged
    chunks; with it ON (where the GPU reads the host's page tables) a device
    kernel copies them in place.  Either way the result must be
    bit-identical to the same pdgemm on device arrays, and C outside the
    sub-matrix untouched."""
    import torch
    from cosma_gb300 import descinit, host_copy_route, load, pxgemm
    monkeypatch.setenv("COSMA_GPU_HOST_DIRECT", direct)
    m, n, k = 1500, 1300, 12000            # A^T: 12000 x 1500 x 8 B = 144 MB, B: 125 MB
    lda, ldb, ldc = k + 3, k, m + 5
    A = oracle.uniform((lda, m), 11)
    B = oracle.uniform((ldb, n), 12)
    C = oracle.uniform((ldc, n + 2), 13)
    desca = descinit(k, m, 128, 128, 0, 0, 0, lda)
    descb = descinit(k, n, 128, 128, 0, 0, 0, ldb)
    descc = descinit(m, n + 2, 128, 128, 0, 0, 0, ldc)
    dA = torch.from_numpy(A.reshape(-1, order="F").copy()).cuda()
    dB = torch.from_numpy(B.reshape(-1, order="F").copy()).cuda()
    dC = torch.from_numpy(C.reshape(-1, order="F").copy()).cuda()
    pxgemm("T", "N", m, n, k, 1.5, dA, 1, 1, desca, dB, 1, 1, descb, 0.5, dC, 1, 2, descc, scalar="d")
    Ch = C.copy(order="F")
    pxgemm("T", "N", m, n, k, 1.5, A, 1, 1, desca, B, 1, 1, descb, 0.5, Ch, 1, 2, descc)
    dev = dC.cpu().numpy().reshape(n + 2, ldc).T
    assert Ch.tobytes() == np.asfortranarray(dev).tobytes()
    assert Ch[:, 0].tobytes() == C[:, 0].tobytes()   # column outside jc..jc+n-1
    route = host_copy_route(A)
    assert route == ("staged" if direct == "OFF" else route)
    assert route in ("staged", "direct")
    assert host_copy_route(dA) == "memcpy"


def test_host_direct_copies_odd_layouts(native_lib, cuda, monkeypatch):
    """The in-place device copy handles 4-byte alignment (psgemm with odd
    leading dimensions and offsets) and bit-matches the staged route."""
    from cosma_gb300 import descinit, pxgemm
    m, n, k = 37, 29, 53
    lda, ldb, ldc = k + 1, k + 3, m + 7
    A = oracle.uniform((lda, m + 1), 21, dtype=np.float32)
    B = oracle.uniform((ldb, n + 2), 22, dtype=np.float32)
    C = oracle.uniform((ldc, n + 1), 23, dtype=np.float32)
    desca = descinit(lda, m + 1, 8, 8, 0, 0, 0, lda)
    descb = descinit(ldb, n + 2, 8, 8, 0, 0, 0, ldb)
    descc = descinit(ldc, n + 1, 8, 8, 0, 0, 0, ldc)
    outs = []
    for direct in ("OFF", "ON"):
        monkeypatch.setenv("COSMA_GPU_HOST_DIRECT", direct)
        Ch = C.copy(order="F")
        pxgemm("T", "N", m, n, k, 1.0, A, 2, 2, desca, B, 1, 3, descb, 0.5, Ch, 3, 2, descc)
        outs.append(Ch.tobytes())
    assert outs[0] == outs[1]


@pytest.mark.parametrize("ta,beta", [("T", 0.5), ("N", 0.0), ("C", -1.0)])
def test_overlapped_pdgemm_host_arrays(native_lib, cuda, monkeypatch, ta, beta):
    """pdgemm_ on host (pageable numpy) arrays under the Chinese-remainder
    method, large enough for the overlapped one-step form (2 x 2 panels):
    bit-identical to the staged form (COSMA_GPU_OZAKI2_OVERLAP=OFF) and to the
    same call on device arrays; C outside the sub-matrix untouched, and C not
    read when beta == 0 (NaN there)."""
    import torch
    from cosma_gb300 import descinit, pxgemm, pxgemm_last_transfers, pxgemm_set_method
    m, n, k = 2100, 2300, 300
    am, an = (m, k) if ta == "N" else (k, m)
    lda, ldb, ldc = am + 3, k + 1, m + 5
    A = oracle.exp_spread((lda, an + 1), 91, 6)
    B = oracle.exp_spread((ldb, n + 2), 92, 6)
    C0 = oracle.uniform((ldc, n + 2), 93)
    if beta == 0:
        C0[2:2 + m, 1:1 + n] = np.nan
    desca = descinit(lda, an + 1, 64, 64, 0, 0, 0, lda)
    descb = descinit(ldb, n + 2, 64, 64, 0, 0, 0, ldb)
    descc = descinit(ldc, n + 2, 64, 64, 0, 0, 0, ldc)
    args = lambda a, b, c: (ta, "N", m, n, k, 0.75, a, 2, 2, desca, b, 2, 3, descb, beta, c, 3, 2, descc)
    pxgemm_set_method("ozaki2")
    try:
        outs = {}
        for mode in ("ON", "OFF"):
            monkeypatch.setenv("COSMA_GPU_OZAKI2_OVERLAP", mode)
            Ch = C0.copy(order="F")
            pxgemm(*args(np.asfortranarray(A), np.asfortranarray(B), Ch))
            outs[mode] = (Ch, pxgemm_last_transfers())
        dA = torch.from_numpy(A.reshape(-1, order="F").copy()).cuda()
        dB = torch.from_numpy(B.reshape(-1, order="F").copy()).cuda()
        dC = torch.from_numpy(C0.reshape(-1, order="F").copy()).cuda()
        pxgemm(*args(dA, dB, dC), scalar="d")
        dev_moved = pxgemm_last_transfers()
    finally:
        pxgemm_set_method("native")
    on, (h2d, d2h, overlapped) = outs["ON"]
    off, (h2d_off, d2h_off, overlapped_off) = outs["OFF"]
    assert overlapped and not overlapped_off
    assert on.tobytes() == off.tobytes()
    assert on.tobytes() == np.asfortranarray(dC.cpu().numpy().reshape(n + 2, ldc).T).tobytes()
    mask = np.ones(on.shape, bool)
    mask[2:2 + m, 1:1 + n] = False
    assert on[mask].tobytes() == C0[mask].tobytes()
    assert not np.isnan(on[2:2 + m, 1:1 + n]).any()
    moved = 8 * (m * k + k * n + (m * n if beta != 0 else 0))
    assert (h2d, d2h) == (moved, 8 * m * n) == (h2d_off, d2h_off)
    assert dev_moved == (0, 0, False)
