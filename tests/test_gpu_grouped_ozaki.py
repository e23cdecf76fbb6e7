"""Grouped Ozaki-split FP64 GEMM (one CUDA graph over the whole batch) vs the oracle.

* every problem bit-exact against the CPU restatement (oracle/ozaki.py) with
  the slice count the plan chose for it, alpha/beta applied as
  fl(fl(alpha*r) + fl(beta*C));
* uneven shapes, ops N/T/C, k = 0, alpha = 0 and empty problems in one batch;
* replays with new data: a problem whose spread outgrew its planned slice
  count, or that holds Inf/NaN, is recomputed on the single-problem path.
"""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, to_dev
from oracle import ozaki as oz

pytestmark = pytest.mark.gpu


def _batch(rng, count, lo, hi, phi=4):
    probs, host = [], []
    for i in range(count):
        m, n, k = (int(x) for x in rng.integers(lo, hi + 1, 3))
        ta, tb = str(rng.choice(["N", "T", "C"])), str(rng.choice(["N", "T"]))
        A = oracle.exp_spread((m, k) if ta == "N" else (k, m), 10 * i + 1, phi)
        B = oracle.exp_spread((k, n) if tb == "N" else (n, k), 10 * i + 2, phi)
        C0 = oracle.uniform((m, n), 10 * i + 3)
        alpha = float(rng.choice([1.0, -0.5, 2.0]))
        beta = float(rng.choice([0.0, 1.0, 0.25]))
        lda, ldb, ldc = max(A.shape[0], 1) + int(rng.integers(0, 3)), max(B.shape[0], 1), max(m, 1) + int(rng.integers(0, 2))
        dA, dB = to_dev(A, lda), to_dev(B, ldb)
        dC = to_dev(C0, ldc, fill=np.nan if beta == 0 else None)
        probs.append((ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc))
        host.append([A, B, C0])
    return probs, host


def _expected(ta, tb, alpha, A, B, beta, C0, S):
    r = oz.ozaki_gemm(ta, tb, A, B, S)
    if alpha != 1.0:
        r = alpha * r
    if beta != 0.0:
        r = r + beta * C0
    return r


def test_grouped_ozaki_bit_exact_per_problem(native_lib, cuda):
    import torch
    from cosma_gb300 import GroupedPlan
    rng = np.random.default_rng(5)
    probs, host = _batch(rng, 36, 1, 300)
    # edge problems: k = 0, alpha = 0, empty
    for (m, n, k, al) in ((20, 30, 0, 1.0), (17, 9, 40, 0.0), (0, 5, 7, 1.0)):
        A, B, C0 = oracle.uniform((m, k), 1), oracle.uniform((k, n), 2), oracle.uniform((m, n), 3)
        probs.append(("N", "N", m, n, k, al, to_dev(A, max(m, 1)), max(m, 1), to_dev(B, max(k, 1)), max(k, 1), 0.5,
                      to_dev(C0, max(m, 1)), max(m, 1)))
        host.append([A, B, C0])
    plan = GroupedPlan(probs, method="ozaki", autotune=False)
    plan.run()
    torch.cuda.synchronize()
    S = plan.slices()
    for i, ((ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc), (A, B, C0)) in enumerate(zip(probs, host)):
        if m == 0 or n == 0:
            continue
        got = from_dev(dC, m, n, ldc)
        if k == 0 or alpha == 0.0:
            np.testing.assert_array_equal(got, beta * C0)
            assert S[i] == 0
            continue
        assert 2 <= S[i] <= 16
        np.testing.assert_array_equal(got, _expected(ta, tb, alpha, A, B, beta, C0, S[i]), err_msg=str(i))
    info = plan.info()
    assert info["tiles"] > 0 and info["padded_flops"] > 0
    plan.close()


def test_grouped_ozaki_replay_with_new_data(native_lib, cuda):
    import torch
    from cosma_gb300 import GroupedPlan
    rng = np.random.default_rng(9)
    count = 12
    probs, host = [], []
    for i in range(count):
        m, n, k = (int(x) for x in rng.integers(40, 260, 3))
        A, B = oracle.exp_spread((m, k), i + 1, 0), oracle.exp_spread((k, n), i + 50, 0)
        dA, dB, dC = to_dev(A, m), to_dev(B, k), to_dev(np.zeros((m, n)), m)
        probs.append(("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dC, m))
        host.append((A, B))
    plan = GroupedPlan(probs, method="ozaki", autotune=True)
    S0 = plan.slices()
    # new data in place: problem 3 gets a wide exponent spread, problem 7 an Inf
    new = []
    for i, (ta, tb, m, n, k, *_rest) in enumerate(probs):
        phi = 32 if i == 3 else 0
        A, B = oracle.exp_spread((m, k), 100 + i, phi), oracle.exp_spread((k, n), 200 + i, phi)
        if i == 7:
            A[1, 2] = np.inf
        probs[i][6].copy_(to_dev(A, m))
        probs[i][8].copy_(to_dev(B, k))
        new.append((A, B))
    plan.run()
    torch.cuda.synchronize()
    for i, ((ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc), (A, B)) in enumerate(zip(probs, new)):
        got = from_dev(dC, m, n, ldc)
        if i == 7:
            assert np.isinf(got[1]).any() or np.isnan(got[1]).any()
            continue
        if i == 3:  # recomputed with its own (larger) slice count: accurate
            rows, cols = np.arange(m) % m, np.arange(m) % n
            hi, lo, ab = oracle.gemm_dd_sampled("N", "N", A, B, rows, cols)
            st = oracle.error_stats(got[rows, cols], hi, lo, ab)
            assert st["max_err_over_absab"] <= 2.0 ** -52, st
            continue
        np.testing.assert_array_equal(got, oz.ozaki_gemm("N", "N", A, B, S0[i]))
    plan.close()


def test_grouped_ozaki_long_k_goes_through_exact_passes(native_lib, cuda):
    """A problem with k above one exact accumulator pass (65536 terms) is run
    on the single-problem path, which cuts K into exact passes."""
    import torch
    from cosma_gb300 import GroupedPlan
    shapes = [(8, 6, 70000), (50, 40, 60)]
    probs, host = [], []
    for i, (m, n, k) in enumerate(shapes):
        A, B = oracle.uniform((m, k), 40 + i), oracle.uniform((k, n), 50 + i)
        probs.append(("N", "N", m, n, k, 1.0, to_dev(A, m), m, to_dev(B, k), k, 0.0, to_dev(np.zeros((m, n)), m), m))
        host.append((A, B))
    plan = GroupedPlan(probs, method="ozaki", autotune=False)
    plan.run()
    torch.cuda.synchronize()
    S = plan.slices()
    assert S[0] == 0 and S[1] > 0
    for (ta, tb, m, n, k, al, dA, lda, dB, ldb, be, dC, ldc), (A, B) in zip(probs, host):
        got = from_dev(dC, m, n, ldc)
        hi, lo, ab = oracle.gemm_dd("N", "N", A, B)
        assert oracle.error_stats(got, hi, lo, ab)["max_err_over_absab"] <= 2.0 ** -51
    plan.close()
