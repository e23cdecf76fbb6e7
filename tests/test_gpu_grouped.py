"""Grouped FP64 GEMM (one persistent launch, CUDA graph) vs the oracle, per problem."""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, gemm_bound, to_dev

pytestmark = pytest.mark.gpu


def _batch(rng, count, lo, hi, with_beta=True):
    probs, host = [], []
    for i in range(count):
        m, n, k = (int(x) for x in rng.integers(lo, hi + 1, 3))
        ta, tb = rng.choice(["N", "T"]), rng.choice(["N", "T"])
        A = oracle.uniform((m, k) if ta == "N" else (k, m), 10 * i + 1)
        B = oracle.uniform((k, n) if tb == "N" else (n, k), 10 * i + 2)
        C0 = oracle.uniform((m, n), 10 * i + 3)
        alpha = float(rng.choice([1.0, -0.5, 2.0]))
        beta = float(rng.choice([0.0, 1.0, 0.25])) if with_beta else 0.0
        lda, ldb, ldc = A.shape[0] + int(rng.integers(0, 3)), B.shape[0], m + int(rng.integers(0, 2))
        dA, dB = to_dev(A, lda), to_dev(B, ldb)
        dC = to_dev(C0, ldc, fill=np.nan if beta == 0 else None)
        probs.append((ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc))
        host.append((A, B, C0))
    return probs, host


def _check(probs, host):
    for (ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc), (A, B, C0) in zip(probs, host):
        got = from_dev(dC, m, n, ldc)
        ref = oracle.gemm(ta, tb, alpha, A, B, beta, C0.copy(order="F"))
        assert np.all(np.abs(got - ref) <= gemm_bound(ta, tb, alpha, A, B, beta, C0, k)), (ta, tb, m, n, k)


@pytest.mark.parametrize("autotune", [False, True])
def test_grouped_uneven_batch(native_lib, cuda, autotune):
    import torch
    from cosma_gb300 import GroupedPlan
    rng = np.random.default_rng(3 + autotune)
    probs, host = _batch(rng, 120, 1, 140)
    plan = GroupedPlan(probs, autotune=autotune)
    plan.run()
    torch.cuda.synchronize()
    _check(probs, host)
    info = plan.info()
    assert info["tiles"] > 0 and info["padded_flops"] >= info["useful_flops"]
    plan.close()


def test_grouped_graph_replay_is_deterministic(native_lib, cuda):
    import torch
    from cosma_gb300 import GroupedPlan
    rng = np.random.default_rng(11)
    probs, host = _batch(rng, 40, 16, 200, with_beta=False)
    plan = GroupedPlan(probs, autotune=False)
    plan.run()
    torch.cuda.synchronize()
    first = [from_dev(p[11], p[2], p[3], p[12]) for p in probs]
    for _ in range(3):
        plan.run()
    torch.cuda.synchronize()
    for p, f in zip(probs, first):
        np.testing.assert_array_equal(from_dev(p[11], p[2], p[3], p[12]), f)
    _check(probs, host)
    plan.close()


def test_grouped_zero_sizes_and_k_zero(native_lib, cuda):
    import torch
    from cosma_gb300 import GroupedPlan
    C0 = oracle.uniform((5, 4), 1)
    dC = to_dev(C0)
    d1 = to_dev(np.ones((5, 1)))
    probs = [("N", "N", 5, 4, 0, 1.0, d1, 5, d1, 1, 0.5, dC, 5),   # k == 0: C <- beta*C
             ("N", "N", 0, 4, 3, 1.0, d1, 1, d1, 3, 0.0, d1, 1)]   # m == 0: nothing
    plan = GroupedPlan(probs, autotune=False)
    plan.run()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(from_dev(dC, 5, 4), 0.5 * C0)
    plan.close()


def test_grouped_one_shot_entry_point(native_lib, cuda):
    import ctypes
    from cosma_gb300 import _native
    rng = np.random.default_rng(5)
    probs, host = _batch(rng, 10, 8, 64)
    arr = (_native.GemmProblem * len(probs))()
    for i, (ta, tb, m, n, k, al, A, lda, B, ldb, be, Cm, ldc) in enumerate(probs):
        arr[i] = _native.GemmProblem(ta.encode(), tb.encode(), m, n, k, al, be, A.data_ptr(), lda, B.data_ptr(), ldb,
                                     Cm.data_ptr(), ldc)
    assert native_lib.cosma_gpu_dgemm_grouped_device(1, len(probs), arr, None) == 0
    _check(probs, host)
    del ctypes
