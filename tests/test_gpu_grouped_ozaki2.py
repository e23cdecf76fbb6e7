"""Grouped Chinese-remainder FP64 GEMM (one CUDA graph over the whole batch) vs the oracle.

* every problem bit-exact against the CPU restatement (oracle/ozaki2.py: the
  exact integer product of the rounded operands, rounded once) with the
  plan's modulus count and the fraction bits it gives at the problem's depth,
  alpha/beta applied as fl(fl(alpha*r) + fl(beta*C));
* uneven shapes, several tiles per problem, K beyond one exact FP32
  accumulation (1024), ops N/T/C, k = 0, alpha = 0 and empty problems in one
  batch, NaN in C with beta = 0;
* replays with new data: a problem whose data outgrew its planned fraction
  bits, or that holds Inf/NaN, is recomputed on the single-problem path;
* K above the grouped limit runs on the single-problem path;
* accuracy against the double-double oracle: correctly rounded where every
  input bit is kept.
"""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, to_dev
from oracle import ozaki2 as o2

pytestmark = pytest.mark.gpu


def _problem(rng, i, m, n, k, phi, ta=None, tb=None):
    ta = ta or str(rng.choice(["N", "T", "C"]))
    tb = tb or str(rng.choice(["N", "T"]))
    A = oracle.exp_spread((m, k) if ta == "N" else (k, m), 10 * i + 1, phi)
    B = oracle.exp_spread((k, n) if tb == "N" else (n, k), 10 * i + 2, phi)
    C0 = oracle.uniform((m, n), 10 * i + 3)
    alpha = float(rng.choice([1.0, -0.5, 2.0]))
    beta = float(rng.choice([0.0, 1.0, 0.25]))
    lda = max(A.shape[0], 1) + int(rng.integers(0, 3))
    ldb = max(B.shape[0], 1)
    ldc = max(m, 1) + int(rng.integers(0, 2))
    dA, dB = to_dev(A, lda), to_dev(B, ldb)
    dC = to_dev(C0, ldc, fill=np.nan if beta == 0 else None)
    return (ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc), [A, B, C0]


def _fraction_bits(nmod, k):
    return min(o2.max_fraction_bits(nmod, k), 116)


def test_grouped_ozaki2_bit_exact_per_problem(native_lib, cuda):
    import torch
    from cosma_gb300 import GroupedPlan
    rng = np.random.default_rng(15)
    probs, host = [], []
    for i in range(20):
        m, n, k = (int(x) for x in rng.integers(1, 90, 3))
        p, h = _problem(rng, i, m, n, k, 4)
        probs.append(p)
        host.append(h)
    # several tiles per problem, K over two exact accumulations, thin shapes
    for i, (m, n, k) in enumerate([(200, 150, 40), (30, 20, 2100), (129, 131, 65), (1, 257, 33), (140, 1, 7)]):
        p, h = _problem(rng, 100 + i, m, n, k, 6)
        probs.append(p)
        host.append(h)
    # edge problems: k = 0, alpha = 0, empty
    for (m, n, k, al) in ((20, 30, 0, 1.0), (17, 9, 40, 0.0), (0, 5, 7, 1.0)):
        A, B, C0 = oracle.uniform((m, k), 1), oracle.uniform((k, n), 2), oracle.uniform((m, n), 3)
        probs.append(("N", "N", m, n, k, al, to_dev(A, max(m, 1)), max(m, 1), to_dev(B, max(k, 1)), max(k, 1), 0.5,
                      to_dev(C0, max(m, 1)), max(m, 1)))
        host.append([A, B, C0])
    plan = GroupedPlan(probs, method="ozaki2", autotune=False)
    plan.run()
    torch.cuda.synchronize()
    N = plan.slices()
    nmods = {x for x in N if x}
    assert len(nmods) == 1  # one modulus count for the batch
    for i, ((ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc), (A, B, C0)) in enumerate(zip(probs, host)):
        if m == 0 or n == 0:
            continue
        got = from_dev(dC, m, n, ldc)
        if k == 0 or alpha == 0.0:
            np.testing.assert_array_equal(got, beta * C0)
            assert N[i] == 0
            continue
        assert 2 <= N[i] <= o2.MAX_MODULI
        want = o2.ozaki2_gemm(ta, tb, A, B, _fraction_bits(N[i], k), alpha, beta, C0)
        np.testing.assert_array_equal(got, want, err_msg=str(i))
    info = plan.info()
    assert info["tiles"] > 0 and info["padded_flops"] >= info["useful_flops"] > 0
    assert info["tile_policy"] == 4
    plan.close()


def test_grouped_ozaki2_autotuned_matches_untuned(native_lib, cuda):
    """Both tile orders (and the tuning replays) give the same bits."""
    import torch
    from cosma_gb300 import GroupedPlan
    rng = np.random.default_rng(21)
    outs = []
    for tune in (False, True):
        probs = []
        for i in range(30):
            m, n, k = (int(x) for x in rng.integers(20, 300, 3))
            A, B = oracle.uniform((m, k), 300 + i), oracle.uniform((k, n), 400 + i)
            probs.append(("N", "T" if i % 2 else "N", m, n, k, 1.0, to_dev(A, m), m,
                          to_dev(B if i % 2 == 0 else B.T.copy(), k if i % 2 == 0 else n), k if i % 2 == 0 else n,
                          0.0, to_dev(np.zeros((m, n)), m), m))
        plan = GroupedPlan(probs, method="ozaki2", autotune=tune)
        plan.run()
        torch.cuda.synchronize()
        outs.append([from_dev(p[11], p[2], p[3], p[12]) for p in probs])
        plan.close()
        rng = np.random.default_rng(21)
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)


def test_grouped_ozaki2_replay_with_new_data(native_lib, cuda):
    import torch
    from cosma_gb300 import GroupedPlan, dgemm_ozaki2_device
    count = 10
    rng = np.random.default_rng(9)
    probs = []
    for i in range(count):
        m, n, k = (int(x) for x in rng.integers(40, 200, 3))
        A, B = oracle.exp_spread((m, k), i + 1, 0), oracle.exp_spread((k, n), i + 50, 0)
        probs.append(("N", "N", m, n, k, 1.0, to_dev(A, m), m, to_dev(B, k), k, 0.0, to_dev(np.zeros((m, n)), m), m))
    plan = GroupedPlan(probs, method="ozaki2", autotune=True)
    N0 = plan.slices()
    # new data in place: problem 3 gets a wide exponent spread, problem 7 an Inf
    new = []
    for i, (ta, tb, m, n, k, *_rest) in enumerate(probs):
        phi = 40 if i == 3 else 0
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
            assert np.isfinite(np.delete(got, 1, axis=0)).all()
            continue
        if i == 3:  # recomputed on the single-problem path, with its own modulus count
            dC2 = to_dev(np.zeros((m, n)), m)
            dgemm_ozaki2_device("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dC2, m)
            np.testing.assert_array_equal(got, from_dev(dC2, m, n, m))
            continue
        np.testing.assert_array_equal(got, o2.ozaki2_gemm("N", "N", A, B, _fraction_bits(N0[i], k)))
    plan.close()


def test_grouped_ozaki2_long_k_goes_to_single_problem_path(native_lib, cuda):
    import torch
    from cosma_gb300 import GroupedPlan
    shapes = [(8, 6, 70000), (50, 40, 60)]
    probs, host = [], []
    for i, (m, n, k) in enumerate(shapes):
        A, B = oracle.uniform((m, k), 40 + i), oracle.uniform((k, n), 50 + i)
        probs.append(("N", "N", m, n, k, 1.0, to_dev(A, m), m, to_dev(B, k), k, 0.0, to_dev(np.zeros((m, n)), m), m))
        host.append((A, B))
    plan = GroupedPlan(probs, method="ozaki2", autotune=False)
    plan.run()
    torch.cuda.synchronize()
    N = plan.slices()
    assert N[0] == 0 and N[1] > 0
    for (ta, tb, m, n, k, al, dA, lda, dB, ldb, be, dC, ldc), (A, B) in zip(probs, host):
        got = from_dev(dC, m, n, ldc)
        hi, lo, ab = oracle.gemm_dd("N", "N", A, B)
        assert oracle.error_stats(got, hi, lo, ab)["max_err_over_absab"] <= 2.0 ** -52
    plan.close()


def test_grouped_ozaki2_correctly_rounded_uniform(native_lib, cuda):
    """U[-1, 1] entries at these depths keep every input bit within the
    planned fraction bits: each entry is the exact product rounded once."""
    import torch
    from cosma_gb300 import GroupedPlan
    rng = np.random.default_rng(33)
    probs, host = [], []
    for i in range(12):
        m, n, k = (int(x) for x in rng.integers(16, 160, 3))
        A, B = oracle.uniform((m, k), 500 + i), oracle.uniform((k, n), 600 + i)
        probs.append(("N", "N", m, n, k, 1.0, to_dev(A, m), m, to_dev(B, k), k, 0.0, to_dev(np.zeros((m, n)), m), m))
        host.append((A, B))
    plan = GroupedPlan(probs, method="ozaki2", autotune=False)
    plan.run()
    torch.cuda.synchronize()
    for (ta, tb, m, n, k, al, dA, lda, dB, ldb, be, dC, ldc), (A, B) in zip(probs, host):
        got = from_dev(dC, m, n, ldc)
        hi, lo, ab = oracle.gemm_dd("N", "N", A, B)
        st = oracle.error_stats(got, hi, lo, ab)
        assert st["max_rel_err"] <= 2.0 ** -52 and st["max_err_over_absab"] <= 2.0 ** -53, st
    plan.close()
