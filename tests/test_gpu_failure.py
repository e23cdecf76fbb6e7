"""Failure detection on the GPU without a fault.

A kernel waits, through the pipelines' own bounded wait, on a barrier that
nothing arrives on.  The wait must give up after its limit, the host must
report COSMA_GPU_ERROR_DEVICE_TIMEOUT with a message, and the context must
stay usable: a GEMM right after it is still correct.
"""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, gemm_bound, to_dev

pytestmark = pytest.mark.gpu

DEVICE_TIMEOUT = 5


def test_bounded_wait_times_out_and_context_survives(native_lib, cuda):
    import time

    import cosma_gb300 as cg
    lib = cg.load()
    t0 = time.perf_counter()
    st = lib.cosma_gpu_selftest_wait_timeout(50_000_000, None)  # 50 ms
    dt = time.perf_counter() - t0
    assert st == DEVICE_TIMEOUT
    assert b"as designed" in lib.cosma_gpu_last_error_string()
    assert 0.04 < dt < 5.0
    # the context is intact: a GEMM still runs and is correct
    m, n, k = 70, 50, 90
    A, B = oracle.uniform((m, k), 1), oracle.uniform((k, n), 2)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(np.zeros((m, n)))
    cg.gemm_device("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dC, m, method="native")
    got = from_dev(dC, m, n)
    ref = oracle.gemm("N", "N", 1.0, A, B, 0.0, np.zeros((m, n), order="F"))
    assert np.all(np.abs(got - ref) <= gemm_bound("N", "N", 1.0, A, B, 0.0, None, k))


def test_selftest_rejects_limits_outside_the_window(native_lib, cuda):
    import cosma_gb300 as cg
    lib = cg.load()
    assert lib.cosma_gpu_selftest_wait_timeout(10, None) == 1          # INVALID_ARGUMENT
    assert lib.cosma_gpu_selftest_wait_timeout(10 ** 10, None) == 1
