"""Host-side fault injection (cosma_gpu_test_fail_next), CPU part: the hook's
argument checks and bookkeeping.  The reference throws on every CUDA error
(src/cosma/gpu/utils.hpp:7-13); this library returns a status instead, and
these hooks let the tests drive those paths without faulting a GPU.  The GPU
part (the error paths themselves) is tests/test_gpu_fault_injection.py."""
import pytest

DEVICE_ALLOC, HOST_REGISTER, PINNED_ALLOC, HOST_COPY = 1, 2, 3, 4


def test_hook_arms_and_disarms_each_site(native_lib):
    lib = native_lib
    for site in (DEVICE_ALLOC, HOST_REGISTER, PINNED_ALLOC, HOST_COPY):
        assert lib.cosma_gpu_test_fail_next(site, 3) == 0
        assert lib.cosma_gpu_test_faults_pending(site) == 3
        assert lib.cosma_gpu_test_fail_next(site, 0) == 0
        assert lib.cosma_gpu_test_faults_pending(site) == 0


@pytest.mark.parametrize("site,count", [(0, 1), (5, 1), (-1, 1), (1, -1)])
def test_hook_rejects_bad_arguments(native_lib, site, count):
    lib = native_lib
    assert lib.cosma_gpu_test_fail_next(site, count) == 1  # COSMA_GPU_ERROR_INVALID_ARGUMENT
    assert b"site" in lib.cosma_gpu_last_error_string()
    assert lib.cosma_gpu_test_faults_pending(0) == -1
