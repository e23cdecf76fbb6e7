"""Error paths on the GPU, driven by host-side fault injection
(cosma_gpu_test_fail_next): a refused device allocation, a refused
page-locking of caller memory and a refused pinned staging allocation.  No
GPU fault is involved: the library sees the refusal on the host.  Each case
checks the status and message, the fall-back where there is one (same bits
as without the fault), and that the handle / context stays usable.  The
reference throws std::runtime_error on any such CUDA error
(src/cosma/gpu/utils.hpp:7-13) and pins through cudaHostRegister
(src/cosma/pinned_buffers.cpp:6-35)."""
import numpy as np
import pytest

import oracle
from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu

DEVICE_ALLOC, HOST_REGISTER, PINNED_ALLOC, HOST_COPY = 1, 2, 3, 4
OUT_OF_MEMORY, CUDA_ERROR = 3, 2


@pytest.fixture(autouse=True)
def disarm(native_lib):
    yield
    for site in (DEVICE_ALLOC, HOST_REGISTER, PINNED_ALLOC, HOST_COPY):
        native_lib.cosma_gpu_test_fail_next(site, 0)


def _problem(m=96, n=80, k=112, seed=1):
    return oracle.uniform((m, k), seed), oracle.uniform((k, n), seed + 1)


@pytest.mark.parametrize("site,method", [(DEVICE_ALLOC, "ozaki"), (DEVICE_ALLOC, "ozaki2"),
                                         (PINNED_ALLOC, "ozaki"), (PINNED_ALLOC, "ozaki2")])
def test_workspace_allocation_failure_then_recovery(native_lib, cuda, site, method):
    import torch

    import cosma_gb300 as cg
    from cosma_gb300 import CosmaGpuError
    A, B = _problem()
    m, k = A.shape
    n = B.shape[1]
    dA, dB = to_dev(A), to_dev(B)
    fn = cg.dgemm_ozaki_device if method == "ozaki" else cg.dgemm_ozaki2_device
    want = to_dev(np.zeros((m, n)))
    fn("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, want, m)
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    cg.release_workspaces(stream)  # pooled streams are reused: start from no workspace, so allocations run now
    dC = to_dev(np.zeros((m, n)))
    native_lib.cosma_gpu_test_fail_next(site, 1)
    with pytest.raises(CosmaGpuError) as e:
        fn("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dC, m, stream=stream)
    assert e.value.code == OUT_OF_MEMORY
    msg = str(e.value)
    assert ("injected" in msg) if site == DEVICE_ALLOC else ("pinned staging" in msg)
    assert native_lib.cosma_gpu_test_faults_pending(site) == 0
    # the same call on the same stream now succeeds, bit for bit
    fn("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dC, m, stream=stream)
    stream.synchronize()
    np.testing.assert_array_equal(from_dev(dC, m, n), from_dev(want, m, n))


def test_tile_buffer_allocation_failure_keeps_the_handle_usable(native_lib, cuda):
    import cosma_gb300 as cg
    from cosma_gb300 import CosmaGpuError
    A, B = _problem(300, 200, 250, seed=3)
    m, k = A.shape
    n = B.shape[1]
    h = cg.make_context("d", 2, 128, 128, 128)
    try:
        Cm = np.zeros((m, n), order="F")
        native_lib.cosma_gpu_test_fail_next(DEVICE_ALLOC, 1)
        with pytest.raises(CosmaGpuError) as e:
            cg.gemm(h, "N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cm, m)
        assert e.value.code == OUT_OF_MEMORY and "injected" in str(e.value)
        cg.gemm(h, "N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cm, m)
        ref = np.zeros((m, n), order="F")
        cg.gemm(h, "N", "N", m, n, k, 1.0, A, m, B, k, 0.0, ref, m)
        np.testing.assert_array_equal(Cm, ref)
        assert np.max(np.abs(Cm - A @ B) / (np.abs(A) @ np.abs(B))) < 1e-13
    finally:
        h.close()


def test_failed_page_locking_falls_back_with_the_same_bits(native_lib, cuda, monkeypatch):
    """With the in-place route off the streamer page-locks the caller's arrays;
    refused registrations leave them pageable and the copies take the
    unregistered route: same C."""
    import cosma_gb300 as cg
    monkeypatch.setenv("COSMA_GPU_HOST_DIRECT", "OFF")
    A, B = _problem(260, 190, 150, seed=5)
    m, k = A.shape
    n = B.shape[1]
    h = cg.make_context("d", 3, 128, 128, 128)
    try:
        ref = np.zeros((m, n), order="F")
        cg.gemm(h, "N", "N", m, n, k, 1.0, A, m, B, k, 0.0, ref, m, pin_host_buffers=True)
        got = np.zeros((m, n), order="F")
        native_lib.cosma_gpu_test_fail_next(HOST_REGISTER, 3)  # A, B and C
        cg.gemm(h, "N", "N", m, n, k, 1.0, A, m, B, k, 0.0, got, m, pin_host_buffers=True)
        assert native_lib.cosma_gpu_test_faults_pending(HOST_REGISTER) == 0  # all three were refused
        np.testing.assert_array_equal(got, ref)
    finally:
        h.close()


def test_failed_staging_allocation_falls_back_to_driver_copies(native_lib, cuda, monkeypatch):
    """Pageable host arrays through the pdgemm wrapper with the in-place route
    off: refused staging buffers leave the copies to the driver; same C."""
    import cosma_gb300 as cg
    monkeypatch.setenv("COSMA_GPU_HOST_DIRECT", "OFF")
    m, n, k = 200, 150, 180
    A, B = oracle.uniform((m, k), 7), oracle.uniform((k, n), 8)
    C0 = oracle.uniform((m, n), 9)
    desca = cg.descinit(m, k, 64, 64, 0, 0, 0, m)
    descb = cg.descinit(k, n, 64, 64, 0, 0, 0, k)
    descc = cg.descinit(m, n, 64, 64, 0, 0, 0, m)
    cg.pxgemm_set_method("native")
    native_lib.cosma_gpu_test_fail_next(PINNED_ALLOC, 2)
    got = C0.copy(order="F")
    cg.pxgemm("N", "N", m, n, k, 1.0, A, 1, 1, desca, B, 1, 1, descb, 0.5, got, 1, 1, descc)
    consumed = native_lib.cosma_gpu_test_faults_pending(PINNED_ALLOC) < 2
    native_lib.cosma_gpu_test_fail_next(PINNED_ALLOC, 0)
    ref = C0.copy(order="F")  # staging buffers allocated now (the refusal is retried)
    cg.pxgemm("N", "N", m, n, k, 1.0, A, 1, 1, desca, B, 1, 1, descb, 0.5, ref, 1, 1, descc)
    np.testing.assert_array_equal(got, ref)
    if not consumed:
        pytest.skip("the process-wide staging buffers already existed: no allocation was attempted")


def test_overlapped_form_allocation_failure_falls_back(native_lib, cuda, monkeypatch):
    """A refused device allocation inside the overlapped one-step form
    (page-locked host operands, Chinese-remainder method), before it touches
    C, gives way to the regular one-step path: the same bits as with the
    overlap switched off, and the handle stays usable."""
    import torch

    import cosma_gb300 as cg
    m, n, k = 2100, 2300, 300
    A, B = oracle.uniform((m, k), 91), oracle.uniform((k, n), 92)
    pin = lambda X: torch.from_numpy(np.ascontiguousarray(X.T).reshape(-1)).pin_memory()
    hA, hB = pin(A), pin(B)

    def run(h):
        hC = torch.zeros(m * n, dtype=torch.float64).pin_memory()
        cg.gemm(h, "N", "N", m, n, k, 1.0, hA, m, hB, k, 0.0, hC, m)
        return hC.numpy().copy(), h.ozaki_info()

    monkeypatch.setenv("COSMA_GPU_OZAKI2_OVERLAP", "OFF")
    h = cg.make_context("d", 2)
    h.set_method("ozaki2", 0)
    want, _ = run(h)
    h.close()
    monkeypatch.setenv("COSMA_GPU_OZAKI2_OVERLAP", "ON")
    h = cg.make_context("d", 2)  # fresh streams: the overlapped form allocates its buffers now
    h.set_method("ozaki2", 0)
    native_lib.cosma_gpu_test_fail_next(DEVICE_ALLOC, 1)
    got, info = run(h)
    assert native_lib.cosma_gpu_test_faults_pending(DEVICE_ALLOC) == 0
    assert info["gemm_ms"] > 0.0  # the regular one-step path ran (the overlapped form times no phases)
    np.testing.assert_array_equal(got, want)
    again, info = run(h)  # the next call takes the overlapped form
    assert info["gemm_ms"] == 0.0
    np.testing.assert_array_equal(again, want)
    h.close()


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
def test_overlapped_form_copy_failure_reported(native_lib, cuda, monkeypatch, pinned):
    """A host copy refused inside the overlapped form's copy thread (the first
    operand panel after the lead panels) fails the call with the copy's
    status and message, reported on the calling thread; C is untouched, and
    the next call on the same handle gives the bits of the form without
    overlap."""
    import torch

    import cosma_gb300 as cg
    from cosma_gb300 import CosmaGpuError
    m, n, k = 2100, 2300, 300
    A, B = oracle.uniform((m, k), 93), oracle.uniform((k, n), 94)
    C0 = oracle.uniform((m, n), 95)

    def host(X):
        if not pinned:
            return np.asfortranarray(X.copy())
        return torch.from_numpy(np.ascontiguousarray(X.T).reshape(-1)).pin_memory()

    def values(hC):
        return hC.copy() if not pinned else hC.numpy().reshape(n, m).T.copy()

    hA, hB = host(A), host(B)
    monkeypatch.setenv("COSMA_GPU_OZAKI2_OVERLAP", "OFF")
    h = cg.make_context("d", 2)
    h.set_method("ozaki2", 0)
    hC = host(C0)
    cg.gemm(h, "N", "N", m, n, k, 1.0, hA, m, hB, k, 0.5, hC, m)
    want = values(hC)
    h.close()
    monkeypatch.setenv("COSMA_GPU_OZAKI2_OVERLAP", "ON")
    h = cg.make_context("d", 2)
    h.set_method("ozaki2", 0)
    hC = host(C0)
    native_lib.cosma_gpu_test_fail_next(HOST_COPY, 1)
    with pytest.raises(CosmaGpuError) as err:
        cg.gemm(h, "N", "N", m, n, k, 1.0, hA, m, hB, k, 0.5, hC, m)
    assert native_lib.cosma_gpu_test_faults_pending(HOST_COPY) == 0
    assert err.value.code == CUDA_ERROR
    assert "overlapped host copy" in str(err.value) and "injected" in str(err.value)
    np.testing.assert_array_equal(values(hC), C0)  # nothing was written
    cg.gemm(h, "N", "N", m, n, k, 1.0, hA, m, hB, k, 0.5, hC, m)
    assert h.ozaki_info()["gemm_ms"] == 0.0  # the overlapped form ran
    np.testing.assert_array_equal(values(hC), want)
    h.close()
