"""Helpers shared by the GPU tests: column-major device buffers and error bounds."""
import numpy as np

_TORCH_DT = {np.dtype(np.float64): "float64", np.dtype(np.float32): "float32",
             np.dtype(np.complex128): "complex128", np.dtype(np.complex64): "complex64"}


def to_dev(A, ld=None, fill=None):
    """Flat CUDA tensor holding column-major A with leading dimension ld."""
    import torch
    A = np.asarray(A)
    rows, cols = A.shape
    ld = ld or max(rows, 1)
    host = np.zeros((max(cols, 1), ld), dtype=A.dtype)  # row j of host = column j of A
    if fill is not None:
        host[:] = fill
    host[:cols, :rows] = A.T
    t = torch.from_numpy(host.reshape(-1).copy()).to("cuda")
    return t


def from_dev(t, rows, cols, ld=None):
    ld = ld or max(rows, 1)
    h = t.cpu().numpy().reshape(max(cols, 1), ld)
    return np.asfortranarray(h[:cols, :rows].T)


def gemm_bound(ta, tb, alpha, A, B, beta, C0, k, c=2.0, u=2.0 ** -53):
    """c*(k+2)*u*(|alpha||op(A)||op(B)| + |beta||C0|) elementwise."""
    opA = A if ta in "Nn" else A.T
    opB = B if tb in "Nn" else B.T
    b = abs(alpha) * (np.abs(opA) @ np.abs(opB))
    if beta != 0:
        b = b + abs(beta) * np.abs(C0)
    return c * (k + 2) * u * b + 1e-300
