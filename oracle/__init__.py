"""Oracle for COSMA's one-rank GEMM path (test infrastructure only).

Python side of the CPU restatement in ``oracle/oracle.c``: ctypes bindings,
the reference's own result checkers restated, and seeded input generators
for the benchmark configurations.  Only ``tests/``, the smoke check and
``bench.py``'s CPU-baseline leg import this package; the library never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(str(path))
        i64, dbl, vp, ch, i32 = C.c_int64, C.c_double, C.c_void_p, C.c_char, C.c_int
        sig = {
            "oracle_local_multiply_cpu_d": [vp, vp, vp, i32, i32, i32, dbl, dbl],
            "oracle_gemm_d": [ch, ch, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64],
            "oracle_gemm_z": [ch, ch, i64, i64, i64, vp, vp, i64, vp, i64, vp, vp, i64],
            "oracle_gemm_s": [ch, ch, i64, i64, i64, C.c_float, vp, i64, vp, i64, C.c_float, vp, i64],
            "oracle_gemm_dd": [ch, ch, i64, i64, i64, vp, i64, vp, i64, vp, vp, vp, i64],
            "oracle_gemm_dd_sampled": [ch, ch, i64, vp, i64, vp, i64, i64, vp, vp, vp, vp, vp],
            "oracle_numroc": [i32, i32, i32, i32, i32],
            "oracle_bc_coords": [i64, i32, i32, i32, vp, vp],
            "oracle_scatter_block_cyclic": [i32, vp, i64, i64, i64, i32, i32, i32, i32, i32, i32, i32, i32, vp, i64],
            "oracle_pack": [ch, i32, i32, i64, i64, vp, i64, vp, i64],
            "oracle_unpack_d": [i64, i64, dbl, vp, i64, dbl, vp, i64],
            "oracle_unpack_z": [i64, i64, vp, vp, i64, vp, vp, i64],
            "oracle_scale_d": [i64, i64, dbl, vp, i64],
        }
        for name, args in sig.items():
            f = getattr(_lib, name)
            f.argtypes = args
            f.restype = C.c_int if name == "oracle_numroc" else None
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _ld(a):
    """Leading dimension (in elements) of a Fortran-ordered 2-D array."""
    assert a.flags.f_contiguous or a.shape[1] <= 1
    return max(1, a.shape[0])


def _b(c):
    return c.encode() if isinstance(c, str) else c


def op_shape(op, a):
    return a.shape if op in "Nn" else (a.shape[1], a.shape[0])


def gemm(ta, tb, alpha, A, B, beta, Cm):
    """BLAS-semantics GEMM (in place on Fortran array Cm)."""
    m, k = op_shape(ta, A)
    n = op_shape(tb, B)[1]
    L = lib()
    if A.dtype == np.float64:
        L.oracle_gemm_d(_b(ta), _b(tb), m, n, k, alpha, _p(A), _ld(A), _p(B), _ld(B), beta, _p(Cm), _ld(Cm))
    elif A.dtype == np.complex128:
        al = np.array([complex(alpha).real, complex(alpha).imag])
        be = np.array([complex(beta).real, complex(beta).imag])
        L.oracle_gemm_z(_b(ta), _b(tb), m, n, k, _p(al), _p(A), _ld(A), _p(B), _ld(B), _p(be), _p(Cm), _ld(Cm))
    elif A.dtype == np.float32:
        L.oracle_gemm_s(_b(ta), _b(tb), m, n, k, alpha, _p(A), _ld(A), _p(B), _ld(B), beta, _p(Cm), _ld(Cm))
    else:
        raise TypeError(A.dtype)
    return Cm


def local_multiply_cpu(A, B, Cm, alpha, beta):
    """The reference's naive checker loop (local_multiply.cpp:278-297), in place."""
    m, k = A.shape
    n = B.shape[1]
    lib().oracle_local_multiply_cpu_d(_p(A), _p(B), _p(Cm), m, n, k, alpha, beta)
    return Cm


def gemm_dd(ta, tb, A, B):
    """Double-double op(A)*op(B): returns (hi, lo, |A||B|)."""
    m, k = op_shape(ta, A)
    n = op_shape(tb, B)[1]
    hi = np.zeros((m, n), order="F")
    lo = np.zeros((m, n), order="F")
    ab = np.zeros((m, n), order="F")
    lib().oracle_gemm_dd(_b(ta), _b(tb), m, n, k, _p(A), _ld(A), _p(B), _ld(B), _p(hi), _p(lo), _p(ab), max(1, m))
    return hi, lo, ab


def gemm_dd_sampled(ta, tb, A, B, rows, cols):
    """Double-double entries (rows[s], cols[s]) of op(A)*op(B)."""
    k = op_shape(ta, A)[1]
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    ns = rows.size
    hi, lo, ab = np.zeros(ns), np.zeros(ns), np.zeros(ns)
    lib().oracle_gemm_dd_sampled(_b(ta), _b(tb), k, _p(A), _ld(A), _p(B), _ld(B), ns, _p(rows), _p(cols), _p(hi),
                                 _p(lo), _p(ab))
    return hi, lo, ab


def numroc(n, nb, iproc, isrc, nprocs):
    return lib().oracle_numroc(n, nb, iproc, isrc, nprocs)


def bc_coords(g, nb, nprocs, src):
    o, l = C.c_int(), C.c_int64()
    lib().oracle_bc_coords(g, nb, nprocs, src, C.byref(o), C.byref(l))
    return o.value, l.value


def scatter_block_cyclic(G, mb, nb, prow, pcol, rsrc, csrc, myrow, mycol, lld=None):
    M, N = G.shape
    lr = numroc(M, mb, myrow, rsrc, prow)
    lc = numroc(N, nb, mycol, csrc, pcol)
    lld = lld or max(1, lr)
    L = np.zeros((lld, max(lc, 1)), dtype=G.dtype, order="F")
    lib().oracle_scatter_block_cyclic(G.itemsize, _p(G), M, N, _ld(G), mb, nb, prow, pcol, rsrc, csrc, myrow, mycol,
                                      _p(L), lld)
    return L


def pack(op, src, rows, cols, dst=None):
    """dst(rows x cols) = op(src), bit-exact."""
    cplx = np.iscomplexobj(src)
    if dst is None:
        dst = np.zeros((rows, cols), dtype=src.dtype, order="F")
    lib().oracle_pack(_b(op), int(cplx), src.itemsize, rows, cols, _p(src), _ld(src), _p(dst), _ld(dst))
    return dst


def unpack(alpha, src, beta, dst):
    """dst = alpha*src + beta*dst (no read of dst when beta == 0), in place."""
    rows, cols = dst.shape
    if src.dtype != dst.dtype:
        raise TypeError("unpack: src and dst types differ")
    if dst.dtype == np.float64:
        lib().oracle_unpack_d(rows, cols, alpha, _p(src), _ld(src), beta, _p(dst), _ld(dst))
    elif dst.dtype == np.complex128:
        al = np.array([complex(alpha).real, complex(alpha).imag])
        be = np.array([complex(beta).real, complex(beta).imag])
        lib().oracle_unpack_z(rows, cols, _p(al), _p(src), _ld(src), _p(be), _p(dst), _ld(dst))
    elif dst.dtype in (np.float32, np.complex64):
        # single precision: numpy rounds every product and sum to the type
        t = dst.dtype.type
        ft = np.float32
        if dst.dtype == np.float32:
            v = t(alpha) * src[:rows, :cols]
            if beta != 0:
                v = v + t(beta) * dst[:rows, :cols]
        else:
            ar, ai = ft(complex(alpha).real), ft(complex(alpha).imag)
            sr, si = src.real.astype(ft), src.imag.astype(ft)
            vr, vi = ar * sr - ai * si, ar * si + ai * sr
            if complex(beta) != 0:
                br, bi = ft(complex(beta).real), ft(complex(beta).imag)
                dr, di = dst.real.astype(ft), dst.imag.astype(ft)
                vr, vi = vr + (br * dr - bi * di), vi + (br * di + bi * dr)
            v = vr + 1j * vi
        dst[:rows, :cols] = v
    else:
        raise TypeError(f"unpack: unsupported dtype {dst.dtype}")
    return dst


def scale(beta, Cm):
    if Cm.dtype != np.float64:
        raise TypeError("scale: float64 only")
    lib().oracle_scale_d(Cm.shape[0], Cm.shape[1], beta, _p(Cm), _ld(Cm))
    return Cm


# ------------------------------------------------ the reference's checkers

def validate_results(v1, v2, epsilon=1e-6):
    """Restates validate_results (utils/pxgemm_utils.hpp:415-449): fails on any
    NaN, else |v1-v2| / max(1e-3, |v1|, |v2|) <= epsilon elementwise."""
    v1 = np.asarray(v1).ravel()
    v2 = np.asarray(v2).ravel()
    if v1.size != v2.size:
        return False
    if v1.size == 0:
        return True
    if np.isnan(v1).any() or np.isnan(v2).any():
        return False
    scale_ = np.maximum(np.maximum(np.abs(v1), np.abs(v2)), 1e-3)
    return bool(np.all(np.abs(v1 - v2) / scale_ <= epsilon))


def cosma_check(glob_c, check_c, epsilon=1e-8, is_fp32=False):
    """Restates test_cosma's comparison (utils/cosma_utils.hpp:365-377):
    relative error where max(|c|,|c_ref|) > 1e-10, absolute otherwise;
    tolerance 1e-5 for 4-byte types, epsilon otherwise."""
    a = np.asarray(glob_c).ravel()
    b = np.asarray(check_c).ravel()
    if a.size != b.size:
        return False
    err = np.abs(a - b)
    sc = np.maximum(np.abs(a), np.abs(b))
    rel = np.where(sc > 1e-10, err / np.where(sc > 1e-10, sc, 1.0), err)
    tol = 1e-5 if is_fp32 else epsilon
    return bool(np.all(rel < tol))


# --------------------------------------------------------- seeded inputs

def uniform(shape, seed, lo=-1.0, hi=1.0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    if np.dtype(dtype).kind == "c":
        re = rng.uniform(lo, hi, size=shape)
        im = rng.uniform(lo, hi, size=shape)
        return np.asfortranarray((re + 1j * im).astype(dtype))
    return np.asfortranarray(rng.uniform(lo, hi, size=shape).astype(dtype))


def normal(shape, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal(size=shape).astype(dtype))


def exp_spread(shape, seed, phi):
    """u * 2**e with u ~ U[-1, 1] and integer e ~ U{-phi..phi} (precision config)."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1.0, 1.0, size=shape)
    e = rng.integers(-phi, phi + 1, size=shape) if phi > 0 else np.zeros(shape, dtype=np.int64)
    return np.asfortranarray(np.ldexp(u, e))


# ---------------------------------------------------------- error metrics

def error_stats(c, hi, lo, absab):
    """Max/mean elementwise relative error of c against the double-double
    value hi+lo, and the max error normalised by |A||B| (componentwise)."""
    c = np.asarray(c, dtype=np.float64).ravel()
    hi = np.asarray(hi).ravel()
    lo = np.asarray(lo).ravel()
    absab = np.asarray(absab).ravel()
    d = (c - hi) - lo
    den = np.abs(hi)
    nz = den > 0
    rel = np.abs(d[nz]) / den[nz]
    nab = np.abs(d) / np.where(absab > 0, absab, 1.0)
    return {
        "max_rel_err": float(rel.max()) if rel.size else 0.0,
        "mean_rel_err": float(rel.mean()) if rel.size else 0.0,
        "max_err_over_absab": float(nab.max()) if nab.size else 0.0,
    }


def openblas_threads():
    return int(os.environ.get("OPENBLAS_NUM_THREADS", os.cpu_count() or 1))
