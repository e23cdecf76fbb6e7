"""Python mirror of the reference interfaces for the one-rank GEMM path.

Names, argument order and meaning follow the reference:
  * ``make_context`` / ``gemm``      -> Tiled-MM ``gpu::make_context`` / ``gpu::gemm``
    (call sites src/cosma/context.cpp:24-25, src/cosma/local_multiply.cpp:245-260)
  * ``local_multiply``               -> ``cosma::local_multiply`` (src/cosma/local_multiply.hpp:6-49)
  * ``pxgemm``                       -> ``cosma::pxgemm`` / ``p?gemm_`` (src/cosma/cosma_pxgemm.cpp:16-34)
Matrices are column-major buffers: numpy arrays (host) or torch tensors
(host or CUDA).  A 2-D torch tensor is taken in column-major form when
``stride(0) == 1``; any buffer may also be passed flat with explicit sizes
and leading dimensions, exactly as through the C ABI.  Every call goes
through the CUDA library; failures raise ``CosmaGpuError``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

_DT = {"s": np.float32, "d": np.float64, "c": np.complex64, "z": np.complex128}


def _scalar_of(dtype) -> str:
    dt = str(dtype).replace("torch.", "")
    table = {"float32": "s", "float64": "d", "complex64": "c", "complex128": "z"}
    if dt not in table:
        raise TypeError(f"unsupported dtype {dtype}")
    return table[dt]


def ptr(buf) -> int:
    """Raw address of a numpy array or torch tensor."""
    if buf is None:
        return 0
    if isinstance(buf, int):
        return buf
    if isinstance(buf, np.ndarray):
        return buf.ctypes.data
    return buf.data_ptr()  # torch tensor


def _cplx_pair(v, real_t):
    v = complex(v)
    arr = (real_t * 2)(v.real, v.imag)
    return arr


def _stream_ptr(stream) -> int:
    if stream is None:
        return 0
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


class MMHandle:
    """A Tiled-MM ``mm_handle<T>`` (owns streams and HBM tile buffers)."""

    def __init__(self, scalar="d", streams=0, tile_m=0, tile_n=0, tile_k=0):
        self.lib = N.load()
        self.scalar = scalar
        self._h = self.lib.cosma_gpu_tmm_make_context(scalar.encode(), streams, tile_m, tile_n, tile_k)
        if not self._h:
            N.check(self.lib.cosma_gpu_last_error() or N.CosmaGpuError(6, "make_context failed").code)

    @property
    def handle(self):
        return self._h

    def set_method(self, method="native", slices=0):
        m = N.METHODS[method] if isinstance(method, str) else int(method)
        N.check(self.lib.cosma_gpu_tmm_set_method(self._h, m, slices))

    def ozaki_info(self):
        info = N.OzakiInfo()
        N.check(self.lib.cosma_gpu_tmm_last_ozaki_info(self._h, C.byref(info)))
        return info.as_dict()

    def set_memory_limit(self, nbytes):
        """Square tiles whose device footprint fits in nbytes (see tiles_for_memory)."""
        N.check(self.lib.cosma_gpu_tmm_set_memory_limit(self._h, int(nbytes)))

    def tiles(self):
        t = [C.c_int(), C.c_int(), C.c_int()]
        N.check(self.lib.cosma_gpu_tmm_tiles(self._h, *(C.byref(x) for x in t)))
        return tuple(x.value for x in t)

    def last_overlapped(self) -> bool:
        """Whether the last gemm call ran in an overlapped one-step form."""
        return bool(self.lib.cosma_gpu_tmm_last_overlapped(self._h))

    def transfer_bytes(self):
        """(host->device, device->host) bytes moved by the last gemm call."""
        h2d, d2h = C.c_int64(), C.c_int64()
        N.check(self.lib.cosma_gpu_tmm_last_transfer_bytes(self._h, C.byref(h2d), C.byref(d2h)))
        return h2d.value, d2h.value

    def device_buffer_c(self) -> int:
        return self.lib.cosma_gpu_tmm_device_buffer_c(self._h) or 0

    def close(self):
        if self._h:
            self.lib.cosma_gpu_tmm_destroy_context(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tiles_for_memory(scalar, method, nbytes):
    """Largest square tiles (multiple of 256) whose handle footprint fits in nbytes."""
    lib = N.load()
    t = [C.c_int(), C.c_int(), C.c_int()]
    meth = N.METHODS[method] if isinstance(method, str) else int(method)
    N.check(lib.cosma_gpu_tmm_tiles_for_memory(scalar.encode(), meth, int(nbytes), *(C.byref(x) for x in t)))
    return tuple(x.value for x in t)


def make_context(scalar="d", streams=0, tile_m=0, tile_n=0, tile_k=0) -> MMHandle:
    return MMHandle(scalar, streams, tile_m, tile_n, tile_k)


def gemm(handle: MMHandle, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc,
         pin_host_buffers=True, copy_c_back=True):
    """Tiled-MM gpu::gemm: C = alpha*op(A)*op(B) + beta*C on host or device buffers."""
    lib = handle.lib
    s = handle.scalar
    ta, tb = transa.encode(), transb.encode()
    args = (m, n, k)
    if s in "sd":
        f = lib.cosma_gpu_tmm_gemm_d if s == "d" else lib.cosma_gpu_tmm_gemm_s
        st = f(handle.handle, ta, tb, *args, alpha, ptr(A), lda, ptr(B), ldb, beta, ptr(Cm), ldc,
               int(pin_host_buffers), int(copy_c_back))
    else:
        rt = C.c_double if s == "z" else C.c_float
        f = lib.cosma_gpu_tmm_gemm_z if s == "z" else lib.cosma_gpu_tmm_gemm_c
        st = f(handle.handle, ta, tb, *args, _cplx_pair(alpha, rt), ptr(A), lda, ptr(B), ldb,
               _cplx_pair(beta, rt), ptr(Cm), ldc, int(pin_host_buffers), int(copy_c_back))
    N.check(st)


def local_multiply(a, b, c, m, n, k, alpha, beta, copy_c_back=True, ctx: MMHandle | None = None):
    """cosma::local_multiply on one rank: C = alpha*A*B + beta*C, ld = m, k, m."""
    lib = N.load()
    s = ctx.scalar if ctx is not None else _scalar_of(a.dtype)
    h = ctx.handle if ctx is not None else None
    if s in "sd":
        f = lib.cosma_gpu_local_multiply_d if s == "d" else lib.cosma_gpu_local_multiply_s
        st = f(h, ptr(a), ptr(b), ptr(c), m, n, k, alpha, beta, int(copy_c_back))
    else:
        rt = C.c_double if s == "z" else C.c_float
        f = lib.cosma_gpu_local_multiply_z if s == "z" else lib.cosma_gpu_local_multiply_c
        st = f(h, ptr(a), ptr(b), ptr(c), m, n, k, _cplx_pair(alpha, rt), _cplx_pair(beta, rt), int(copy_c_back))
    N.check(st)


def _ip(v):
    return C.byref(C.c_int(int(v)))


def descinit(m, n, mb, nb, rsrc, csrc, ictxt, lld):
    """The 9-integer ScaLAPACK array descriptor (dtype 1 = dense block-cyclic)."""
    return np.array([1, ictxt, m, n, mb, nb, rsrc, csrc, lld], dtype=np.int32)


def pxgemm(transa, transb, m, n, k, alpha, a, ia, ja, desca, b, ib, jb, descb, beta, c, ic, jc, descc,
           scalar=None, prefix="p", suffix="_"):
    """ScaLAPACK p?gemm on a 1x1 grid through the library's interposed symbol."""
    lib = N.load()
    s = scalar or _scalar_of(a.dtype)
    name = f"{prefix}{s}gemm{suffix}" if prefix.islower() or prefix == "cosma_p" else f"{prefix}{s.upper()}GEMM{suffix}"
    f = getattr(lib, name)
    rt = C.c_double if s in "dz" else C.c_float
    if s in "sd":
        al, be = (rt * 1)(alpha), (rt * 1)(beta)
    else:
        al, be = _cplx_pair(alpha, rt), _cplx_pair(beta, rt)
    da = np.ascontiguousarray(desca, dtype=np.int32)
    db = np.ascontiguousarray(descb, dtype=np.int32)
    dc = np.ascontiguousarray(descc, dtype=np.int32)
    f(C.c_char_p(transa.encode()), C.c_char_p(transb.encode()), _ip(m), _ip(n), _ip(k), al, C.c_void_p(ptr(a)),
      _ip(ia), _ip(ja), da.ctypes.data_as(C.c_void_p), C.c_void_p(ptr(b)), _ip(ib), _ip(jb),
      db.ctypes.data_as(C.c_void_p), be, C.c_void_p(ptr(c)), _ip(ic), _ip(jc), dc.ctypes.data_as(C.c_void_p))
    N.check(lib.cosma_gpu_last_error())


def pxgemm_set_method(method="native"):
    lib = N.load()
    N.check(lib.cosma_gpu_pxgemm_set_method(N.METHODS[method] if isinstance(method, str) else int(method)))


def pxgemm_last_transfers():
    """(h2d_bytes, d2h_bytes, overlapped) of the last p?gemm call: the bytes
    its host arrays moved, and whether the overlapped one-step form ran it."""
    lib = N.load()
    h2d, d2h, ov = C.c_int64(0), C.c_int64(0), C.c_int(0)
    N.check(lib.cosma_gpu_pxgemm_last_transfers(C.byref(h2d), C.byref(d2h), C.byref(ov)))
    return h2d.value, d2h.value, bool(ov.value)


HOST_COPY_ROUTES = {0: "memcpy", 1: "staged", 2: "direct"}


def host_copy_route(array):
    """Route the host-pointer entry points take for `array` (a numpy array,
    a torch tensor or an address): "memcpy" (device / pinned memory),
    "staged" (pageable, through pinned buffers) or "direct" (pageable, read
    and written in place by a device copy kernel)."""
    if hasattr(array, "data_ptr"):
        ptr = array.data_ptr()
    elif hasattr(array, "ctypes"):
        ptr = array.ctypes.data
    else:
        ptr = int(array)
    return HOST_COPY_ROUTES[N.load().cosma_gpu_host_copy_route(ptr)]


# ------------------------------------------------------ device-pointer API

def gemm_device(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc, method="native", stream=None,
                scalar=None):
    """Stream-ordered GEMM on CUDA buffers (no synchronisation)."""
    lib = N.load()
    s = scalar or _scalar_of(A.dtype)
    meth = N.METHODS[method] if isinstance(method, str) else int(method)
    ta, tb, sp = transa.encode(), transb.encode(), _stream_ptr(stream)
    if s == "d":
        st = lib.cosma_gpu_dgemm_device(meth, ta, tb, m, n, k, alpha, ptr(A), lda, ptr(B), ldb, beta, ptr(Cm), ldc, sp)
    elif s == "s":
        st = lib.cosma_gpu_sgemm_device(meth, ta, tb, m, n, k, alpha, ptr(A), lda, ptr(B), ldb, beta, ptr(Cm), ldc, sp)
    elif s == "z":
        st = lib.cosma_gpu_zgemm_device(meth, ta, tb, m, n, k, _cplx_pair(alpha, C.c_double), ptr(A), lda, ptr(B),
                                        ldb, _cplx_pair(beta, C.c_double), ptr(Cm), ldc, sp)
    else:
        st = lib.cosma_gpu_cgemm_device(meth, ta, tb, m, n, k, _cplx_pair(alpha, C.c_float), ptr(A), lda, ptr(B), ldb,
                                        _cplx_pair(beta, C.c_float), ptr(Cm), ldc, sp)
    N.check(st)


def dgemm_ozaki_device(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc, slices=0, stream=None):
    """FP64-accurate Ozaki-split DGEMM on CUDA buffers; returns the slice statistics."""
    lib = N.load()
    info = N.OzakiInfo()
    N.check(lib.cosma_gpu_dgemm_ozaki_device(transa.encode(), transb.encode(), m, n, k, alpha, ptr(A), lda, ptr(B),
                                             ldb, beta, ptr(Cm), ldc, slices, _stream_ptr(stream), C.byref(info)))
    return info.as_dict()


def zgemm_ozaki_device(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc, slices=0, stream=None):
    """FP64-accurate Ozaki-split ZGEMM (complex128 CUDA buffers, op N/T/C);
    returns the slice statistics."""
    lib = N.load()
    info = N.OzakiInfo()
    al, be = _cplx_pair(alpha, C.c_double), _cplx_pair(beta, C.c_double)
    N.check(lib.cosma_gpu_zgemm_ozaki_device(transa.encode(), transb.encode(), m, n, k, al, ptr(A), lda, ptr(B),
                                             ldb, be, ptr(Cm), ldc, slices, _stream_ptr(stream), C.byref(info)))
    return info.as_dict()


def dgemm_ozaki2_device(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc, moduli=0, stream=None):
    """FP64-accurate DGEMM by the Chinese-remainder (Ozaki scheme II) form on
    CUDA buffers; returns the statistics (slices = modulus count,
    fraction_bits = P)."""
    lib = N.load()
    info = N.OzakiInfo()
    N.check(lib.cosma_gpu_dgemm_ozaki2_device(transa.encode(), transb.encode(), m, n, k, alpha, ptr(A), lda, ptr(B),
                                              ldb, beta, ptr(Cm), ldc, moduli, _stream_ptr(stream), C.byref(info)))
    return info.as_dict()


def zgemm_ozaki2_device(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc, moduli=0, stream=None):
    """The Chinese-remainder form for complex128 CUDA buffers (op N/T/C)."""
    lib = N.load()
    info = N.OzakiInfo()
    al, be = _cplx_pair(alpha, C.c_double), _cplx_pair(beta, C.c_double)
    N.check(lib.cosma_gpu_zgemm_ozaki2_device(transa.encode(), transb.encode(), m, n, k, al, ptr(A), lda, ptr(B),
                                              ldb, be, ptr(Cm), ldc, moduli, _stream_ptr(stream), C.byref(info)))
    return info.as_dict()


def dgemm_ozaki2_residual(transa, transb, m, n, k, A, lda, B, ldb, Ct, ldt, E, Rx, ldo, moduli=28, stream=None):
    """E = op(A) op(B) - Ct (exact before one rounding) and Rx = op(A) op(B)
    rounded once, on CUDA buffers; returns the statistics."""
    lib = N.load()
    info = N.OzakiInfo()
    N.check(lib.cosma_gpu_dgemm_ozaki2_residual(transa.encode(), transb.encode(), m, n, k, ptr(A), lda, ptr(B), ldb,
                                                ptr(Ct), ldt, moduli, ptr(E), ptr(Rx), ldo, _stream_ptr(stream),
                                                C.byref(info)))
    return info.as_dict()


def release_workspaces(stream=None):
    """Frees the precision forms' workspaces kept for `stream` (call before
    the stream is destroyed; its work must be complete)."""
    N.check(N.load().cosma_gpu_release_workspaces(_stream_ptr(stream)))


def ozaki2_choose(k, spread_bits=0.0, moduli=0, exact_bits=0):
    """(modulus count, fraction bits P) the Chinese-remainder form uses (host only)."""
    lib = N.load()
    nm, P = C.c_int(), C.c_int()
    N.check(lib.cosma_gpu_ozaki2_choose(int(k), float(spread_bits), int(exact_bits), int(moduli), C.byref(nm),
                                        C.byref(P)))
    return nm.value, P.value


class BlockLayout:
    """A matrix described block by block, as the reference's C `layout`:
    block (r, c) covers rows rowsplit[r]:rowsplit[r+1] and columns
    colsplit[c]:colsplit[c+1]; `blocks[(r, c)] = (buffer, ld)` with a
    column-major host array or CUDA tensor.  All blocks belong to rank 0."""

    def __init__(self, rowsplit, colsplit, blocks, owners=None):
        self.rowsplit = (C.c_int * len(rowsplit))(*rowsplit)
        self.colsplit = (C.c_int * len(colsplit))(*colsplit)
        nb = (len(rowsplit) - 1) * (len(colsplit) - 1)
        self.owners = (C.c_int * max(1, nb))(*(owners or [0] * nb))
        items = list(blocks.items())
        self.blocks = (N.Block * max(1, len(items)))()
        for i, ((r, c), (buf, ld)) in enumerate(items):
            self.blocks[i] = N.Block(ptr(buf), int(ld), int(r), int(c))
        self._keep = blocks
        self.c = N.Layout(len(rowsplit) - 1, len(colsplit) - 1, self.rowsplit, self.colsplit, self.owners,
                          len(items), self.blocks)


def multiply_using_layout(transa, transb, alpha, a: BlockLayout, b: BlockLayout, beta, c: BlockLayout, scalar="d"):
    """cosma::multiply_using_layout on one rank (the reference's C interface):
    C = alpha * op(A) * op(B) + beta * C over block layouts."""
    lib = N.load()
    rt = C.c_double if scalar in "dz" else C.c_float
    al = (rt * 1)(alpha) if scalar in "sd" else _cplx_pair(alpha, rt)
    be = (rt * 1)(beta) if scalar in "sd" else _cplx_pair(beta, rt)
    f = getattr(lib, f"cosma_gpu_{scalar}multiply_using_layout")
    N.check(f(transa.encode(), transb.encode(), C.cast(al, C.c_void_p), C.byref(a.c), C.byref(b.c),
              C.cast(be, C.c_void_p), C.byref(c.c)))


class GroupedPlan:
    """A grouped FP64 GEMM over many device problems, one persistent launch
    replayed from a CUDA graph (method "native", "ozaki" or "ozaki2").  `problems` is a list of tuples
    (transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc) with device
    buffers (torch tensors or raw addresses)."""

    def __init__(self, problems, method="native", autotune=True, stream=None):
        self.lib = N.load()
        arr = (N.GemmProblem * max(1, len(problems)))()
        for i, (ta, tb, m, n, k, al, A, lda, B, ldb, be, Cm, ldc) in enumerate(problems):
            arr[i] = N.GemmProblem(ta.encode(), tb.encode(), m, n, k, al, be, ptr(A), lda, ptr(B), ldb, ptr(Cm), ldc)
        self._keep = problems  # the device buffers must outlive the plan
        meth = N.METHODS[method] if isinstance(method, str) else int(method)
        self._p = self.lib.cosma_gpu_grouped_plan_create(meth, len(problems), arr, int(autotune), _stream_ptr(stream))
        if not self._p:
            N.check(self.lib.cosma_gpu_last_error() or 6)

    def run(self, stream=None):
        N.check(self.lib.cosma_gpu_grouped_plan_run(self._p, _stream_ptr(stream)))

    def info(self):
        inf = N.GroupedInfo()
        N.check(self.lib.cosma_gpu_grouped_plan_info(self._p, C.byref(inf)))
        return inf.as_dict()

    def slices(self):
        """Planned slice count per problem of an "ozaki" plan, the batch's
        modulus count for each problem of an "ozaki2" plan (0 where a problem
        is not on the grouped path, and for native plans)."""
        out = (C.c_int * max(1, len(self._keep)))()
        N.check(self.lib.cosma_gpu_grouped_plan_slices(self._p, out))
        return list(out)[:len(self._keep)]

    def close(self):
        if self._p:
            self.lib.cosma_gpu_grouped_plan_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pack(op, rows, cols, src, ld_src, dst, ld_dst, is_complex=False, elem_bytes=8, stream=None):
    """COSTA 1x1 pack: dst(rows x cols) = op(src) on CUDA buffers."""
    lib = N.load()
    N.check(lib.costa_gpu_pack(op.encode(), int(is_complex), elem_bytes, rows, cols, ptr(src), ld_src, ptr(dst),
                               ld_dst, _stream_ptr(stream)))


def unpack(rows, cols, alpha, src, ld_src, beta, dst, ld_dst, scalar="d", stream=None):
    """COSTA 1x1 back-transform: dst = alpha*src + beta*dst on CUDA buffers."""
    lib = N.load()
    sp = _stream_ptr(stream)
    if scalar == "d":
        st = lib.costa_gpu_unpack_d(rows, cols, alpha, ptr(src), ld_src, beta, ptr(dst), ld_dst, sp)
    elif scalar == "s":
        st = lib.costa_gpu_unpack_s(rows, cols, alpha, ptr(src), ld_src, beta, ptr(dst), ld_dst, sp)
    elif scalar == "z":
        st = lib.costa_gpu_unpack_z(rows, cols, _cplx_pair(alpha, C.c_double), ptr(src), ld_src,
                                    _cplx_pair(beta, C.c_double), ptr(dst), ld_dst, sp)
    else:
        st = lib.costa_gpu_unpack_c(rows, cols, _cplx_pair(alpha, C.c_float), ptr(src), ld_src,
                                    _cplx_pair(beta, C.c_float), ptr(dst), ld_dst, sp)
    N.check(st)
