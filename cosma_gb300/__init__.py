"""cosma_gb300: COSMA's one-rank GEMM path, rebuilt for GB300 (sm_103a).

The compute lives in the in-tree CUDA library ``_lib/libcosma_gb300.so``
(C ABI: ``include/cosma_gb300.h``); this package is its Python mirror.
"""
from ._native import (CosmaGpuError, METHOD_AUTO, METHOD_BF16X3, METHOD_NATIVE, METHOD_OZAKI, LIB_PATH,  # noqa: F401
                      load)
from .api import (BlockLayout, GroupedPlan, MMHandle, dgemm_ozaki_device, multiply_using_layout, descinit, gemm,  # noqa: F401
                  gemm_device, host_copy_route, local_multiply, make_context, pack, pxgemm, pxgemm_set_method,
                  tiles_for_memory, unpack, zgemm_ozaki_device)

__version__ = "0.1.0"
