"""cosma_gb300: COSMA's one-rank GEMM path, rebuilt for GB300 (sm_103a).

The compute lives in the in-tree CUDA library ``_lib/libcosma_gb300.so``
(C ABI: ``include/cosma_gb300.h``); this package is its Python mirror.
"""
from ._native import (CosmaGpuError, METHOD_AUTO, METHOD_BF16X3, METHOD_NATIVE, METHOD_OZAKI, METHOD_OZAKI2,  # noqa: F401
                      LIB_PATH, load)
from .api import (BlockLayout, GroupedPlan, MMHandle, dgemm_ozaki_device, dgemm_ozaki2_device,  # noqa: F401
                  multiply_using_layout, descinit, gemm, gemm_device, host_copy_route, local_multiply, make_context,
                  dgemm_ozaki2_residual, ozaki2_choose, pack, pxgemm, pxgemm_last_transfers, pxgemm_set_method,
                  release_workspaces,
                  tiles_for_memory, unpack, zgemm_ozaki_device,
                  zgemm_ozaki2_device)

__version__ = "0.1.0"
