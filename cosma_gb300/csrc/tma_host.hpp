// Host-side TMA tensor-map creation through the driver entry point (no
// link-time dependency on libcuda).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include "common.cuh"

namespace cgb {

inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        else
            cudaGetLastError();
    }
    return fn;
}

// 2-D row-major byte matrix [rows][cols] (cols contiguous, row pitch
// `pitch_bytes`), box = box_rows x box_cols elements, 128-byte swizzle.
// elem: CU_TENSOR_MAP_DATA_TYPE_UINT8 or _BFLOAT16.
inline int make_tmap_2d(CUtensorMap* map, CUtensorMapDataType dtype, size_t elem_bytes, const void* base,
                        uint64_t cols, uint64_t rows, uint64_t pitch_bytes, uint32_t box_cols, uint32_t box_rows) {
    auto enc = tensor_map_encoder();
    if (!enc) return set_error(COSMA_GPU_ERROR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
    if (((uintptr_t)base % 16) || (pitch_bytes % 16) || ((box_cols * elem_bytes) % 16))
        return set_error(COSMA_GPU_ERROR_INTERNAL, "tensor map: misaligned base, pitch or box");
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {pitch_bytes};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, dtype, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(COSMA_GPU_ERROR_CUDA, "cuTensorMapEncodeTiled failed");
    return COSMA_GPU_SUCCESS;
}

}  // namespace cgb
