// multiply_using_layout on one rank: C = alpha * op(A) * op(B) + beta * C for
// matrices described block by block (the reference's C interface,
// src/cosma/cinterface.cpp:55-147, over multiply_using_layout,
// src/cosma/multiply.cpp:78-213).
//
// With one rank every block is local, COSMA's strategy is empty and COSTA's
// transforms reduce to gathers: each operand's blocks are gathered into one
// dense column-major matrix in HBM (host blocks through the staged copier,
// device blocks by device copies), one device GEMM runs with the process-wide
// method, and C's blocks are scattered back.  Corner cases follow the
// reference (multiply.cpp:99-109): m or n == 0 is a no-op, k == 0 or
// alpha == 0 scales C by beta, beta == 0 never reads C.
#include "common.cuh"
#include "runtime.hpp"

#include <algorithm>
#include <cctype>
#include <mutex>
#include <string>
#include <vector>

namespace cgb {
namespace {

struct Dense {
    int64_t rows = 0, cols = 0;
};

bool on_device(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Checks that `L` is a complete one-rank layout; returns its global shape.
int check_layout(const char* name, const cosma_gpu_layout* L, Dense* d) {
    const std::string who = std::string("multiply_using_layout: ") + name + ": ";
    if (!L || L->rowblocks < 0 || L->colblocks < 0 || (L->rowblocks && !L->rowsplit) ||
        (L->colblocks && !L->colsplit) || L->nlocalblocks < 0 || (L->nlocalblocks && !L->localblocks))
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, who + "malformed layout");
    for (int i = 0; i < L->rowblocks; ++i)
        if (L->rowsplit[i] > L->rowsplit[i + 1]) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, who + "rowsplit");
    for (int j = 0; j < L->colblocks; ++j)
        if (L->colsplit[j] > L->colsplit[j + 1]) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, who + "colsplit");
    if ((L->rowblocks && L->rowsplit[0] != 0) || (L->colblocks && L->colsplit[0] != 0))
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, who + "splits must start at 0");
    if (L->owners)
        for (int i = 0; i < L->rowblocks * L->colblocks; ++i)
            if (L->owners[i] != 0)
                return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, who + "blocks owned by other ranks (one-rank build)");
    std::vector<char> seen((size_t)L->rowblocks * L->colblocks, 0);
    for (int b = 0; b < L->nlocalblocks; ++b) {
        const cosma_gpu_block& blk = L->localblocks[b];
        if (blk.row < 0 || blk.row >= L->rowblocks || blk.col < 0 || blk.col >= L->colblocks)
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, who + "block index out of range");
        char& s = seen[(size_t)blk.row * L->colblocks + blk.col];
        if (s) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, who + "block listed twice");
        s = 1;
        const int rows = L->rowsplit[blk.row + 1] - L->rowsplit[blk.row];
        const int cols = L->colsplit[blk.col + 1] - L->colsplit[blk.col];
        if (rows > 0 && cols > 0 && (!blk.data || blk.ld < rows))
            return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, who + "block data / leading dimension");
    }
    for (char s : seen)
        if (!s) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, who + "a block is missing");
    d->rows = L->rowblocks ? L->rowsplit[L->rowblocks] : 0;
    d->cols = L->colblocks ? L->colsplit[L->colblocks] : 0;
    return COSMA_GPU_SUCCESS;
}

// Copies every block of `L` into (to_dense) or out of the dense matrix
// `dense` (leading dimension ld, element size es).
int move_blocks(const cosma_gpu_layout* L, char* dense, int64_t ld, size_t es, bool to_dense, cudaStream_t s) {
    for (int b = 0; b < L->nlocalblocks; ++b) {
        const cosma_gpu_block& blk = L->localblocks[b];
        const int64_t r0 = L->rowsplit[blk.row], c0 = L->colsplit[blk.col];
        const int64_t rows = L->rowsplit[blk.row + 1] - r0, cols = L->colsplit[blk.col + 1] - c0;
        if (rows == 0 || cols == 0) continue;
        char* d = dense + (r0 + c0 * ld) * es;
        const size_t width = (size_t)rows * es, dpitch = (size_t)ld * es, bpitch = (size_t)blk.ld * es;
        if (on_device(blk.data)) {
            if (to_dense)
                CGB_CUDA(cudaMemcpy2DAsync(d, dpitch, blk.data, bpitch, width, cols, cudaMemcpyDeviceToDevice, s));
            else
                CGB_CUDA(cudaMemcpy2DAsync(blk.data, bpitch, d, dpitch, width, cols, cudaMemcpyDeviceToDevice, s));
        } else if (to_dense) {
            CGB_CHECK(copy_h2d_2d(d, dpitch, blk.data, bpitch, width, (size_t)cols, s));
        } else {
            CGB_CHECK(copy_d2h_2d(blk.data, bpitch, d, dpitch, width, (size_t)cols, s));
        }
    }
    return COSMA_GPU_SUCCESS;
}

std::mutex g_lay_mu;
cudaStream_t g_lay_stream = nullptr;
DeviceBuffer g_lay_buf[3];

int multiply_using_layout(Scalar sc, const char* transa, const char* transb, const double* alpha,
                          const cosma_gpu_layout* LA, const cosma_gpu_layout* LB, const double* beta,
                          const cosma_gpu_layout* LC) {
    if (!transa || !transb || !alpha || !beta)
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "multiply_using_layout: null argument");
    const int opa = parse_op((char)std::toupper(*transa)), opb = parse_op((char)std::toupper(*transb));
    if (opa < 0 || opb < 0)
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "multiply_using_layout: trans must be N, T or C");
    Dense a, b, c;
    CGB_CHECK(check_layout("A", LA, &a));
    CGB_CHECK(check_layout("B", LB, &b));
    CGB_CHECK(check_layout("C", LC, &c));
    const int64_t m = opa == 0 ? a.rows : a.cols, k = opa == 0 ? a.cols : a.rows;
    const int64_t kb = opb == 0 ? b.rows : b.cols, n = opb == 0 ? b.cols : b.rows;
    if (k != kb || c.rows != m || c.cols != n)
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "multiply_using_layout: shapes of op(A), op(B), C differ");
    if (m == 0 || n == 0) return COSMA_GPU_SUCCESS;
    const bool cplx = scalar_complex(sc);
    const bool alpha_zero = alpha[0] == 0.0 && (!cplx || alpha[1] == 0.0);
    const bool beta_zero = beta[0] == 0.0 && (!cplx || beta[1] == 0.0);
    const bool beta_one = beta[0] == 1.0 && (!cplx || beta[1] == 0.0);
    const size_t es = scalar_bytes(sc);

    std::lock_guard<std::mutex> lock(g_lay_mu);
    if (!g_lay_stream) CGB_CUDA(cudaStreamCreateWithFlags(&g_lay_stream, cudaStreamNonBlocking));
    cudaStream_t s = g_lay_stream;
    CGB_CHECK(g_lay_buf[2].reserve(std::max<size_t>((size_t)m * n * es, 16), s));
    char* dC = (char*)g_lay_buf[2].ptr;
    if (k == 0 || alpha_zero) {  // C <- beta * C (multiply.cpp:101-106)
        if (beta_one) return COSMA_GPU_SUCCESS;
        if (!beta_zero) CGB_CHECK(move_blocks(LC, dC, m, es, true, s));
        CGB_CHECK(scale_matrix_device(sc, m, n, beta, dC, m, s));
        CGB_CHECK(move_blocks(LC, dC, m, es, false, s));
        CGB_CUDA(cudaStreamSynchronize(s));
        return COSMA_GPU_SUCCESS;
    }
    CGB_CHECK(g_lay_buf[0].reserve(std::max<size_t>((size_t)a.rows * a.cols * es, 16), s));
    CGB_CHECK(g_lay_buf[1].reserve(std::max<size_t>((size_t)b.rows * b.cols * es, 16), s));
    char* dA = (char*)g_lay_buf[0].ptr;
    char* dB = (char*)g_lay_buf[1].ptr;
    CGB_CHECK(move_blocks(LA, dA, std::max<int64_t>(a.rows, 1), es, true, s));
    CGB_CHECK(move_blocks(LB, dB, std::max<int64_t>(b.rows, 1), es, true, s));
    if (!beta_zero) CGB_CHECK(move_blocks(LC, dC, m, es, true, s));
    GemmDesc g = make_gemm_desc(sc, *transa, *transb, m, n, k, alpha, dA, std::max<int64_t>(a.rows, 1), dB,
                                std::max<int64_t>(b.rows, 1), beta, dC, m);
    CGB_CHECK(gemm_device(g, process_gemm_method(), 0, s, nullptr));
    CGB_CHECK(move_blocks(LC, dC, m, es, false, s));
    CGB_CUDA(cudaStreamSynchronize(s));
    return COSMA_GPU_SUCCESS;
}

}  // namespace
}  // namespace cgb

extern "C" {

int cosma_gpu_smultiply_using_layout(const char* ta, const char* tb, const float* alpha, const cosma_gpu_layout* a,
                                     const cosma_gpu_layout* b, const float* beta, const cosma_gpu_layout* c) {
    cgb::clear_error();
    if (!alpha || !beta) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "multiply_using_layout: null scalar");
    const double al[2] = {*alpha, 0.0}, be[2] = {*beta, 0.0};
    return cgb::multiply_using_layout(cgb::Scalar::S, ta, tb, al, a, b, be, c);
}
int cosma_gpu_dmultiply_using_layout(const char* ta, const char* tb, const double* alpha, const cosma_gpu_layout* a,
                                     const cosma_gpu_layout* b, const double* beta, const cosma_gpu_layout* c) {
    cgb::clear_error();
    if (!alpha || !beta) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "multiply_using_layout: null scalar");
    const double al[2] = {*alpha, 0.0}, be[2] = {*beta, 0.0};
    return cgb::multiply_using_layout(cgb::Scalar::D, ta, tb, al, a, b, be, c);
}
int cosma_gpu_cmultiply_using_layout(const char* ta, const char* tb, const float* alpha, const cosma_gpu_layout* a,
                                     const cosma_gpu_layout* b, const float* beta, const cosma_gpu_layout* c) {
    cgb::clear_error();
    if (!alpha || !beta) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "multiply_using_layout: null scalar");
    const double al[2] = {alpha[0], alpha[1]}, be[2] = {beta[0], beta[1]};
    return cgb::multiply_using_layout(cgb::Scalar::C, ta, tb, al, a, b, be, c);
}
int cosma_gpu_zmultiply_using_layout(const char* ta, const char* tb, const double* alpha, const cosma_gpu_layout* a,
                                     const cosma_gpu_layout* b, const double* beta, const cosma_gpu_layout* c) {
    cgb::clear_error();
    if (!alpha || !beta) return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "multiply_using_layout: null scalar");
    return cgb::multiply_using_layout(cgb::Scalar::Z, ta, tb, alpha, a, b, beta, c);
}

}  // extern "C"
