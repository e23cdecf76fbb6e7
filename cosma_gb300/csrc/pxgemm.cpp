// ScaLAPACK p?gemm on a 1x1 process grid.
//
// Follows cosma::pxgemm<T> (src/cosma/cosma_pxgemm.cpp:16-388) for P = 1:
//   1. corner cases: m == 0 or n == 0 -> return; k == 0 or alpha == 0 ->
//      C(ic:, jc:) <- beta * C (no-op for beta == 1)        (:39-46, :393-460)
//   2. trans flags are case-insensitive                      (:57-58)
//   3. descriptors: desc[2..3] global size, desc[4..5] block size,
//      desc[6..7] source process, desc[8] LLD              (scalapack.hpp:11-47)
//   4. transform A, B from the block-cyclic layout to COSMA's blocked
//      column-major layout with op(A), op(B) applied          (:338-343)
//   5. multiply with alpha = 1, beta = 0                     (:350)
//   6. transform C back with C_sc <- alpha*C_cosma + beta*C_sc   (:362-364)
// On a 1x1 grid the block-cyclic layout of every matrix is a single
// column-major buffer of leading dimension LLD, so step 4 is the pack kernel
// (layout.cu) and step 6 the unpack kernel.  The whole problem is staged in
// HBM (host pointers are copied in once; device pointers are used in place).
#include "common.cuh"
#include "runtime.hpp"

#include <algorithm>
#include <cctype>
#include <dlfcn.h>
#include <mutex>
#include <string>

// BLACS is optional: when a BLACS library is linked its grid query is used
// to insist on a 1x1 grid, otherwise the grid is taken to be 1x1.
extern "C" void Cblacs_gridinfo(int ctxt, int* nprow, int* npcol, int* myrow, int* mycol) __attribute__((weak));

namespace cgb {
namespace {

std::mutex g_px_mu;
int g_px_method = -1;
cudaStream_t g_px_stream = nullptr;
cudaStream_t g_px_copy[2] = {nullptr, nullptr};  // host-to-device, device-to-host (the overlapped form)
DeviceBuffer g_px_buf[6];  // A_sc, A_cosma, B_sc, B_cosma, C_cosma, C_sc
// the last call's host<->HBM bytes and whether the overlapped form ran it
int64_t g_px_h2d = 0, g_px_d2h = 0;
int g_px_overlapped = 0;

int px_method() {
    if (g_px_method < 0) g_px_method = default_method();
    return g_px_method;
}

bool is_dev(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Checks that descriptor `d` describes a matrix usable on a 1x1 grid and that
// the (sub_rows x sub_cols) sub-matrix starting at 1-based (i, j) lies inside it.
int check_desc(const char* name, const int* d, int i, int j, int64_t sub_rows, int64_t sub_cols) {
    if (!d) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, std::string("p?gemm: null descriptor ") + name);
    const int M = d[2], N = d[3], MB = d[4], NB = d[5], RSRC = d[6], CSRC = d[7], LLD = d[8];
    if (MB <= 0 || NB <= 0) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, std::string("p?gemm: block size of ") + name);
    if (RSRC != 0 || CSRC != 0)
        return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, std::string("p?gemm: source process of ") + name + " must be 0 on a 1x1 grid");
    if (M < 0 || N < 0 || LLD < std::max(1, M))
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, std::string("p?gemm: global size / LLD of ") + name);
    if (i < 1 || j < 1 || (int64_t)i - 1 + sub_rows > M || (int64_t)j - 1 + sub_cols > N)
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, std::string("p?gemm: sub-matrix out of range in ") + name);
    return COSMA_GPU_SUCCESS;
}

int check_grid(int ctxt) {
    if (Cblacs_gridinfo) {
        int nprow = 0, npcol = 0, myrow = 0, mycol = 0;
        Cblacs_gridinfo(ctxt, &nprow, &npcol, &myrow, &mycol);
        if (nprow != 1 || npcol != 1)
            return set_error(COSMA_GPU_ERROR_NOT_SUPPORTED, "p?gemm: only a 1x1 process grid is supported");
    }
    return COSMA_GPU_SUCCESS;
}

// Brings a (rows x cols, ld) host/device sub-matrix into HBM; returns the
// device pointer and its leading dimension.
int stage_in(const void* p, int64_t rows, int64_t cols, int64_t ld, size_t es, DeviceBuffer& buf, bool copy,
             const void** dptr, int64_t* dld, cudaStream_t s) {
    if (is_dev(p)) {
        *dptr = p;
        *dld = ld;
        return COSMA_GPU_SUCCESS;
    }
    CGB_CHECK(buf.reserve(std::max<size_t>((size_t)rows * cols * es, 16), s));
    *dptr = buf.ptr;
    *dld = std::max<int64_t>(rows, 1);
    if (copy && rows > 0 && cols > 0) {
        CGB_CHECK(copy_h2d_2d(buf.ptr, (size_t)*dld * es, p, (size_t)ld * es, (size_t)rows * es, (size_t)cols, s));
        g_px_h2d += rows * cols * (int64_t)es;
    }
    return COSMA_GPU_SUCCESS;
}

int pxgemm_impl(Scalar sc, const char* transa, const char* transb, const int* pm, const int* pn, const int* pk,
                const double* alpha, const void* a, const int* pia, const int* pja, const int* desca, const void* b,
                const int* pib, const int* pjb, const int* descb, const double* beta, void* c, const int* pic,
                const int* pjc, const int* descc) {
    if (!transa || !transb || !pm || !pn || !pk || !pia || !pja || !pib || !pjb || !pic || !pjc)
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "p?gemm: null argument");
    const int m = *pm, n = *pn, k = *pk;
    if (m < 0 || n < 0 || k < 0) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "p?gemm: negative size");
    if (m == 0 || n == 0) return COSMA_GPU_SUCCESS;
    const bool cplx = scalar_complex(sc);
    const bool alpha_zero = alpha[0] == 0.0 && (!cplx || alpha[1] == 0.0);
    const char ta = (char)std::toupper(*transa), tb = (char)std::toupper(*transb);
    const int opa = parse_op(ta), opb = parse_op(tb);
    if (opa < 0 || opb < 0) return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "p?gemm: trans must be N, T or C");
    CGB_CHECK(check_desc("C", descc, *pic, *pjc, m, n));
    CGB_CHECK(check_grid(descc[1]));
    const size_t es = scalar_bytes(sc);
    const int64_t lldc = descc[8];
    char* csub = (char*)c + ((int64_t)(*pic - 1) + (int64_t)(*pjc - 1) * lldc) * es;

    std::lock_guard<std::mutex> lock(g_px_mu);
    g_px_h2d = g_px_d2h = 0;
    g_px_overlapped = 0;
    if (!g_px_stream) CGB_CUDA(cudaStreamCreateWithFlags(&g_px_stream, cudaStreamNonBlocking));
    cudaStream_t s = g_px_stream;
    const bool c_dev = is_dev(c);

    if (k == 0 || alpha_zero) {  // scale_matrix(descc, c, ic, jc, m, n, beta)
        const bool beta_one = beta[0] == 1.0 && (!cplx || beta[1] == 0.0);
        if (beta_one) return COSMA_GPU_SUCCESS;
        const bool beta_zero = beta[0] == 0.0 && (!cplx || beta[1] == 0.0);
        const void* dC;
        int64_t ldC;
        CGB_CHECK(stage_in(csub, m, n, lldc, es, g_px_buf[5], !beta_zero, &dC, &ldC, s));
        CGB_CHECK(scale_matrix_device(sc, m, n, beta, (void*)dC, ldC, s));
        if (!c_dev) {
            CGB_CHECK(copy_d2h_2d(csub, lldc * es, dC, ldC * es, (size_t)m * es, n, s));
            g_px_d2h = (int64_t)m * n * (int64_t)es;
        }
        CGB_CUDA(cudaStreamSynchronize(s));
        return COSMA_GPU_SUCCESS;
    }

    // sub-matrix shapes as stored (before op), cosma_pxgemm.cpp:87-94
    const int64_t a_subm = opa == 0 ? m : k, a_subn = opa == 0 ? k : m;
    const int64_t b_subm = opb == 0 ? k : n, b_subn = opb == 0 ? n : k;
    CGB_CHECK(check_desc("A", desca, *pia, *pja, a_subm, a_subn));
    CGB_CHECK(check_desc("B", descb, *pib, *pjb, b_subm, b_subn));
    if (desca[1] != descc[1] || descb[1] != descc[1])
        return set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "p?gemm: A, B and C must share one BLACS context");
    const int64_t llda = desca[8], lldb = descb[8];
    const char* asub = (const char*)a + ((int64_t)(*pia - 1) + (int64_t)(*pja - 1) * llda) * es;
    const char* bsub = (const char*)b + ((int64_t)(*pib - 1) + (int64_t)(*pjb - 1) * lldb) * es;

    // Host A, B and C of a real double problem under the Chinese-remainder
    // method: the overlapped one-step form copies op(A) row panels and op(B)
    // column panels straight from the ScaLAPACK buffers while earlier blocks
    // compute and sends C blocks back while later ones do.  Its reconstruction
    // rounds fl(fl(alpha * fl(A B)) + fl(beta * C)), which is steps 3 and 4
    // below to the bit (the product rounded once, then the unpack's scaling).
    // When its first panels would choose another modulus count than the whole
    // data, or the data holds Inf/NaN, or a buffer is refused before C is
    // touched, the staged path below runs.
    // (pzgemm keeps the staged form: its unpack multiplies by alpha + 0i as a
    // complex number, whose zero imaginary products can change the sign of a
    // zero result, which the reconstruction's real scaling would not.)
    if (sc == Scalar::D && px_method() == COSMA_GPU_METHOD_OZAKI2 && !c_dev && !is_dev(asub) && !is_dev(bsub) &&
        env_bool("COSMA_GPU_OZAKI2_OVERLAP", true)) {
        for (auto& cs : g_px_copy)
            if (!cs) CGB_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        const GemmDesc g = make_gemm_desc(sc, ta, tb, m, n, k, alpha, asub, llda, bsub, lldb, beta, csub, lldc);
        int64_t h2d = 0, d2h = 0;
        bool taken = false;
        const int st = ozaki2_gemm_host(g, 0, s, g_px_copy[0], g_px_copy[1], nullptr, &h2d, &d2h, &taken);
        if (taken && st == COSMA_GPU_SUCCESS) {
            g_px_h2d = h2d;
            g_px_d2h = d2h;
            g_px_overlapped = 1;
        }
        if (taken || (st != COSMA_GPU_SUCCESS && st != COSMA_GPU_ERROR_OUT_OF_MEMORY)) return st;
        clear_error();
    }

    // 1. stage the ScaLAPACK sub-matrices in HBM
    const void *dAsc, *dBsc, *dCsc;
    int64_t ldAsc, ldBsc, ldCsc;
    const bool beta_zero = beta[0] == 0.0 && (!cplx || beta[1] == 0.0);
    CGB_CHECK(stage_in(asub, a_subm, a_subn, llda, es, g_px_buf[0], true, &dAsc, &ldAsc, s));
    CGB_CHECK(stage_in(bsub, b_subm, b_subn, lldb, es, g_px_buf[2], true, &dBsc, &ldBsc, s));
    CGB_CHECK(stage_in(csub, m, n, lldc, es, g_px_buf[5], !beta_zero, &dCsc, &ldCsc, s));
    // 2. transform into COSMA's blocked layout: A_cosma = op(A) (m x k),
    //    B_cosma = op(B) (k x n), both column-major with ld = rows
    CGB_CHECK(g_px_buf[1].reserve(std::max<size_t>((size_t)m * k * es, 16), s));
    CGB_CHECK(g_px_buf[3].reserve(std::max<size_t>((size_t)k * n * es, 16), s));
    CGB_CHECK(g_px_buf[4].reserve(std::max<size_t>((size_t)m * n * es, 16), s));
    void* dA = g_px_buf[1].ptr;
    void* dB = g_px_buf[3].ptr;
    void* dCc = g_px_buf[4].ptr;
    CGB_CHECK(pack_device(opa, cplx, (int)es, m, k, dAsc, ldAsc, dA, m, s));
    CGB_CHECK(pack_device(opb, cplx, (int)es, k, n, dBsc, ldBsc, dB, k, s));
    // 3. C_cosma = A_cosma * B_cosma (alpha = 1, beta = 0)
    const double one[2] = {1.0, 0.0}, zero[2] = {0.0, 0.0};
    GemmDesc g = make_gemm_desc(sc, 'N', 'N', m, n, k, one, dA, m, dB, k, zero, dCc, m);
    CGB_CHECK(gemm_device(g, px_method(), 0, s, nullptr));
    // 4. C_sc = alpha * C_cosma + beta * C_sc
    CGB_CHECK(unpack_device(sc, m, n, alpha, dCc, m, beta, (void*)dCsc, ldCsc, s));
    if (!c_dev) {
        CGB_CHECK(copy_d2h_2d(csub, lldc * es, dCsc, ldCsc * es, (size_t)m * es, n, s));
        g_px_d2h = (int64_t)m * n * (int64_t)es;
    }
    CGB_CUDA(cudaStreamSynchronize(s));
    return COSMA_GPU_SUCCESS;
}

}  // namespace

int process_gemm_method() {
    std::lock_guard<std::mutex> lock(g_px_mu);
    return px_method();
}

}  // namespace cgb

namespace cgb {
namespace {

// COSMA_DIM_THRESHOLD (default 0, i.e. never): a problem with
// min(m, n, k) below it goes to the next p?gemm_ in the dynamic symbol
// search order, the real ScaLAPACK linked after this library, as the
// reference's interposed entry points do (src/cosma/pxgemm.cpp,
// src/cosma/cosma_pxgemm.cpp:652-655, default in
// src/cosma/environment_variables.hpp:92).  Without a next definition the
// problem stays here.
bool too_small(const int* m, const int* n, const int* k) {
    const long long t = env_ll("COSMA_DIM_THRESHOLD", 0);
    if (t <= 0 || !m || !n || !k) return false;
    return (long long)std::min(*m, std::min(*n, *k)) < t;
}

void* next_definition(const char* name) { return dlsym(RTLD_NEXT, name); }

}  // namespace
}  // namespace cgb

// The ScaLAPACK entry points are void (as in the reference); their status is
// available through cosma_gpu_last_error().  Every spelling falls through to
// the Fortran symbol REAL (p?gemm_) of the next library.
#define CGB_PX_NEXT(T, REAL)                                                                                         \
    if (cgb::too_small(m, n, k)) {                                                                                   \
        using Next = void (*)(COSMA_GPU_PXGEMM_ARGS(T));                                                            \
        static const Next next = (Next)cgb::next_definition(#REAL);                                                  \
        if (next) {                                                                                                  \
            cgb::clear_error();                                                                                      \
            next(transa, transb, m, n, k, alpha, a, ia, ja, desca, b, ib, jb, descb, beta, c, ic, jc, descc);        \
            return;                                                                                                  \
        }                                                                                                            \
    }
#define CGB_PX_REAL(NAME, T, SC, REAL)                                                                               \
    void NAME(COSMA_GPU_PXGEMM_ARGS(T)) {                                                                           \
        CGB_PX_NEXT(T, REAL)                                                                                         \
        cgb::clear_error();                                                                                          \
        double al[2] = {alpha ? (double)alpha[0] : 0.0, 0.0}, be[2] = {beta ? (double)beta[0] : 0.0, 0.0};          \
        cgb::pxgemm_impl(SC, transa, transb, m, n, k, al, a, ia, ja, desca, b, ib, jb, descb, be, c, ic, jc, descc); \
    }
#define CGB_PX_CPLX(NAME, T, SC, REAL)                                                                               \
    void NAME(COSMA_GPU_PXGEMM_ARGS(T)) {                                                                           \
        CGB_PX_NEXT(T, REAL)                                                                                         \
        cgb::clear_error();                                                                                          \
        double al[2] = {alpha ? (double)alpha[0] : 0.0, alpha ? (double)alpha[1] : 0.0};                            \
        double be[2] = {beta ? (double)beta[0] : 0.0, beta ? (double)beta[1] : 0.0};                                \
        cgb::pxgemm_impl(SC, transa, transb, m, n, k, al, a, ia, ja, desca, b, ib, jb, descb, be, c, ic, jc, descc); \
    }
#define CGB_PX_FAMILY(NS, ND, NC, NZ)                          \
    CGB_PX_REAL(NS, float, cgb::Scalar::S, psgemm_)           \
    CGB_PX_REAL(ND, double, cgb::Scalar::D, pdgemm_)          \
    CGB_PX_CPLX(NC, float, cgb::Scalar::C, pcgemm_)           \
    CGB_PX_CPLX(NZ, double, cgb::Scalar::Z, pzgemm_)

extern "C" {

CGB_PX_FAMILY(psgemm, pdgemm, pcgemm, pzgemm)
CGB_PX_FAMILY(psgemm_, pdgemm_, pcgemm_, pzgemm_)
CGB_PX_FAMILY(PSGEMM, PDGEMM, PCGEMM, PZGEMM)
CGB_PX_FAMILY(PSGEMM_, PDGEMM_, PCGEMM_, PZGEMM_)
CGB_PX_FAMILY(cosma_psgemm, cosma_pdgemm, cosma_pcgemm, cosma_pzgemm)
CGB_PX_FAMILY(cosma_psgemm_, cosma_pdgemm_, cosma_pcgemm_, cosma_pzgemm_)
CGB_PX_FAMILY(COSMA_PSGEMM, COSMA_PDGEMM, COSMA_PCGEMM, COSMA_PZGEMM)
CGB_PX_FAMILY(COSMA_PSGEMM_, COSMA_PDGEMM_, COSMA_PCGEMM_, COSMA_PZGEMM_)

int cosma_gpu_pxgemm_set_method(int method) {
    if (method < COSMA_GPU_METHOD_AUTO || method > COSMA_GPU_METHOD_OZAKI2)
        return cgb::set_error(COSMA_GPU_ERROR_INVALID_ARGUMENT, "pxgemm_set_method: unknown method");
    std::lock_guard<std::mutex> lock(cgb::g_px_mu);
    cgb::g_px_method = method;
    return COSMA_GPU_SUCCESS;
}

int cosma_gpu_pxgemm_last_transfers(int64_t* h2d_bytes, int64_t* d2h_bytes, int* overlapped) {
    std::lock_guard<std::mutex> lock(cgb::g_px_mu);
    if (h2d_bytes) *h2d_bytes = cgb::g_px_h2d;
    if (d2h_bytes) *d2h_bytes = cgb::g_px_d2h;
    if (overlapped) *overlapped = cgb::g_px_overlapped;
    return COSMA_GPU_SUCCESS;
}

}  // extern "C"
