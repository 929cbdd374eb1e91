// Host runtime of libelhlprop.so: device context, the reference's drop-in
// symbols and the native trajectory API (include/elhl_prop.h).
//
// Per nuclear step (ElHl_Chebyshev, ElHl_Chebyshev.f:148-291) everything stays
// on the device: S and h from coordinates (build_sh.cu), the Cholesky factor
// S = L L^T with its inverse G = L^-1 and H' = S^-1 h = G^T (G h) (factor.cu,
// dgemm.cu; replacing the reference's LU inverse + dsymm, Taylor_gpu.cpp:686-697),
// the propagation (taylor.cu, cheb.cu) and the populations.  Host traffic per
// step is the coordinates in and the populations out.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "elhl_internal.cuh"

using namespace elhl;

namespace elhl {
std::atomic<long long> g_own_launches{0};
void count_launch(long long n) { g_own_launches.fetch_add(n, std::memory_order_relaxed); }
long long own_launches() { return g_own_launches.load(std::memory_order_relaxed); }
}  // namespace elhl

namespace {

thread_local int g_last_status = ELHL_OK;
constexpr int kGemmMinCols = 16;  // ket columns (one per particle) from which H.Psi runs as one GEMM per order
#ifndef ELHL_GEMM_MIN_N
#define ELHL_GEMM_MIN_N 2048
#endif
constexpr int kGemmMinN = ELHL_GEMM_MIN_N;  // ... on a basis at least this large (smaller ones stay on the row kernel)

#define CU_TRY(expr)                                                                  \
    do {                                                                              \
        cudaError_t e_ = (expr);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            fprintf(stderr, "elhlprop: %s failed: %s (%s:%d)\n", #expr,               \
                    cudaGetErrorString(e_), __FILE__, __LINE__);                      \
            return e_ == cudaErrorMemoryAllocation ? ELHL_ERR_OOM : ELHL_ERR_CUDA;   \
        }                                                                             \
    } while (0)

#define SOLVER_TRY(expr)                                                              \
    do {                                                                              \
        cusolverStatus_t s_ = (expr);                                                 \
        if (s_ != CUSOLVER_STATUS_SUCCESS) {                                          \
            fprintf(stderr, "elhlprop: %s failed: status %d\n", #expr, (int)s_);      \
            return ELHL_ERR_CUDA;                                                     \
        }                                                                             \
    } while (0)

template <typename T>
int dev_alloc(T **p, size_t n) {
    *p = nullptr;
    if (n == 0) return ELHL_OK;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return e == cudaErrorMemoryAllocation ? ELHL_ERR_OOM : ELHL_ERR_CUDA;
    }
    return ELHL_OK;
}

template <typename T>
void dev_free(T *&p) {
    if (p) cudaFree((void *)p);
    p = nullptr;
}

// ---- process-wide context -------------------------------------------------
struct Context {
    bool ready = false;
    int device = -1, sms = 0, grid = 0;
    cudaStream_t stream = nullptr, copy_stream = nullptr, own_stream = nullptr;
    cusolverDnHandle_t solver = nullptr;
    cublasHandle_t blas = nullptr;
    cublasHandle_t blas_tc = nullptr;  // tensor-core emulated FP32 GEMMs (GEMM regime), fixed workspace
    void *tc_ws = nullptr;
    unsigned *bar = nullptr;  // [2] count, gen
    int *err = nullptr;
    double *partials = nullptr;
    // 0/1 propagation begin/end, 2/3 rebuild begin/end, 4 S/h built, 5 factorised, 6 inverse formed
    cudaEvent_t ev[7] = {};
    // the factorisation's second stream: G11^T L21^T of a split runs there while the
    // main stream factors the trailing block (ev_l21: L21 ready, ev_side: side work done)
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t ev_l21 = nullptr, ev_side = nullptr;
    std::mutex mu;
};
Context g_ctx;

// Copies ordered with the library stream.  The library's streams are created
// non-blocking, so a plain cudaMemcpy (legacy default stream) is not ordered
// with their work; device-to-host copies also wait for the data.
cudaError_t copy_h2d(void *dst, const void *src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g_ctx.stream);
}
cudaError_t copy_d2h(void *dst, const void *src, size_t bytes) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g_ctx.stream);
    return e != cudaSuccess ? e : cudaStreamSynchronize(g_ctx.stream);
}

int ensure_context_locked(int device) {
    if (g_ctx.ready && (device < 0 || device == g_ctx.device)) return ELHL_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ELHL_ERR_NO_DEVICE;
    if (device < 0) device = 0;
    device %= ndev;
    CU_TRY(cudaSetDevice(device));
    g_ctx.device = device;
    CU_TRY(cudaDeviceGetAttribute(&g_ctx.sms, cudaDevAttrMultiProcessorCount, device));
    if (taylor_grid_size(kTaylorBlock, &g_ctx.grid)) return ELHL_ERR_CUDA;
    CU_TRY(init_build_tables());
    CU_TRY(cudaStreamCreateWithFlags(&g_ctx.own_stream, cudaStreamNonBlocking));
    g_ctx.stream = g_ctx.own_stream;
    CU_TRY(cudaStreamCreateWithFlags(&g_ctx.copy_stream, cudaStreamNonBlocking));
    CU_TRY(cudaStreamCreateWithFlags(&g_ctx.aux_stream, cudaStreamNonBlocking));
    CU_TRY(cudaEventCreateWithFlags(&g_ctx.ev_l21, cudaEventDisableTiming));
    CU_TRY(cudaEventCreateWithFlags(&g_ctx.ev_side, cudaEventDisableTiming));
    SOLVER_TRY(cusolverDnCreate(&g_ctx.solver));
    SOLVER_TRY(cusolverDnSetStream(g_ctx.solver, g_ctx.stream));
    if (cublasCreate(&g_ctx.blas) != CUBLAS_STATUS_SUCCESS) return ELHL_ERR_CUDA;
    if (cublasSetStream(g_ctx.blas, g_ctx.stream) != CUBLAS_STATUS_SUCCESS) return ELHL_ERR_CUDA;
    if (cublasCreate(&g_ctx.blas_tc) != CUBLAS_STATUS_SUCCESS) return ELHL_ERR_CUDA;
    if (cublasSetStream(g_ctx.blas_tc, g_ctx.stream) != CUBLAS_STATUS_SUCCESS) return ELHL_ERR_CUDA;
    CU_TRY(cudaMalloc(&g_ctx.tc_ws, 64u << 20));
    if (cublasSetWorkspace(g_ctx.blas_tc, g_ctx.tc_ws, 64u << 20) != CUBLAS_STATUS_SUCCESS) return ELHL_ERR_CUDA;
    cublasSetMathMode(g_ctx.blas_tc, CUBLAS_FP32_EMULATED_BF16X9_MATH);
    cublasSetEmulationStrategy(g_ctx.blas_tc, CUBLAS_EMULATION_STRATEGY_EAGER);
    if (int rc = dev_alloc(&g_ctx.bar, 2)) return rc;
    if (int rc = dev_alloc(&g_ctx.err, 1)) return rc;
    if (int rc = dev_alloc(&g_ctx.partials, (size_t)2 * 2 * g_ctx.grid * 16)) return rc;
    CU_TRY(cudaMemset(g_ctx.bar, 0, 2 * sizeof(unsigned)));
    CU_TRY(cudaMemset(g_ctx.err, 0, sizeof(int)));
    for (auto &e : g_ctx.ev) CU_TRY(cudaEventCreate(&e));
    // make the allocation-free entry point's fixed array resident now, before
    // a caller's pool allocator or stream capture can start
    if (int rc = fixed_scratch_prepare()) return rc;
    g_ctx.ready = true;
    return ELHL_OK;
}

int ensure_context(int device = -1) {
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    return ensure_context_locked(device);
}

// ---- small kernels -----------------------------------------------------------
// complex vector (interleaved) <-> two real columns (re | im), ld = ldm
__global__ void split_complex(const double2 *__restrict__ z, double *__restrict__ m, int n, int ldm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double2 v = z[i];
        m[i] = v.x;
        m[ldm + i] = v.y;
    }
}
__global__ void join_complex(const double *__restrict__ m, double2 *__restrict__ z, int n, int ldm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = make_double2(m[i], m[ldm + i]);
}

// Embed fragment eigenvector (column `col` of V, ldf) into the full basis with
// the sign convention "largest |component| positive" (first index on ties).
// One block; ket_full must be zeroed by the caller.
__global__ void embed_fmo(const double *__restrict__ V, int ldf, int nf, int col, const int *__restrict__ aos,
                          double2 *__restrict__ ket_full, int stride) {
    __shared__ double s_val[256];
    __shared__ int s_idx[256];
    const double *c = V + (size_t)col * ldf;
    double best = -1.0;
    int bi = 0x7fffffff;
    for (int k = threadIdx.x; k < nf; k += blockDim.x) {
        const double a = fabs(c[k]);
        if (a > best) { best = a; bi = k; }
    }
    s_val[threadIdx.x] = best;
    s_idx[threadIdx.x] = bi;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            const double v2 = s_val[threadIdx.x + o];
            const int i2 = s_idx[threadIdx.x + o];
            if (v2 > s_val[threadIdx.x] || (v2 == s_val[threadIdx.x] && i2 < s_idx[threadIdx.x])) {
                s_val[threadIdx.x] = v2;
                s_idx[threadIdx.x] = i2;
            }
        }
        __syncthreads();
    }
    const double sign = c[s_idx[0]] < 0.0 ? -1.0 : 1.0;
    for (int k = threadIdx.x; k < nf; k += blockDim.x) ket_full[(size_t)aos[k] * stride] = make_double2(sign * c[k], 0.0);
}

// bra = S ket for a ket supported on the AO list `aos` (real coefficients)
__global__ void s_times_sparse(const double *__restrict__ S, int ld, int n, const int *__restrict__ aos, int nf,
                               const double2 *__restrict__ ket, double2 *__restrict__ bra, int stride) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = 0.0;
    for (int k = 0; k < nf; ++k) {
        const int j = aos[k];
        acc += S[(size_t)j * ld + i] * ket[(size_t)j * stride].x;  // S symmetric: S(i, j) = S(j, i)
    }
    bra[(size_t)i * stride] = make_double2(acc, 0.0);
}

__global__ void zero_strided(double2 *v, int n, int stride) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[(size_t)i * stride] = make_double2(0.0, 0.0);
}

// ---- S = L L^T and G = L^-1 in FP64 (hand-written) ------------------------------
// zero the strictly upper triangle and the padding rows of an ld x n matrix
__global__ void lower_only_kernel(double *A, int n, int ld) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i < ld && j < n && (i < j || i >= n)) A[(size_t)j * ld + i] = 0.0;
}

// Cholesky factor and its inverse together, in place, FP64 on the FP64 pipe:
//   L11, G11 = chol_inv(A11);   L21 = A21 G11^T;   A22 -= L21 L21^T;
//   L22, G22 = chol_inv(A22);   G21 = -G22 (L21 G11),
// N^3/3 + N^3/3 flops in dgemm64 products (triangular operands at half cost),
// 64-row diagonal blocks as leaves (leaf_chol_inv64), splits on multiples of 64.
// G11^T L21^T, the first factor of G21 = -G22 (L21 G11) stored transposed in the
// unused upper block G12, runs on a second stream while the main stream does the
// Schur update and factors A22 (whose single-CTA leaves leave most SMs free).
// It replaces the reference's LU inverse of S (MAGMA dgetrf + dgetri,
// GPU_Interface.cpp:910-928; CPU dsytrf + dsytri, :936-947): S is symmetric
// positive definite, so its Cholesky factor gives S^-1 = G^T G.  W holds the
// n2 x n1 off-diagonal block of each split (leading dimension ld).  The upper
// triangles of A and G are left undefined.
bool chol_inv_fits(int n, int ld, size_t wcap) {
    const int leaf = leaf_rows();
    if (n <= leaf) return true;
    const int n1 = round_up(n / 2, leaf), n2 = n - n1;
    return (size_t)ld * n1 <= wcap && chol_inv_fits(n1, ld, wcap) && chol_inv_fits(n2, ld, wcap);
}

// An FP64 product of the factorisations: on the tensor cores from exact slices
// (ozgemm) when tc is set and the product is large enough to fill the GPU, else
// on the FP64 pipe (dgemm64).
// Below 320 rows the FP64 pipe of all SMs (dgemm64's 16- and 32-row tiles) beats
// the three launches of a sliced product: the factorisation at N = 3720 took
// 15.7 ms with the cut at 64 rows, 12.4 at 192, 11.7 at 320, 11.8 at 448 and
// 12.6 at 640.
constexpr int kOzGemmMin = 320;
cudaError_t fgemm(bool tc, int m, int n, int k, double alpha, const double *A, int lda, bool transA, const double *B,
                  int ldb, bool transB, double beta, double *C, int ldc, cudaStream_t st, int tri = 0, int lane = 0) {
    if (tc && m >= kOzGemmMin && n >= kOzGemmMin && k >= kOzGemmMin)
        return ozgemm(m, n, k, alpha, A, lda, transA, B, ldb, transB, beta, C, ldc, st, tri, lane);
    return dgemm64(m, n, k, alpha, A, lda, transA, B, ldb, transB, beta, C, ldc, st, tri, lane);
}

// ELHL_ERR_TIMEOUT if a tensor-core product gave up a wait since the last check (then cleared)
int ozgemm_status() {
    for (int lane = 0; lane < 2; ++lane) {
        int *e = ozgemm_error(lane);
        if (!e) continue;
        int h = 0;
        CU_TRY(cudaMemcpy(&h, e, sizeof(int), cudaMemcpyDeviceToHost));
        if (h) {
            CU_TRY(cudaMemset(e, 0, sizeof(int)));
            return h;
        }
    }
    return ELHL_OK;
}

int chol_inv64(double *A, double *G, int n, int ld, int row0, double *W, int *info, bool tc = false) {
    cudaStream_t st = g_ctx.stream;
    const int leaf = leaf_rows();
    if (n <= leaf) {
        CU_TRY(leaf_chol_inv64(A, G, n, ld, row0, info, st));
        return ELHL_OK;
    }
    const int n1 = round_up(n / 2, leaf), n2 = n - n1;
    double *A21 = A + n1, *A22 = A + (size_t)n1 * ld + n1;
    double *G21 = G + n1, *G22 = G + (size_t)n1 * ld + n1;
    double *G12 = G + (size_t)n1 * ld;  // n1 x n2, above the diagonal: free until lower_only
    cudaStream_t side = g_ctx.aux_stream;
    if (int rc = chol_inv64(A, G, n1, ld, row0, W, info, tc)) return rc;
    CU_TRY(cudaMemcpy2DAsync(W, ld * sizeof(double), A21, ld * sizeof(double), n2 * sizeof(double), n1,
                             cudaMemcpyDeviceToDevice, st));
    CU_TRY(fgemm(tc, n2, n1, n1, 1.0, W, ld, false, G, ld, true, 0.0, A21, ld, st, kTriBt));       // L21
    CU_TRY(cudaEventRecord(g_ctx.ev_l21, st));
    CU_TRY(cudaStreamWaitEvent(side, g_ctx.ev_l21, 0));
    CU_TRY(fgemm(tc, n1, n2, n1, 1.0, G, ld, true, A21, ld, true, 0.0, G12, ld, side, kTriAt, 1));  // (L21 G11)^T
    CU_TRY(cudaEventRecord(g_ctx.ev_side, side));
    CU_TRY(fgemm(tc, n2, n2, n1, -1.0, A21, ld, false, A21, ld, true, 1.0, A22, ld, st, kTriLowerC));  // Schur
    if (int rc = chol_inv64(A22, G22, n2, ld, row0 + n1, W, info, tc)) return rc;
    // the side stream is serial: its last recorded event covers this split's product
    CU_TRY(cudaStreamWaitEvent(st, g_ctx.ev_side, 0));
    CU_TRY(fgemm(tc, n2, n1, n2, -1.0, G22, ld, false, G12, ld, true, 0.0, G21, ld, st, kTriA));  // G21
    return ELHL_OK;
}

// ---- H' = S^-1 h = G^T (G h) ---------------------------------------------------
struct Factor {
    int N = 0, ld = 0;
    double *L = nullptr;     // Cholesky factor (lower, zero above the diagonal), N x N, ld
    double *G = nullptr;     // G = L^-1 (lower, zero above the diagonal), unless factor() put it elsewhere
    double *W = nullptr;     // ld x N workspace: the factorisation's off-diagonal blocks, then G h
    int *info = nullptr;     // [2]: first non-positive pivot (1-based global column), 0 = positive definite
    double *cols = nullptr;  // 2 x (N x 2) scratch (S^-1 applied to a complex vector)
    bool tc = false;         // large products on the tensor cores from exact slices (ELHL_PREC_OZ64)
    int reserve(int N_, int ld_) {
        if (N_ <= N && ld_ == ld && L) return ELHL_OK;
        release();
        N = N_;
        ld = ld_;
        if (int rc = dev_alloc(&L, (size_t)ld * N)) return rc;
        if (int rc = dev_alloc(&G, (size_t)ld * N)) return rc;
        if (int rc = dev_alloc(&W, (size_t)ld * N)) return rc;
        if (int rc = dev_alloc(&info, 2)) return rc;
        CU_TRY(cudaMemset(info, 0, 2 * sizeof(int)));
        if (int rc = dev_alloc(&cols, (size_t)4 * ld)) return rc;
        return ELHL_OK;
    }
    void release() {
        dev_free(L); dev_free(G); dev_free(W); dev_free(info); dev_free(cols);
        N = 0;
    }
    // L <- chol(S) and Gdst (this->G when null) <- L^-1, both with zero upper
    // triangles and padding rows.  Every block of the recursion is checked
    // against the workspace before the first launch.  Asynchronous.
    int factor(const double *S, int n, double *Gdst = nullptr) {
        cudaStream_t st = g_ctx.stream;
        double *g = Gdst ? Gdst : G;
        if (!chol_inv_fits(n, ld, (size_t)ld * N)) return ELHL_ERR_OOM;
        CU_TRY(cudaMemsetAsync(info, 0, 2 * sizeof(int), st));
        CU_TRY(cudaMemcpy2DAsync(L, ld * sizeof(double), S, ld * sizeof(double), n * sizeof(double), n,
                                 cudaMemcpyDeviceToDevice, st));
        if (int rc = chol_inv64(L, g, n, ld, 0, W, info, tc)) return rc;
        const dim3 grid((ld + 127) / 128, n);
        lower_only_kernel<<<grid, 128, 0, st>>>(L, n, ld);
        count_launch();
        lower_only_kernel<<<grid, 128, 0, st>>>(g, n, ld);
        count_launch();
        CU_TRY(cudaGetLastError());
        return ELHL_OK;
    }
    // L, G from S; Hp <- G^T (G h) = S^-1 h, 2 N^3 flops with triangular G.  Asynchronous.
    int form_hprime(const double *S, const double *h, double *Hp, int n) {
        cudaStream_t st = g_ctx.stream;
        if (int rc = factor(S, n)) return rc;
        CU_TRY(fgemm(tc, n, n, n, 1.0, G, ld, false, h, ld, false, 0.0, W, ld, st, kTriA));    // G h
        CU_TRY(fgemm(tc, n, n, n, 1.0, G, ld, true, W, ld, false, 0.0, Hp, ld, st, kTriAt));   // G^T (G h)
        return ELHL_OK;
    }
    // out = S^-1 z = G^T (G z) for a complex vector z (device), using the factor.
    int apply_sinv(const double2 *z, double2 *out, int n) {
        cudaStream_t st = g_ctx.stream;
        const int tb = 256, nb = (n + tb - 1) / tb;
        double *c2 = cols + 2 * ld;
        split_complex<<<nb, tb, 0, st>>>(z, cols, n, ld);
        count_launch();
        CU_TRY(dgemm64(n, 2, n, 1.0, G, ld, false, cols, ld, false, 0.0, c2, ld, st, kTriA));
        CU_TRY(dgemm64(n, 2, n, 1.0, G, ld, true, c2, ld, false, 0.0, cols, ld, st, kTriAt));
        join_complex<<<nb, tb, 0, st>>>(cols, out, n, ld);
        count_launch();
        CU_TRY(cudaGetLastError());
        return ELHL_OK;
    }
    // status of the last factorisation; waits for it on the library stream
    int check_info(bool = true) {
        int h[2] = {0, 0};
        CU_TRY(cudaMemcpyAsync(h, info, 2 * sizeof(int), cudaMemcpyDeviceToHost, g_ctx.stream));
        CU_TRY(cudaStreamSynchronize(g_ctx.stream));
        if (tc)
            if (int rc = ozgemm_status()) return rc;
        if (h[0] > 0) return ELHL_ERR_NOT_POSITIVE_DEFINITE;
        if (h[0] < 0) return ELHL_ERR_BAD_ARG;
        return ELHL_OK;
    }
};

// ---- one Taylor launch -------------------------------------------------------
struct TaylorBuffers {
    int N = 0, ldv = 0, P = 0;
    double2 *slots = nullptr;
    TaylorParticle *part = nullptr;
    double *tfinal = nullptr;
    int reserve(int N_, int P_) {
        const int ldv_ = round_up(N_, 32);
        if (slots && N_ <= N && P_ <= P && ldv_ <= ldv) return ELHL_OK;
        release();
        N = N_;
        P = P_;
        ldv = ldv_;
        if (int rc = dev_alloc(&slots, (size_t)P * kSlots * 2 * ldv)) return rc;
        if (int rc = dev_alloc(&part, (size_t)P)) return rc;
        if (int rc = dev_alloc(&tfinal, 1)) return rc;
        CU_TRY(cudaMemset(slots, 0, (size_t)P * kSlots * 2 * ldv * sizeof(double2)));
        return ELHL_OK;
    }
    void release() {
        dev_free(slots); dev_free(part); dev_free(tfinal);
        N = 0;
        P = 0;
    }
    double2 *bra(int p) { return slots + (size_t)(p * kSlots) * 2 * ldv; }
    double2 *ket(int p) { return slots + ((size_t)(p * kSlots) * 2 + 1) * ldv; }
};

int run_taylor(const double *Hp, int N, int ld, TaylorBuffers &tb, int P, const double *tau_in, double t_init,
               double t_max, double tol, double norm_tol, int max_conv, int nsteps, int it0, double dt_frame,
               double tau_max, double *d_pops, const int *ao_frag, int nfrag) {
    cudaStream_t st = g_ctx.stream;
    std::vector<TaylorParticle> hp(P);
    for (int p = 0; p < P; ++p) {
        memset(&hp[p], 0, sizeof(TaylorParticle));
        hp[p].tau_in = tau_in[p];
    }
    CU_TRY(cudaMemcpyAsync(tb.part, hp.data(), P * sizeof(TaylorParticle), cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemsetAsync(g_ctx.err, 0, sizeof(int), st));
    CU_TRY(cudaMemsetAsync(g_ctx.bar, 0, 2 * sizeof(unsigned), st));  // fresh barrier every launch
    TaylorLaunch L{};
    L.H = Hp;
    L.N = N;
    L.ld = ld;
    L.nparticles = P;
    L.slots = tb.slots;
    L.ldv = tb.ldv;
    L.part = tb.part;
    L.t_init = t_init;
    L.t_max = t_max;
    L.tol = tol;
    L.norm_tol = norm_tol;
    L.max_conv_calls = max_conv;
    L.nsteps = nsteps;
    L.it0 = it0;
    L.dt_frame = dt_frame;
    L.tau_max = tau_max;
    L.pops = d_pops;
    L.ao_frag = ao_frag;
    L.nfrag = nfrag;
    L.t_final = tb.tfinal;
    L.partials = g_ctx.partials;
    L.bar_count = g_ctx.bar;
    L.error = g_ctx.err;
    CU_TRY(cudaEventRecord(g_ctx.ev[0], st));
    CU_TRY(launch_taylor(L, g_ctx.grid, kTaylorBlock, st));
    CU_TRY(cudaEventRecord(g_ctx.ev[1], st));
    return ELHL_OK;
}

// elapsed ms between two recorded events (after a synchronize)
double event_ms(int a, int b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, g_ctx.ev[a], g_ctx.ev[b]) != cudaSuccess) return 0.0;
    return ms;
}

int collect_taylor(TaylorBuffers &tb, int P, std::vector<TaylorParticle> &out, double *tfinal) {
    out.resize(P);
    int err = 0;
    CU_TRY(cudaMemcpyAsync(out.data(), tb.part, P * sizeof(TaylorParticle), cudaMemcpyDeviceToHost, g_ctx.stream));
    CU_TRY(cudaMemcpyAsync(&err, g_ctx.err, sizeof(int), cudaMemcpyDeviceToHost, g_ctx.stream));
    if (tfinal) CU_TRY(cudaMemcpyAsync(tfinal, tb.tfinal, sizeof(double), cudaMemcpyDeviceToHost, g_ctx.stream));
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    if (err) return err;
    for (int p = 0; p < P; ++p)
        if (out[p].status) return out[p].status;
    return ELHL_OK;
}

// ---- drop-in state (function-static in the reference, Taylor_gpu.cpp:650-673) --
struct DropIn {
    int N = 0, ld = 0;
    double *S = nullptr, *h = nullptr, *Hp = nullptr;
    Factor fac;
    TaylorBuffers tb;
    double2 *ao = nullptr;
    cudaEvent_t hp_ready = nullptr;  // H' formed: the copy stream may read it
    int reserve(int N_) {
        const int ld_ = round_up(N_, 32);
        if (!(S && N_ <= N && ld_ == ld)) {
            release();
            N = N_;
            ld = ld_;
            if (int rc = dev_alloc(&S, (size_t)ld * N)) return rc;
            if (int rc = dev_alloc(&h, (size_t)ld * N)) return rc;
            if (int rc = dev_alloc(&Hp, (size_t)ld * N)) return rc;
            if (int rc = dev_alloc(&ao, (size_t)ld)) return rc;
            if (int rc = fac.reserve(N, ld)) return rc;
            if (int rc = tb.reserve(N, 1)) return rc;
        }
        if (!hp_ready) CU_TRY(cudaEventCreateWithFlags(&hp_ready, cudaEventDisableTiming));
        return ELHL_OK;
    }
    void release() {
        dev_free(S); dev_free(h); dev_free(Hp); dev_free(ao);
        fac.release();
        tb.release();
        if (hp_ready) cudaEventDestroy(hp_ready);
        hp_ready = nullptr;
        N = 0;
    }
};
DropIn g_drop;

// Waits for the copy stream when it goes out of scope, so that no return path
// leaves a copy into the caller's host buffer in flight.
struct CopyStreamJoin {
    ~CopyStreamJoin() { cudaStreamSynchronize(g_ctx.copy_stream); }
};

int dropin_elhl(int n, const double *hS, const double *hh, double *hH, elhl_zcomplex *hAO_bra, elhl_zcomplex *hbra,
                elhl_zcomplex *hket, double t_init, double t_max, double tau, double *save_tau) {
    if (n <= 0 || !hS || !hh || !hbra || !hket) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (int rc = ensure_context_locked(-1)) return rc;
    if (int rc = g_drop.reserve(n)) return rc;
    DropIn &d = g_drop;
    cudaStream_t st = g_ctx.stream;
    const size_t col = n * sizeof(double), ldb = d.ld * sizeof(double);
    CU_TRY(cudaMemcpy2DAsync(d.S, ldb, hS, col, col, n, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpy2DAsync(d.h, ldb, hh, col, col, n, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(d.tb.bra(0), hbra, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(d.tb.ket(0), hket, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    if (int rc = d.fac.form_hprime(d.S, d.h, d.Hp, n)) return rc;
    // A factorisation that failed (S not positive definite) ends the call here,
    // before anything is propagated or copied back.
    if (int frc = d.fac.check_info()) return frc;
    // H' back to the host on a second stream, overlapped with the propagation (Taylor_gpu.cpp:700)
    CopyStreamJoin join;
    CU_TRY(cudaEventRecord(d.hp_ready, st));
    CU_TRY(cudaStreamWaitEvent(g_ctx.copy_stream, d.hp_ready, 0));
    if (hH) CU_TRY(cudaMemcpy2DAsync(hH, col, d.Hp, ldb, col, n, cudaMemcpyDeviceToHost, g_ctx.copy_stream));
    const double tau_in[1] = {tau};
    const double dt = t_max - t_init;
    if (int rc = run_taylor(d.Hp, n, d.ld, d.tb, 1, tau_in, t_init, t_max, 1.0e-8, 1.0e-8, 10000, 1, 2, dt,
                            tau, nullptr, nullptr, 0))
        return rc;
    // AO_bra = S^-1 PSI_bra (Taylor_gpu.cpp:717-721), not conjugated
    if (hAO_bra) {
        if (int rc = d.fac.apply_sinv(d.tb.bra(0), d.ao, n)) return rc;
    }
    CU_TRY(cudaMemcpyAsync(hbra, d.tb.bra(0), n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaMemcpyAsync(hket, d.tb.ket(0), n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    if (hAO_bra) CU_TRY(cudaMemcpyAsync(hAO_bra, d.ao, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    std::vector<TaylorParticle> res;
    int rc = collect_taylor(d.tb, 1, res, nullptr);
    CU_TRY(cudaStreamSynchronize(g_ctx.copy_stream));
    if (int frc = d.fac.check_info()) return frc;
    if (save_tau) *save_tau = res[0].save_tau;
    return rc;
}

int dropin_single(int n, double tau, double *save_tau, double t_init, double t_max, elhl_zcomplex *hbra,
                  elhl_zcomplex *hket, const double *hH) {
    if (n <= 0 || !hH || !hbra || !hket) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (int rc = ensure_context_locked(-1)) return rc;
    if (int rc = g_drop.reserve(n)) return rc;
    DropIn &d = g_drop;
    cudaStream_t st = g_ctx.stream;
    const size_t col = n * sizeof(double), ldb = d.ld * sizeof(double);
    CU_TRY(cudaMemcpy2DAsync(d.Hp, ldb, hH, col, col, n, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(d.tb.bra(0), hbra, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(d.tb.ket(0), hket, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    const double tau_in[1] = {tau};
    if (int rc = run_taylor(d.Hp, n, d.ld, d.tb, 1, tau_in, t_init, t_max, 1.0e-8, 1.0e-8, 10000, 1, 2,
                            t_max - t_init, tau, nullptr, nullptr, 0))
        return rc;
    CU_TRY(cudaMemcpyAsync(hbra, d.tb.bra(0), n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaMemcpyAsync(hket, d.tb.ket(0), n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    std::vector<TaylorParticle> res;
    int rc = collect_taylor(d.tb, 1, res, nullptr);
    if (save_tau) *save_tau = res[0].save_tau;
    return rc;
}

#define BLAS_TRY(expr)                                                                \
    do {                                                                              \
        cublasStatus_t b_ = (expr);                                                   \
        if (b_ != CUBLAS_STATUS_SUCCESS) {                                            \
            fprintf(stderr, "elhlprop: %s failed: status %d\n", #expr, (int)b_);      \
            return ELHL_ERR_CUDA;                                                     \
        }                                                                             \
    } while (0)

// ---- Chebyshev state of one problem ------------------------------------------
// H~ = L^-1 h L^-T (FP64), its scaled copy Hs = (H~ - a)/b in the launch
// precision, the expansion coefficients and the column buffers.
template <typename T>
__global__ void scale_kernel(const double *__restrict__ Ht, T *__restrict__ Hs, int n, int ld, double a, double binv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= ld || j >= n) return;
    const double v = (i < n) ? (Ht[(size_t)j * ld + i] - (i == j ? a : 0.0)) * binv : 0.0;
    Hs[(size_t)j * ld + i] = (T)v;
}

// dcorr[i] = Hs_ii - (float) Hs_ii (rounded to FP32) for the FP32 Hs of
// scale_kernel: the diagonal (the on-site energies, the largest entries of Hs)
// is the part of the FP32 rounding that shifts every eigenvalue coherently, so
// the row kernel adds it back before each order's single rounding (in numpy
// replays with exact propagators over 200 steps of the trajectory mix, the FP32
// Hs moved populations by up to 9.6e-7, the FP32 off-diagonal with the exact
// diagonal by 6.7e-8 on the same member; on the GPU the served 512-member mix
// went from 1.36e-6 to 7.9e-7 at most against FP64)
__global__ void diag_corr_kernel(const double *__restrict__ Ht, float *__restrict__ dcorr, int n, int ld, double a,
                                 double binv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = (Ht[(size_t)i * ld + i] - a) * binv;
    dcorr[i] = (float)(v - (double)(float)v);
}

// pops[p*(nfrag+1) + f] = Re sum_{i in f} conj(psi_ip) bra_ip over column p of
// [ld][m] arrays; one block per particle, fixed-order tree reduction.
__global__ void populations_kernel(const double2 *__restrict__ psi, const double2 *__restrict__ bra, int n, int m,
                                   const int *__restrict__ ao_frag, int nfrag, double *__restrict__ pops) {
    __shared__ double red[kMaxFrag + 1][256];
    const int p = blockIdx.x;
    double acc[kMaxFrag + 1];
    for (int f = 0; f <= kMaxFrag; ++f) acc[f] = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 a = psi[(size_t)i * m + p], b = bra[(size_t)i * m + p];
        const double v = a.x * b.x + a.y * b.y;
        if (ao_frag) {
            const int f = ao_frag[i];
            if (f >= 0 && f < nfrag && f < kMaxFrag) acc[f] += v;
        }
        acc[kMaxFrag] += v;
    }
    for (int f = 0; f <= kMaxFrag; ++f) red[f][threadIdx.x] = acc[f];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int f = 0; f <= kMaxFrag; ++f) red[f][threadIdx.x] += red[f][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int f = 0; f < nfrag && f < kMaxFrag; ++f) pops[(size_t)p * (nfrag + 1) + f] = red[f][0];
        pops[(size_t)p * (nfrag + 1) + nfrag] = red[kMaxFrag][0];
    }
}

// After a reduced-precision step: scale particle p's propagated columns (ket
// column p and, when bra columns are carried, column P + p) so that its total
// population returns to the target (FP64 norm control).
__global__ void renormalize_kernel(double2 *cols, int n, int m, int P, const double *pops, int nfrag,
                                   const double *target) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int p = 0; p < P; ++p) {
        const double tot = pops[(size_t)p * (nfrag + 1) + nfrag];
        const double s = (tot > 0.0 && target[p] > 0.0) ? sqrt(target[p] / tot) : 1.0;
        double2 a = cols[(size_t)i * m + p];
        cols[(size_t)i * m + p] = make_double2(a.x * s, a.y * s);
        if (m == 2 * P) {
            double2 b = cols[(size_t)i * m + P + p];
            cols[(size_t)i * m + P + p] = make_double2(b.x * s, b.y * s);
        }
    }
}

// 8-byte storage per real element: FP64, or a DF64 (hi, lo) pair of FP32
constexpr int kLzPart = 1024;  // per-CTA partial sums of the Lanczos launch: 2 per SM, up to 512 SMs
inline bool wide_storage(int prec) { return prec == ELHL_PREC_FP64 || prec == ELHL_PREC_DF64; }
// reduced precision: renormalised every step, GEMM regime possible
inline bool reduced_precision(int prec) { return prec == ELHL_PREC_FP32 || prec == ELHL_PREC_BF16X3; }

// x -> (hi, lo) FP32 pair (DF64 storage), zero rows >= n
__global__ void split_df_kernel(const double *__restrict__ src, float2 *__restrict__ dst, int n, int ld, double a,
                                double binv, bool transpose_lower) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= ld || j >= n) return;
    double v = 0.0;
    if (i < n) {
        if (transpose_lower) v = (j >= i) ? src[(size_t)i * ld + j] : 0.0;  // dst(i, j) = src(j, i), j >= i
        else v = (src[(size_t)j * ld + i] - (i == j ? a : 0.0)) * binv;
    }
    const float h = __double2float_rn(v);
    dst[(size_t)j * ld + i] = make_float2(h, __double2float_rn(v - (double)h));
}

// Resources of ELHL_PREC_OZ64 (ozaki.cu): the BF16 slices of Hs with their row
// scales, the FP64 series vectors in [ld][8] rows, their sliced copies, the
// block schedule and the launch's partial tiles and counters.
struct OzRes {
    int N = 0, ld = 0, ntiles = 0, grid = 0;
    __nv_bfloat16 *s = nullptr;   // [slices][N][ld]
    double *r = nullptr;          // [tiles * 128] row scales (0 past N)
    double *v = nullptr, *part = nullptr;
    unsigned char *xs = nullptr;  // [3][2 tiles] sliced vectors (oz_vector_tile_bytes each)
    int *xe = nullptr;            // [3][2 tiles][8] their scale exponents, then [3][8] column maxima
    unsigned *cnt = nullptr;
    OzSeg *segs = nullptr;
    int *begin = nullptr, *base = nullptr, *count = nullptr;
    size_t xs_bytes() const { return (size_t)3 * 2 * ntiles * oz_vector_tile_bytes(); }
    int init(int N_, int ld_, int grid_) {
        N = N_;
        ld = ld_;
        grid = grid_;
        ntiles = (N + oz_tile_rows() - 1) / oz_tile_rows();
        if (int rc = dev_alloc(&v, (size_t)3 * ld * 8)) return rc;
        CU_TRY(cudaMemset(v, 0, (size_t)3 * ld * 8 * sizeof(double)));
        CU_TRY(cudaMalloc(&xs, xs_bytes()));
        CU_TRY(cudaMemset(xs, 0, xs_bytes()));  // the zero slots of every tile stay zero
        if (int rc = dev_alloc(&xe, (size_t)3 * 2 * ntiles * 8 + 3 * 8)) return rc;
        CU_TRY(cudaMalloc(&cnt, (size_t)ntiles * sizeof(unsigned)));
        std::vector<OzSeg> sg;
        std::vector<int> b, pb, pc;
        oz_schedule(N, grid, sg, b, pb, pc);
        CU_TRY(cudaMalloc(&segs, std::max<size_t>(sg.size(), 1) * sizeof(OzSeg)));
        if (int rc = dev_alloc(&begin, b.size())) return rc;
        if (int rc = dev_alloc(&base, pb.size())) return rc;
        if (int rc = dev_alloc(&count, pc.size())) return rc;
        if (!sg.empty()) CU_TRY(copy_h2d(segs, sg.data(), sg.size() * sizeof(OzSeg)));
        CU_TRY(copy_h2d(begin, b.data(), b.size() * sizeof(int)));
        CU_TRY(copy_h2d(base, pb.data(), pb.size() * sizeof(int)));
        CU_TRY(copy_h2d(count, pc.data(), pc.size() * sizeof(int)));
        return dev_alloc(&part, std::max<size_t>(sg.size(), 1) * oz_tile_rows() * 16);  // 128-bit partials
    }
    // slices and row scales of Hs (FP64), allocated on first use
    int slice(const double *Hs, cudaStream_t st) {
        if (!s) {
            CU_TRY(cudaMalloc(&s, (size_t)oz_slices() * N * ld * sizeof(__nv_bfloat16)));
            const size_t nr = (size_t)ntiles * oz_tile_rows();
            if (int rc = dev_alloc(&r, nr)) return rc;
            CU_TRY(cudaMemset(r, 0, nr * sizeof(double)));  // rows past N: scale 0
        }
        CU_TRY(oz_slice_matrix(Hs, N, ld, s, r, st));
        return ELHL_OK;
    }
    void release() {
        if (s) cudaFree(s);
        if (segs) cudaFree(segs);
        if (xs) cudaFree(xs);
        if (cnt) cudaFree(cnt);
        s = nullptr;
        segs = nullptr;
        xs = nullptr;
        cnt = nullptr;
        dev_free(r); dev_free(begin); dev_free(base); dev_free(count);
        dev_free(v); dev_free(xe); dev_free(part);
    }
};

struct ChebState {
    int N = 0, ld = 0, m = 0, precision = ELHL_PREC_FP64, K = 0;
    int parity = 0;            // phi/acc role of col[0], col[1] for the device read-out path
    void *A = nullptr, *B = nullptr;   // L^-1, L^T in the launch precision (fixed nuclei read-out)
    bool readout_ready = false, cols_current = false;
    double *scale = nullptr;   // [P] pending renormalisation factor (reduced precision), 1 otherwise
    double *drift = nullptr;   // norm drift word of the GEMM-regime step (plans keep their own)
    double *ntot = nullptr;    // [kMaxCols] FP64 totals of the last step's columns (renormalisation)
    double2 *saved = nullptr;  // [ld][m] input columns at the start of a call, for redone steps
    double guard = 0.01;       // Lanczos interval guard, fraction of the width
    OzRes *oz = nullptr;       // ELHL_PREC_OZ64: operator products on the tensor cores (FP64 otherwise)
    bool ro64 = false;         // read-out matrices A, B in FP64 (else the launch precision)
    size_t ab_tsz = 0;         // element size A and B were allocated with
    // read-out outputs, owned by the trajectory
    int P = 0, nfrag = 0;
    double2 *psi_out = nullptr, *bra_out = nullptr;
    const int *ao_frag = nullptr;
    double *target = nullptr;
    double2 *cin() { return parity ? acc : phi; }
    // GEMM regime (many columns, FP32): tensor-core GEMMs per order, one CUDA graph per step parity
    bool gemm = false;
    float *Y = nullptr;        // [ld][m] complex (2m x ld real), GEMM output
    float *Vf = nullptr;       // [ld][m] complex FP32 copy of the propagated columns (read-out input)
    double *gpops = nullptr;   // [P][nfrag+1] populations of the last step
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    long long graph_kernels = 0;  // kernels of this library in one step graph
    // BF16X3 on the hand-written tcgen05 GEMM: Hs and the order's block split in three BF16 terms
    bool umma = false;
    int usplits = 1;           // K split of the tensor-core GEMM (partial tiles in Y)
    __nv_bfloat16 *hsplit[3] = {nullptr, nullptr, nullptr};  // N rows of ld (Hs symmetric: row = column)
    __nv_bfloat16 *vsplit[3] = {nullptr, nullptr, nullptr};  // 2m rows of ld (K-major block)
    double *Ht = nullptr;    // FP64 H~
    void *Hs = nullptr;      // scaled, launch precision
    void *vbuf = nullptr;
    double2 *phi = nullptr, *acc = nullptr;  // [ld][m]
    double2 *coef = nullptr;
    int coef_cap = 0;
    double emin = 0.0, emax = 0.0, a = 0.0, b = 1.0;
    double2 c0{1.0, 0.0};    // host copy of the order-0 coefficient
    double *lz = nullptr;    // Lanczos vectors [6][ld], partial sums [kLzPart], record [128]
    float *dcorr = nullptr;  // explicit FP32 Hs: [ld] the rounding residual of its diagonal
    // implicit operator (geometry changing every step): Ht holds G = L^-1 in FP64,
    // Hs = h/b, A = G and Gt = G^T in the launch precision; no H~ is formed
    bool implicit = false;
    void *Gt = nullptr;
    void *wb = nullptr;      // [2][ld][m] launch precision (phase intermediates)
    // FP64 L^T and G^T for the column transforms of the implicit operator: B and
    // Gt on the FP64 path, own copies in the other precisions
    double *Lt64 = nullptr, *Gt64 = nullptr;
    const double *lt64() const { return precision == ELHL_PREC_FP64 ? static_cast<const double *>(B) : Lt64; }
    const double *gt64() const { return precision == ELHL_PREC_FP64 ? static_cast<const double *>(Gt) : Gt64; }
    double *cscratch = nullptr;  // [2m][ld] column-transform output
    int alloc(int N_, int m_, int prec) {
        N = N_;
        ld = round_up(N, 32);
        m = m_;
        precision = prec;
        const size_t tsz = wide_storage(prec) ? sizeof(double) : sizeof(float);
        if (int rc = dev_alloc(&Ht, (size_t)ld * N)) return rc;
        CU_TRY(cudaMalloc(&Hs, (size_t)ld * N * tsz));
        CU_TRY(cudaMalloc(&vbuf, (size_t)3 * ld * m * 2 * tsz));
        CU_TRY(cudaMemset(vbuf, 0, (size_t)3 * ld * m * 2 * tsz));
        if (int rc = dev_alloc(&phi, (size_t)ld * m)) return rc;
        if (int rc = dev_alloc(&acc, (size_t)ld * m)) return rc;
        CU_TRY(cudaMemset(phi, 0, (size_t)ld * m * sizeof(double2)));
        CU_TRY(cudaMemset(acc, 0, (size_t)ld * m * sizeof(double2)));
        // 6 Lanczos vectors, per-CTA partial sums, the tridiagonal record
        if (int rc = dev_alloc(&lz, (size_t)6 * ld + kLzPart + 128)) return rc;
        if (int rc = dev_alloc(&cscratch, (size_t)2 * m * ld)) return rc;
        if (int rc = dev_alloc(&scale, (size_t)kMaxCols)) return rc;
        if (int rc = dev_alloc(&drift, 1)) return rc;
        if (int rc = dev_alloc(&ntot, (size_t)kMaxCols)) return rc;
        CU_TRY(cudaMemset(drift, 0, sizeof(double)));
        std::vector<double> ones(kMaxCols, 1.0);
        CU_TRY(copy_h2d(scale, ones.data(), kMaxCols * sizeof(double)));
        return ELHL_OK;
    }
    void release() {
        for (auto &g : graph) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
        if (Y) cudaFree(Y);
        if (Vf) cudaFree(Vf);
        Y = Vf = nullptr;
        for (int t = 0; t < 3; ++t) {
            if (hsplit[t]) cudaFree(hsplit[t]);
            if (vsplit[t]) cudaFree(vsplit[t]);
            hsplit[t] = vsplit[t] = nullptr;
        }
        umma = false;
        if (oz) {
            oz->release();
            delete oz;
            oz = nullptr;
        }
        if (Gt) cudaFree(Gt);
        if (wb) cudaFree(wb);
        Gt = wb = nullptr;
        dev_free(Lt64);
        dev_free(Gt64);
        dev_free(cscratch);
        implicit = false;
        dev_free(gpops);
        dev_free(Ht); dev_free(phi); dev_free(acc); dev_free(coef); dev_free(lz); dev_free(scale);
        dev_free(drift); dev_free(saved); dev_free(ntot);
        if (dcorr) cudaFree(dcorr);
        dcorr = nullptr;
        if (Hs) cudaFree(Hs);
        if (vbuf) cudaFree(vbuf);
        if (A) cudaFree(A);
        if (B) cudaFree(B);
        Hs = vbuf = A = B = nullptr;
        coef_cap = 0;
        readout_ready = false;
    }
};

// A(j, i) = A(i, j) for i > j: the upper triangle from the lower one
__global__ void mirror_lower_kernel(double *A, int n, int ld) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i < n && j < n && i > j) A[(size_t)i * ld + j] = A[(size_t)j * ld + i];
}

// H~ = G h G^T with G = L^-1 (lower, zero upper triangle): W = G h, then the
// lower triangle of W G^T (symmetric result, N^3 + N^3/2 flops), mirrored.
// tc: products of 320 or more rows on the tensor cores from exact slices.
int form_htilde(ChebState &cs, const double *G, const double *h, int ld, double *W, bool tc) {
    cudaStream_t st = g_ctx.stream;
    const int n = cs.N;
    CU_TRY(fgemm(tc, n, n, n, 1.0, G, ld, false, h, ld, false, 0.0, W, ld, st, kTriA));
    CU_TRY(fgemm(tc, n, n, n, 1.0, W, ld, false, G, ld, true, 0.0, cs.Ht, cs.ld, st, kTriBt | kTriLowerC));
    mirror_lower_kernel<<<dim3((n + 127) / 128, n), 128, 0, st>>>(cs.Ht, n, cs.ld);
    count_launch();
    CU_TRY(cudaGetLastError());
    return ELHL_OK;
}

// Lanczos steps of the spectral bounds: a fixed-nuclei set-up runs once per
// trajectory and every step propagates on its interval, so it takes 40; a
// moving-nuclei rebuild runs every step and takes 20 (N = 3720: 0.9 ms less per
// step for 0.7 % more Chebyshev orders than 40; 16 steps gave 1.2 % more).
constexpr int kLanczosFixed = 40, kLanczosMoving = 20;

// Spectral bounds of H~ by Lanczos (k steps, no reorthogonalisation) with a
// guard of |beta_k s_k| + cs.guard of the width around the extreme Ritz
// values, in FP64 on the device in one cooperative launch (lanczos.cu):
// h == nullptr: H~ is cs.Ht (both triangles stored); otherwise H~ = G h G^T
// with G = L^-1 in cs.Ht (zero upper triangle) and its transpose Gt (FP64).
// The tridiagonal matrix is read back once.
int lanczos_bounds(ChebState &cs, int ksteps, const double *h = nullptr, const double *Gt = nullptr) {
    const int n = cs.N, ld = cs.ld;
    cudaStream_t st = g_ctx.stream;
    const int k = std::min(std::min(ksteps, n), 63);
    double *part = cs.lz + 6 * ld, *rec = part + kLzPart;  // rec: [2k + 1] <= 127 doubles
    if (h && !Gt) return ELHL_ERR_BAD_ARG;
    CU_TRY(cudaMemsetAsync(rec, 0, (2 * k + 1) * sizeof(double), st));
    CU_TRY(cudaMemsetAsync(g_ctx.err, 0, sizeof(int), st));
    CU_TRY(launch_lanczos64(n, ld, k, h ? h : cs.Ht, h ? cs.Ht : nullptr, Gt, cs.lz, cs.lz + 4 * ld, part, kLzPart,
                            rec, g_ctx.bar, g_ctx.err, st));
    int err = 0;
    CU_TRY(copy_d2h(&err, g_ctx.err, sizeof(int)));
    if (err) return err;
    std::vector<double> r(2 * k + 1);
    CU_TRY(copy_d2h(r.data(), rec, r.size() * sizeof(double)));
    const int used = r[2 * k] > 0.0 ? (int)r[2 * k] : k;
    const double *alpha = r.data(), *beta = r.data() + k;
    double lo = 0.0, hi = 0.0;
    tridiagonal_extremes(alpha, beta, used, &lo, &hi);
    const double bk = beta[used - 1];
    const double rlo = bk * tridiagonal_last_component(alpha, beta, used, lo);
    const double rhi = bk * tridiagonal_last_component(alpha, beta, used, hi);
    const double width = hi - lo;
    cs.emin = lo - rlo - cs.guard * width;
    cs.emax = hi + rhi + cs.guard * width;
    if (!(cs.emax > cs.emin) || !std::isfinite(cs.emin) || !std::isfinite(cs.emax)) return ELHL_ERR_NO_CONVERGENCE;
    return ELHL_OK;
}

// Hs and the coefficients for step dt on the current bounds.  Explicit:
// Hs = (H~ - a)/b from cs.Ht; implicit (h given): Hs = h/b, the shift a/b is
// applied by the kernel.
int cheb_prepare(ChebState &cs, double dt, double tol, const double *h = nullptr) {
    cudaStream_t st = g_ctx.stream;
    cs.a = 0.5 * (cs.emax + cs.emin);
    cs.b = 0.5 * (cs.emax - cs.emin);
    const double binv = 1.0 / cs.b;
    dim3 grid((cs.ld + 127) / 128, cs.N);
    const double *src = h ? h : cs.Ht;
    const double a = h ? 0.0 : cs.a;
    if (cs.precision == ELHL_PREC_DF64) {
        split_df_kernel<<<grid, 128, 0, st>>>(src, (float2 *)cs.Hs, cs.N, cs.ld, a, binv, false);
        count_launch();
    } else if (cs.precision == ELHL_PREC_FP64) {
        scale_kernel<double><<<grid, 128, 0, st>>>(src, (double *)cs.Hs, cs.N, cs.ld, a, binv);
        count_launch();
    } else {
        scale_kernel<float><<<grid, 128, 0, st>>>(src, (float *)cs.Hs, cs.N, cs.ld, a, binv);
        count_launch();
        if (!h) {  // explicit FP32 Hs: the FP64 correction of its diagonal
            if (!cs.dcorr) CU_TRY(cudaMalloc(&cs.dcorr, (size_t)cs.ld * sizeof(float)));
            diag_corr_kernel<<<(cs.N + 255) / 256, 256, 0, st>>>(src, cs.dcorr, cs.N, cs.ld, a, binv);
            count_launch();
        }
    }
    CU_TRY(cudaGetLastError());
    std::vector<double> cre, cim;
    int K = 0;
    if (int rc = chebyshev_coefficients(dt, cs.emin, cs.emax, tol, 20000, cre, cim, &K)) return rc;
    if (K + 1 > cs.coef_cap) {
        dev_free(cs.coef);
        if (int rc = dev_alloc(&cs.coef, (size_t)K + 1)) return rc;
        cs.coef_cap = K + 1;
    }
    std::vector<double2> c(K + 1);
    for (int k = 0; k <= K; ++k) c[k] = make_double2(cre[k], cim[k]);
    cs.c0 = c[0];
    for (auto &g : cs.graph) {  // recorded with the old coefficients
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
    CU_TRY(cudaMemcpyAsync(cs.coef, c.data(), (K + 1) * sizeof(double2), cudaMemcpyHostToDevice, st));
    CU_TRY(cudaStreamSynchronize(st));  // c is a host temporary
    cs.K = K;
    if (cs.oz)  // the tensor-core propagation reads Hs as BF16 slices
        if (int rc = cs.oz->slice(static_cast<const double *>(cs.Hs), st)) return rc;
    if (cs.umma && !h) {  // the tensor-core GEMM reads Hs as three BF16 terms
        if (int rc = split3_bf16(reinterpret_cast<const float *>(cs.Hs), cs.N, cs.N, cs.ld, cs.hsplit, cs.ld, false, st))
            return rc;
    }
    return ELHL_OK;
}

// dst(i, j) = src(j, i) if transpose else src(i, j), in T, keeping only the
// lower triangle of src (the factorisations leave the other triangle undefined); rows >= n are zero
template <typename T>
__global__ void convert_kernel(const double *__restrict__ src, T *__restrict__ dst, int n, int ld, bool transpose) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= ld || j >= n) return;
    double v = 0.0;
    if (i < n) {
        if (transpose) v = (j >= i) ? src[(size_t)i * ld + j] : 0.0;  // src(j, i), j >= i
        else v = (i >= j) ? src[(size_t)j * ld + i] : 0.0;            // src(i, j), i >= j
    }
    dst[(size_t)j * ld + i] = (T)v;
}

// Read-out matrices in FP64 for the reduced precisions too: the populations
// of an FP32 read-out carry about 1e-7 of noise (up to 1e-6 on some members of
// the 512-trajectory mix), while the FP32 propagation itself stays within 5e-8
// of FP64 over 200 steps.  Exceptions: the GEMM regime, whose read-out is two
// tensor-core GEMMs of the FP32 block, and bases whose FP64 vector would not fit
// in shared memory for the read-out kernel.
bool gemm_eligible(const ChebState &cs) {
    return reduced_precision(cs.precision) && cs.m == cs.P && cs.P >= kGemmMinCols && cs.N >= kGemmMinN;
}
bool readout_fp64(const ChebState &cs) {
    if (cs.precision == ELHL_PREC_FP64) return true;
    return reduced_precision(cs.precision) && !gemm_eligible(cs) && cheb_group_size(ELHL_PREC_FP64, 1, cs.ld) > 0;
}

// A = L^-1 and B = L^T for the device read-out of fixed nuclei, in FP64
// (readout_fp64) or the launch precision.  L and G = L^-1 both FP64 with zero
// upper triangles.
int cheb_prepare_readout(ChebState &cs, const double *Lfac, const double *G) {
    cudaStream_t st = g_ctx.stream;
    const int n = cs.N, ld = cs.ld;
    const bool wide = readout_fp64(cs);
    const size_t tsz = wide ? sizeof(double) : sizeof(float);
    if (cs.A && cs.ab_tsz != tsz) {  // allocated by the implicit operator in the launch precision
        cudaFree(cs.A);
        cudaFree(cs.B);
        cs.A = cs.B = nullptr;
    }
    if (!cs.A) CU_TRY(cudaMalloc(&cs.A, (size_t)ld * n * tsz));
    if (!cs.B) CU_TRY(cudaMalloc(&cs.B, (size_t)ld * n * tsz));
    cs.ab_tsz = tsz;
    cs.ro64 = wide;
    dim3 grid((ld + 127) / 128, n);
    if (wide) {
        convert_kernel<double><<<grid, 128, 0, st>>>(G, (double *)cs.A, n, ld, false);
        count_launch();
        convert_kernel<double><<<grid, 128, 0, st>>>(Lfac, (double *)cs.B, n, ld, true);
        count_launch();
    } else {
        convert_kernel<float><<<grid, 128, 0, st>>>(G, (float *)cs.A, n, ld, false);
        count_launch();
        convert_kernel<float><<<grid, 128, 0, st>>>(Lfac, (float *)cs.B, n, ld, true);
        count_launch();
    }
    CU_TRY(cudaGetLastError());
    CU_TRY(cudaStreamSynchronize(st));
    cs.readout_ready = true;
    return ELHL_OK;
}

// Implicit operator for the current factor and h: G = L^-1 (FP64, in cs.Ht,
// formed with L at N^3/3 flops instead of the 2 N^3 of forming H~), bounds by
// Lanczos on G h G^T, Hs = h/b, and A = G, Gt = G^T, B = L^T in the launch
// precision.
int cheb_prepare_implicit(ChebState &cs, const double *Lfac, const double *h, double dt, double tol) {
    cudaStream_t st = g_ctx.stream;
    const int n = cs.N, ld = cs.ld;
    const size_t tsz = wide_storage(cs.precision) ? sizeof(double) : sizeof(float);
    if (cs.A && cs.ab_tsz != tsz) {  // FP64 read-out matrices of an earlier fixed-nuclei set-up
        cudaFree(cs.A);
        cudaFree(cs.B);
        cs.A = cs.B = nullptr;
    }
    if (!cs.A) CU_TRY(cudaMalloc(&cs.A, (size_t)ld * n * tsz));
    if (!cs.B) CU_TRY(cudaMalloc(&cs.B, (size_t)ld * n * tsz));
    cs.ab_tsz = tsz;
    cs.ro64 = cs.precision == ELHL_PREC_FP64;
    if (!cs.Gt) CU_TRY(cudaMalloc(&cs.Gt, (size_t)ld * n * tsz));
    if (!cs.wb) {
        CU_TRY(cudaMalloc(&cs.wb, (size_t)2 * ld * cs.m * 2 * tsz));
        CU_TRY(cudaMemset(cs.wb, 0, (size_t)2 * ld * cs.m * 2 * tsz));
    }
    // L with a zero upper triangle (the recursion leaves S's there): the dense column transforms read all of it
    lower_only_kernel<<<dim3((ld + 127) / 128, n), 128, 0, st>>>(const_cast<double *>(Lfac), n, ld);
    count_launch();
    CU_TRY(cudaGetLastError());
    CU_TRY(cudaEventRecord(g_ctx.ev[6], st));
    lower_only_kernel<<<dim3((ld + 127) / 128, n), 128, 0, st>>>(cs.Ht, n, ld);
    count_launch();
    CU_TRY(cudaGetLastError());
    dim3 grid((ld + 127) / 128, n);
    // FP64 G^T: the bounds' G (.) products, then the column transforms (and the
    // FP64 propagation); FP64 L^T for the transforms of the other precisions
    if (cs.precision != ELHL_PREC_FP64) {
        if (!cs.Lt64)
            if (int rc = dev_alloc(&cs.Lt64, (size_t)ld * n)) return rc;
        if (!cs.Gt64)
            if (int rc = dev_alloc(&cs.Gt64, (size_t)ld * n)) return rc;
        convert_kernel<double><<<grid, 128, 0, st>>>(Lfac, cs.Lt64, n, ld, true);
        count_launch();
    }
    convert_kernel<double><<<grid, 128, 0, st>>>(cs.Ht, const_cast<double *>(cs.gt64()), n, ld, true);
    count_launch();
    CU_TRY(cudaGetLastError());
    if (int rc = lanczos_bounds(cs, kLanczosMoving, h, cs.gt64())) return rc;
    if (int rc = cheb_prepare(cs, dt, tol, h)) return rc;
    if (cs.precision == ELHL_PREC_DF64) {  // G and G^T as (hi, lo) pairs; no device read-out matrices
        split_df_kernel<<<grid, 128, 0, st>>>(cs.Ht, (float2 *)cs.A, n, ld, 0.0, 1.0, false);
        count_launch();
        split_df_kernel<<<grid, 128, 0, st>>>(cs.Ht, (float2 *)cs.Gt, n, ld, 0.0, 1.0, true);
        count_launch();
        CU_TRY(cudaGetLastError());
        cs.implicit = true;
        cs.readout_ready = false;  // read-out through the FP64 dense transforms
        return ELHL_OK;
    }
    if (cs.precision == ELHL_PREC_FP64) {  // G^T (cs.Gt) is in place already
        convert_kernel<double><<<grid, 128, 0, st>>>(cs.Ht, (double *)cs.A, n, ld, false);
        count_launch();
        convert_kernel<double><<<grid, 128, 0, st>>>(Lfac, (double *)cs.B, n, ld, true);
        count_launch();
    } else {
        convert_kernel<float><<<grid, 128, 0, st>>>(cs.Ht, (float *)cs.A, n, ld, false);
        count_launch();
        convert_kernel<float><<<grid, 128, 0, st>>>(cs.Ht, (float *)cs.Gt, n, ld, true);
        count_launch();
        convert_kernel<float><<<grid, 128, 0, st>>>(Lfac, (float *)cs.B, n, ld, true);
        count_launch();
    }
    CU_TRY(cudaGetLastError());
    cs.implicit = true;
    cs.readout_ready = true;
    return ELHL_OK;
}

// ---- norm control ------------------------------------------------------------
// In the symmetrised basis the exact step exp(-i H~ dt / hbar) is unitary, so
// each propagated column keeps its squared norm.  For column c: n_in = s^2
// |col_in|^2 (s: the pending renormalisation factor applied to the input, 1
// without) and n_out = |col_out|^2 before any renormalisation; the relative
// drift |n_out / n_in - 1| is the counterpart of the Taylor path's test
// |<bra|ket>| - norm_ref (Taylor.f:103-104).  One block of kDriftBlock threads
// per column, fixed-order FP64 sums; the largest drift is kept in *drift by an
// integer max on the bits of the non-negative double (exact, independent of
// the order in which blocks finish).  A non-finite norm counts as 1e300.
constexpr int kDriftBlock = 256;

__device__ void drift_column(const double2 *__restrict__ in, const double2 *__restrict__ out, int n, int m, int c,
                             double s2, double *drift) {
    __shared__ double ra[kDriftBlock], rb[kDriftBlock];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += kDriftBlock) {
        const double2 x = in[(size_t)i * m + c], y = out[(size_t)i * m + c];
        a += x.x * x.x + x.y * x.y;
        b += y.x * y.x + y.y * y.y;
    }
    ra[threadIdx.x] = a;
    rb[threadIdx.x] = b;
    __syncthreads();
    for (int o = kDriftBlock / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            ra[threadIdx.x] += ra[threadIdx.x + o];
            rb[threadIdx.x] += rb[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double nin = ra[0] * s2, nout = rb[0];
        double d = nin > 0.0 ? fabs(nout / nin - 1.0) : (nout > 0.0 ? 1.0e300 : 0.0);
        if (!(d <= 1.0e300)) d = 1.0e300;
        atomicMax(reinterpret_cast<unsigned long long *>(drift), (unsigned long long)__double_as_longlong(d));
    }
}

// every problem of a plan after a propagation launch of this parity (block (q, c))
__global__ void __launch_bounds__(kDriftBlock) norm_drift_kernel(const ChebProblem *probs, int parity) {
    const ChebProblem &pb = probs[blockIdx.x];
    const int c = blockIdx.y;
    if (!pb.drift || c >= pb.m) return;
    const double s = pb.scale ? pb.scale[c % pb.P] : 1.0;
    drift_column(pb.col[parity], pb.col[parity ^ 1], pb.N, pb.m, c, s * s, pb.drift);
}

// one problem's columns (GEMM regime), block c
__global__ void __launch_bounds__(kDriftBlock) norm_drift_cols_kernel(const double2 *in, const double2 *out, int n,
                                                                      int m, int P, const double *scale, double *drift) {
    const int c = blockIdx.x;
    const double s = scale ? scale[c % P] : 1.0;
    drift_column(in, out, n, m, c, s * s, drift);
}

// Total population of particle p after a step, in FP64 from the propagated
// columns of the symmetrised basis: |phi_p|^2 for ket-only problems (m = P),
// Re <phi_p|chi_p> with bra columns (m = 2P); one block per (problem, particle),
// fixed-order sums.
__device__ void total_column(const double2 *__restrict__ out, int n, int m, int P, int p, double *dst) {
    __shared__ double r[kDriftBlock];
    double a = 0.0;
    for (int i = threadIdx.x; i < n; i += kDriftBlock) {
        const double2 x = out[(size_t)i * m + p];
        const double2 y = m == 2 * P ? out[(size_t)i * m + P + p] : x;
        a += x.x * y.x + x.y * y.y;
    }
    r[threadIdx.x] = a;
    __syncthreads();
    for (int o = kDriftBlock / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) r[threadIdx.x] += r[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *dst = r[0];
}

__global__ void __launch_bounds__(kDriftBlock) norm_total_kernel(const ChebProblem *probs, int parity) {
    const ChebProblem &pb = probs[blockIdx.x];
    if (!pb.ntot || (int)blockIdx.y >= pb.P) return;
    total_column(pb.col[parity ^ 1], pb.N, pb.m, pb.P, blockIdx.y, pb.ntot + blockIdx.y);
}

__global__ void __launch_bounds__(kDriftBlock) norm_total_cols_kernel(const double2 *out, int n, int m, int P,
                                                                      double *ntot) {
    total_column(out, n, m, P, blockIdx.x, ntot + blockIdx.x);
}

// ---- GEMM regime kernels (complex columns [ld][m], element-wise) -------------
__global__ void gemm_order0_kernel(const double2 *__restrict__ phi, const double *__restrict__ scale, int P, int n,
                                   int m, double2 c0, float2 *__restrict__ v0, double2 *__restrict__ acc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n * m) return;
    double2 p = phi[q];
    const double sc = scale ? scale[(q % m) % P] : 1.0;
    p.x *= sc;
    p.y *= sc;
    v0[q] = make_float2((float)p.x, (float)p.y);
    acc[q] = make_double2(c0.x * p.x - c0.y * p.y, c0.x * p.y + c0.y * p.x);
}

// y = sum of the nsplit partial products (FP64, fixed order), v_k = 2 y - v_{k-2}
// (v_1 = y) rounded to FP32, acc += c_k v_k in FP64
__global__ void gemm_epilogue_kernel(const float2 *__restrict__ Y, int nsplit, size_t split_stride,
                                     const float2 *__restrict__ vprev2, float2 *__restrict__ vout,
                                     double2 *__restrict__ acc, const double2 *coef, int k, int nm) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nm) return;
    double yx = 0.0, yy = 0.0;
    for (int s = 0; s < nsplit; ++s) {
        const float2 t = Y[s * split_stride + q];
        yx += (double)t.x;
        yy += (double)t.y;
    }
    float2 v;
    if (k == 1) {
        v = make_float2((float)yx, (float)yy);
    } else {
        const float2 w = vprev2[q];
        v = make_float2((float)(2.0 * yx - (double)w.x), (float)(2.0 * yy - (double)w.y));
    }
    vout[q] = v;
    const double2 c = coef[k];
    double2 a = acc[q];
    a.x += c.x * (double)v.x - c.y * (double)v.y;
    a.y += c.x * (double)v.y + c.y * (double)v.x;
    acc[q] = a;
}

__global__ void to_float2_kernel(const double2 *__restrict__ src, float2 *__restrict__ dst, int nm) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nm) dst[q] = make_float2((float)src[q].x, (float)src[q].y);
}

__global__ void to_double2_kernel(const float2 *__restrict__ src, double2 *__restrict__ dst, int nm) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nm) dst[q] = make_double2((double)src[q].x, (double)src[q].y);
}

// renormalisation factor s = sqrt(target / total) for the next step, the total
// in FP64 from the propagated columns (ntot); the populations become those of
// the renormalised state (each times s^2)
__global__ void scale_from_pops_kernel(double *pops, int P, int nfrag, const double *target, const double *ntot,
                                       double *scale) {
    const int p = threadIdx.x;
    if (p < P) {
        const double tot = ntot[p];
        const bool rn = tot > 0.0 && target[p] > 0.0;
        scale[p] = rn ? sqrt(target[p] / tot) : 1.0;
        if (rn)
            for (int f = 0; f <= nfrag; ++f) pops[(size_t)p * (nfrag + 1) + f] *= target[p] / tot;
    }
}

// Yt (2m x n) = Vt (2m x n, ld 2m) * M (n x n, ld), FP32 data.  ELHL_PREC_FP32:
// FP32 FMAs with round-to-nearest sums (PEDANTIC: no reduced-precision path);
// ELHL_PREC_BF16X3: tensor cores with each operand split in three BF16 terms.
int gemm_vt(cublasHandle_t h, int precision, int m2, int n, const float *Vt, const float *M, int ld, float *Yt) {
    const float one = 1.0f, zero = 0.0f;
    const cublasComputeType_t ct =
        precision == ELHL_PREC_BF16X3 ? CUBLAS_COMPUTE_32F_EMULATED_16BFX9 : CUBLAS_COMPUTE_32F_PEDANTIC;
    BLAS_TRY(cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, m2, n, n, &one, Vt, CUDA_R_32F, m2, M, CUDA_R_32F, ld, &zero,
                          Yt, CUDA_R_32F, m2, ct, CUBLAS_GEMM_DEFAULT));
    return ELHL_OK;
}

// Enqueue one GEMM-regime step (fixed nuclei, FP32, ket columns only) on the
// context stream: order 0, K x (tensor-core GEMM + recurrence epilogue), read-out
// GEMMs with A = L^-1 and B = L^T, populations into cs.gpops, renormalisation factor.
int cheb_gemm_enqueue(ChebState &cs, int parity) {
    cudaStream_t st = g_ctx.stream;
    const int n = cs.N, m = cs.m, nm = n * m, tb = 256, nb = (nm + tb - 1) / tb;
    float2 *vb = reinterpret_cast<float2 *>(cs.vbuf);
    const size_t vs = (size_t)cs.ld * m;
    const double2 *in = parity ? cs.acc : cs.phi;
    double2 *out = parity ? cs.phi : cs.acc;
    const bool renorm = true;
    gemm_order0_kernel<<<nb, tb, 0, st>>>(in, renorm ? cs.scale : nullptr, cs.P, n, m, cs.c0, vb, out);
    count_launch();
    for (int k = 1; k <= cs.K; ++k) {
        const float *vprev = reinterpret_cast<const float *>(vb + ((k + 2) % 3) * vs);
        if (cs.umma) {  // Y (N x 2m) = Hs V^T on the tensor cores (Hs symmetric), three BF16 terms each
            if (int rc = split3_bf16(vprev, n, 2 * m, 2 * m, cs.vsplit, cs.ld, true, st)) return rc;
            if (int rc = umma_bf16x3_gemm(cs.hsplit, cs.ld, cs.vsplit, cs.ld, n, n, 2 * m, cs.usplits, cs.Y,
                                          g_ctx.err, st))
                return rc;
        } else if (int rc = gemm_vt(g_ctx.blas_tc, cs.precision, 2 * m, n, vprev,
                                    reinterpret_cast<const float *>(cs.Hs), cs.ld, cs.Y)) {
            return rc;
        }
        gemm_epilogue_kernel<<<nb, tb, 0, st>>>(reinterpret_cast<const float2 *>(cs.Y), cs.umma ? cs.usplits : 1,
                                                (size_t)n * m, vb + ((k + 1) % 3) * vs,
                                                vb + (k % 3) * vs, out, cs.coef, k, nm);
        count_launch();
    }
    norm_drift_cols_kernel<<<m, kDriftBlock, 0, st>>>(in, out, n, m, cs.P, renorm ? cs.scale : nullptr, cs.drift);
    count_launch();
    norm_total_cols_kernel<<<cs.P, kDriftBlock, 0, st>>>(out, n, m, cs.P, cs.ntot);
    count_launch();
    to_float2_kernel<<<nb, tb, 0, st>>>(out, reinterpret_cast<float2 *>(cs.Vf), nm);
    count_launch();
    if (int rc = gemm_vt(g_ctx.blas_tc, cs.precision, 2 * m, n, cs.Vf, reinterpret_cast<const float *>(cs.A), cs.ld,
                         cs.Y))
        return rc;
    to_double2_kernel<<<nb, tb, 0, st>>>(reinterpret_cast<const float2 *>(cs.Y), cs.psi_out, nm);
    count_launch();
    if (int rc = gemm_vt(g_ctx.blas_tc, cs.precision, 2 * m, n, cs.Vf, reinterpret_cast<const float *>(cs.B), cs.ld,
                         cs.Y))
        return rc;
    to_double2_kernel<<<nb, tb, 0, st>>>(reinterpret_cast<const float2 *>(cs.Y), cs.bra_out, nm);
    count_launch();
    populations_kernel<<<cs.P, 256, 0, st>>>(cs.psi_out, cs.bra_out, n, cs.P, cs.ao_frag, cs.nfrag, cs.gpops);
    count_launch();
    scale_from_pops_kernel<<<1, kMaxCols, 0, st>>>(cs.gpops, cs.P, cs.nfrag, cs.target, cs.ntot, cs.scale);
    count_launch();
    CU_TRY(cudaGetLastError());
    return ELHL_OK;
}

// one GEMM-regime step: replay the step graph of this parity (captured on first use)
int cheb_gemm_step(ChebState &cs) {
    cudaStream_t st = g_ctx.stream;
    cudaGraphExec_t &ge = cs.graph[cs.parity];
    if (!ge) {
        cudaGraph_t g = nullptr;
        CU_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const long long before = own_launches();
        int rc = cheb_gemm_enqueue(cs, cs.parity);
        cs.graph_kernels = own_launches() - before;  // recorded, not launched: counted at each replay
        count_launch(-cs.graph_kernels);
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        CU_TRY(e);
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        CU_TRY(e);
    }
    CU_TRY(cudaEventRecord(g_ctx.ev[0], st));
    CU_TRY(cudaGraphLaunch(ge, st));
    count_launch(cs.graph_kernels);
    CU_TRY(cudaEventRecord(g_ctx.ev[1], st));
    cs.parity ^= 1;
    return ELHL_OK;
}

// Launch plan for a set of problems: row segments balanced by matrix elements.
struct ChebPlan {
    std::vector<ChebProblem> probs;
    std::vector<ChebSegment> segs;
    std::vector<int> seg_begin;
    std::vector<int> prob_seg0;
    std::vector<ChebSegment> segs_full;  // implicit operator: even row split of the full phase
    std::vector<int> seg_full_begin;
    ChebProblem *d_probs = nullptr;
    ChebSegment *d_segs = nullptr, *d_segs_full = nullptr;
    int *d_seg_begin = nullptr, *d_prob_seg0 = nullptr, *d_seg_full_begin = nullptr;
    double *d_seg_pops = nullptr;
    double *d_drift = nullptr;  // [problem] norm drift of the steps since the last reset
    int grid = 0, max_ld = 0, kmax = 0, mg = 0, mg_read = 0, precision = 0, parity = 0;
    int ro_precision = 0;      // element type of the read-out matrices (FP64 or the launch precision)
    int nphase = 1;            // 3: one implicit problem
    int mgcd = 0;              // gcd of the problems' column counts
    bool tuned = false;        // tile measured (on the plan's first run)
    OzRes *oz = nullptr;       // one ELHL_PREC_OZ64 trajectory: the tensor-core propagation
    size_t pops_per_step = 0;  // populations of all problems in one step
    void release() {
        dev_free(d_probs); dev_free(d_segs); dev_free(d_seg_begin); dev_free(d_prob_seg0); dev_free(d_seg_pops);
        dev_free(d_drift); dev_free(d_segs_full); dev_free(d_seg_full_begin);
    }
};

int tune_plan(ChebPlan &pl, int mgcd);

int cheb_plan(ChebPlan &pl, const std::vector<ChebState *> &states) {
    pl.release();
    pl.probs.clear();
    pl.segs.clear();
    if (states.empty()) return ELHL_ERR_BAD_ARG;
    if (cheb_grid_size(&pl.grid)) return ELHL_ERR_CUDA;
    if (int rc = dev_alloc(&pl.d_drift, states.size())) return rc;
    CU_TRY(cudaMemsetAsync(pl.d_drift, 0, states.size() * sizeof(double), g_ctx.stream));
    pl.max_ld = 0;
    pl.kmax = 0;
    pl.precision = states[0]->precision;
    double work = 0.0;
    int mgcd = 0;  // staged group size must divide every problem's column count
    for (auto *cs : states) {
        if (cs->precision != pl.precision || cs->m <= 0) return ELHL_ERR_BAD_ARG;
        pl.max_ld = std::max(pl.max_ld, cs->ld);
        work += (double)cs->N * cs->ld;
        int a = cs->m, b = mgcd;
        while (b) { const int t = a % b; a = b; b = t; }
        mgcd = a;
    }
    const bool implicit_plan = states[0]->implicit;
    pl.mg = cheb_group_size(pl.precision, mgcd, pl.max_ld, !implicit_plan);
    if (!pl.mg) return ELHL_ERR_UNSUPPORTED;
    int pgcd = 0;  // read-out groups must divide every problem's ket columns
    for (auto *cs : states) {
        int a = std::max(cs->P, 1), b = pgcd;
        while (b) { const int t = a % b; a = b; b = t; }
        pgcd = a;
    }
    pl.ro_precision = states[0]->ro64 ? ELHL_PREC_FP64 : pl.precision;
    for (auto *cs : states)
        if (cs->readout_ready && cs->ro64 != states[0]->ro64) return ELHL_ERR_UNSUPPORTED;  // one read-out type
    pl.mg_read = cheb_group_size(pl.ro_precision, pgcd, pl.max_ld);
    pl.pops_per_step = 0;
    pl.parity = states[0]->parity;
    const bool implicit = states[0]->implicit;
    if (implicit && states.size() != 1) return ELHL_ERR_UNSUPPORTED;
    pl.nphase = implicit ? 3 : 1;
    for (auto *cs : states) {
        ChebProblem p{};
        p.N = cs->N; p.ld = cs->ld; p.ldv = cs->ld; p.m = cs->m; p.K = cs->K;
        p.H = cs->Hs; p.vbuf = cs->vbuf; p.col[0] = cs->phi; p.col[1] = cs->acc; p.coef = cs->coef;
        p.P = cs->P;
        const bool dev = cs->readout_ready && pl.mg_read;
        p.A = dev ? cs->A : nullptr;
        p.B = dev ? cs->B : nullptr;
        p.psi = cs->psi_out; p.bra = cs->bra_out; p.ao_frag = cs->ao_frag; p.nfrag = cs->nfrag;
        p.pops_off = (int)pl.pops_per_step;
        const bool renorm = dev && reduced_precision(cs->precision);
        p.scale = renorm ? cs->scale : nullptr;
        p.scale_out = renorm ? cs->scale : nullptr;
        p.target = renorm ? cs->target : nullptr;
        p.ntot = renorm ? cs->ntot : nullptr;
        if (cs->implicit) {
            p.G = cs->A;
            p.Gt = cs->Gt;
            p.wb = cs->wb;
            p.shift = cs->a / cs->b;
        } else if (reduced_precision(cs->precision)) {
            p.dcorr = cs->dcorr;
        }
        p.drift = pl.d_drift + pl.probs.size();
        pl.pops_per_step += (size_t)cs->P * (cs->nfrag + 1);
        pl.probs.push_back(p);
        pl.kmax = std::max(pl.kmax, cs->K);
        if (cs->parity != pl.parity) return ELHL_ERR_BAD_ARG;
    }
    pl.seg_begin.assign(pl.grid + 1, 0);
    pl.segs_full.clear();
    pl.seg_full_begin.clear();
    if (implicit) {
        // the full phase: CTA c owns rows [N c / grid, N (c + 1) / grid), 24 or 25 rows at N = 3720
        const int N = states[0]->N;
        pl.seg_full_begin.assign(pl.grid + 1, 0);
        for (int c = 0; c < pl.grid; ++c) {
            const int r0 = (int)((long long)N * c / pl.grid), r1 = (int)((long long)N * (c + 1) / pl.grid);
            if (r1 > r0) pl.segs_full.push_back({0, r0, r1});
            pl.seg_full_begin[c + 1] = (int)pl.segs_full.size();
        }
    }
    if (implicit) {
        // 2 x grid equal row chunks, CTA c owning chunks c and 2 grid - 1 - c: the
        // triangular phases (G^T: j >= i, G: j <= i) then cost every CTA the same
        const int N = states[0]->N, nch = 2 * pl.grid;
        for (int c = 0; c < pl.grid; ++c) {
            for (int q : {c, nch - 1 - c}) {
                const int r0 = (int)((long long)N * q / nch), r1 = (int)((long long)N * (q + 1) / nch);
                if (r1 > r0) pl.segs.push_back({0, r0, r1});
            }
            pl.seg_begin[c + 1] = (int)pl.segs.size();
        }
    }
    // greedy split of the concatenated rows: CTA c fills up to (c+1)/grid of the work
    const double per = work / pl.grid;
    int c = implicit ? pl.grid : 0;
    double acc_w = 0.0;
    for (int q = 0; q < (int)states.size() && !implicit; ++q) {
        const ChebState *cs = states[q];
        const double rw = cs->ld;  // work per row
        int r = 0;
        while (r < cs->N) {
            int take = cs->N - r;
            if (c < pl.grid - 1) {
                const double room = per * (c + 1) - acc_w;
                take = std::min(take, std::max(1, (int)std::floor(room / rw + 0.5)));
            }
            pl.segs.push_back({q, r, r + take});
            acc_w += take * rw;
            r += take;
            if (c < pl.grid - 1 && acc_w >= per * (c + 1) - 0.5 * rw) {
                ++c;
                pl.seg_begin[c] = (int)pl.segs.size();
            }
        }
    }
    if (!implicit)
        for (int cc = c + 1; cc <= pl.grid; ++cc) pl.seg_begin[cc] = (int)pl.segs.size();
    pl.prob_seg0.assign(states.size() + 1, 0);
    for (size_t i = 0; i < pl.segs.size(); ++i) pl.prob_seg0[pl.segs[i].prob + 1] = (int)i + 1;
    for (size_t q = 1; q <= states.size(); ++q) pl.prob_seg0[q] = std::max(pl.prob_seg0[q], pl.prob_seg0[q - 1]);
    if (int rc = dev_alloc(&pl.d_prob_seg0, pl.prob_seg0.size())) return rc;
    CU_TRY(copy_h2d(pl.d_prob_seg0, pl.prob_seg0.data(), pl.prob_seg0.size() * sizeof(int)));
    if (int rc = dev_alloc(&pl.d_seg_pops, pl.segs.size() * kMaxCols * (kMaxFrag + 1))) return rc;
    if (int rc = dev_alloc(&pl.d_probs, pl.probs.size())) return rc;
    if (int rc = dev_alloc(&pl.d_segs, pl.segs.size())) return rc;
    if (int rc = dev_alloc(&pl.d_seg_begin, pl.seg_begin.size())) return rc;
    CU_TRY(copy_h2d(pl.d_probs, pl.probs.data(), pl.probs.size() * sizeof(ChebProblem)));
    CU_TRY(copy_h2d(pl.d_segs, pl.segs.data(), pl.segs.size() * sizeof(ChebSegment)));
    CU_TRY(copy_h2d(pl.d_seg_begin, pl.seg_begin.data(), pl.seg_begin.size() * sizeof(int)));
    if (!pl.segs_full.empty()) {
        if (int rc = dev_alloc(&pl.d_segs_full, pl.segs_full.size())) return rc;
        if (int rc = dev_alloc(&pl.d_seg_full_begin, pl.seg_full_begin.size())) return rc;
        CU_TRY(copy_h2d(pl.d_segs_full, pl.segs_full.data(), pl.segs_full.size() * sizeof(ChebSegment)));
        CU_TRY(copy_h2d(pl.d_seg_full_begin, pl.seg_full_begin.data(), pl.seg_full_begin.size() * sizeof(int)));
    }
    pl.mgcd = mgcd;
    pl.tuned = false;  // measured on the first run (plans of batch members never run)
    pl.oz = states.size() == 1 ? states[0]->oz : nullptr;
    return ELHL_OK;
}

// refresh per-problem order counts and coefficient pointers after cheb_prepare
int cheb_plan_refresh(ChebPlan &pl, const std::vector<ChebState *> &states) {
    if (pl.nphase != (states[0]->implicit ? 3 : 1)) return cheb_plan(pl, states);  // operator form changed
    pl.kmax = 0;
    for (size_t q = 0; q < states.size(); ++q) {
        pl.probs[q].K = states[q]->K;
        pl.probs[q].coef = states[q]->coef;
        if (states[q]->implicit) pl.probs[q].shift = states[q]->a / states[q]->b;
        pl.kmax = std::max(pl.kmax, states[q]->K);
    }
    CU_TRY(copy_h2d(pl.d_probs, pl.probs.data(), pl.probs.size() * sizeof(ChebProblem)));
    return ELHL_OK;
}

ChebLaunch plan_launch(const ChebPlan &pl) {
    ChebLaunch L{};
    L.probs = pl.d_probs;
    L.segs = pl.d_segs;
    L.seg_begin = pl.d_seg_begin;
    L.kmax = pl.kmax;
    L.max_ld = pl.max_ld;
    L.grid = pl.grid;
    L.bar_count = g_ctx.bar;
    L.error = g_ctx.err;
    L.prob_seg0 = pl.d_prob_seg0;
    L.parity = pl.parity;
    L.seg_pops = pl.d_seg_pops;
    L.nphase = pl.nphase;
    L.segs_full = pl.d_segs_full;
    L.seg_full_begin = pl.d_seg_full_begin;
    return L;
}

// Autotuner of the propagation tile: the number of complex columns staged per
// pass over the matrix (4, 2 or 1 where it divides every problem's column count
// and fits in shared memory) sets the accumulator tile of every warp (row tile x
// columns) and the passes per order.  Each candidate runs the plan itself for
// up to 4 orders (twice; the second run is timed with CUDA events); the fastest
// is kept per (precision, column gcd, phases, padded size, total elements).  A
// trial only writes the output columns and recurrence buffers, which the next
// real launch overwrites.
std::map<std::tuple<int, int, int, int, int>, int> g_tile_cache;

int tune_plan(ChebPlan &pl, int mgcd) {
    std::vector<int> cand;
    for (int mg : {4, 2, 1})
        if (mgcd % mg == 0 && cheb_group_size(pl.precision, mg, pl.max_ld, pl.nphase == 1) == mg) cand.push_back(mg);
    if (cand.size() < 2 || pl.kmax < 1) return ELHL_OK;
    double elems = 0.0;
    for (const auto &p : pl.probs) elems += (double)p.N * p.ld;
    const auto key = std::make_tuple(pl.precision, mgcd, pl.nphase, (pl.max_ld + 255) / 256, (int)std::log2(elems + 1));
    auto it = g_tile_cache.find(key);
    if (it != g_tile_cache.end()) {
        pl.mg = it->second;
        return ELHL_OK;
    }
    cudaStream_t st = g_ctx.stream;
    ChebLaunch L = plan_launch(pl);
    L.kmax = std::min(pl.kmax, 4);
    float best = 3.0e38f;
    int best_mg = pl.mg;
    for (int mg : cand) {
        float ms = 0.0f;
        for (int rep = 0; rep < 2; ++rep) {
            CU_TRY(cudaMemsetAsync(g_ctx.err, 0, sizeof(int), st));
            CU_TRY(cudaMemsetAsync(g_ctx.bar, 0, 2 * sizeof(unsigned), st));
            CU_TRY(cudaEventRecord(g_ctx.ev[0], st));
            CU_TRY(launch_cheb(L, pl.precision, mg, st));
            CU_TRY(cudaEventRecord(g_ctx.ev[1], st));
        }
        CU_TRY(cudaEventSynchronize(g_ctx.ev[1]));
        CU_TRY(cudaEventElapsedTime(&ms, g_ctx.ev[0], g_ctx.ev[1]));
        int err = 0;
        CU_TRY(copy_d2h(&err, g_ctx.err, sizeof(int)));
        if (err) return err;
        if (ms < best) {
            best = ms;
            best_mg = mg;
        }
    }
    pl.mg = best_mg;
    g_tile_cache[key] = best_mg;
    return ELHL_OK;
}

// Failure-detection test hook (elhl_debug_barrier): the grid-barrier limit of
// the propagation launches and a one-shot early exit of one CTA.
unsigned long long g_dbg_barrier_ns = 0;
int g_dbg_exit_cta1 = 0;

// The propagation launch of an ELHL_PREC_OZ64 plan (one problem, m <= 4, explicit Hs).
int oz_run(ChebPlan &pl) {
    cudaStream_t st = g_ctx.stream;
    OzRes &oz = *pl.oz;
    const ChebProblem &p = pl.probs[0];
    if (p.m > 4 || !oz.s || pl.nphase != 1) return ELHL_ERR_UNSUPPORTED;
    OzLaunch L{};
    L.N = p.N; L.ld = p.ld; L.K = p.K; L.m = p.m; L.P = p.P;
    L.coef = p.coef;
    L.phi = p.col[pl.parity];
    L.acc = p.col[pl.parity ^ 1];
    L.scale = p.scale;
    L.v = oz.v;
    for (int b = 0; b < 3; ++b) {
        L.xs[b] = oz.xs + (size_t)b * 2 * oz.ntiles * oz_vector_tile_bytes();
        L.xe[b] = oz.xe + (size_t)b * 2 * oz.ntiles * 8;
        L.emax[b] = oz.xe + (size_t)3 * 2 * oz.ntiles * 8 + b * 8;
    }
    L.rscale = oz.r;
    L.segs = oz.segs;
    L.seg_begin = oz.begin;
    L.part_base = oz.base;
    L.part_count = oz.count;
    L.part = oz.part;
    L.tile_cnt = oz.cnt;
    L.bar_count = g_ctx.bar;
    L.error = g_ctx.err;
    L.barrier_ns = g_dbg_barrier_ns;
    L.exit_cta1 = g_dbg_exit_cta1;
    g_dbg_exit_cta1 = 0;  // one launch only
    CU_TRY(cudaMemsetAsync(g_ctx.err, 0, sizeof(int), st));
    CU_TRY(cudaMemsetAsync(g_ctx.bar, 0, 2 * sizeof(unsigned), st));
    CU_TRY(cudaMemsetAsync(oz.cnt, 0, (size_t)oz.ntiles * sizeof(unsigned), st));
    CU_TRY(cudaMemsetAsync(oz.xe + (size_t)3 * 2 * oz.ntiles * 8, 0x80, 3 * 8 * sizeof(int), st));  // column maxima
    CU_TRY(cudaEventRecord(g_ctx.ev[0], st));
    CU_TRY(launch_oz_cheb(L, oz.s, oz.grid, st));
    CU_TRY(cudaEventRecord(g_ctx.ev[1], st));
    return ELHL_OK;
}

int cheb_run(ChebPlan &pl) {
    cudaStream_t st = g_ctx.stream;
    if (pl.oz) return oz_run(pl);
    if (!pl.tuned) {
        if (int rc = tune_plan(pl, pl.mgcd)) return rc;
        pl.tuned = true;
    }
    CU_TRY(cudaMemsetAsync(g_ctx.err, 0, sizeof(int), st));
    CU_TRY(cudaMemsetAsync(g_ctx.bar, 0, 2 * sizeof(unsigned), st));
    ChebLaunch L{};
    L.probs = pl.d_probs;
    L.segs = pl.d_segs;
    L.seg_begin = pl.d_seg_begin;
    L.kmax = pl.kmax;
    L.max_ld = pl.max_ld;
    L.grid = pl.grid;
    L.bar_count = g_ctx.bar;
    L.error = g_ctx.err;
    L.prob_seg0 = pl.d_prob_seg0;
    L.parity = pl.parity;
    L.seg_pops = pl.d_seg_pops;
    L.nphase = pl.nphase;
    L.segs_full = pl.d_segs_full;
    L.seg_full_begin = pl.d_seg_full_begin;
    L.barrier_ns = g_dbg_barrier_ns;
    L.exit_cta1 = g_dbg_exit_cta1;
    g_dbg_exit_cta1 = 0;  // one launch only
    CU_TRY(cudaEventRecord(g_ctx.ev[0], st));
    CU_TRY(launch_cheb(L, pl.precision, pl.mg, st));
    CU_TRY(cudaEventRecord(g_ctx.ev[1], st));
    return ELHL_OK;
}

int launch_norm_drift(const ChebPlan &pl) {
    int mmax = 0;
    for (const auto &p : pl.probs) mmax = std::max(mmax, p.m);
    norm_drift_kernel<<<dim3((unsigned)pl.probs.size(), mmax), kDriftBlock, 0, g_ctx.stream>>>(pl.d_probs, pl.parity);
    count_launch();
    bool totals = false;
    int pmax = 0;
    for (const auto &p : pl.probs) {
        totals |= p.ntot != nullptr;
        pmax = std::max(pmax, p.P);
    }
    if (totals) {
        norm_total_kernel<<<dim3((unsigned)pl.probs.size(), pmax), kDriftBlock, 0, g_ctx.stream>>>(pl.d_probs,
                                                                                                    pl.parity);
        count_launch();
    }
    CU_TRY(cudaGetLastError());
    return ELHL_OK;
}

// drift tolerance of a configuration: <= 0 selects the precision's default
double cheb_norm_tolerance(const elhl_traj_config &c) {
    if (c.cheb_norm_tol > 0.0) return c.cheb_norm_tol;
    return reduced_precision(c.precision) ? 1.0e-4 : 1.0e-8;
}

// One fixed-nuclei step with the device read-out: propagation launch, norm
// drift of the step, read-out launch (+ population reduction), then the
// columns swap roles.  No host sync.
int cheb_dev_step(ChebPlan &pl, const std::vector<ChebState *> &states, double *d_pops_step) {
    if (int rc = cheb_run(pl)) return rc;
    if (int rc = launch_norm_drift(pl)) return rc;
    ChebLaunch L{};
    L.probs = pl.d_probs;
    L.segs = pl.d_segs;
    L.seg_begin = pl.d_seg_begin;
    L.prob_seg0 = pl.d_prob_seg0;
    L.max_ld = pl.max_ld;
    L.grid = pl.grid;
    L.parity = pl.parity;
    L.seg_pops = pl.d_seg_pops;
    L.pops = d_pops_step;
    CU_TRY(launch_readout(L, (int)pl.probs.size(), pl.ro_precision, pl.mg_read, g_ctx.stream));
    pl.parity ^= 1;
    for (auto *cs : states) cs->parity = pl.parity;
    return ELHL_OK;
}

// apply the pending renormalisation factor to the next input columns and the
// AO-basis outputs, then reset it to 1 (end of a multi-step call)
__global__ void settle_scale_kernel(double2 *cols, int m, double2 *psi, double2 *bra, int n, int P, double *scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        for (int c = 0; c < m; ++c) {
            const double sc = scale[c % P];
            double2 v = cols[(size_t)i * m + c];
            cols[(size_t)i * m + c] = make_double2(v.x * sc, v.y * sc);
        }
        for (int p = 0; p < P; ++p) {
            const double sc = scale[p];
            double2 a = psi[(size_t)i * P + p], b = bra[(size_t)i * P + p];
            psi[(size_t)i * P + p] = make_double2(a.x * sc, a.y * sc);
            bra[(size_t)i * P + p] = make_double2(b.x * sc, b.y * sc);
        }
    }
}

__global__ void ones_kernel(double *v, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = 1.0;
}

int cheb_settle(const std::vector<ChebState *> &states) {
    cudaStream_t st = g_ctx.stream;
    for (auto *cs : states) {
        if (!reduced_precision(cs->precision)) continue;
        settle_scale_kernel<<<(cs->N + 255) / 256, 256, 0, st>>>(cs->cin(), cs->m, cs->psi_out, cs->bra_out, cs->N,
                                                                 cs->P, cs->scale);
        count_launch();
        ones_kernel<<<1, kMaxCols, 0, st>>>(cs->scale, kMaxCols);
        count_launch();
    }
    CU_TRY(cudaGetLastError());
    return ELHL_OK;
}

// Complex columns stored [ld][m] (interleaved) are the rows of a 2m x N
// column-major real matrix X; right-side triangular operations act on every
// column at once:  X L  = (L^T x)^T,  X L^-1 = (L^-T x)^T,
//                  X L^T = (L x)^T,   X L^-T = (L^-1 x)^T.
// Y (R x n) = X M for an R x n X (column k at X + k ldx) and a triangular FP64
// M: Y(r, j) = sum_k X(r, k) M(k, j) over the non-zero part of column j of M
// (k >= j for a lower M, k <= j for an upper one).  One warp per column j:
// coalesced reads of the column, the R <= kMaxTransformRows values of X(., k)
// from L1/L2, FP64 FMAs, then fixed-order warp sums.  The DGEMM it replaces,
// with 4 rows, ran at about 0.9 ms at N = 3720.
constexpr int kMaxTransformRows = 8;
template <bool LOWER>
__global__ void cols_mt_kernel(const double *__restrict__ M, int ld, int n, const double *__restrict__ X, int ldx,
                               int R, double *__restrict__ Y) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
    if (j >= n) return;
    const int k0 = LOWER ? j : 0, k1 = LOWER ? n : j + 1;
    const double *col = M + (size_t)j * ld;
    double acc[kMaxTransformRows];
#pragma unroll
    for (int r = 0; r < kMaxTransformRows; ++r) acc[r] = 0.0;
    for (int k = k0 + lane; k < k1; k += 32) {
        const double mk = col[k];
        const double *x = X + (size_t)k * ldx;
#pragma unroll
        for (int r = 0; r < kMaxTransformRows; ++r)
            if (r < R) acc[r] = fma(mk, x[r], acc[r]);
    }
#pragma unroll
    for (int r = 0; r < kMaxTransformRows; ++r)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
#pragma unroll
    for (int r = 0; r < kMaxTransformRows; ++r)
        if (r < R && lane == r) Y[(size_t)j * R + r] = acc[r];
}

// The same four transforms with dense FP64 factors (zeros above the diagonal):
// M = G = L^-1 for the inverse ones, M = L otherwise, X op(M) into scratch
// (2 ncols x n) and a strided copy back.  op(M) = M, and op(M) = M^T when the
// FP64 transpose Mt (Lt for L, Gt for G) is resident, run as cols_mt_kernel;
// otherwise one DGEMM.  The implicit operator keeps both factors, and either
// costs one read of M, where a right-side TRSM with 4 rows runs as a long
// chain of small launches.
int cols_apply_dense(const double *L, const double *G, int ld, int n, double2 *cols, int m, int col0, int ncols,
                     bool transpose, bool inverse, double *scratch, const double *Lt = nullptr,
                     const double *Gt = nullptr) {
    double *X = reinterpret_cast<double *>(cols) + 2 * col0;
    const int rows = 2 * ncols, ldx = 2 * m;
    const double *Mt = inverse ? Gt : Lt;
    if (rows <= kMaxTransformRows && (!transpose || Mt)) {
        const int warps_per_block = 8, grid = (n + warps_per_block - 1) / warps_per_block;
        if (!transpose) {
            cols_mt_kernel<true><<<grid, 32 * warps_per_block, 0, g_ctx.stream>>>(inverse ? G : L, ld, n, X, ldx, rows,
                                                                                   scratch);
            count_launch();
        } else {  // X M^T = X (Mt)^T with Mt upper triangular
            cols_mt_kernel<false><<<grid, 32 * warps_per_block, 0, g_ctx.stream>>>(Mt, ld, n, X, ldx, rows, scratch);
            count_launch();
        }
        CU_TRY(cudaGetLastError());
    } else {
        CU_TRY(dgemm64(rows, n, n, 1.0, X, ldx, false, inverse ? G : L, ld, transpose, 0.0, scratch, rows, g_ctx.stream,
                       transpose ? kTriBt : kTriB));
    }
    CU_TRY(cudaMemcpy2DAsync(X, ldx * sizeof(double), scratch, rows * sizeof(double), rows * sizeof(double), n,
                             cudaMemcpyDeviceToDevice, g_ctx.stream));
    return ELHL_OK;
}

// ---- Ehrenfest force kernel pieces ---------------------------------------------
// K = X o A (Hadamard), then K -= H A by one FP64 product (dgemm64, beta = 1):
// the K = X o A - H A of hadamard_minus (Chebyshev_gpu_kernels.cu:358-389) with
// ehrenfestkernel_gpu_ (Taylor_gpu.cpp:743-791).
__global__ void hadamard_kernel(const double *__restrict__ X, const double *__restrict__ A, double *__restrict__ K,
                                int n, int ld) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i < n && j < n) K[(size_t)j * ld + i] = X[(size_t)j * ld + i] * A[(size_t)j * ld + i];
}

// A = (rho + rho^T)/2, rho_ij = Re(ket_j1 bra_i1) - Re(ket_j2 bra_i2)
// (calculate_A / calculate_rho_kernel, Chebyshev_gpu_kernels.cu:394-455); bra/ket [2][n]
__global__ void ehrenfest_a_kernel(const double2 *__restrict__ bra, const double2 *__restrict__ ket, double *A,
                                   int n, int ld) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= n || j >= n) return;
    auto rho = [&](int r, int c) {
        const double2 k1 = ket[c], b1 = bra[r], k2 = ket[n + c], b2 = bra[n + r];
        return (k1.x * b1.x - k1.y * b1.y) - (k2.x * b2.x - k2.y * b2.y);
    };
    A[(size_t)j * ld + i] = 0.5 * (rho(i, j) + rho(j, i));
}

struct EhrenfestBuffers {
    int n = 0, ld = 0;
    double *H = nullptr, *A = nullptr, *X = nullptr, *K = nullptr;
    double2 *bk = nullptr;
    int reserve(int n_) {
        if (H && n_ <= n) return ELHL_OK;
        dev_free(H); dev_free(A); dev_free(X); dev_free(K); dev_free(bk);
        n = n_;
        ld = round_up(n, 32);
        if (int rc = dev_alloc(&H, (size_t)ld * n)) return rc;
        if (int rc = dev_alloc(&A, (size_t)ld * n)) return rc;
        if (int rc = dev_alloc(&X, (size_t)ld * n)) return rc;
        if (int rc = dev_alloc(&K, (size_t)ld * n)) return rc;
        return dev_alloc(&bk, (size_t)4 * n);
    }
};
EhrenfestBuffers g_ehr;

int ehrenfest_impl(int n, const double *hH, const double *hA, const elhl_zcomplex *hbra, const elhl_zcomplex *hket,
                   const double *hX, double *hK) {
    if (n <= 0 || !hH || !hX || !hK || (!hA && (!hbra || !hket))) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (int rc = ensure_context_locked(-1)) return rc;
    if (int rc = g_ehr.reserve(n)) return rc;
    cudaStream_t st = g_ctx.stream;
    const int ld = g_ehr.ld;
    const size_t col = n * sizeof(double), ldb = ld * sizeof(double);
    dim3 grid((n + 127) / 128, n);
    CU_TRY(cudaMemcpy2DAsync(g_ehr.H, ldb, hH, col, col, n, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpy2DAsync(g_ehr.X, ldb, hX, col, col, n, cudaMemcpyHostToDevice, st));
    if (hA) {
        CU_TRY(cudaMemcpy2DAsync(g_ehr.A, ldb, hA, col, col, n, cudaMemcpyHostToDevice, st));
    } else {
        CU_TRY(cudaMemcpyAsync(g_ehr.bk, hbra, 2 * n * sizeof(double2), cudaMemcpyHostToDevice, st));
        CU_TRY(cudaMemcpyAsync(g_ehr.bk + 2 * n, hket, 2 * n * sizeof(double2), cudaMemcpyHostToDevice, st));
        ehrenfest_a_kernel<<<grid, 128, 0, st>>>(g_ehr.bk, g_ehr.bk + 2 * n, g_ehr.A, n, ld);
        count_launch();
    }
    hadamard_kernel<<<grid, 128, 0, st>>>(g_ehr.X, g_ehr.A, g_ehr.K, n, ld);
    count_launch();
    CU_TRY(cudaGetLastError());
    CU_TRY(dgemm64(n, n, n, -1.0, g_ehr.H, ld, false, g_ehr.A, ld, false, 1.0, g_ehr.K, ld, st));  // K -= H' A
    CU_TRY(cudaMemcpy2DAsync(hK, col, g_ehr.K, ldb, col, n, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    return ELHL_OK;
}

}  // namespace

// =============================== trajectories ===================================
struct elhl_traj {
    DevBasis basis;
    // host copy of the basis (fragment sub-bases for the initial states)
    std::vector<int> h_ao0, h_nao, h_n, h_l, h_m, h_nz;
    std::vector<double> h_zeta, h_coef, h_ip, h_kwh, h_vs;
    const double *last_coords = nullptr;  // device coordinates of the current S, h
    int N = 0, ld = 0, natoms = 0, nfrag = 0, P = 2;
    elhl_traj_config cfg;
    double *S = nullptr, *h = nullptr, *Hp = nullptr, *coords = nullptr, *pops = nullptr;
    int pops_cap = 0, coords_cap = 0;
    Factor fac;
    TaylorBuffers tb;
    double t = 0.0;
    int it = 1;
    bool first_call = true;
    double save_tau[2] = {0.0, 0.0};
    elhl_traj_stats stats{};
    // Chebyshev method: AO-basis Psi_ket / Psi_bra as [ld][2] (row i, particle p)
    ChebState cs;
    ChebPlan plan;
    double2 *psi_ao = nullptr, *bra_ao = nullptr, *ro_ket = nullptr, *ro_bra = nullptr;
    double *target = nullptr;  // per-particle total population to hold (reduced precision)
    bool cheb() const { return cfg.method == ELHL_METHOD_CHEBYSHEV; }
};

namespace {

int upload_basis(DevBasis &d, const elhl_basis_desc *b) {
    d.natoms = b->natoms;
    d.nao = b->nao;
    d.nfrag = b->nfrag;
    auto up_i = [](int **dst, const int *src, size_t n) -> int {
        if (int rc = dev_alloc(dst, n)) return rc;
        CU_TRY(copy_h2d(*dst, src, n * sizeof(int)));
        return ELHL_OK;
    };
    auto up_d = [](double **dst, const double *src, size_t n) -> int {
        if (int rc = dev_alloc(dst, n)) return rc;
        CU_TRY(copy_h2d(*dst, src, n * sizeof(double)));
        return ELHL_OK;
    };
    int rc = 0;
    rc |= up_i(&d.atom_ao0, b->atom_ao0, b->natoms);
    rc |= up_i(&d.atom_nao, b->atom_nao, b->natoms);
    rc |= up_i(&d.ao_n, b->ao_n, b->nao);
    rc |= up_i(&d.ao_l, b->ao_l, b->nao);
    rc |= up_i(&d.ao_m, b->ao_m, b->nao);
    rc |= up_i(&d.ao_nzeta, b->ao_nzeta, b->nao);
    rc |= up_d(&d.ao_zeta, b->ao_zeta, 2 * (size_t)b->nao);
    rc |= up_d(&d.ao_coef, b->ao_coef, 2 * (size_t)b->nao);
    rc |= up_d(&d.ao_ip, b->ao_ip, b->nao);
    rc |= up_d(&d.ao_kwh, b->ao_kwh, b->nao);
    rc |= up_d(&d.ao_vshift, b->ao_vshift, b->nao);
    if (b->ao_frag) rc |= up_i(&d.ao_frag, b->ao_frag, b->nao);
    // atoms grouped by kind: AO count, then each AO's (n, l, zetas), so that the
    // S/h build's warps see few distinct pair kinds
    std::vector<int> order(b->natoms);
    for (int a = 0; a < b->natoms; ++a) order[a] = a;
    auto key = [&](int a) {
        std::vector<double> k{(double)b->atom_nao[a]};
        for (int i = b->atom_ao0[a]; i < b->atom_ao0[a] + b->atom_nao[a]; ++i) {
            k.push_back(b->ao_n[i]);
            k.push_back(b->ao_l[i]);
            k.push_back(b->ao_nzeta[i]);
            for (int z = 0; z < b->ao_nzeta[i]; ++z) k.push_back(b->ao_zeta[2 * i + z]);
        }
        return k;
    };
    std::vector<std::vector<double>> keys(b->natoms);
    for (int a = 0; a < b->natoms; ++a) keys[a] = key(a);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return keys[x] < keys[y]; });
    rc |= up_i(&d.atom_order, order.data(), b->natoms);
    return rc ? ELHL_ERR_CUDA : ELHL_OK;
}

void free_basis(DevBasis &d) {
    dev_free(d.atom_ao0); dev_free(d.atom_nao); dev_free(d.ao_n); dev_free(d.ao_l); dev_free(d.ao_m);
    dev_free(d.ao_nzeta); dev_free(d.ao_zeta); dev_free(d.ao_coef); dev_free(d.ao_ip); dev_free(d.ao_kwh);
    dev_free(d.ao_vshift); dev_free(d.ao_frag); dev_free(d.atom_order);
}

int validate_basis(const elhl_basis_desc *b) {
    if (!b || b->natoms <= 0 || b->nao <= 0 || !b->atom_ao0 || !b->atom_nao || !b->ao_n || !b->ao_l || !b->ao_m ||
        !b->ao_nzeta || !b->ao_zeta || !b->ao_coef || !b->ao_ip || !b->ao_kwh || !b->ao_vshift)
        return ELHL_ERR_BAD_ARG;
    if (b->nfrag < 0 || b->nfrag > kMaxFrag) return ELHL_ERR_BAD_ARG;
    int count = 0;
    for (int a = 0; a < b->natoms; ++a) {
        if (b->atom_ao0[a] != count || b->atom_nao[a] <= 0) return ELHL_ERR_BAD_ARG;
        count += b->atom_nao[a];
    }
    if (count != b->nao) return ELHL_ERR_BAD_ARG;
    for (int i = 0; i < b->nao; ++i) {
        if (b->ao_n[i] < 1 || b->ao_n[i] > 3 || b->ao_l[i] < 0 || b->ao_l[i] > 1) return ELHL_ERR_UNSUPPORTED;
        if (b->ao_m[i] < -b->ao_l[i] || b->ao_m[i] > b->ao_l[i]) return ELHL_ERR_BAD_ARG;
        if (b->ao_nzeta[i] < 1 || b->ao_nzeta[i] > 2) return ELHL_ERR_BAD_ARG;
        if (b->ao_frag && (b->ao_frag[i] < 0 || b->ao_frag[i] >= (b->nfrag > 0 ? b->nfrag : 1))) return ELHL_ERR_BAD_ARG;
    }
    return ELHL_OK;
}

// S, h, H' for the coordinates currently in tr->coords (+ offset)
int rebuild(elhl_traj *tr, const double *d_coords) {
    tr->last_coords = d_coords;
    CU_TRY(cudaEventRecord(g_ctx.ev[2], g_ctx.stream));
    CU_TRY(launch_build_sh(tr->basis, d_coords, tr->cfg.cutoff, tr->S, tr->h, tr->ld, g_ctx.stream));
    int rc = tr->cheb() ? ELHL_OK : tr->fac.form_hprime(tr->S, tr->h, tr->Hp, tr->N);
    CU_TRY(cudaEventRecord(g_ctx.ev[3], g_ctx.stream));
    return rc;
}

// Cholesky factor, then the operator for the current S, h: explicit H~ (formed
// once for fixed nuclei, 2 N^3 flops) or implicit G h G^T (a geometry that
// changes every step, N^3/3 flops); bounds and coefficients.
int cheb_rebuild_operator(elhl_traj *tr, bool implicit = false) {
    cudaStream_t st = g_ctx.stream;
    ChebState &cs = tr->cs;
    // S = L L^T and G = L^-1 in one recursion, in FP64 for every precision: on the
    // FP64 pipe for FP64 propagation (the plain FP64 path), with the products of
    // 320 or more rows exact on the tensor cores for the others (Factor::tc).
    // The implicit operator keeps G in cs.Ht, the explicit one in the factor's G.
    if (implicit && cs.oz) {
        // ELHL_PREC_OZ64: with every product on the tensor cores, forming H~ = G h G^T
        // (1.5 N^3 flops) costs less than the implicit operator's extra phases (2 N^2
        // elements and three grid phases per order instead of N^2 and one), so moving
        // nuclei use the explicit operator too.  FP64 L^T and G^T serve the column transforms.
        if (int rc = tr->fac.factor(tr->S, tr->N)) return rc;
        CU_TRY(cudaEventRecord(g_ctx.ev[5], st));
        if (int rc = tr->fac.check_info(false)) return rc;
        cs.implicit = false;
        if (int rc = form_htilde(cs, tr->fac.G, tr->h, tr->ld, tr->fac.W, tr->fac.tc)) return rc;
        CU_TRY(cudaEventRecord(g_ctx.ev[6], st));
        if (int rc = lanczos_bounds(cs, kLanczosMoving)) return rc;
        if (int rc = cheb_prepare(cs, tr->cfg.dt * tr->cfg.frame_step, tr->cfg.cheb_tol)) return rc;
        if (int rc = cheb_prepare_readout(cs, tr->fac.L, tr->fac.G)) return rc;  // A = G, B = L^T in FP64
        if (!cs.Gt) CU_TRY(cudaMalloc(&cs.Gt, (size_t)cs.ld * cs.N * sizeof(double)));
        convert_kernel<double><<<dim3((cs.ld + 127) / 128, cs.N), 128, 0, st>>>(tr->fac.G, (double *)cs.Gt, cs.N,
                                                                                cs.ld, true);
        count_launch();
        CU_TRY(cudaGetLastError());
        return ELHL_OK;
    }
    if (int rc = tr->fac.factor(tr->S, tr->N, implicit ? cs.Ht : nullptr)) return rc;
    CU_TRY(cudaEventRecord(g_ctx.ev[5], st));
    if (int rc = tr->fac.check_info(false)) return rc;
    if (implicit) return cheb_prepare_implicit(cs, tr->fac.L, tr->h, tr->cfg.dt * tr->cfg.frame_step, tr->cfg.cheb_tol);
    cs.implicit = false;
    if (int rc = form_htilde(cs, tr->fac.G, tr->h, tr->ld, tr->fac.W, tr->fac.tc)) return rc;
    if (int rc = lanczos_bounds(cs, kLanczosFixed)) return rc;
    return cheb_prepare(cs, tr->cfg.dt * tr->cfg.frame_step, tr->cfg.cheb_tol);
}

// G = L^-1 of the trajectory's current factor: in cs.Ht for the implicit
// operator, in the factor's own buffer otherwise
const double *traj_inverse(const elhl_traj *tr) { return tr->cs.implicit ? tr->cs.Ht : tr->fac.G; }

// phi <- transformed columns of (psi_ao, bra_ao) with the current factor
int cheb_load_columns(elhl_traj *tr) {
    cudaStream_t st = g_ctx.stream;
    ChebState &cs = tr->cs;
    const int P = tr->P, n = tr->N;
    const size_t e = sizeof(double2);
    double2 *in = cs.cin();
    CU_TRY(cudaMemcpy2DAsync(in, cs.m * e, tr->psi_ao, P * e, P * e, n, cudaMemcpyDeviceToDevice, st));
    if (cs.m == 2 * P)
        CU_TRY(cudaMemcpy2DAsync(in + P, cs.m * e, tr->bra_ao, P * e, P * e, n, cudaMemcpyDeviceToDevice, st));
    if (cs.implicit) {  // dense L (zeroed upper triangle) and G = L^-1
        const double *Lt = cs.lt64(), *Gt = cs.gt64();
        if (int rc = cols_apply_dense(tr->fac.L, cs.Ht, tr->ld, n, in, cs.m, 0, P, false, false, cs.cscratch, Lt, Gt))
            return rc;
        if (cs.m == 2 * P)
            if (int rc = cols_apply_dense(tr->fac.L, cs.Ht, tr->ld, n, in, cs.m, P, P, true, true, cs.cscratch, Lt, Gt))
                return rc;
        cs.cols_current = true;
        return ELHL_OK;
    }
    const double *G = traj_inverse(tr);
    const double *Lt = cs.oz ? cs.lt64() : nullptr, *Gt = cs.oz ? cs.gt64() : nullptr;  // FP64 transposes
    if (int rc = cols_apply_dense(tr->fac.L, G, tr->ld, n, in, cs.m, 0, P, false, false, cs.cscratch, Lt, Gt))
        return rc;  // L^T psi
    if (cs.m == 2 * P)
        if (int rc = cols_apply_dense(tr->fac.L, G, tr->ld, n, in, cs.m, P, P, true, true, cs.cscratch, Lt, Gt))
            return rc;  // L^-1 bra
    cs.cols_current = true;
    return ELHL_OK;
}

// psi_ao, bra_ao <- back-transformed columns of acc; populations into d_pops
int cheb_readout(elhl_traj *tr, const double2 *cols, double *d_pops) {
    cudaStream_t st = g_ctx.stream;
    ChebState &cs = tr->cs;
    const int P = tr->P, n = tr->N;
    const size_t e = sizeof(double2);
    CU_TRY(cudaMemcpy2DAsync(tr->psi_ao, P * e, cols, cs.m * e, P * e, n, cudaMemcpyDeviceToDevice, st));
    const double2 *bsrc = (cs.m == 2 * P) ? cols + P : cols;
    CU_TRY(cudaMemcpy2DAsync(tr->bra_ao, P * e, bsrc, cs.m * e, P * e, n, cudaMemcpyDeviceToDevice, st));
    if (cs.implicit) {
        if (int rc = cols_apply_dense(tr->fac.L, cs.Ht, tr->ld, n, tr->psi_ao, P, 0, P, false, true, cs.cscratch,
                                      cs.lt64(), cs.gt64()))
            return rc;  // L^-T phi
        if (int rc = cols_apply_dense(tr->fac.L, cs.Ht, tr->ld, n, tr->bra_ao, P, 0, P, true, false, cs.cscratch,
                                      cs.lt64(), cs.gt64()))
            return rc;  // L chi
    } else {
        const double *G = traj_inverse(tr);
        const double *Lt = cs.oz ? cs.lt64() : nullptr, *Gt = cs.oz ? cs.gt64() : nullptr;  // FP64 transposes
        if (int rc = cols_apply_dense(tr->fac.L, G, tr->ld, n, tr->psi_ao, P, 0, P, false, true, cs.cscratch, Lt, Gt))
            return rc;  // L^-T phi
        if (int rc = cols_apply_dense(tr->fac.L, G, tr->ld, n, tr->bra_ao, P, 0, P, true, false, cs.cscratch, Lt, Gt))
            return rc;  // L chi
    }
    if (d_pops) {
        populations_kernel<<<P, 256, 0, st>>>(tr->psi_ao, tr->bra_ao, n, P, tr->basis.ao_frag, tr->nfrag, d_pops);
        count_launch();
        CU_TRY(cudaGetLastError());
    }
    return ELHL_OK;
}

// ---- norm control of the trajectory's steps ----------------------------------
// Widen the spectral interval by half its width (a quarter on each side) and
// redo the scaled operator, the coefficients and the plan's order counts.
int cheb_widen(elhl_traj *tr) {
    ChebState &cs = tr->cs;
    const double w = cs.emax - cs.emin;
    cs.emin -= 0.25 * w;
    cs.emax += 0.25 * w;
    if (int rc = cheb_prepare(cs, tr->cfg.dt * tr->cfg.frame_step, tr->cfg.cheb_tol, cs.implicit ? tr->h : nullptr))
        return rc;
    if (tr->plan.probs.empty()) return ELHL_OK;  // GEMM regime: no row-kernel plan
    std::vector<ChebState *> one{&cs};
    return cheb_plan_refresh(tr->plan, one);
}

// Input columns and pending renormalisation factors at the start of a
// multi-step call (column roles: the caller keeps the parity), so that the
// whole call can be redone.
int cheb_save_state(ChebState &cs) {
    cudaStream_t st = g_ctx.stream;
    if (!cs.saved)
        if (int rc = dev_alloc(&cs.saved, (size_t)cs.ld * cs.m + kMaxCols / 2)) return rc;
    CU_TRY(cudaMemcpyAsync(cs.saved, cs.cin(), (size_t)cs.ld * cs.m * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    CU_TRY(cudaMemcpyAsync(cs.saved + (size_t)cs.ld * cs.m, cs.scale, kMaxCols * sizeof(double),
                           cudaMemcpyDeviceToDevice, st));
    return ELHL_OK;
}

int cheb_restore_state(elhl_traj *tr, int parity) {
    cudaStream_t st = g_ctx.stream;
    ChebState &cs = tr->cs;
    cs.parity = parity;
    tr->plan.parity = parity;
    CU_TRY(cudaMemcpyAsync(cs.cin(), cs.saved, (size_t)cs.ld * cs.m * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    CU_TRY(cudaMemcpyAsync(cs.scale, cs.saved + (size_t)cs.ld * cs.m, kMaxCols * sizeof(double),
                           cudaMemcpyDeviceToDevice, st));
    return ELHL_OK;
}

// One propagation launch of the trajectory's plan with the norm check: redone
// from its input columns (which the launch does not write) on a widened
// interval while the drift exceeds the tolerance, at most cheb_max_retries
// times.  Synchronises with the stream; *drift receives the accepted drift.
int cheb_run_checked(elhl_traj *tr, double *drift) {
    cudaStream_t st = g_ctx.stream;
    const double ntol = cheb_norm_tolerance(tr->cfg);
    for (int attempt = 0;; ++attempt) {
        CU_TRY(cudaMemsetAsync(tr->plan.d_drift, 0, sizeof(double), st));
        if (int rc = cheb_run(tr->plan)) return rc;
        if (int rc = launch_norm_drift(tr->plan)) return rc;
        int err = 0;
        double d = 0.0;
        CU_TRY(cudaMemcpyAsync(&err, g_ctx.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaMemcpyAsync(&d, tr->plan.d_drift, sizeof(double), cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaStreamSynchronize(st));
        if (err) return err;
        *drift = d;
        if (d <= ntol) return ELHL_OK;
        if (attempt >= tr->cfg.cheb_max_retries) return ELHL_ERR_NO_CONVERGENCE;
        if (int rc = cheb_widen(tr)) return rc;
        tr->stats.cheb_retries += 1;
    }
}

int cheb_step_impl(elhl_traj *tr, const double *coords, bool coords_on_device, int nsteps, double *d_pops) {
    cudaStream_t st = g_ctx.stream;
    ChebState &cs = tr->cs;
    const int P = tr->P, nf = tr->nfrag;
    const size_t pop_per_step = (size_t)P * (nf + 1);
    const size_t nc = (size_t)tr->natoms * 3;
    std::vector<ChebState *> one{&cs};
    int rc = ELHL_OK;
    if (!coords && cs.implicit && cs.gemm) {
        // GEMM regime after moving steps: form H~ for the current geometry
        if ((rc = cheb_rebuild_operator(tr, false))) return rc;
        if ((rc = cheb_prepare_readout(cs, tr->fac.L, traj_inverse(tr)))) return rc;
        if ((rc = cheb_plan(tr->plan, one))) return rc;
    }
    if (!coords && !cs.readout_ready && tr->fac.L && cs.precision != ELHL_PREC_DF64) {
        // fixed nuclei after moving steps: factor-based read-out matrices for the current L
        if ((rc = cheb_prepare_readout(cs, tr->fac.L, traj_inverse(tr)))) return rc;
        if ((rc = cheb_plan(tr->plan, one))) return rc;
    }
    if (!coords && cs.readout_ready && (tr->plan.mg_read || cs.gemm)) {
        // ---- fixed nuclei, device read-out: two launches (or one graph) per step, no host sync;
        // the norm drift of every step is kept on the device and read once at the end
        if (!cs.cols_current && (rc = cheb_load_columns(tr))) return rc;
        if ((rc = cheb_save_state(cs))) return rc;
        const int parity0 = cs.parity;
        const double ntol = cheb_norm_tolerance(tr->cfg);
        double *d_drift = cs.gemm ? cs.drift : tr->plan.d_drift;
        double drift = 0.0;
        for (int attempt = 0;; ++attempt) {
            CU_TRY(cudaMemsetAsync(d_drift, 0, sizeof(double), st));
            CU_TRY(cudaEventRecord(g_ctx.ev[2], st));
            for (int s = 0; s < nsteps; ++s) {
                if (cs.gemm) {
                    if ((rc = cheb_gemm_step(cs))) return rc;
                    tr->plan.parity = cs.parity;
                    if (d_pops)
                        CU_TRY(cudaMemcpyAsync(d_pops + s * pop_per_step, cs.gpops, pop_per_step * sizeof(double),
                                               cudaMemcpyDeviceToDevice, st));
                    continue;
                }
                if ((rc = cheb_dev_step(tr->plan, one, d_pops ? d_pops + s * pop_per_step : nullptr))) return rc;
            }
            CU_TRY(cudaEventRecord(g_ctx.ev[3], st));
            if ((rc = cheb_settle(one))) return rc;
            int err = 0;
            CU_TRY(cudaMemcpyAsync(&err, g_ctx.err, sizeof(int), cudaMemcpyDeviceToHost, st));
            CU_TRY(cudaMemcpyAsync(&drift, d_drift, sizeof(double), cudaMemcpyDeviceToHost, st));
            CU_TRY(cudaStreamSynchronize(st));
            if (err) return err;
            if (drift <= ntol) break;
            tr->stats.norm_drift = drift;
            if (attempt >= tr->cfg.cheb_max_retries) return ELHL_ERR_NO_CONVERGENCE;
            // redo the whole call from its saved input on a widened interval
            if ((rc = cheb_restore_state(tr, parity0))) return rc;
            if ((rc = cheb_widen(tr))) return rc;
            tr->stats.cheb_retries += 1;
        }
        tr->stats.norm_drift = drift;
        tr->stats.prop_ms += event_ms(0, 1) * nsteps;  // last launch x launches
        tr->stats.rebuild_ms += 0.0;
        tr->stats.prop_launches += nsteps;
        tr->stats.orders += (long long)cs.K * cs.m * nsteps;
        tr->stats.substeps += nsteps;
        for (int s = 0; s < nsteps; ++s) tr->t = tr->t + tr->cfg.dt * tr->cfg.frame_step;
        tr->it += nsteps;
        tr->first_call = false;
        for (int p = 0; p < P && p < 2; ++p) tr->save_tau[p] = tr->cfg.dt / kHbar;  // electron, hole
        return ELHL_OK;
    }
    // ---- moving nuclei (or no device read-out): factor-based read-out through cuBLAS
    const bool renorm = reduced_precision(cs.precision);
    double *pops_tmp = nullptr;
    if (!d_pops && renorm) {
        if ((rc = dev_alloc(&pops_tmp, pop_per_step))) return rc;
    }
    if (!coords && !cs.cols_current) rc = cheb_load_columns(tr);
    for (int s = 0; s < nsteps && !rc; ++s) {
        if (coords) {
            const double *dc;
            if (coords_on_device) {
                dc = coords + s * nc;
            } else {
                if (cudaMemcpyAsync(tr->coords, coords + s * nc, nc * sizeof(double), cudaMemcpyHostToDevice, st) !=
                    cudaSuccess) { rc = ELHL_ERR_CUDA; break; }
                dc = tr->coords;
            }
            tr->last_coords = dc;
            if (cudaEventRecord(g_ctx.ev[2], st) != cudaSuccess) { rc = ELHL_ERR_CUDA; break; }
            if (launch_build_sh(tr->basis, dc, tr->cfg.cutoff, tr->S, tr->h, tr->ld, st) != cudaSuccess) {
                rc = ELHL_ERR_CUDA;
                break;
            }
            if (cudaEventRecord(g_ctx.ev[4], st) != cudaSuccess) { rc = ELHL_ERR_CUDA; break; }
            if ((rc = cheb_rebuild_operator(tr, true))) break;  // implicit: A, B follow the new L
            if ((rc = cheb_load_columns(tr))) break;
            if (cudaEventRecord(g_ctx.ev[3], st) != cudaSuccess) { rc = ELHL_ERR_CUDA; break; }
            if ((rc = cheb_plan_refresh(tr->plan, one))) break;
        }
        double drift = 0.0;
        if ((rc = cheb_run_checked(tr, &drift))) break;
        tr->stats.norm_drift = std::max(tr->stats.norm_drift, drift);
        double2 *out = cs.parity ? cs.phi : cs.acc;
        double *pp = d_pops ? d_pops + s * pop_per_step : pops_tmp;
        if ((rc = cheb_readout(tr, out, pp))) break;
        if (renorm) {
            renormalize_kernel<<<(tr->N + 255) / 256, 256, 0, st>>>(out, tr->N, cs.m, P, pp, nf, tr->target);
            count_launch();
            if (cudaGetLastError() != cudaSuccess) { rc = ELHL_ERR_CUDA; break; }
            if ((rc = cheb_readout(tr, out, pp))) break;  // AO state and populations of the renormalised columns
        }
        tr->plan.parity ^= 1;
        cs.parity = tr->plan.parity;
        tr->stats.prop_ms += event_ms(0, 1);  // the events completed before the checked run returned
        tr->stats.prop_launches += 1;
        tr->stats.orders += (long long)cs.K * cs.m;
        if (coords) {
            tr->stats.rebuild_ms += event_ms(2, 3);
            tr->stats.sh_ms += event_ms(2, 4);
            tr->stats.factor_ms += event_ms(4, 5);
            tr->stats.inverse_ms += event_ms(5, 6);
            tr->stats.rebuild_count += 1;
        }
        tr->stats.substeps += 1;
        tr->t = tr->t + tr->cfg.dt * tr->cfg.frame_step;
        tr->it += 1;
        tr->first_call = false;
    }
    dev_free(pops_tmp);
    for (int p = 0; p < P && p < 2; ++p) tr->save_tau[p] = tr->cfg.dt / kHbar;  // electron, hole
    tr->stats.status = rc;
    return rc;
}

int traj_step_impl(elhl_traj *tr, const double *coords, bool coords_on_device, int nsteps, double *pops,
                   bool pops_on_device) {
    if (!tr || nsteps <= 0) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (int rc = ensure_context_locked(-1)) return rc;
    cudaStream_t st = g_ctx.stream;
    const int P = tr->P, nf = tr->nfrag;
    const size_t pop_per_step = (size_t)P * (nf + 1);
    double *d_pops = pops_on_device ? pops : nullptr;
    if (pops && !pops_on_device) {
        if ((int)(nsteps * pop_per_step) > tr->pops_cap) {
            dev_free(tr->pops);
            if (int rc = dev_alloc(&tr->pops, nsteps * pop_per_step)) return rc;
            tr->pops_cap = (int)(nsteps * pop_per_step);
        }
        d_pops = tr->pops;
    }
    const double dt_frame = tr->cfg.dt * tr->cfg.frame_step;
    const double tau_max = tr->cfg.dt / kHbar;
    std::vector<TaylorParticle> res;
    auto tau_for_step = [&](double *taus) {
        for (int p = 0; p < P; ++p) {
            const double t = tr->first_call ? tau_max : tr->save_tau[p] * 1.15;
            taus[p] = t > tau_max ? tau_max : t;
        }
    };
    memset(&tr->stats, 0, sizeof(tr->stats));
    if (tr->cheb()) {
        const int rc = cheb_step_impl(tr, coords, coords_on_device, nsteps, d_pops);
        tr->stats.tile_cols = tr->cs.gemm ? 0 : tr->plan.mg;
        tr->stats.phases = tr->plan.nphase;
        if (rc) return rc;
        if (pops && !pops_on_device)
            CU_TRY(copy_d2h(pops, d_pops, nsteps * pop_per_step * sizeof(double)));
        return ELHL_OK;
    }
    if (!coords) {
        // fixed nuclei: S, h, H' unchanged; the whole run is one launch
        double taus[2];
        tau_for_step(taus);
        const int it0 = tr->it + 1;
        if (int rc = run_taylor(tr->Hp, tr->N, tr->ld, tr->tb, P, taus, tr->t, dt_frame * (double)(it0 - 1),
                                tr->cfg.tol, tr->cfg.norm_tol, tr->cfg.max_conv_calls, nsteps, it0, dt_frame,
                                tau_max, d_pops, tr->basis.ao_frag, nf))
            return rc;
        double tf = 0.0;
        int rc = collect_taylor(tr->tb, P, res, &tf);
        tr->stats.prop_ms += event_ms(0, 1);
        tr->stats.prop_launches += 1;
        for (int p = 0; p < P; ++p) {
            tr->save_tau[p] = res[p].save_tau;
            tr->stats.orders += res[p].orders;
            tr->stats.conv_calls += res[p].conv_calls;
            tr->stats.substeps += res[p].substeps;
        }
        if (rc) { tr->stats.status = rc; return rc; }
        tr->t = tf;
        tr->it += nsteps;
        tr->first_call = false;
    } else {
        const size_t nc = (size_t)tr->natoms * 3;
        if (!coords_on_device && tr->coords_cap < (int)nc) {
            dev_free(tr->coords);
            if (int rc = dev_alloc(&tr->coords, nc)) return rc;
            tr->coords_cap = (int)nc;
        }
        for (int s = 0; s < nsteps; ++s) {
            const double *dc;
            if (coords_on_device) {
                dc = coords + s * nc;
            } else {
                CU_TRY(cudaMemcpyAsync(tr->coords, coords + s * nc, nc * sizeof(double), cudaMemcpyHostToDevice, st));
                dc = tr->coords;
            }
            if (int rc = rebuild(tr, dc)) return rc;
            double taus[2];
            tau_for_step(taus);
            const int it0 = tr->it + 1;
            if (int rc = run_taylor(tr->Hp, tr->N, tr->ld, tr->tb, P, taus, tr->t, dt_frame * (double)(it0 - 1),
                                    tr->cfg.tol, tr->cfg.norm_tol, tr->cfg.max_conv_calls, 1, it0, dt_frame,
                                    tau_max, d_pops ? d_pops + s * pop_per_step : nullptr, tr->basis.ao_frag, nf))
                return rc;
            double tf = 0.0;
            int rc = collect_taylor(tr->tb, P, res, &tf);
            tr->stats.prop_ms += event_ms(0, 1);
            tr->stats.rebuild_ms += event_ms(2, 3);
            tr->stats.prop_launches += 1;
            tr->stats.rebuild_count += 1;
            for (int p = 0; p < P; ++p) {
                tr->save_tau[p] = res[p].save_tau;
                tr->stats.orders += res[p].orders;
                tr->stats.conv_calls += res[p].conv_calls;
                tr->stats.substeps += res[p].substeps;
            }
            if (rc) { tr->stats.status = rc; return rc; }
            if (int frc = tr->fac.check_info()) { tr->stats.status = frc; return frc; }
            tr->t = tf;
            tr->it += 1;
            tr->first_call = false;
        }
    }
    if (pops && !pops_on_device)
        CU_TRY(copy_d2h(pops, d_pops, nsteps * pop_per_step * sizeof(double)));
    return ELHL_OK;
}

// Initial state of particle p from fragment MO `state` (1-based).
int fmo_particle(elhl_traj *tr, int nat, const int *atoms, int state, double2 *ket, double2 *bra, int stride) {
    if (nat <= 0 || !atoms || state < 1 || !tr->S) return ELHL_ERR_BAD_ARG;
    std::vector<int> ao0, nao, n, l, m, nz, aos;
    std::vector<double> zeta, coef, ip, kwh, vs;
    for (int a = 0; a < nat; ++a) {
        const int at = atoms[a];
        if (at < 0 || at >= tr->natoms || (a > 0 && at <= atoms[a - 1])) return ELHL_ERR_BAD_ARG;
        ao0.push_back((int)n.size());
        nao.push_back(tr->h_nao[at]);
        for (int j = 0; j < tr->h_nao[at]; ++j) {
            const int i = tr->h_ao0[at] + j;
            aos.push_back(i);
            n.push_back(tr->h_n[i]); l.push_back(tr->h_l[i]); m.push_back(tr->h_m[i]); nz.push_back(tr->h_nz[i]);
            zeta.push_back(tr->h_zeta[2 * i]); zeta.push_back(tr->h_zeta[2 * i + 1]);
            coef.push_back(tr->h_coef[2 * i]); coef.push_back(tr->h_coef[2 * i + 1]);
            ip.push_back(tr->h_ip[i]); kwh.push_back(tr->h_kwh[i]); vs.push_back(tr->h_vs[i]);
        }
    }
    const int nf = (int)aos.size();
    if (state > nf) return ELHL_ERR_BAD_ARG;
    // fragment coordinates gathered from the current device coordinates
    std::vector<double> all((size_t)tr->natoms * 3), sub((size_t)nat * 3);
    CU_TRY(copy_d2h(all.data(), tr->last_coords, all.size() * sizeof(double)));
    for (int a = 0; a < nat; ++a)
        for (int k = 0; k < 3; ++k) sub[3 * a + k] = all[3 * (size_t)atoms[a] + k];
    elhl_basis_desc d{};
    d.natoms = nat; d.nao = nf; d.atom_ao0 = ao0.data(); d.atom_nao = nao.data(); d.ao_n = n.data();
    d.ao_l = l.data(); d.ao_m = m.data(); d.ao_nzeta = nz.data(); d.ao_zeta = zeta.data(); d.ao_coef = coef.data();
    d.ao_ip = ip.data(); d.ao_kwh = kwh.data(); d.ao_vshift = vs.data(); d.ao_frag = nullptr; d.nfrag = 0;
    DevBasis fb;
    int rc = upload_basis(fb, &d);
    const int ldf = round_up(nf, 32);
    double *Sf = nullptr, *hf = nullptr, *w = nullptr, *dc = nullptr, *work = nullptr;
    int *info = nullptr, *daos = nullptr, lwork = 0;
    cudaStream_t st = g_ctx.stream;
    if (!rc) rc = dev_alloc(&Sf, (size_t)ldf * nf);
    if (!rc) rc = dev_alloc(&hf, (size_t)ldf * nf);
    if (!rc) rc = dev_alloc(&w, (size_t)nf);
    if (!rc) rc = dev_alloc(&dc, sub.size());
    if (!rc) rc = dev_alloc(&info, 1);
    if (!rc) rc = dev_alloc(&daos, (size_t)nf);
    if (!rc && copy_h2d(dc, sub.data(), sub.size() * sizeof(double)) != cudaSuccess) rc = ELHL_ERR_CUDA;
    if (!rc && copy_h2d(daos, aos.data(), nf * sizeof(int)) != cudaSuccess) rc = ELHL_ERR_CUDA;
    if (!rc && launch_build_sh(fb, dc, tr->cfg.cutoff, Sf, hf, ldf, st) != cudaSuccess) rc = ELHL_ERR_CUDA;
    if (!rc && cusolverDnDsygvd_bufferSize(g_ctx.solver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                           CUBLAS_FILL_MODE_LOWER, nf, hf, ldf, Sf, ldf, w, &lwork) !=
                   CUSOLVER_STATUS_SUCCESS)
        rc = ELHL_ERR_CUDA;
    if (!rc) rc = dev_alloc(&work, (size_t)lwork + 1);
    if (!rc && cusolverDnDsygvd(g_ctx.solver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                nf, hf, ldf, Sf, ldf, w, work, lwork, info) != CUSOLVER_STATUS_SUCCESS)
        rc = ELHL_ERR_CUDA;
    if (!rc) {
        zero_strided<<<(tr->N + 255) / 256, 256, 0, st>>>(ket, tr->N, stride);
        count_launch();
        embed_fmo<<<1, 256, 0, st>>>(hf, ldf, nf, state - 1, daos, ket, stride);
        count_launch();
        s_times_sparse<<<(tr->N + 127) / 128, 128, 0, st>>>(tr->S, tr->ld, tr->N, daos, nf, ket, bra, stride);
        count_launch();
        if (cudaGetLastError() != cudaSuccess) rc = ELHL_ERR_CUDA;
    }
    int hinfo = 0;
    if (!rc && cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) rc = ELHL_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = ELHL_ERR_CUDA;
    if (!rc && hinfo != 0) rc = hinfo > nf ? ELHL_ERR_NOT_POSITIVE_DEFINITE : ELHL_ERR_CUDA;
    free_basis(fb);
    dev_free(Sf); dev_free(hf); dev_free(w); dev_free(dc); dev_free(work); dev_free(info); dev_free(daos);
    return rc;
}

int cheb_set_target(elhl_traj *tr);

// Psi (host, column-major N x P) into the [ld][P] AO arrays; bra = S ket when
// bra is NULL.  The norm target of each particle is its initial total population.
int cheb_set_psi(elhl_traj *tr, const elhl_zcomplex *bra, const elhl_zcomplex *ket) {
    if (!bra && !tr->S) return ELHL_ERR_BAD_ARG;  // S was released by elhl_batch_compact
    const size_t e = sizeof(double2);
    const int P = tr->P, n = tr->N;
    for (int p = 0; p < P; ++p)
        CU_TRY(cudaMemcpy2D(tr->psi_ao + p, P * e, ket + (size_t)p * n, e, e, n, cudaMemcpyHostToDevice));
    if (bra) {
        for (int p = 0; p < P; ++p)
            CU_TRY(cudaMemcpy2D(tr->bra_ao + p, P * e, bra + (size_t)p * n, e, e, n, cudaMemcpyHostToDevice));
    } else {
        // bra = S ket: the complex columns as a 2P x N real matrix times S (symmetric)
        CU_TRY(dgemm64(2 * P, n, n, 1.0, (const double *)tr->psi_ao, 2 * P, false, tr->S, tr->ld, false, 0.0,
                       (double *)tr->bra_ao, 2 * P, g_ctx.stream));
    }
    return cheb_set_target(tr);
}

// norm target of each particle = its current total population
int cheb_set_target(elhl_traj *tr) {
    const int P = tr->P, n = tr->N;
    tr->cs.cols_current = false;  // a new state: columns reload from psi_ao / bra_ao
    double *pops = nullptr;
    if (int rc = dev_alloc(&pops, (size_t)P * (tr->nfrag + 1))) return rc;
    populations_kernel<<<P, 256, 0, g_ctx.stream>>>(tr->psi_ao, tr->bra_ao, n, P, tr->basis.ao_frag, tr->nfrag, pops);
    count_launch();
    std::vector<double> h((size_t)P * (tr->nfrag + 1)), tgt(P);
    cudaError_t ce = cudaMemcpyAsync(h.data(), pops, h.size() * sizeof(double), cudaMemcpyDeviceToHost, g_ctx.stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(g_ctx.stream);
    dev_free(pops);
    CU_TRY(ce);
    for (int p = 0; p < P; ++p) tgt[p] = h[(size_t)p * (tr->nfrag + 1) + tr->nfrag];
    CU_TRY(copy_h2d(tr->target, tgt.data(), P * sizeof(double)));
    return ELHL_OK;
}

}  // namespace

// =============================== exported ========================================
extern "C" {

int elhl_last_status(void) { return g_last_status; }

const char *elhl_status_string(int s) {
    switch (s) {
        case ELHL_OK: return "ok";
        case ELHL_ERR_BAD_ARG: return "bad argument";
        case ELHL_ERR_NO_CONVERGENCE: return "no convergence (tau retries exhausted)";
        case ELHL_ERR_TIMEOUT: return "device wait timed out";
        case ELHL_ERR_OOM: return "out of device memory";
        case ELHL_ERR_CUDA: return "CUDA error";
        case ELHL_ERR_NOT_POSITIVE_DEFINITE: return "overlap matrix not positive definite";
        case ELHL_ERR_NO_DEVICE: return "no CUDA device";
        case ELHL_ERR_UNSUPPORTED: return "unsupported basis";
        default: return "unknown status";
    }
}

int elhl_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

int elhl_debug_barrier(double limit_s, int exit_cta) {
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (limit_s > 10.0 || exit_cta < -1 || exit_cta >= 1 << 20) return ELHL_ERR_BAD_ARG;
    g_dbg_barrier_ns = limit_s > 0.0 ? (unsigned long long)(limit_s * 1e9) : 0ULL;
    g_dbg_exit_cta1 = exit_cta + 1;
    return ELHL_OK;
}

int elhl_set_stream(void *stream) {
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (int rc = ensure_context_locked(-1)) return rc;
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    g_ctx.stream = stream ? (cudaStream_t)stream : g_ctx.own_stream;
    SOLVER_TRY(cusolverDnSetStream(g_ctx.solver, g_ctx.stream));
    if (cublasSetStream(g_ctx.blas, g_ctx.stream) != CUBLAS_STATUS_SUCCESS) return ELHL_ERR_CUDA;
    if (cublasSetStream(g_ctx.blas_tc, g_ctx.stream) != CUBLAS_STATUS_SUCCESS) return ELHL_ERR_CUDA;
    return ELHL_OK;
}

long long elhl_kernel_launches(void) { return own_launches(); }

int elhl_sm_count(void) {
    if (ensure_context()) return 0;
    return g_ctx.sms;
}

void gpu_init_(const int *myid, const int *procs_per_dev) {
    // device = (myid / procs_per_dev) % ndev (GPU_Interface.cpp:226-263)
    int id = myid ? *myid : 0, per = (procs_per_dev && *procs_per_dev > 0) ? *procs_per_dev : 1;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    g_last_status = ensure_context_locked(id / per);
    if (g_last_status) fprintf(stderr, "elhlprop: gpu_init_: %s\n", elhl_status_string(g_last_status));
}

void gpu_finalize_(void) {
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (!g_ctx.ready) return;
    cudaDeviceSynchronize();
    g_drop.release();
    dev_free(g_ctx.bar);
    dev_free(g_ctx.err);
    dev_free(g_ctx.partials);
    if (g_ctx.solver) cusolverDnDestroy(g_ctx.solver);
    if (g_ctx.blas) cublasDestroy(g_ctx.blas);
    if (g_ctx.blas_tc) cublasDestroy(g_ctx.blas_tc);
    g_ctx.blas = g_ctx.blas_tc = nullptr;
    if (g_ctx.tc_ws) cudaFree(g_ctx.tc_ws);
    g_ctx.tc_ws = nullptr;
    if (g_ctx.own_stream) cudaStreamDestroy(g_ctx.own_stream);
    if (g_ctx.copy_stream) cudaStreamDestroy(g_ctx.copy_stream);
    if (g_ctx.aux_stream) cudaStreamDestroy(g_ctx.aux_stream);
    if (g_ctx.ev_l21) cudaEventDestroy(g_ctx.ev_l21);
    if (g_ctx.ev_side) cudaEventDestroy(g_ctx.ev_side);
    g_ctx.aux_stream = nullptr;
    g_ctx.ev_l21 = g_ctx.ev_side = nullptr;
    g_ctx.solver = nullptr;
    g_ctx.stream = g_ctx.copy_stream = g_ctx.own_stream = nullptr;
    g_ctx.ready = false;
}

void gpu_pin_(void *ptr, const int *bytes) {
    if (!ptr || !bytes || *bytes <= 0) { g_last_status = ELHL_ERR_BAD_ARG; return; }
    cudaError_t e = cudaHostRegister(ptr, (size_t)*bytes, cudaHostRegisterPortable);
    g_last_status = e == cudaSuccess ? ELHL_OK : ELHL_ERR_CUDA;
    if (e != cudaSuccess) fprintf(stderr, "elhlprop: gpu_pin_: %s\n", cudaGetErrorString(e));
}

void gpu_unpin_(void *ptr) {
    if (!ptr) { g_last_status = ELHL_ERR_BAD_ARG; return; }
    cudaError_t e = cudaHostUnregister(ptr);
    g_last_status = e == cudaSuccess ? ELHL_OK : ELHL_ERR_CUDA;
}

void ehrenfestkernel_gpu_(const int *N, const double *h_H, const double *h_A, const double *h_X, double *h_K) {
    g_last_status = N ? ehrenfest_impl(*N, h_H, h_A, nullptr, nullptr, h_X, h_K) : ELHL_ERR_BAD_ARG;
    if (g_last_status) fprintf(stderr, "elhlprop: ehrenfestkernel_gpu_: %s\n", elhl_status_string(g_last_status));
}

void ehrenfestkernel2_gpu_(const int *N, const elhl_zcomplex *h_bra, const elhl_zcomplex *h_ket, const double *h_H,
                           const double *h_X, double *h_K) {
    g_last_status = N ? ehrenfest_impl(*N, h_H, nullptr, h_bra, h_ket, h_X, h_K) : ELHL_ERR_BAD_ARG;
    if (g_last_status) fprintf(stderr, "elhlprop: ehrenfestkernel2_gpu_: %s\n", elhl_status_string(g_last_status));
}

void propagation_gpucaller_(const int *n, double *tau, double *save_tau, const double *t_init, const double *t_max,
                            elhl_zcomplex *h_PSI_bra, elhl_zcomplex *h_PSI_ket, const double *h_H) {
    if (!n || !tau || !t_init || !t_max) { g_last_status = ELHL_ERR_BAD_ARG; return; }
    g_last_status = dropin_single(*n, *tau, save_tau, *t_init, *t_max, h_PSI_bra, h_PSI_ket, h_H);
    if (g_last_status) fprintf(stderr, "elhlprop: propagation_gpucaller_: %s\n", elhl_status_string(g_last_status));
}

void propagationelhl_gpucaller_(const int *N, const double *h_S, const double *h_h, double *h_H,
                                elhl_zcomplex *h_AO_bra, elhl_zcomplex *h_AO_ket, elhl_zcomplex *h_PSI_bra,
                                elhl_zcomplex *h_PSI_ket, const double *t_init, const double *t_max, double *tau,
                                double *save_tau) {
    (void)h_AO_ket;  // unused by the reference as well
    if (!N || !t_init || !t_max || !tau) { g_last_status = ELHL_ERR_BAD_ARG; return; }
    g_last_status = dropin_elhl(*N, h_S, h_h, h_H, h_AO_bra, h_PSI_bra, h_PSI_ket, *t_init, *t_max, *tau, save_tau);
    if (g_last_status)
        fprintf(stderr, "elhlprop: propagationelhl_gpucaller_: %s\n", elhl_status_string(g_last_status));
}

void elhl_traj_config_default(elhl_traj_config *c) {
    if (!c) return;
    c->method = ELHL_METHOD_TAYLOR_REF;
    c->precision = ELHL_PREC_FP64;
    c->dt = 1.0e-4;
    c->frame_step = 1;
    c->tol = 1.0e-8;
    c->norm_tol = 1.0e-8;
    c->cheb_tol = 1.0e-12;
    c->cutoff = 12.0;
    c->max_conv_calls = 2000;
    c->ncols = 2;
    c->nparticles = 2;
    c->cheb_norm_tol = 0.0;  // by precision
    c->cheb_max_retries = 3;
    c->lanczos_guard = 0.01;
}

int elhl_ehrenfest_forces(const elhl_basis_desc *basis, const double *coords, const double *kernel, double delta,
                          double cutoff, double *forces) {
    if (!coords || !kernel || !forces) return ELHL_ERR_BAD_ARG;
    if (int rc = validate_basis(basis)) return rc;
    if (!(delta > 0.0)) delta = 1.0e-8;   // diabatic-Ehren.f:32
    if (!(cutoff > 0.0)) cutoff = 12.0;   // cutoff_Angs
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (int rc = ensure_context_locked(-1)) return rc;
    cudaStream_t st = g_ctx.stream;
    const int nat = basis->natoms, n = basis->nao;
    DevBasis db{};
    double *d_coords = nullptr, *d_kernel = nullptr, *d_F = nullptr, *d_force = nullptr;
    int rc = upload_basis(db, basis);
    if (!rc) rc = dev_alloc(&d_coords, (size_t)nat * 3);
    if (!rc) rc = dev_alloc(&d_kernel, (size_t)n * n);
    if (!rc) rc = dev_alloc(&d_F, (size_t)nat * nat * 3);
    if (!rc) rc = dev_alloc(&d_force, (size_t)nat * 3);
    if (!rc && (cudaMemcpyAsync(d_coords, coords, (size_t)nat * 3 * sizeof(double), cudaMemcpyHostToDevice, st) ||
                cudaMemcpyAsync(d_kernel, kernel, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice, st)))
        rc = ELHL_ERR_CUDA;
    if (!rc && launch_pulay_forces(db, d_coords, cutoff, delta, d_kernel, n, d_F, 2.0 * 1.602176565e-9, d_force, st))
        rc = ELHL_ERR_CUDA;
    if (!rc && (cudaMemcpyAsync(forces, d_force, (size_t)nat * 3 * sizeof(double), cudaMemcpyDeviceToHost, st) ||
                cudaStreamSynchronize(st)))
        rc = ELHL_ERR_CUDA;
    free_basis(db);
    dev_free(d_coords); dev_free(d_kernel); dev_free(d_F); dev_free(d_force);
    return rc;
}

int elhl_huckel_with_fields(const elhl_basis_desc *basis, const double *coords, const double *S, const double *dp_ao,
                            const double *dp4, double cutoff, double *h) {
    if (!coords || !S || !dp_ao || !dp4 || !h) return ELHL_ERR_BAD_ARG;
    if (int rc = validate_basis(basis)) return rc;
    if (!(cutoff > 0.0)) cutoff = 12.0;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (int rc = ensure_context_locked(-1)) return rc;
    cudaStream_t st = g_ctx.stream;
    const int nat = basis->natoms, n = basis->nao;
    const size_t nn = (size_t)n * n, aa = (size_t)nat * nat;
    DevBasis db{};
    double *d_coords = nullptr, *d_S = nullptr, *d_dp = nullptr, *d_dp4 = nullptr, *d_h = nullptr;
    int rc = upload_basis(db, basis);
    if (!rc) rc = dev_alloc(&d_coords, (size_t)nat * 3);
    if (!rc) rc = dev_alloc(&d_S, nn);
    if (!rc) rc = dev_alloc(&d_dp, 3 * nn);
    if (!rc) rc = dev_alloc(&d_dp4, 4 * aa);
    if (!rc) rc = dev_alloc(&d_h, nn);
    if (!rc && (copy_h2d(d_coords, coords, (size_t)nat * 3 * sizeof(double)) ||
                copy_h2d(d_S, S, nn * sizeof(double)) || copy_h2d(d_dp, dp_ao, 3 * nn * sizeof(double)) ||
                copy_h2d(d_dp4, dp4, 4 * aa * sizeof(double)) ||
                cudaMemsetAsync(d_h, 0, nn * sizeof(double), st)))
        rc = ELHL_ERR_CUDA;
    if (!rc && launch_huckel_fields(db, d_coords, cutoff, d_S, n, d_dp, d_dp4, d_h, n, st)) rc = ELHL_ERR_CUDA;
    if (!rc && copy_d2h(h, d_h, nn * sizeof(double))) rc = ELHL_ERR_CUDA;
    free_basis(db);
    dev_free(d_coords); dev_free(d_S); dev_free(d_dp); dev_free(d_dp4); dev_free(d_h);
    return rc;
}

int elhl_traj_create(const elhl_basis_desc *basis, const double *coords, const elhl_traj_config *cfg,
                     elhl_traj **out) {
    if (!out || !coords) return ELHL_ERR_BAD_ARG;
    *out = nullptr;
    if (int rc = validate_basis(basis)) return rc;
    if (int rc = ensure_context()) return rc;
    elhl_traj *tr = new elhl_traj();
    if (cfg) tr->cfg = *cfg; else elhl_traj_config_default(&tr->cfg);
    const bool taylor_ok = tr->cfg.method == ELHL_METHOD_TAYLOR_REF && tr->cfg.precision == ELHL_PREC_FP64;
    const bool taylor_p = tr->cfg.nparticles == 2;
    const bool cheb_ok = tr->cfg.method == ELHL_METHOD_CHEBYSHEV &&
                         (tr->cfg.precision == ELHL_PREC_FP64 || tr->cfg.precision == ELHL_PREC_FP32 ||
                          tr->cfg.precision == ELHL_PREC_BF16X3 || tr->cfg.precision == ELHL_PREC_DF64 ||
                          (tr->cfg.precision == ELHL_PREC_OZ64 && tr->cfg.ncols <= 4)) &&
                         tr->cfg.nparticles >= 1 && tr->cfg.nparticles <= 64 &&
                         (tr->cfg.ncols == tr->cfg.nparticles || tr->cfg.ncols == 2 * tr->cfg.nparticles) &&
                         tr->cfg.cheb_tol > 0.0;
    const bool control_ok = tr->cfg.cheb_max_retries >= 0 && tr->cfg.lanczos_guard > -0.45 &&
                            tr->cfg.lanczos_guard < 10.0 && !(tr->cfg.cheb_norm_tol < 0.0);
    if (!((taylor_ok && taylor_p) || cheb_ok) || !control_ok || tr->cfg.dt <= 0 || tr->cfg.frame_step <= 0 ||
        tr->cfg.max_conv_calls <= 0) {
        delete tr;
        return ELHL_ERR_UNSUPPORTED;
    }
    tr->N = basis->nao;
    tr->ld = round_up(tr->N, 32);
    tr->P = tr->cfg.nparticles;
    tr->h_ao0.assign(basis->atom_ao0, basis->atom_ao0 + basis->natoms);
    tr->h_nao.assign(basis->atom_nao, basis->atom_nao + basis->natoms);
    tr->h_n.assign(basis->ao_n, basis->ao_n + basis->nao);
    tr->h_l.assign(basis->ao_l, basis->ao_l + basis->nao);
    tr->h_m.assign(basis->ao_m, basis->ao_m + basis->nao);
    tr->h_nz.assign(basis->ao_nzeta, basis->ao_nzeta + basis->nao);
    tr->h_zeta.assign(basis->ao_zeta, basis->ao_zeta + 2 * basis->nao);
    tr->h_coef.assign(basis->ao_coef, basis->ao_coef + 2 * basis->nao);
    tr->h_ip.assign(basis->ao_ip, basis->ao_ip + basis->nao);
    tr->h_kwh.assign(basis->ao_kwh, basis->ao_kwh + basis->nao);
    tr->h_vs.assign(basis->ao_vshift, basis->ao_vshift + basis->nao);
    tr->natoms = basis->natoms;
    tr->nfrag = basis->nfrag;
    int rc = upload_basis(tr->basis, basis);
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (!rc) rc = dev_alloc(&tr->S, (size_t)tr->ld * tr->N);
    if (!rc) rc = dev_alloc(&tr->h, (size_t)tr->ld * tr->N);
    if (!rc && !tr->cheb()) rc = dev_alloc(&tr->Hp, (size_t)tr->ld * tr->N);
    if (!rc) rc = dev_alloc(&tr->coords, (size_t)tr->natoms * 3);
    if (!rc) tr->coords_cap = tr->natoms * 3;
    if (!rc) rc = tr->fac.reserve(tr->N, tr->ld);
    if (!rc && !tr->cheb()) rc = tr->tb.reserve(tr->N, tr->P);
    if (!rc && copy_h2d(tr->coords, coords, tr->natoms * 3 * sizeof(double)) != cudaSuccess)
        rc = ELHL_ERR_CUDA;
    if (!rc) rc = rebuild(tr, tr->coords);
    if (!rc && cudaStreamSynchronize(g_ctx.stream) != cudaSuccess) rc = ELHL_ERR_CUDA;
    if (!rc && !tr->cheb()) rc = tr->fac.check_info();  // the Chebyshev set-up factors S below
    if (!rc && tr->cheb()) {
        const bool oz = tr->cfg.precision == ELHL_PREC_OZ64;  // FP64 state, tensor-core propagation
        tr->fac.tc = tr->cfg.precision != ELHL_PREC_FP64;      // FP64 factorisation, large products sliced
        rc = tr->cs.alloc(tr->N, tr->cfg.ncols, oz ? ELHL_PREC_FP64 : tr->cfg.precision);
        if (!rc && oz) {
            int grid = 0;
            tr->cs.oz = new OzRes();
            rc = cheb_grid_size(&grid) ? ELHL_ERR_CUDA : tr->cs.oz->init(tr->N, tr->ld, grid);
        }
        tr->cs.guard = tr->cfg.lanczos_guard;
        if (!rc) rc = dev_alloc(&tr->psi_ao, (size_t)tr->ld * tr->P);
        if (!rc) rc = dev_alloc(&tr->bra_ao, (size_t)tr->ld * tr->P);
        if (!rc) rc = dev_alloc(&tr->target, (size_t)tr->P);
        if (!rc && cudaMemset(tr->psi_ao, 0, (size_t)tr->ld * tr->P * sizeof(double2)) != cudaSuccess) rc = ELHL_ERR_CUDA;
        if (!rc && cudaMemset(tr->bra_ao, 0, (size_t)tr->ld * tr->P * sizeof(double2)) != cudaSuccess) rc = ELHL_ERR_CUDA;
        const bool df = tr->cfg.precision == ELHL_PREC_DF64;  // DF64: implicit operator from the start
        if (!rc) rc = cheb_rebuild_operator(tr, df);
        ChebState &cs = tr->cs;
        cs.P = tr->P; cs.nfrag = tr->nfrag; cs.psi_out = tr->psi_ao; cs.bra_out = tr->bra_ao;
        cs.ao_frag = tr->basis.ao_frag; cs.target = tr->target;
        if (!rc && !df) rc = cheb_prepare_readout(cs, tr->fac.L, traj_inverse(tr));
        // GEMM regime: many ket columns in FP32 / BF16X3 -> one GEMM per order
        if (!rc && gemm_eligible(cs)) {
            cs.gemm = true;
            if (cudaMalloc(&cs.Y, (size_t)cs.ld * cs.m * sizeof(float2)) != cudaSuccess ||
                cudaMalloc(&cs.Vf, (size_t)cs.ld * cs.m * sizeof(float2)) != cudaSuccess)
                rc = ELHL_ERR_OOM;
            if (!rc) rc = dev_alloc(&cs.gpops, (size_t)cs.P * (cs.nfrag + 1));
            // BF16X3 with 16, 32 or 64 columns: the hand-written tcgen05 GEMM (else cuBLAS emulation)
            if (!rc && cs.precision == ELHL_PREC_BF16X3 && umma_supported_n2(2 * cs.m)) {
                for (int t = 0; t < 3 && !rc; ++t)
                    if (cudaMalloc(&cs.hsplit[t], (size_t)cs.ld * cs.N * sizeof(__nv_bfloat16)) != cudaSuccess ||
                        cudaMalloc(&cs.vsplit[t], (size_t)cs.ld * 2 * cs.m * sizeof(__nv_bfloat16)) != cudaSuccess)
                        rc = ELHL_ERR_OOM;
                cs.usplits = umma_splits(cs.N, cs.N);
                if (!rc && cs.usplits > 1) {  // Y holds one partial tile per split
                    cudaFree(cs.Y);
                    cs.Y = nullptr;
                    if (cudaMalloc(&cs.Y, (size_t)cs.usplits * cs.N * cs.m * sizeof(float2)) != cudaSuccess)
                        rc = ELHL_ERR_OOM;
                }
                if (!rc) {
                    cs.umma = true;
                    rc = split3_bf16(reinterpret_cast<const float *>(cs.Hs), cs.N, cs.N, cs.ld, cs.hsplit, cs.ld,
                                     false, g_ctx.stream);
                }
            }
        }
        std::vector<ChebState *> one{&tr->cs};
        if (!rc) rc = cheb_plan(tr->plan, one);
    }
    if (rc) {
        free_basis(tr->basis);
        dev_free(tr->S); dev_free(tr->h); dev_free(tr->Hp); dev_free(tr->coords);
        tr->fac.release();
        tr->tb.release();
        delete tr;
        return rc;
    }
    *out = tr;
    return ELHL_OK;
}

int elhl_traj_destroy(elhl_traj *tr) {
    if (!tr) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    cudaStreamSynchronize(g_ctx.stream);
    free_basis(tr->basis);
    dev_free(tr->S); dev_free(tr->h); dev_free(tr->Hp); dev_free(tr->coords); dev_free(tr->pops);
    tr->fac.release();
    tr->tb.release();
    tr->cs.release();
    tr->plan.release();
    dev_free(tr->psi_ao); dev_free(tr->bra_ao); dev_free(tr->target);
    delete tr;
    return ELHL_OK;
}

int elhl_traj_init_fmo(elhl_traj *tr, int n_el_atoms, const int *el_atoms, int electron_state, int n_hl_atoms,
                       const int *hl_atoms, int hole_state) {
    if (!tr) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (tr->cheb()) {
        if (tr->P < 2) return ELHL_ERR_BAD_ARG;
        if (int rc = fmo_particle(tr, n_el_atoms, el_atoms, electron_state, tr->psi_ao, tr->bra_ao, tr->P)) return rc;
        if (int rc = fmo_particle(tr, n_hl_atoms, hl_atoms, hole_state, tr->psi_ao + 1, tr->bra_ao + 1, tr->P))
            return rc;
        return cheb_set_target(tr);
    }
    if (int rc = fmo_particle(tr, n_el_atoms, el_atoms, electron_state, tr->tb.ket(0), tr->tb.bra(0), 1)) return rc;
    return fmo_particle(tr, n_hl_atoms, hl_atoms, hole_state, tr->tb.ket(1), tr->tb.bra(1), 1);
}

int elhl_traj_init_fmo_states(elhl_traj *tr, int n_atoms, const int *atoms, int nstates, const int *states) {
    if (!tr || !tr->cheb() || nstates < 1 || nstates > tr->P || !states) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    for (int c = 0; c < nstates; ++c)
        if (int rc = fmo_particle(tr, n_atoms, atoms, states[c], tr->psi_ao + c, tr->bra_ao + c, tr->P)) return rc;
    return cheb_set_target(tr);
}

int elhl_traj_energies(elhl_traj *tr, elhl_zcomplex *E) {
    // QuasiParticleEnergies (ElHl_Chebyshev.f:329-371): E_p = sum_ij AO_bra_i h_ij AO_ket_j
    // with AO_bra = conj(S^-1 Psi_bra) (ElHl_Chebyshev.f:274-275) and AO_ket = Psi_ket.
    if (!tr || !E || !tr->h || !tr->fac.L) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    cudaStream_t st = g_ctx.stream;
    const int P = tr->P, n = tr->N;
    double2 *ket = nullptr, *bra = nullptr, *hk = nullptr;  // [n][P] each
    double *scr = nullptr;                                  // 2P x n transform output
    int rc = dev_alloc(&ket, (size_t)n * P);
    if (!rc) rc = dev_alloc(&bra, (size_t)n * P);
    if (!rc) rc = dev_alloc(&hk, (size_t)n * P);
    if (!rc) rc = dev_alloc(&scr, (size_t)2 * n * P);
    const size_t e = sizeof(double2);
    for (int p = 0; p < P && !rc; ++p) {
        const double2 *k = tr->cheb() ? tr->psi_ao + p : tr->tb.ket(p);
        const double2 *b = tr->cheb() ? tr->bra_ao + p : tr->tb.bra(p);
        const size_t sp = tr->cheb() ? P * e : e;
        if (cudaMemcpy2DAsync(ket + p, P * e, k, sp, e, n, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
            cudaMemcpy2DAsync(bra + p, P * e, b, sp, e, n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            rc = ELHL_ERR_CUDA;
    }
    // S^-1 bra = G^T G bra: rows of the 2P x n real view times G^T, then times G
    const double *G = tr->cheb() ? traj_inverse(tr) : tr->fac.G;
    if (!rc) rc = cols_apply_dense(tr->fac.L, G, tr->ld, n, bra, P, 0, P, true, true, scr);
    if (!rc) rc = cols_apply_dense(tr->fac.L, G, tr->ld, n, bra, P, 0, P, false, true, scr);
    if (!rc && dgemm64(2 * P, n, n, 1.0, (const double *)ket, 2 * P, false, tr->h, tr->ld, false, 0.0, (double *)hk,
                       2 * P, st) != cudaSuccess)
        rc = ELHL_ERR_CUDA;  // (h ket)^T = ket^T h, h symmetric
    std::vector<double2> hb((size_t)n * P), hh((size_t)n * P);
    if (!rc && (cudaMemcpyAsync(hb.data(), bra, hb.size() * e, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaMemcpyAsync(hh.data(), hk, hh.size() * e, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = ELHL_ERR_CUDA;
    dev_free(ket); dev_free(bra); dev_free(hk); dev_free(scr);
    if (rc) return rc;
    for (int p = 0; p < P; ++p) {
        double er = 0.0, ei = 0.0;
        for (int i = 0; i < n; ++i) {
            const double2 a = hb[(size_t)i * P + p], b = hh[(size_t)i * P + p];  // conj(a) * b
            er += a.x * b.x + a.y * b.y;
            ei += a.x * b.y - a.y * b.x;
        }
        E[p].re = er;
        E[p].im = ei;
    }
    return ELHL_OK;
}

int elhl_traj_set_psi(elhl_traj *tr, const elhl_zcomplex *bra, const elhl_zcomplex *ket) {
    if (!tr || !ket || (!bra && !tr->cheb())) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (tr->cheb()) return cheb_set_psi(tr, bra, ket);
    for (int p = 0; p < tr->P; ++p) {
        CU_TRY(copy_h2d(tr->tb.bra(p), bra + (size_t)p * tr->N, tr->N * sizeof(double2)));
        CU_TRY(copy_h2d(tr->tb.ket(p), ket + (size_t)p * tr->N, tr->N * sizeof(double2)));
    }
    return ELHL_OK;
}

int elhl_traj_get_psi(elhl_traj *tr, elhl_zcomplex *bra, elhl_zcomplex *ket) {
    if (!tr) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    if (tr->cheb()) {
        const size_t e = sizeof(double2);
        for (int p = 0; p < tr->P; ++p) {
            if (ket) CU_TRY(cudaMemcpy2D(ket + (size_t)p * tr->N, e, tr->psi_ao + p, tr->P * e, e, tr->N, cudaMemcpyDeviceToHost));
            if (bra) CU_TRY(cudaMemcpy2D(bra + (size_t)p * tr->N, e, tr->bra_ao + p, tr->P * e, e, tr->N, cudaMemcpyDeviceToHost));
        }
        return ELHL_OK;
    }
    for (int p = 0; p < tr->P; ++p) {
        if (bra) CU_TRY(copy_d2h(bra + (size_t)p * tr->N, tr->tb.bra(p), tr->N * sizeof(double2)));
        if (ket) CU_TRY(copy_d2h(ket + (size_t)p * tr->N, tr->tb.ket(p), tr->N * sizeof(double2)));
    }
    return ELHL_OK;
}

int elhl_traj_step(elhl_traj *tr, const double *coords, int nsteps, double *pops) {
    return traj_step_impl(tr, coords, false, nsteps, pops, false);
}

int elhl_traj_step_device(elhl_traj *tr, const double *d_coords, int nsteps, double *d_pops) {
    return traj_step_impl(tr, d_coords, true, nsteps, d_pops, true);
}

int elhl_traj_get_matrices(elhl_traj *tr, double *S, double *h, double *Hp) {
    if (!tr) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    const size_t col = tr->N * sizeof(double), ldb = tr->ld * sizeof(double);
    if (S) CU_TRY(cudaMemcpy2D(S, col, tr->S, ldb, col, tr->N, cudaMemcpyDeviceToHost));
    if (h) CU_TRY(cudaMemcpy2D(h, col, tr->h, ldb, col, tr->N, cudaMemcpyDeviceToHost));
    if (Hp && tr->Hp) CU_TRY(cudaMemcpy2D(Hp, col, tr->Hp, ldb, col, tr->N, cudaMemcpyDeviceToHost));
    return ELHL_OK;
}

int elhl_traj_get_factor(elhl_traj *tr, double *L, double *G) {
    if (!tr) return ELHL_ERR_BAD_ARG;
    if (!tr->cheb()) return ELHL_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    const size_t col = tr->N * sizeof(double), ldb = tr->ld * sizeof(double);
    if (L) {
        CU_TRY(cudaMemcpy2D(L, col, tr->fac.L, ldb, col, tr->N, cudaMemcpyDeviceToHost));
        for (int j = 1; j < tr->N; ++j)  // the explicit operator's factor keeps S above the diagonal
            std::memset(L + (size_t)j * tr->N, 0, j * sizeof(double));
    }
    if (G) {
        CU_TRY(cudaMemcpy2D(G, col, traj_inverse(tr), ldb, col, tr->N, cudaMemcpyDeviceToHost));
        for (int j = 1; j < tr->N; ++j)  // zero above the diagonal, whatever the recursion left there
            std::memset(G + (size_t)j * tr->N, 0, j * sizeof(double));
    }
    return ELHL_OK;
}

int elhl_traj_get_stats(elhl_traj *tr, elhl_traj_stats *st) {
    if (!tr || !st) return ELHL_ERR_BAD_ARG;
    *st = tr->stats;
    st->emin = tr->cheb() ? tr->cs.emin : 0.0;
    st->emax = tr->cheb() ? tr->cs.emax : 0.0;
    st->save_tau[0] = tr->save_tau[0];
    st->save_tau[1] = tr->save_tau[1];
    st->t = tr->t;
    st->it = tr->it;
    return ELHL_OK;
}

}  // extern "C"

// =============================== checkpoints ====================================
// Security_Copy_Cheb / Restart_State_Cheb (backup.f:329-445): a Fortran
// sequential unformatted file (4-byte record lengths around each record) with
// it, t, the basis size, the particle count, the particle tags, per particle
// the interleaved (DUAL_bra, DUAL_ket) and (AO_bra, AO_ket) pairs, and the
// Net_Charge record (the reference writes the whole array once per atom).  The
// reference's reader stops there; one more record, which it never reads,
// carries what a bit-exact resume of this library's trajectory needs: the
// method and precision, first_call and save_tau (the next step's tau), the
// norm targets, the Chebyshev interval and the symmetrised columns.
namespace {

constexpr char kResumeMagic[8] = {'E', 'L', 'H', 'L', 'R', 'S', 'M', '1'};

struct ResumeHead {
    char magic[8];
    int method, precision, N, P, ncols, first_call, has_cols, pad;
    double save_tau[2], emin, emax;
};

bool put_record(FILE *f, const void *p, size_t n) {
    const uint32_t m = (uint32_t)n;
    return fwrite(&m, 4, 1, f) == 1 && (n == 0 || fwrite(p, 1, n, f) == n) && fwrite(&m, 4, 1, f) == 1;
}

bool get_record(FILE *f, std::vector<char> &buf) {
    uint32_t m = 0, m2 = 0;
    if (fread(&m, 4, 1, f) != 1) return false;
    buf.resize(m);
    if (m && fread(buf.data(), 1, m, f) != m) return false;
    return fread(&m2, 4, 1, f) == 1 && m2 == m;
}

struct FileCloser {
    FILE *f;
    ~FileCloser() { if (f) fclose(f); }
};

// Psi_bra, Psi_ket of every particle (host, column-major N x P)
int traj_psi_host(elhl_traj *tr, std::vector<double2> &bra, std::vector<double2> &ket) {
    const int N = tr->N, P = tr->P;
    bra.resize((size_t)N * P);
    ket.resize((size_t)N * P);
    const size_t e = sizeof(double2);
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    for (int p = 0; p < P; ++p) {
        if (tr->cheb()) {
            CU_TRY(cudaMemcpy2D(ket.data() + (size_t)p * N, e, tr->psi_ao + p, P * e, e, N, cudaMemcpyDeviceToHost));
            CU_TRY(cudaMemcpy2D(bra.data() + (size_t)p * N, e, tr->bra_ao + p, P * e, e, N, cudaMemcpyDeviceToHost));
        } else {
            CU_TRY(cudaMemcpy(bra.data() + (size_t)p * N, tr->tb.bra(p), N * e, cudaMemcpyDeviceToHost));
            CU_TRY(cudaMemcpy(ket.data() + (size_t)p * N, tr->tb.ket(p), N * e, cudaMemcpyDeviceToHost));
        }
    }
    return ELHL_OK;
}

// AO_bra = conj(S^-1 Psi_bra) (ElHl_Chebyshev.f:274-275), S^-1 = G^T G on the device
int traj_ao_bra(elhl_traj *tr, const std::vector<double2> &bra, std::vector<double2> &ao) {
    const int N = tr->N, P = tr->P;
    const size_t e = sizeof(double2);
    double2 *d = nullptr;
    double *scr = nullptr;
    int rc = dev_alloc(&d, (size_t)N * P);
    if (!rc) rc = dev_alloc(&scr, (size_t)2 * N * P);
    for (int p = 0; p < P && !rc; ++p)  // [N][P] row-interleaved: the 2P x N real view
        if (cudaMemcpy2DAsync(d + p, P * e, bra.data() + (size_t)p * N, e, e, N, cudaMemcpyHostToDevice,
                              g_ctx.stream) != cudaSuccess)
            rc = ELHL_ERR_CUDA;
    const double *G = tr->cheb() ? traj_inverse(tr) : tr->fac.G;
    if (!rc) rc = cols_apply_dense(tr->fac.L, G, tr->ld, N, d, P, 0, P, true, true, scr);
    if (!rc) rc = cols_apply_dense(tr->fac.L, G, tr->ld, N, d, P, 0, P, false, true, scr);
    ao.resize((size_t)N * P);
    for (int p = 0; p < P && !rc; ++p)
        if (cudaMemcpy2DAsync(ao.data() + (size_t)p * N, e, d + p, P * e, e, N, cudaMemcpyDeviceToHost,
                              g_ctx.stream) != cudaSuccess)
            rc = ELHL_ERR_CUDA;
    if (!rc && cudaStreamSynchronize(g_ctx.stream) != cudaSuccess) rc = ELHL_ERR_CUDA;
    dev_free(d);
    dev_free(scr);
    for (auto &z : ao) z.y = -z.y;
    return rc;
}

int traj_snapshot_impl(elhl_traj *tr, const char *path) {
    const int N = tr->N, P = tr->P;
    std::vector<double2> bra, ket, ao_bra;
    if (int rc = traj_psi_host(tr, bra, ket)) return rc;
    if (int rc = traj_ao_bra(tr, bra, ao_bra)) return rc;
    ResumeHead rh{};
    memcpy(rh.magic, kResumeMagic, 8);
    rh.method = tr->cfg.method;
    rh.precision = tr->cfg.precision;
    rh.N = N;
    rh.P = P;
    rh.ncols = tr->cfg.ncols;
    rh.first_call = tr->first_call;
    rh.save_tau[0] = tr->save_tau[0];
    rh.save_tau[1] = tr->save_tau[1];
    std::vector<double> target(P, 0.0);
    std::vector<double2> cols;
    if (tr->cheb()) {
        ChebState &cs = tr->cs;
        rh.emin = cs.emin;
        rh.emax = cs.emax;
        CU_TRY(cudaMemcpy(target.data(), tr->target, P * sizeof(double), cudaMemcpyDeviceToHost));
        if (cs.cols_current) {  // fixed-nuclei steps continue from them (moving ones reload them from Psi)
            rh.has_cols = 1;
            cols.resize((size_t)N * cs.m);
            CU_TRY(cudaMemcpy(cols.data(), cs.cin(), cols.size() * sizeof(double2), cudaMemcpyDeviceToHost));
        }
    }
    // Net_Charge(atom) = sum_n sign_n |sum_{i in atom} DUAL_bra_i DUAL_ket_i|, sign -1 el / +1 hl
    // (Populations_mtx, data_output.f:129-134), DUAL_bra = conj(Psi_ket), DUAL_ket = Psi_bra
    std::vector<double> q(tr->natoms, 0.0);
    for (int p = 0; p < P; ++p) {
        const double sg = p % 2 == 0 ? -1.0 : 1.0;
        for (int a = 0; a < tr->natoms; ++a) {
            double re = 0.0, im = 0.0;
            for (int j = 0; j < tr->h_nao[a]; ++j) {
                const size_t i = (size_t)p * N + tr->h_ao0[a] + j;
                const double2 x = make_double2(ket[i].x, -ket[i].y), y = bra[i];
                re += x.x * y.x - x.y * y.y;
                im += x.x * y.y + x.y * y.x;
            }
            q[a] += sg * std::sqrt(re * re + im * im);
        }
    }
    FILE *f = fopen(path, "wb");
    if (!f) return ELHL_ERR_BAD_ARG;
    FileCloser fc{f};
    const int it = tr->it, ntag = P;
    const double t = tr->t;
    bool ok = put_record(f, &it, 4) && put_record(f, &t, 8) && put_record(f, &N, 4) && put_record(f, &P, 4) &&
              put_record(f, &ntag, 4);
    std::string tags;
    for (int p = 0; p < P; ++p) tags += p == 0 ? "el" : p == 1 ? "hl" : "  ";
    ok = ok && put_record(f, tags.data(), tags.size());
    std::vector<double2> pair(2 * (size_t)N);
    for (int p = 0; p < P && ok; ++p) {
        for (int i = 0; i < N; ++i) {  // (DUAL_bra, DUAL_ket) = (conj Psi_ket, Psi_bra)
            const double2 k = ket[(size_t)p * N + i];
            pair[2 * i] = make_double2(k.x, -k.y);
            pair[2 * i + 1] = bra[(size_t)p * N + i];
        }
        ok = put_record(f, pair.data(), pair.size() * sizeof(double2));
        for (int i = 0; i < N; ++i) {  // (AO_bra, AO_ket) = (conj S^-1 Psi_bra, Psi_ket)
            pair[2 * i] = ao_bra[(size_t)p * N + i];
            pair[2 * i + 1] = ket[(size_t)p * N + i];
        }
        ok = ok && put_record(f, pair.data(), pair.size() * sizeof(double2));
    }
    std::vector<double> qrep;
    for (int a = 0; a < tr->natoms; ++a) qrep.insert(qrep.end(), q.begin(), q.end());
    ok = ok && put_record(f, qrep.data(), qrep.size() * sizeof(double));
    std::vector<char> resume(sizeof(ResumeHead) + P * sizeof(double) + cols.size() * sizeof(double2));
    memcpy(resume.data(), &rh, sizeof(rh));
    memcpy(resume.data() + sizeof(rh), target.data(), P * sizeof(double));
    if (!cols.empty()) memcpy(resume.data() + sizeof(rh) + P * sizeof(double), cols.data(), cols.size() * sizeof(double2));
    ok = ok && put_record(f, resume.data(), resume.size());
    return ok ? ELHL_OK : ELHL_ERR_CUDA;
}

int traj_restore_impl(elhl_traj *tr, const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) return ELHL_ERR_BAD_ARG;
    FileCloser fc{f};
    std::vector<char> r;
    int it = 0, N = 0, P = 0, ntag = 0;
    double t = 0.0;
    auto get_int = [&](int &v) { return get_record(f, r) && r.size() == 4 && (memcpy(&v, r.data(), 4), true); };
    if (!get_int(it) || !(get_record(f, r) && r.size() == 8)) return ELHL_ERR_BAD_ARG;
    memcpy(&t, r.data(), 8);
    if (!get_int(N) || !get_int(P) || !get_int(ntag) || !get_record(f, r)) return ELHL_ERR_BAD_ARG;
    if (N != tr->N || P != tr->P) return ELHL_ERR_BAD_ARG;
    std::vector<double2> bra((size_t)N * P), ket((size_t)N * P);
    for (int p = 0; p < P; ++p) {
        if (!get_record(f, r) || r.size() != 2 * (size_t)N * sizeof(double2)) return ELHL_ERR_BAD_ARG;
        const double2 *d = reinterpret_cast<const double2 *>(r.data());
        for (int i = 0; i < N; ++i) bra[(size_t)p * N + i] = d[2 * i + 1];  // Psi_bra = DUAL_ket
        if (!get_record(f, r) || r.size() != 2 * (size_t)N * sizeof(double2)) return ELHL_ERR_BAD_ARG;
        d = reinterpret_cast<const double2 *>(r.data());
        for (int i = 0; i < N; ++i) ket[(size_t)p * N + i] = d[2 * i + 1];  // Psi_ket = AO_ket
    }
    if (!get_record(f, r)) return ELHL_ERR_BAD_ARG;  // Net_Charge
    ResumeHead rh{};
    std::vector<double> target;
    std::vector<char> res;
    if (get_record(f, res) && res.size() >= sizeof(ResumeHead)) {
        memcpy(&rh, res.data(), sizeof(rh));
        if (memcmp(rh.magic, kResumeMagic, 8) || rh.method != tr->cfg.method || rh.precision != tr->cfg.precision ||
            rh.N != N || rh.P != P || rh.ncols != tr->cfg.ncols)
            return ELHL_ERR_BAD_ARG;
        const size_t need = sizeof(rh) + P * sizeof(double) + (rh.has_cols ? (size_t)N * tr->cfg.ncols * 16 : 0);
        if (res.size() != need) return ELHL_ERR_BAD_ARG;
        target.assign(reinterpret_cast<const double *>(res.data() + sizeof(rh)),
                      reinterpret_cast<const double *>(res.data() + sizeof(rh)) + P);
    } else {
        res.clear();  // a checkpoint of the reference itself: Psi, t and it only
    }
    const size_t e = sizeof(double2);
    if (tr->cheb()) {
        ChebState &cs = tr->cs;
        for (int p = 0; p < P; ++p) {
            CU_TRY(cudaMemcpy2D(tr->psi_ao + p, P * e, ket.data() + (size_t)p * N, e, e, N, cudaMemcpyHostToDevice));
            CU_TRY(cudaMemcpy2D(tr->bra_ao + p, P * e, bra.data() + (size_t)p * N, e, e, N, cudaMemcpyHostToDevice));
        }
        if (res.empty()) {
            if (int rc = cheb_set_target(tr)) return rc;
        } else {
            CU_TRY(cudaMemcpy(tr->target, target.data(), P * sizeof(double), cudaMemcpyHostToDevice));
            cs.cols_current = false;
            if (!cs.implicit && (rh.emin != cs.emin || rh.emax != cs.emax)) {  // an interval widened by norm control
                cs.emin = rh.emin;
                cs.emax = rh.emax;
                if (int rc = cheb_prepare(cs, tr->cfg.dt * tr->cfg.frame_step, tr->cfg.cheb_tol)) return rc;
                if (!tr->plan.probs.empty()) {
                    std::vector<ChebState *> one{&cs};
                    if (int rc = cheb_plan_refresh(tr->plan, one)) return rc;
                }
            }
            if (rh.has_cols) {
                CU_TRY(cudaMemcpy(cs.cin(), res.data() + sizeof(rh) + P * sizeof(double), (size_t)N * cs.m * e,
                                  cudaMemcpyHostToDevice));
                cs.cols_current = true;
            }
        }
    } else {
        for (int p = 0; p < P; ++p) {
            CU_TRY(cudaMemcpy(tr->tb.bra(p), bra.data() + (size_t)p * N, N * e, cudaMemcpyHostToDevice));
            CU_TRY(cudaMemcpy(tr->tb.ket(p), ket.data() + (size_t)p * N, N * e, cudaMemcpyHostToDevice));
        }
    }
    tr->t = t;
    tr->it = it;
    if (!res.empty()) {
        tr->first_call = rh.first_call != 0;
        tr->save_tau[0] = rh.save_tau[0];
        tr->save_tau[1] = rh.save_tau[1];
    } else {
        tr->first_call = true;  // the reference's checkpoint has no tau: restart at tau_max
    }
    return ELHL_OK;
}

}  // namespace

extern "C" {

int elhl_traj_snapshot(elhl_traj *tr, const char *path) {
    if (!tr || !path) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    return traj_snapshot_impl(tr, path);
}

int elhl_traj_restore(elhl_traj *tr, const char *path) {
    if (!tr || !path) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    return traj_restore_impl(tr, path);
}

}  // extern "C"

// =============================== batches ========================================
// Many Chebyshev trajectories (fixed nuclei) advanced together: one cooperative
// launch per nuclear step covers every member's orders (persistent kernel over
// a row-segment work list balanced by matrix elements), then each member's
// columns are read out and its populations reduced.
struct elhl_batch {
    std::vector<elhl_traj *> members;
    ChebPlan plan;
    std::vector<ChebState *> states;
    double *pops = nullptr;
    size_t pops_cap = 0;
    bool compact = false;
    elhl_traj_stats stats{};
};

extern "C" {

int elhl_batch_create(int ntraj, const elhl_basis_desc *bases, const double *const *coords,
                      const elhl_traj_config *cfg, elhl_batch **out) {
    if (!out || ntraj <= 0 || !bases || !coords || !cfg) return ELHL_ERR_BAD_ARG;
    if (cfg->method != ELHL_METHOD_CHEBYSHEV || cfg->precision == ELHL_PREC_OZ64) return ELHL_ERR_UNSUPPORTED;
    *out = nullptr;
    elhl_batch *b = new elhl_batch();
    int rc = ELHL_OK;
    for (int i = 0; i < ntraj && !rc; ++i) {
        elhl_traj *tr = nullptr;
        rc = elhl_traj_create(&bases[i], coords[i], cfg, &tr);
        if (!rc) {
            b->members.push_back(tr);
            b->states.push_back(&tr->cs);
            if (tr->nfrag != b->members[0]->nfrag || tr->P != b->members[0]->P) rc = ELHL_ERR_BAD_ARG;
        }
    }
    if (!rc) {
        std::lock_guard<std::mutex> lk(g_ctx.mu);
        rc = cheb_plan(b->plan, b->states);
    }
    if (rc) {
        for (auto *tr : b->members) elhl_traj_destroy(tr);
        b->plan.release();
        delete b;
        return rc;
    }
    *out = b;
    return ELHL_OK;
}

int elhl_batch_size(elhl_batch *b) { return b ? (int)b->members.size() : 0; }

elhl_traj *elhl_batch_member(elhl_batch *b, int i) {
    if (!b || i < 0 || i >= (int)b->members.size()) return nullptr;
    return b->members[i];
}

int elhl_batch_compact(elhl_batch *b) {
    if (!b) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    for (auto *tr : b->members) {
        dev_free(tr->S); dev_free(tr->h); dev_free(tr->cs.Ht); dev_free(tr->cs.lz);
        tr->tb.release();
    }
    b->compact = true;
    return ELHL_OK;
}

int elhl_batch_step(elhl_batch *b, int nsteps, double *pops) {
    if (!b || nsteps <= 0) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    cudaStream_t st = g_ctx.stream;
    const int nt = (int)b->members.size(), P = b->members[0]->P, nf = b->members[0]->nfrag;
    const size_t per_traj = (size_t)P * (nf + 1), per_step = per_traj * nt;
    if (per_step * nsteps > b->pops_cap) {
        dev_free(b->pops);
        if (int rc = dev_alloc(&b->pops, per_step * nsteps)) return rc;
        b->pops_cap = per_step * nsteps;
    }
    memset(&b->stats, 0, sizeof(b->stats));
    if (!b->plan.mg_read) return ELHL_ERR_UNSUPPORTED;
    for (auto *tr : b->members)
        if (!tr->cs.cols_current)
            if (int rc = cheb_load_columns(tr)) return rc;
    (void)per_traj;
    CU_TRY(cudaMemsetAsync(b->plan.d_drift, 0, nt * sizeof(double), st));
    for (int s = 0; s < nsteps; ++s) {
        if (int rc = cheb_dev_step(b->plan, b->states, b->pops + s * per_step)) return rc;
        for (auto *tr : b->members) {
            tr->t = tr->t + tr->cfg.dt * tr->cfg.frame_step;
            tr->it += 1;
            tr->first_call = false;
        }
    }
    if (int rc = cheb_settle(b->states)) return rc;
    int err = 0;
    std::vector<double> drift(nt, 0.0);
    CU_TRY(cudaMemcpyAsync(&err, g_ctx.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaMemcpyAsync(drift.data(), b->plan.d_drift, nt * sizeof(double), cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    if (err) return err;
    // norm control: a member whose step changed a column's norm beyond the
    // tolerance fails the call (its stats carry the drift)
    bool diverged = false;
    for (int i = 0; i < nt; ++i) {
        b->members[i]->stats.norm_drift = drift[i];
        b->stats.norm_drift = std::max(b->stats.norm_drift, drift[i]);
        diverged |= !(drift[i] <= cheb_norm_tolerance(b->members[i]->cfg));
    }
    if (diverged) return ELHL_ERR_NO_CONVERGENCE;
    b->stats.prop_ms += event_ms(0, 1) * nsteps;
    b->stats.prop_launches += nsteps;
    b->stats.tile_cols = b->plan.mg;
    b->stats.phases = b->plan.nphase;
    for (auto *cs : b->states) b->stats.orders += (long long)cs->K * cs->m * nsteps;
    b->stats.substeps += (long long)nt * nsteps;
    if (pops) CU_TRY(copy_d2h(pops, b->pops, per_step * nsteps * sizeof(double)));
    return ELHL_OK;
}

int elhl_batch_get_stats(elhl_batch *b, elhl_traj_stats *st) {
    if (!b || !st) return ELHL_ERR_BAD_ARG;
    *st = b->stats;
    return ELHL_OK;
}

int elhl_batch_destroy(elhl_batch *b) {
    if (!b) return ELHL_ERR_BAD_ARG;
    for (auto *tr : b->members) elhl_traj_destroy(tr);
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    b->plan.release();
    dev_free(b->pops);
    delete b;
    return ELHL_OK;
}

}  // extern "C"

// =============================== serving ========================================
// Continuous batching of propagation requests: requests wait FIFO until their
// estimated device memory fits the HBM budget, are set up on the device
// (S, h, L, H~, bounds, fragment-MO initial columns), join the running batch at
// the next step boundary, and leave it when their step count is reached.  Every
// server step is one cooperative launch over all active requests.
#include <chrono>
#include <deque>
#include <map>

struct ServerRequest {
    long long id = 0;
    int nsteps = 0, done_steps = 0, P = 0, nfrag = 0, natoms = 0, nao = 0;
    std::vector<int> ao0, naoat, n, l, m, nz, frag, frag_atoms, states;
    std::vector<double> zeta, coef, ip, kwh, vs, coords;
    double bytes = 0.0;
    elhl_traj *tr = nullptr;
    std::vector<double> pops;          // last populations, P x (nfrag+1)
    std::vector<double2> psi;          // final ket, N x P (column-major)
    int status = ELHL_OK;
    double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;  // seconds, host steady clock
    std::string restart;               // checkpoint to resume from at admission (empty: initial states)
    int group = -1;                    // row-kernel group index, or -1: GEMM regime (own step graph)
    size_t pops_off = 0;               // offset of its populations in the group's block
};

// Requests whose bases allow the same staged column-group size (4, 2 or 1:
// the whole previous vector of a group sits in shared memory) share one plan
// and one cooperative launch per server step, so that one large basis does
// not force single columns on every other request.
struct ServerGroup {
    std::vector<ServerRequest *> reqs;
    ChebPlan plan;
    bool dirty = true;
    int parity = 0;
    double *pops = nullptr;
    size_t pops_cap = 0;
};
constexpr int kServerGroups = 4;  // FP64 read-out with column-group size 4, 2, 1; read-out in the launch precision

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct elhl_server {
    elhl_traj_config cfg;
    double budget = 0.0, used = 0.0;
    std::deque<ServerRequest *> pending;
    std::vector<ServerRequest *> active;  // admission order
    std::map<long long, ServerRequest *> finished;
    std::vector<long long> newly_done;
    ServerGroup groups[kServerGroups];
    long long next_id = 1;
    long long steps_done = 0;
};

static double request_bytes(const elhl_traj_config &cfg, int nao, int P) {
    const double ld = (double)round_up(nao, 32), tsz = wide_storage(cfg.precision) ? 8.0 : 4.0;
    // set-up peak: S, h, H~, L, G (FP64) + Hs + read-out matrices (FP64) + vectors, and
    // for the sliced set-up products (every precision but FP64) the slices of both
    // operands of an N x N x N product: 2 x 7 BF16 slices of N^2 elements
    const double slices = (cfg.precision != ELHL_PREC_FP64 && nao >= 320) ? 28.0 * nao * nao : 0.0;
    return ld * nao * (5 * 8.0 + tsz + 2 * 8.0) + ld * cfg.ncols / cfg.nparticles * P * (3 * 2 * tsz + 2 * 16.0) +
           slices + 1e6;
}

static int server_admit(elhl_server *sv, ServerRequest *r) {
    elhl_basis_desc d{};
    d.natoms = r->natoms; d.nao = r->nao;
    d.atom_ao0 = r->ao0.data(); d.atom_nao = r->naoat.data();
    d.ao_n = r->n.data(); d.ao_l = r->l.data(); d.ao_m = r->m.data(); d.ao_nzeta = r->nz.data();
    d.ao_zeta = r->zeta.data(); d.ao_coef = r->coef.data(); d.ao_ip = r->ip.data(); d.ao_kwh = r->kwh.data();
    d.ao_vshift = r->vs.data(); d.ao_frag = r->frag.data(); d.nfrag = r->nfrag;
    elhl_traj_config c = sv->cfg;
    c.nparticles = r->P;
    c.ncols = r->P;  // ket columns only (fixed nuclei: bra = S ket)
    if (int rc = elhl_traj_create(&d, r->coords.data(), &c, &r->tr)) return rc;
    if (int rc = elhl_traj_init_fmo_states(r->tr, (int)r->frag_atoms.size(), r->frag_atoms.data(), r->P,
                                           r->states.data()))
        return rc;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    elhl_traj *tr = r->tr;
    if (tr->cs.gemm) {
        r->group = -1;  // many columns on a large basis: one GEMM per order, its own step graph
    } else {
        const ChebState &cs = tr->cs;
        const int mg = cheb_group_size(cs.ro64 ? ELHL_PREC_FP64 : tr->cfg.precision, 4, tr->ld);
        if (!mg) return ELHL_ERR_UNSUPPORTED;  // the vector does not fit in shared memory
        r->group = !cs.ro64 ? 3 : mg == 4 ? 0 : mg == 2 ? 1 : 2;
        tr->cs.parity = sv->groups[r->group].parity;  // join the running group's column roles
    }
    if (!r->restart.empty())
        if (int rc = traj_restore_impl(tr, r->restart.c_str())) return rc;
    if (!tr->cs.cols_current)
        if (int rc = cheb_load_columns(tr)) return rc;
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    dev_free(tr->S); dev_free(tr->h); dev_free(tr->cs.Ht); dev_free(tr->cs.lz);
    return ELHL_OK;
}

extern "C" {

int elhl_server_create(double hbm_budget_bytes, const elhl_traj_config *cfg, elhl_server **out) {
    if (!out || !cfg || !(hbm_budget_bytes > 0.0)) return ELHL_ERR_BAD_ARG;
    if (cfg->method != ELHL_METHOD_CHEBYSHEV || cfg->precision == ELHL_PREC_OZ64) return ELHL_ERR_UNSUPPORTED;
    if (int rc = ensure_context()) return rc;
    elhl_server *sv = new elhl_server();
    sv->cfg = *cfg;
    sv->budget = hbm_budget_bytes;
    *out = sv;
    return ELHL_OK;
}

static int server_submit(elhl_server *sv, const elhl_request *q, const char *restart, long long *id);

int elhl_server_submit(elhl_server *sv, const elhl_request *q, long long *id) {
    return server_submit(sv, q, nullptr, id);
}

int elhl_server_submit_restart(elhl_server *sv, const elhl_request *q, const char *path, long long *id) {
    if (!path) return ELHL_ERR_BAD_ARG;
    return server_submit(sv, q, path, id);
}

int elhl_server_snapshot(elhl_server *sv, long long id, const char *path) {
    if (!sv || !path) return ELHL_ERR_BAD_ARG;
    for (auto *r : sv->active) {
        if (r->id != id) continue;
        std::lock_guard<std::mutex> lk(g_ctx.mu);
        std::vector<ChebState *> one{&r->tr->cs};
        if (int rc = cheb_settle(one)) return rc;  // apply the pending renormalisation (bit-neutral)
        return traj_snapshot_impl(r->tr, path);
    }
    return ELHL_ERR_BAD_ARG;  // not admitted yet, or finished
}

static int server_submit(elhl_server *sv, const elhl_request *q, const char *restart, long long *id) {
    if (!sv || !q || !q->basis || !q->coords || q->nsteps <= 0 || q->nparticles < 1 || q->nparticles > 64 ||
        !q->frag_atoms || q->n_frag_atoms <= 0 || !q->states)
        return ELHL_ERR_BAD_ARG;
    if (int rc = validate_basis(q->basis)) return rc;
    const elhl_basis_desc *b = q->basis;
    ServerRequest *r = new ServerRequest();
    r->nsteps = q->nsteps; r->P = q->nparticles; r->nfrag = b->nfrag; r->natoms = b->natoms; r->nao = b->nao;
    r->ao0.assign(b->atom_ao0, b->atom_ao0 + b->natoms);
    r->naoat.assign(b->atom_nao, b->atom_nao + b->natoms);
    r->n.assign(b->ao_n, b->ao_n + b->nao); r->l.assign(b->ao_l, b->ao_l + b->nao);
    r->m.assign(b->ao_m, b->ao_m + b->nao); r->nz.assign(b->ao_nzeta, b->ao_nzeta + b->nao);
    r->zeta.assign(b->ao_zeta, b->ao_zeta + 2 * b->nao); r->coef.assign(b->ao_coef, b->ao_coef + 2 * b->nao);
    r->ip.assign(b->ao_ip, b->ao_ip + b->nao); r->kwh.assign(b->ao_kwh, b->ao_kwh + b->nao);
    r->vs.assign(b->ao_vshift, b->ao_vshift + b->nao);
    if (b->ao_frag) r->frag.assign(b->ao_frag, b->ao_frag + b->nao); else r->frag.assign(b->nao, 0);
    r->coords.assign(q->coords, q->coords + 3 * b->natoms);
    r->frag_atoms.assign(q->frag_atoms, q->frag_atoms + q->n_frag_atoms);
    r->states.assign(q->states, q->states + q->nparticles);
    if (restart) r->restart = restart;
    r->bytes = request_bytes(sv->cfg, b->nao, r->P);
    if (r->bytes > sv->budget) {
        delete r;
        return ELHL_ERR_OOM;  // can never be admitted
    }
    r->id = sv->next_id++;
    r->t_submit = now_s();
    sv->pending.push_back(r);
    if (id) *id = r->id;
    return ELHL_OK;
}

int elhl_server_step(elhl_server *sv, int *n_active, int *n_pending) {
    if (!sv) return ELHL_ERR_BAD_ARG;
    // admission, FIFO, within the budget
    while (!sv->pending.empty() && sv->used + sv->pending.front()->bytes <= sv->budget) {
        ServerRequest *r = sv->pending.front();
        sv->pending.pop_front();
        r->t_admit = now_s();
        int rc = server_admit(sv, r);
        if (rc) {
            r->status = rc;
            r->t_done = now_s();
            if (r->tr) elhl_traj_destroy(r->tr);
            r->tr = nullptr;
            sv->finished[r->id] = r;
            sv->newly_done.push_back(r->id);
            continue;
        }
        sv->used += r->bytes;
        sv->active.push_back(r);
        if (r->group >= 0) {
            sv->groups[r->group].reqs.push_back(r);
            sv->groups[r->group].dirty = true;
        }
    }
    if (!sv->active.empty()) {
        std::lock_guard<std::mutex> lk(g_ctx.mu);
        cudaStream_t st = g_ctx.stream;
        // one cooperative launch per non-empty group, one step graph per GEMM-regime request
        for (auto &g : sv->groups) {
            if (g.reqs.empty()) continue;
            std::vector<ChebState *> states;
            for (auto *r : g.reqs) states.push_back(&r->tr->cs);
            if (g.dirty) {
                if (int rc = cheb_plan(g.plan, states)) return rc;
                if (!g.plan.mg_read) return ELHL_ERR_UNSUPPORTED;
                g.dirty = false;
            }
            size_t need = 0;
            for (auto *r : g.reqs) {
                r->pops_off = need;
                need += (size_t)r->P * (r->nfrag + 1);
            }
            if (need > g.pops_cap) {
                dev_free(g.pops);
                if (int rc = dev_alloc(&g.pops, need)) return rc;
                g.pops_cap = need;
            }
            CU_TRY(cudaMemsetAsync(g.plan.d_drift, 0, g.reqs.size() * sizeof(double), st));
            if (int rc = cheb_dev_step(g.plan, states, g.pops)) return rc;
            g.parity = g.plan.parity;
        }
        for (auto *r : sv->active) {
            if (r->group >= 0) continue;
            CU_TRY(cudaMemsetAsync(r->tr->cs.drift, 0, sizeof(double), st));
            if (int rc = cheb_gemm_step(r->tr->cs)) return rc;
        }
        std::vector<ChebState *> leaving;
        for (auto *r : sv->active)
            if (r->done_steps + 1 >= r->nsteps) leaving.push_back(&r->tr->cs);
        if (!leaving.empty())
            if (int rc = cheb_settle(leaving)) return rc;
        int err = 0;
        std::vector<double> drift(sv->active.size(), 0.0);
        CU_TRY(cudaMemcpyAsync(&err, g_ctx.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        for (size_t q = 0; q < sv->active.size(); ++q) {
            const ServerRequest *r = sv->active[q];
            const double *d = r->group < 0 ? r->tr->cs.drift : sv->groups[r->group].plan.d_drift;
            if (r->group >= 0) {
                const auto &reqs = sv->groups[r->group].reqs;
                d += std::find(reqs.begin(), reqs.end(), r) - reqs.begin();
            }
            CU_TRY(cudaMemcpyAsync(&drift[q], d, sizeof(double), cudaMemcpyDeviceToHost, st));
        }
        CU_TRY(cudaStreamSynchronize(st));
        if (err) return err;
        sv->steps_done += (long long)sv->active.size();
        // retire finished requests, and requests whose step failed the norm control
        // (status ELHL_ERR_NO_CONVERGENCE, results as of that step)
        std::vector<ServerRequest *> keep;
        for (size_t q = 0; q < sv->active.size(); ++q) {
            ServerRequest *r = sv->active[q];
            r->done_steps += 1;
            r->tr->t += r->tr->cfg.dt * r->tr->cfg.frame_step;
            r->tr->it += 1;
            r->tr->first_call = false;
            const size_t np = (size_t)r->P * (r->nfrag + 1);
            if (!(drift[q] <= cheb_norm_tolerance(r->tr->cfg))) r->status = ELHL_ERR_NO_CONVERGENCE;
            if (r->done_steps >= r->nsteps || r->status) {
                r->pops.resize(np);
                const double *src = r->group < 0 ? r->tr->cs.gpops : sv->groups[r->group].pops + r->pops_off;
                CU_TRY(copy_d2h(r->pops.data(), src, np * sizeof(double)));
                r->psi.resize((size_t)r->nao * r->P);
                const size_t e = sizeof(double2);
                for (int p = 0; p < r->P; ++p)
                    CU_TRY(cudaMemcpy2D(r->psi.data() + (size_t)p * r->nao, e, r->tr->psi_ao + p, r->P * e, e, r->nao,
                                        cudaMemcpyDeviceToHost));
                r->t_done = now_s();
                sv->used -= r->bytes;
                if (r->group >= 0) {
                    auto &g = sv->groups[r->group];
                    g.reqs.erase(std::find(g.reqs.begin(), g.reqs.end(), r));
                    g.dirty = true;
                }
                sv->finished[r->id] = r;
                sv->newly_done.push_back(r->id);
            } else {
                keep.push_back(r);
            }
        }
        sv->active.swap(keep);
    }
    // destroy retired trajectories outside the context lock
    for (auto id : sv->newly_done) {
        ServerRequest *r = sv->finished[id];
        if (r->tr) {
            elhl_traj_destroy(r->tr);
            r->tr = nullptr;
        }
    }
    if (n_active) *n_active = (int)sv->active.size();
    if (n_pending) *n_pending = (int)sv->pending.size();
    return ELHL_OK;
}

int elhl_server_poll(elhl_server *sv, long long *ids, int max, int *n) {
    if (!sv || !n || (max > 0 && !ids)) return ELHL_ERR_BAD_ARG;
    int k = 0;
    while (k < max && !sv->newly_done.empty()) {
        ids[k++] = sv->newly_done.front();
        sv->newly_done.erase(sv->newly_done.begin());
    }
    *n = k;
    return ELHL_OK;
}

int elhl_server_result(elhl_server *sv, long long id, double *pops, elhl_zcomplex *psi_ket, double *times) {
    if (!sv) return ELHL_ERR_BAD_ARG;
    auto it = sv->finished.find(id);
    if (it == sv->finished.end()) return ELHL_ERR_BAD_ARG;
    ServerRequest *r = it->second;
    if (pops && !r->pops.empty()) memcpy(pops, r->pops.data(), r->pops.size() * sizeof(double));
    if (psi_ket && !r->psi.empty()) memcpy(psi_ket, r->psi.data(), r->psi.size() * sizeof(double2));
    if (times) {
        times[0] = r->t_submit;
        times[1] = r->t_admit;
        times[2] = r->t_done;
    }
    const int st = r->status;
    sv->finished.erase(it);
    delete r;
    return st;
}

int elhl_server_destroy(elhl_server *sv) {
    if (!sv) return ELHL_ERR_BAD_ARG;
    for (auto *r : sv->pending) delete r;
    for (auto *r : sv->active) {
        if (r->tr) elhl_traj_destroy(r->tr);
        delete r;
    }
    for (auto &kv : sv->finished) {
        if (kv.second->tr) elhl_traj_destroy(kv.second->tr);
        delete kv.second;
    }
    {
        std::lock_guard<std::mutex> lk(g_ctx.mu);
        for (auto &g : sv->groups) {
            g.plan.release();
            dev_free(g.pops);
        }
    }
    delete sv;
    return ELHL_OK;
}

}  // extern "C"
