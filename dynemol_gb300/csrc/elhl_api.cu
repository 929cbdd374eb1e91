// Host runtime of libelhlprop.so: device context, the reference's drop-in
// symbols and the native trajectory API (include/elhl_prop.h).
//
// Per nuclear step (ElHl_Chebyshev, ElHl_Chebyshev.f:148-291) everything stays
// on the device: S and h from coordinates (build_sh.cu), the Cholesky factor
// S = L L^T and H' = S^-1 h by two triangular solves (cuSOLVER potrf/potrs,
// replacing the reference's LU inverse + dsymm, Taylor_gpu.cpp:686-697), the
// propagation (taylor.cu) and the populations.  Host traffic per step is the
// coordinates in and the populations out.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "elhl_internal.cuh"

using namespace elhl;

namespace {

thread_local int g_last_status = ELHL_OK;

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
    unsigned *bar = nullptr;  // [2] count, gen
    int *err = nullptr;
    double *partials = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // prop begin/end, rebuild begin/end
    std::mutex mu;
};
Context g_ctx;

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
    CU_TRY(cudaStreamCreateWithFlags(&g_ctx.own_stream, cudaStreamNonBlocking));
    g_ctx.stream = g_ctx.own_stream;
    CU_TRY(cudaStreamCreateWithFlags(&g_ctx.copy_stream, cudaStreamNonBlocking));
    SOLVER_TRY(cusolverDnCreate(&g_ctx.solver));
    SOLVER_TRY(cusolverDnSetStream(g_ctx.solver, g_ctx.stream));
    if (int rc = dev_alloc(&g_ctx.bar, 2)) return rc;
    if (int rc = dev_alloc(&g_ctx.err, 1)) return rc;
    if (int rc = dev_alloc(&g_ctx.partials, (size_t)2 * 2 * g_ctx.grid * 16)) return rc;
    CU_TRY(cudaMemset(g_ctx.bar, 0, 2 * sizeof(unsigned)));
    CU_TRY(cudaMemset(g_ctx.err, 0, sizeof(int)));
    for (auto &e : g_ctx.ev) CU_TRY(cudaEventCreate(&e));
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
                          double2 *__restrict__ ket_full) {
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
    for (int k = threadIdx.x; k < nf; k += blockDim.x) ket_full[aos[k]] = make_double2(sign * c[k], 0.0);
}

// bra = S ket for a ket supported on the AO list `aos` (real coefficients)
__global__ void s_times_sparse(const double *__restrict__ S, int ld, int n, const int *__restrict__ aos, int nf,
                               const double2 *__restrict__ ket, double2 *__restrict__ bra) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = 0.0;
    for (int k = 0; k < nf; ++k) {
        const int j = aos[k];
        acc += S[(size_t)j * ld + i] * ket[j].x;  // S symmetric: S(i, j) = S(j, i)
    }
    bra[i] = make_double2(acc, 0.0);
}

// ---- H' = S^-1 h via Cholesky ------------------------------------------------
struct Factor {
    int N = 0, ld = 0, lwork = 0;
    double *L = nullptr;     // Cholesky factor (lower), N x N, ld
    double *work = nullptr;
    int *info = nullptr;
    double *cols = nullptr;  // N x 2 scratch (S^-1 applied to a complex vector)
    int reserve(int N_, int ld_) {
        if (N_ <= N && ld_ == ld && L) return ELHL_OK;
        release();
        N = N_;
        ld = ld_;
        if (int rc = dev_alloc(&L, (size_t)ld * N)) return rc;
        if (cusolverDnDpotrf_bufferSize(g_ctx.solver, CUBLAS_FILL_MODE_LOWER, N, L, ld, &lwork) !=
            CUSOLVER_STATUS_SUCCESS)
            return ELHL_ERR_CUDA;
        if (int rc = dev_alloc(&work, (size_t)lwork + 1)) return rc;
        if (int rc = dev_alloc(&info, 2)) return rc;
        if (int rc = dev_alloc(&cols, (size_t)2 * ld)) return rc;
        return ELHL_OK;
    }
    void release() {
        dev_free(L); dev_free(work); dev_free(info); dev_free(cols);
        N = 0;
    }
    // L <- chol(S); Hp <- S^-1 h.  Asynchronous on the context stream.
    int form_hprime(const double *S, const double *h, double *Hp, int n) {
        cudaStream_t st = g_ctx.stream;
        CU_TRY(cudaMemcpy2DAsync(L, ld * sizeof(double), S, ld * sizeof(double), n * sizeof(double), n,
                                 cudaMemcpyDeviceToDevice, st));
        SOLVER_TRY(cusolverDnDpotrf(g_ctx.solver, CUBLAS_FILL_MODE_LOWER, n, L, ld, work, lwork, info));
        CU_TRY(cudaMemcpy2DAsync(Hp, ld * sizeof(double), h, ld * sizeof(double), n * sizeof(double), n,
                                 cudaMemcpyDeviceToDevice, st));
        SOLVER_TRY(cusolverDnDpotrs(g_ctx.solver, CUBLAS_FILL_MODE_LOWER, n, n, L, ld, Hp, ld, info + 1));
        return ELHL_OK;
    }
    // out = S^-1 z for a complex vector z (device), using the factor.
    int apply_sinv(const double2 *z, double2 *out, int n) {
        cudaStream_t st = g_ctx.stream;
        const int tb = 256, nb = (n + tb - 1) / tb;
        split_complex<<<nb, tb, 0, st>>>(z, cols, n, ld);
        SOLVER_TRY(cusolverDnDpotrs(g_ctx.solver, CUBLAS_FILL_MODE_LOWER, n, 2, L, ld, cols, ld, info + 1));
        join_complex<<<nb, tb, 0, st>>>(cols, out, n, ld);
        CU_TRY(cudaGetLastError());
        return ELHL_OK;
    }
    int check_info() {
        int h[2] = {0, 0};
        CU_TRY(cudaMemcpy(h, info, 2 * sizeof(int), cudaMemcpyDeviceToHost));
        if (h[0] > 0) return ELHL_ERR_NOT_POSITIVE_DEFINITE;
        if (h[0] < 0 || h[1] != 0) return ELHL_ERR_BAD_ARG;
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
    L.bar_gen = g_ctx.bar + 1;
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
    int reserve(int N_) {
        const int ld_ = round_up(N_, 32);
        if (S && N_ <= N && ld_ == ld) return ELHL_OK;
        release();
        N = N_;
        ld = ld_;
        if (int rc = dev_alloc(&S, (size_t)ld * N)) return rc;
        if (int rc = dev_alloc(&h, (size_t)ld * N)) return rc;
        if (int rc = dev_alloc(&Hp, (size_t)ld * N)) return rc;
        if (int rc = dev_alloc(&ao, (size_t)ld)) return rc;
        if (int rc = fac.reserve(N, ld)) return rc;
        if (int rc = tb.reserve(N, 1)) return rc;
        return ELHL_OK;
    }
    void release() {
        dev_free(S); dev_free(h); dev_free(Hp); dev_free(ao);
        fac.release();
        tb.release();
        N = 0;
    }
};
DropIn g_drop;

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
    // H' back to the host on a second stream, overlapped with the propagation (Taylor_gpu.cpp:700)
    cudaEvent_t ev;
    CU_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CU_TRY(cudaEventRecord(ev, st));
    CU_TRY(cudaStreamWaitEvent(g_ctx.copy_stream, ev, 0));
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
    cudaEventDestroy(ev);
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
};

namespace {

int upload_basis(DevBasis &d, const elhl_basis_desc *b) {
    d.natoms = b->natoms;
    d.nao = b->nao;
    d.nfrag = b->nfrag;
    auto up_i = [](int **dst, const int *src, size_t n) -> int {
        if (int rc = dev_alloc(dst, n)) return rc;
        CU_TRY(cudaMemcpy(*dst, src, n * sizeof(int), cudaMemcpyHostToDevice));
        return ELHL_OK;
    };
    auto up_d = [](double **dst, const double *src, size_t n) -> int {
        if (int rc = dev_alloc(dst, n)) return rc;
        CU_TRY(cudaMemcpy(*dst, src, n * sizeof(double), cudaMemcpyHostToDevice));
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
    return rc ? ELHL_ERR_CUDA : ELHL_OK;
}

void free_basis(DevBasis &d) {
    dev_free(d.atom_ao0); dev_free(d.atom_nao); dev_free(d.ao_n); dev_free(d.ao_l); dev_free(d.ao_m);
    dev_free(d.ao_nzeta); dev_free(d.ao_zeta); dev_free(d.ao_coef); dev_free(d.ao_ip); dev_free(d.ao_kwh);
    dev_free(d.ao_vshift); dev_free(d.ao_frag);
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
    int rc = tr->fac.form_hprime(tr->S, tr->h, tr->Hp, tr->N);
    CU_TRY(cudaEventRecord(g_ctx.ev[3], g_ctx.stream));
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
        CU_TRY(cudaMemcpy(pops, d_pops, nsteps * pop_per_step * sizeof(double), cudaMemcpyDeviceToHost));
    return ELHL_OK;
}

// Initial state of particle p from fragment MO `state` (1-based).
int fmo_particle(elhl_traj *tr, int nat, const int *atoms, int state, int p) {
    if (nat <= 0 || !atoms || state < 1) return ELHL_ERR_BAD_ARG;
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
    CU_TRY(cudaMemcpy(all.data(), tr->last_coords, all.size() * sizeof(double), cudaMemcpyDeviceToHost));
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
    if (!rc && cudaMemcpy(dc, sub.data(), sub.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) rc = ELHL_ERR_CUDA;
    if (!rc && cudaMemcpy(daos, aos.data(), nf * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) rc = ELHL_ERR_CUDA;
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
        double2 *ket = tr->tb.ket(p), *bra = tr->tb.bra(p);
        if (cudaMemsetAsync(ket, 0, tr->N * sizeof(double2), st) != cudaSuccess) rc = ELHL_ERR_CUDA;
        embed_fmo<<<1, 256, 0, st>>>(hf, ldf, nf, state - 1, daos, ket);
        s_times_sparse<<<(tr->N + 127) / 128, 128, 0, st>>>(tr->S, tr->ld, tr->N, daos, nf, ket, bra);
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

int elhl_set_stream(void *stream) {
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (int rc = ensure_context_locked(-1)) return rc;
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    g_ctx.stream = stream ? (cudaStream_t)stream : g_ctx.own_stream;
    SOLVER_TRY(cusolverDnSetStream(g_ctx.solver, g_ctx.stream));
    return ELHL_OK;
}

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
    if (g_ctx.own_stream) cudaStreamDestroy(g_ctx.own_stream);
    if (g_ctx.copy_stream) cudaStreamDestroy(g_ctx.copy_stream);
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
}

int elhl_traj_create(const elhl_basis_desc *basis, const double *coords, const elhl_traj_config *cfg,
                     elhl_traj **out) {
    if (!out || !coords) return ELHL_ERR_BAD_ARG;
    *out = nullptr;
    if (int rc = validate_basis(basis)) return rc;
    if (int rc = ensure_context()) return rc;
    elhl_traj *tr = new elhl_traj();
    if (cfg) tr->cfg = *cfg; else elhl_traj_config_default(&tr->cfg);
    if (tr->cfg.method != ELHL_METHOD_TAYLOR_REF || tr->cfg.precision != ELHL_PREC_FP64 || tr->cfg.dt <= 0 ||
        tr->cfg.frame_step <= 0 || tr->cfg.max_conv_calls <= 0) {
        delete tr;
        return ELHL_ERR_UNSUPPORTED;
    }
    tr->N = basis->nao;
    tr->ld = round_up(tr->N, 32);
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
    if (!rc) rc = dev_alloc(&tr->Hp, (size_t)tr->ld * tr->N);
    if (!rc) rc = dev_alloc(&tr->coords, (size_t)tr->natoms * 3);
    if (!rc) tr->coords_cap = tr->natoms * 3;
    if (!rc) rc = tr->fac.reserve(tr->N, tr->ld);
    if (!rc) rc = tr->tb.reserve(tr->N, tr->P);
    if (!rc && cudaMemcpy(tr->coords, coords, tr->natoms * 3 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = ELHL_ERR_CUDA;
    if (!rc) rc = rebuild(tr, tr->coords);
    if (!rc && cudaStreamSynchronize(g_ctx.stream) != cudaSuccess) rc = ELHL_ERR_CUDA;
    if (!rc) rc = tr->fac.check_info();
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
    delete tr;
    return ELHL_OK;
}

int elhl_traj_init_fmo(elhl_traj *tr, int n_el_atoms, const int *el_atoms, int electron_state, int n_hl_atoms,
                       const int *hl_atoms, int hole_state) {
    if (!tr) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (int rc = fmo_particle(tr, n_el_atoms, el_atoms, electron_state, 0)) return rc;
    return fmo_particle(tr, n_hl_atoms, hl_atoms, hole_state, 1);
}

int elhl_traj_set_psi(elhl_traj *tr, const elhl_zcomplex *bra, const elhl_zcomplex *ket) {
    if (!tr || !bra || !ket) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    for (int p = 0; p < tr->P; ++p) {
        CU_TRY(cudaMemcpy(tr->tb.bra(p), bra + (size_t)p * tr->N, tr->N * sizeof(double2), cudaMemcpyHostToDevice));
        CU_TRY(cudaMemcpy(tr->tb.ket(p), ket + (size_t)p * tr->N, tr->N * sizeof(double2), cudaMemcpyHostToDevice));
    }
    return ELHL_OK;
}

int elhl_traj_get_psi(elhl_traj *tr, elhl_zcomplex *bra, elhl_zcomplex *ket) {
    if (!tr) return ELHL_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    CU_TRY(cudaStreamSynchronize(g_ctx.stream));
    for (int p = 0; p < tr->P; ++p) {
        if (bra) CU_TRY(cudaMemcpy(bra + (size_t)p * tr->N, tr->tb.bra(p), tr->N * sizeof(double2), cudaMemcpyDeviceToHost));
        if (ket) CU_TRY(cudaMemcpy(ket + (size_t)p * tr->N, tr->tb.ket(p), tr->N * sizeof(double2), cudaMemcpyDeviceToHost));
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
    if (Hp) CU_TRY(cudaMemcpy2D(Hp, col, tr->Hp, ldb, col, tr->N, cudaMemcpyDeviceToHost));
    return ELHL_OK;
}

int elhl_traj_get_stats(elhl_traj *tr, elhl_traj_stats *st) {
    if (!tr || !st) return ELHL_ERR_BAD_ARG;
    *st = tr->stats;
    st->save_tau[0] = tr->save_tau[0];
    st->save_tau[1] = tr->save_tau[1];
    st->t = tr->t;
    st->it = tr->it;
    return ELHL_OK;
}

}  // extern "C"
