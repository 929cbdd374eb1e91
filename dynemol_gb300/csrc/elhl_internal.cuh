// Internal declarations shared by the translation units of libelhlprop.so.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../include/elhl_prop.h"

namespace elhl {

// Kernels of this library launched so far (graph replays counted per kernel
// node), for the launch accounting of benchmarks: count_launch() follows every
// launch site.
void count_launch(long long n = 1);
long long own_launches();

constexpr double kHbar = 6.58264e-4;  // eV ps (constants_m.f:23)
constexpr int kOrder = 25;            // Taylor order cap (Taylor.f:20)
constexpr int kMaxFrag = 8;           // fragments tracked by the population reduction

// ---- device-side STO basis (structure of arrays) --------------------------
struct DevBasis {
    int natoms = 0, nao = 0, nfrag = 0;
    int *atom_ao0 = nullptr, *atom_nao = nullptr;
    int *ao_n = nullptr, *ao_l = nullptr, *ao_m = nullptr, *ao_nzeta = nullptr, *ao_frag = nullptr;
    double *ao_zeta = nullptr, *ao_coef = nullptr, *ao_ip = nullptr, *ao_kwh = nullptr, *ao_vshift = nullptr;
    int *atom_order = nullptr;  // atoms grouped by kind (same AO signature): the S/h build's pair order
};

// One-time per-device fill of the overlap kernel's constant tables.
cudaError_t init_build_tables();

// S and h (both N x N, column-major, leading dimension ld) from coordinates.
// Hueckel Hamiltonian with environment fields (h zeroed by the caller)
cudaError_t launch_huckel_fields(const DevBasis &b, const double *d_coords, double cutoff, const double *d_S, int lds,
                                 const double *d_dp_ao, const double *d_dp4, double *d_h, int ldh, cudaStream_t st);
// Ehrenfest Pulay forces: F (natoms^2 x 3 scratch) and force (natoms x 3) on the device
cudaError_t launch_pulay_forces(const DevBasis &b, const double *d_coords, double cutoff, double delta,
                                const double *d_kernel, int ldk, double *d_F, double scale, double *d_force,
                                cudaStream_t st);
cudaError_t launch_build_sh(const DevBasis &b, const double *d_coords, double cutoff, double *d_S,
                            double *d_h, int ld, cudaStream_t st);

// ---- Taylor persistent engine ---------------------------------------------
// Per-particle control, in device memory.  Written by the host before the
// launch (tau, t_init, t_max) and by the kernel (results).
struct TaylorParticle {
    double tau_in;     // initial tau of the step
    double save_tau;   // out: tau accepted by the first convergence
    double tau_out;    // out: tau at the end (the reference's inout tau)
    long long orders;  // out: expansion orders executed
    int conv_calls;    // out
    int substeps;      // out
    int status;        // out: ELHL_OK / ELHL_ERR_NO_CONVERGENCE / ELHL_ERR_TIMEOUT
    int psi_slot;      // out: slot holding the propagated Psi
};

struct TaylorLaunch {
    const double *H;      // H' (N x N, ld)
    int N, ld;
    int nparticles;       // 1 or 2
    double2 *slots;       // [nparticles][kSlots][2 (bra,ket)][ldv]; Psi in slot 0 in and out
    int ldv;              // vector stride (>= N)
    TaylorParticle *part; // [nparticles]
    double t_init, t_max;
    double tol, norm_tol;
    int max_conv_calls;
    // multi-step mode (fixed nuclei): nsteps > 1 runs the step driver on the device
    int nsteps;
    int it0;              // reference counter `it` before the first step
    double dt_frame;      // dt * frame_step
    double tau_max;
    double *pops;         // [nsteps][nparticles][nfrag+1] or nullptr
    const int *ao_frag;
    int nfrag;
    double *t_final;      // out: time after the last step
    // scratch
    double *partials;     // [2][nparticles][grid][4]
    double *pop_partials; // [grid][nparticles][kMaxFrag+1]
    unsigned *bar_count;  // grid barrier: two words, one 64-bit count (8-byte aligned, zero at the launch)
    int *error;           // global error flag
};
constexpr int kSlots = 6;

cudaError_t launch_taylor(const TaylorLaunch &L, int grid, int block, cudaStream_t st);
int taylor_grid_size(int block, int *grid_out);
// Loads the allocation-free entry point's module on the current device and
// resolves its fixed scratch (noalloc.cu); ELHL_OK or an error status.
int fixed_scratch_prepare();
constexpr int kTaylorBlock = 256;

// ---- Chebyshev engine (cheb.cu, chebcoef.cu) ---------------------------------
constexpr int kMaxCols = 64;  // ket columns per problem (read-out partial layout)
struct ChebProblem {
    int N, ld, ldv, m, K;   // size, matrix/vector leading dims (padded rows are 0), complex columns, last order
    const void *H;          // Hs = (H~ - a)/b in the launch precision, N columns of ld rows (symmetric)
    void *vbuf;             // [3][m/MG][ldv][MG] complex vectors in the launch precision
    double2 *col[2];        // ping-pong columns [ldv][m] (FP64): col[parity] in, col[parity^1] out
    const double2 *coef;    // [K+1] expansion coefficients (phase folded in)
    const double *scale;    // [P] factor applied to the input columns (renormalisation) or nullptr
    // read-out (fixed nuclei): P ket columns; bra from columns P..2P-1 when m == 2P, else from the kets
    int P;
    const void *A, *B;      // L^-1 and L^T in the launch precision (ld x N), nullptr = no device read-out
    double2 *psi, *bra;     // [ldv][P] AO-basis Psi_ket / Psi_bra outputs
    const int *ao_frag;
    int nfrag, pops_off;    // populations of this problem at pops + pops_off, P x (nfrag+1)
    const double *target;   // [P] norm targets for the renormalisation factor, or nullptr
    double *scale_out;      // [P] factor for the next step, or nullptr
    // implicit operator (geometry changing every step): H holds h/b, G = L^-1 (lower,
    // zeros above the diagonal), Gt = G^T (upper), and one order applies
    // Hs v = G (h/b) G^T v - shift v in three grid-synchronised phases.  G == nullptr: explicit Hs.
    const void *G, *Gt;
    void *wb;               // [2][m/MG][ldv][MG] launch precision: w = G^T v, y = (h/b) w
    double shift;           // a / b
    double *drift;          // largest relative change of a column's squared norm over a step (norm control)
    double *ntot;           // [P] total population of each particle after the step, in FP64 from the
                            // propagated columns (reduced precision: the renormalisation divides by it)
    const float *dcorr;     // explicit FP32 Hs: [N] Hs_ii minus its FP32 value (in FP32), or nullptr
};
struct ChebSegment {
    int prob, row0, row1;   // rows [row0, row1) of problem `prob` owned by one CTA
};
struct ChebLaunch {
    const ChebProblem *probs;
    const ChebSegment *segs;
    const int *seg_begin;   // [grid + 1]: CTA c owns segs[seg_begin[c] .. seg_begin[c+1])
    const int *prob_seg0;   // [nprob + 1]: problem q owns segs[prob_seg0[q] .. prob_seg0[q+1])
    int kmax, max_ld, grid, parity;
    unsigned *bar_count;    // grid barrier: two words, one 64-bit count (8-byte aligned, zero at the launch)
    int *error;
    double *seg_pops;       // [nseg][kMaxCols][kMaxFrag+1] read-out partials
    double *pops;           // this step's populations block, or nullptr
    int nphase;             // grid phases per order: 1 (explicit Hs) or 3 (one implicit problem)
    // implicit operator: row ranges of the full phase y = (h/b) w, an even split of
    // the rows over the CTAs (the triangular phases use segs: mirrored chunk pairs)
    const ChebSegment *segs_full;
    const int *seg_full_begin;  // [grid + 1]
    int jwin;                   // explicit Hs: vector window in rows (0: the whole vector); set by the launcher
    // failure-detection test hook (elhl_debug_barrier): grid-barrier limit in ns
    // (0: the default 5 s) and 1 + the CTA that leaves before its first grid
    // barrier (0: none, so a zero-initialised launch has no hook)
    unsigned long long barrier_ns;
    int exit_cta1;
};
constexpr size_t kCheb_part_bytes = 16 * 64 * sizeof(double);  // cross-warp partial sums
constexpr size_t kCheb_smem_limit = 200 * 1024;
int cheb_block();
int cheb_grid_size(int *grid_out);
// columns staged per pass, 0 = unsupported; windowed: the explicit propagation,
// which stages the vector in windows when it does not fit in shared memory
int cheb_group_size(int precision, int m, int max_ld, bool windowed = false);
cudaError_t launch_cheb(const ChebLaunch &L, int precision, int mg, cudaStream_t st);
cudaError_t launch_readout(const ChebLaunch &L, int nprob, int precision, int mg, cudaStream_t st);

// Split-precision tensor-core GEMM (umma_gemm.cu): sum over s < splits of Y_s
// (rows x n2, row-major FP32, Y_s = Y + s rows n2) = sum over the BF16 terms
// (i + j <= 2) of A_i (rows x K, K contiguous, ld lda) times B_j^T (B_j: n2 x K,
// ld ldb).  n2 in {32, 64, 128}; umma_splits picks the K split.
size_t umma_smem_bytes(int n2);
int umma_supported_n2(int n2);
int umma_splits(int rows, int K);
int split3_bf16(const float *src, int rows, int cols, int lds, __nv_bfloat16 *const dst[3], int ldd, bool transpose,
                cudaStream_t st);
int umma_bf16x3_gemm(const __nv_bfloat16 *const A[3], int lda, const __nv_bfloat16 *const B[3], int ldb, int rows,
                     int K, int n2, int splits, float *Y, int *d_error, cudaStream_t st);

// FP64 Chebyshev propagation by exact BF16 slices on the tensor cores
// (ozaki.cu), one grid phase per order on an explicit Hs.  An order's work:
// 64-K blocks of 128-row tiles; OzSeg is one CTA's run of blocks [kb0, kb1) in
// row tile rt, the slot-th segment of that tile.
struct OzSeg {
    int rt, kb0, kb1, slot;
};
struct OzLaunch {
    int N, ld, K, m, P;          // size, padded rows, last order, complex columns (<= 4), particles
    const double2 *coef;         // [K+1] expansion coefficients
    const double2 *phi;          // [ld][m] input columns
    double2 *acc;                // [ld][m] output columns (sum of c_k v_k)
    const double *scale;         // [P] renormalisation factor of the input, or nullptr
    double *v;                   // [3][ld][8] Chebyshev vectors (re, im of 4 columns; padding rows zero)
    unsigned char *xs[3];        // v_k as BF16 slices: [2 tiles] tiles of 64 rows (zero slots 0, 8)
    int *xe[3];                  // [2 tiles][8] exponents e of their scales 2^e, one per 64-row chunk and column
    int *emax[3];                // [8] the largest chunk exponent of each column (integer max)
    const double *rscale;        // [tiles * 128] power-of-two row scales of the sliced Hs
    const OzSeg *segs;
    const int *seg_begin;        // [grid + 1]
    const int *part_base;        // [tiles] first partial slot of a row tile
    const int *part_count;       // [tiles] segments of a row tile
    double *part;                // partial tiles [slot][128][8] as 128-bit integers (16 bytes each)
    unsigned *tile_cnt;          // [tiles] segments written, over all orders of the launch
    unsigned *bar_count;         // grid-barrier arrivals, over all orders of the launch (0 at the launch)
    int *error;
    unsigned long long barrier_ns;  // grid-barrier limit (0: default)
    int exit_cta1;                  // test hook: 1 + the CTA that leaves before its first barrier
};
int oz_slices();
int oz_tile_rows();
int oz_block_k();
size_t oz_vector_tile_bytes();  // bytes of one sliced 64-row tile of a vector
size_t oz_smem_bytes();
// slices [oz_slices()][n][ld] of the n storage columns of M (ld rows), scale per column
cudaError_t oz_slice_matrix(const double *M, int n, int ld, __nv_bfloat16 *out, double *rscale, cudaStream_t st);
// blocks of an n x n operator over grid CTAs
void oz_schedule(int n, int grid, std::vector<OzSeg> &segs, std::vector<int> &seg_begin, std::vector<int> &part_base,
                 std::vector<int> &part_count);
cudaError_t launch_oz_cheb(const OzLaunch &L, const __nv_bfloat16 *hs_slices, int grid, cudaStream_t st);

// Triangular operands of the FP64 products (dgemm64, ozgemm), flags of `tri`:
// kTriA: op(A) = A lower triangular; kTriAt: op(A) = A^T of a lower A; kTriB:
// op(B) = B lower; kTriBt: op(B) = B^T of a lower B; kTriLowerC: a symmetric
// update that writes only the tiles on or below the diagonal.
constexpr int kTriA = 1, kTriB = 2, kTriBt = 4, kTriLowerC = 8, kTriAt = 16;
// C = alpha op(A) op(B) + beta C in FP64 on the FP64 pipe (dgemm.cu), op = the
// transpose when transA / transB, `tri` the triangular flags above.  lane 0 or 1: products that run concurrently (on two streams)
// use different lanes, each with its own scheduler and workspace; lane 1 takes
// three quarters of the resident CTA slots.
cudaError_t dgemm64(int m, int n, int k, double alpha, const double *A, int lda, bool transA, const double *B, int ldb,
                    bool transB, double beta, double *C, int ldc, cudaStream_t st, int tri = 0, int lane = 0);
// The same product on the tensor cores from exact BF16 slices (ozgemm.cu):
// FP64-accurate (each output exact until one rounding, products below 2^-64 of
// the row and column scales dropped), for large products; lane as for dgemm64.
// A timeout of its bounded waits sets *ozgemm_error(lane) to ELHL_ERR_TIMEOUT.
cudaError_t ozgemm(int m, int n, int k, double alpha, const double *A, int lda, bool transA, const double *B, int ldb,
                   bool transB, double beta, double *C, int ldc, cudaStream_t st, int tri = 0, int lane = 0);
int *ozgemm_error(int lane);
size_t ozgemm_smem_bytes();
// Diagonal-block leaves of the recursive factorisation (factor.cu), in shared
// memory, blocks of leaf_rows() = 64 rows: leaf_chol_inv64: A (nb x nb,
// nb <= 64) <- chol(A), G <- its inverse, in FP64; a non-positive pivot sets
// *info (if still 0) to row0 + column + 1.
int leaf_rows();
cudaError_t leaf_chol_inv64(double *A, double *G, int nb, int ld, int row0, int *info, cudaStream_t st);

// Lanczos recursion of k steps for the spectral bounds, FP64, one cooperative
// launch (lanczos.cu): explicit H (G == nullptr; both triangles stored) or
// implicit G H G^T (G lower, Gt = G^T).  r: 4 x ld, t: 2 x ld, part: part_cap
// doubles (at least two per SM), rec: alpha[k], beta[k], steps used (0 = all,
// zeroed by the caller), bar: 2 barrier words, err: ELHL_ERR_TIMEOUT on a
// barrier that gave up.
cudaError_t launch_lanczos64(int n, int ld, int k, const double *H, const double *G, const double *Gt, double *r,
                             double *t, double *part, int part_cap, double *rec, unsigned *bar, int *err,
                             cudaStream_t st);

int bessel_j_sequence(double beta, int kmax, double *J);
int chebyshev_coefficients(double dt, double emin, double emax, double tol, int kcap, std::vector<double> &cre,
                           std::vector<double> &cim, int *K_out);
void tridiagonal_extremes(const double *alpha, const double *beta, int n, double *lo, double *hi);
double tridiagonal_last_component(const double *alpha, const double *beta, int n, double theta);

// ---- small helpers ----------------------------------------------------------
inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace elhl
