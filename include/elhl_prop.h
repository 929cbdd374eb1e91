/*
 * elhl_prop.h -- C ABI of libelhlprop.so, the GB300 (sm_103a) electron-hole
 * wavepacket propagator.
 *
 * Two groups of entry points:
 *
 *  1. Drop-in replacements for the symbols Dynemol's Fortran host binds by
 *     implicit interface (all arguments by reference, column-major matrices,
 *     complex*16 = interleaved double pairs, lowercase name + trailing
 *     underscore, no hidden string lengths).  They keep the reference's
 *     argument meaning and "void + print on error" behaviour; the status of
 *     the last call is available from elhl_last_status().
 *
 *  2. The native API (elhl_*): device-resident trajectories that rebuild S, h
 *     and H' = S^-1 h on the GPU from nuclear coordinates and propagate the
 *     electron and the hole together, returning an explicit status code.
 *
 * All compute runs on the GPU; there is no CPU fallback.  Calls return
 * ELHL_ERR_NO_DEVICE when no CUDA device is present.
 */
#ifndef ELHL_PROP_H
#define ELHL_PROP_H

#ifdef __cplusplus
extern "C" {
#endif

/* complex*16 / cuDoubleComplex layout */
typedef struct {
    double re, im;
} elhl_zcomplex;

/* ---- status codes ------------------------------------------------------- */
enum {
    ELHL_OK = 0,
    ELHL_ERR_BAD_ARG = 1,
    ELHL_ERR_NO_CONVERGENCE = 2, /* tau retries exhausted (the reference loops forever) */
    ELHL_ERR_TIMEOUT = 3,        /* a bounded device-side wait gave up */
    ELHL_ERR_OOM = 4,
    ELHL_ERR_CUDA = 5,
    ELHL_ERR_NOT_POSITIVE_DEFINITE = 6, /* Cholesky of S failed */
    ELHL_ERR_NO_DEVICE = 7,
    ELHL_ERR_UNSUPPORTED = 8
};

/* ======================= 1. drop-in symbols ============================== */

/* GPU_Init (GPU_Interface.cpp:226-263): bind device (myid / procs_per_dev) % ndev. */
void gpu_init_(const int *myid, const int *procs_per_dev);

/* GPU_Finalize (GPU_Interface.cpp:266-282): release library state. */
void gpu_finalize_(void);

/* GPU_Pin (GPU_Interface.cpp:288-295): page-lock `*bytes` bytes at ptr (cudaHostRegister). */
void gpu_pin_(void *ptr, const int *bytes);

/* GPU_Unpin (GPU_Interface.cpp:297-302). */
void gpu_unpin_(void *ptr);

/*
 * propagation_gpucaller_ (Taylor_gpu.cpp:295-330): Taylor propagation of one
 * particle under a given H' (host, N x N, ld = N) from t_init to t_max.
 * tau is read (initial step) and not written back; save_tau receives the tau
 * accepted by the first convergence (Taylor.f:71).  PSI_bra/PSI_ket are in/out.
 */
void propagation_gpucaller_(const int *n, double *tau, double *save_tau, const double *t_init,
                            const double *t_max, elhl_zcomplex *h_PSI_bra, elhl_zcomplex *h_PSI_ket,
                            const double *h_H);

/*
 * propagationelhl_gpucaller_ (Taylor_gpu.cpp:634-736, called from
 * ElHl_Chebyshev_GPU.f:269-272): one particle, one nuclear step.
 *   in : S, h (host, N x N, ld = N), PSI_bra/PSI_ket (length N), t_init, t_max, tau
 *   out: h_H = H' = S^-1 h (host, ld = N); PSI_bra/PSI_ket propagated;
 *        h_AO_bra = S^-1 PSI_bra (not conjugated; the caller conjugates);
 *        save_tau.  h_AO_ket is not touched (as in the reference).
 * Differences from the reference, by design: S^-1 h comes from a Cholesky
 * factorisation instead of LU; device buffers are re-sized when N grows
 * instead of being fixed by the first call; non-convergence stops after a
 * bounded number of tau retries (status ELHL_ERR_NO_CONVERGENCE).
 */
void propagationelhl_gpucaller_(const int *N, const double *h_S, const double *h_h, double *h_H,
                                elhl_zcomplex *h_AO_bra, elhl_zcomplex *h_AO_ket,
                                elhl_zcomplex *h_PSI_bra, elhl_zcomplex *h_PSI_ket,
                                const double *t_init, const double *t_max, double *tau,
                                double *save_tau);

/*
 * Ehrenfest force kernel pieces (Taylor_gpu.cpp:743-791, :795-874; kernels
 * Chebyshev_gpu_kernels.cu:358-455), host N x N column-major, ld = N:
 *   ehrenfestkernel_gpu_ : K = X o A - H A   (o = element-wise product)
 *   ehrenfestkernel2_gpu_: the same with A = (rho + rho^T)/2,
 *       rho_ij = Re(ket_j,1 bra_i,1) - Re(ket_j,2 bra_i,2); bra/ket are N x 2.
 */
void ehrenfestkernel_gpu_(const int *N, const double *h_H, const double *h_A, const double *h_X, double *h_K);
void ehrenfestkernel2_gpu_(const int *N, const elhl_zcomplex *h_bra, const elhl_zcomplex *h_ket, const double *h_H,
                           const double *h_X, double *h_K);

/* Status of the last drop-in call on this thread (ELHL_OK, ...). */
int elhl_last_status(void);
const char *elhl_status_string(int status);

/* ======================= 2. native API =================================== */

/* Propagation method / precision of a trajectory. */
enum {
    ELHL_METHOD_TAYLOR_REF = 0, /* the reference's adaptive-tau Taylor (Taylor.f) on H', bra and ket */
    ELHL_METHOD_CHEBYSHEV = 1   /* Chebyshev on the symmetrised H~ = L^-1 h L^-T, ket only */
};
enum {
    ELHL_PREC_FP64 = 0,
    ELHL_PREC_FP32 = 1,   /* Chebyshev: FP32 H~ and series vectors (the FP32 rounding residual of H~'s
                             diagonal added back in every order), FP64 coefficients, sums, norms,
                             Cholesky factor with inverse and spectral bounds; with >= 16 ket columns
                             (one per particle) and N >= 2048, H~.Psi runs as FP32 GEMMs on the FP32
                             pipes (cuBLAS, FP32 sums along N) */
    ELHL_PREC_DF64 = 3,   /* Chebyshev, implicit operator: operator and series vectors as FP32 pairs
                             hi + lo (48-bit significands) with exact-product / TwoSum arithmetic on the
                             FP32 pipes, FP64 recurrence and sums: FP64-level accuracy (1e-10 populations)
                             without the FP64 pipe; FP64 factor, bounds and read-out */
    ELHL_PREC_BF16X3 = 2, /* Chebyshev: as FP32, but those GEMMs run on the tensor cores with each
                             FP32 operand split in three bf16 terms: a hand-written tcgen05/TMA kernel
                             for 16, 32 or 64 columns (cuBLAS emulation otherwise); outside the GEMM
                             regime it runs as FP32 */
    ELHL_PREC_OZ64 = 4    /* Chebyshev, trajectories with ncols <= 4: FP64 operator, vectors and
                             recurrence, with every operator product computed exactly on the tensor
                             cores from 7 bf16 slices of 8 bits per operand (Ozaki scheme I, products
                             below 2^-64 of a row's scale dropped) and rounded once to FP64; moving
                             nuclei form H~ = G h G^T every step the same way, and the factorisation's
                             products of 320 or more rows too; bounds and read-out in FP64 */
};

/* STO basis of one system (the STO_basis fields the path reads, types_EHT.f:135-165). */
typedef struct {
    int natoms;
    int nao;
    const int *atom_ao0;     /* [natoms] first AO of each atom */
    const int *atom_nao;     /* [natoms] AOs per atom */
    const int *ao_n;         /* [nao] principal quantum number (1..3) */
    const int *ao_l;         /* [nao] 0 or 1 */
    const int *ao_m;         /* [nao] -l..l */
    const int *ao_nzeta;     /* [nao] 1 or 2 */
    const double *ao_zeta;   /* [nao*2] exponents, Angstrom^-1 */
    const double *ao_coef;   /* [nao*2] contraction coefficients */
    const double *ao_ip;     /* [nao] ionisation potential, eV */
    const double *ao_kwh;    /* [nao] Wolfsberg-Helmholz k */
    const double *ao_vshift; /* [nao] on-site shift, eV */
    const int *ao_frag;      /* [nao] fragment id 0..nfrag-1 (populations) */
    int nfrag;
} elhl_basis_desc;

typedef struct {
    int method;          /* ELHL_METHOD_* */
    int precision;       /* ELHL_PREC_* */
    double dt;           /* nuclear step, ps */
    int frame_step;      /* t_max = dt*frame_step*(it-1) (ElHl_Chebyshev.f:176) */
    double tol;          /* Taylor `error` (Taylor.f:21), e.g. 1e-8 or 1e-10 */
    double norm_tol;     /* Taylor `norm_error` (Taylor.f:22) */
    double cheb_tol;     /* Chebyshev truncation |c_k| < cheb_tol */
    double cutoff;       /* overlap cutoff, Angstrom (QM_cutoff, 12) */
    int max_conv_calls;  /* bound on tau retries per particle and step */
    int ncols;           /* Chebyshev: propagated complex columns, nparticles (ket only, bra = S ket)
                            or 2 * nparticles (bra carried as the reference does) */
    int nparticles;      /* wavefunctions per trajectory: 2 (electron, hole) for the Taylor method;
                            1..64 for Chebyshev (ensembles) */
    /* Chebyshev norm and convergence control, the counterpart of the Taylor
     * path's per-sub-step test |<bra|ket>| - norm_ref (Taylor.f:103-114): the
     * exact step is unitary in the symmetrised basis, so after every step each
     * propagated column's squared norm is compared with its value before the
     * step (before any reduced-precision renormalisation).  A relative change
     * above cheb_norm_tol means the expansion did not converge (for example a
     * spectral interval that misses part of the spectrum): the step is redone
     * from its saved input on an interval widened by half its width each time,
     * at most cheb_max_retries times, and then the call returns
     * ELHL_ERR_NO_CONVERGENCE (batch and server members: the member fails). */
    double cheb_norm_tol;  /* <= 0: 1e-8 for FP64 / DF64 (the reference's norm_error), 1e-4 for FP32 / BF16X3 */
    int cheb_max_retries;  /* redone steps per step (default 3) */
    double lanczos_guard;  /* spectral interval = Lanczos extremes + residual bounds, widened on each side by
                              this fraction of the width (default 0.01) */
} elhl_traj_config;

typedef struct elhl_traj elhl_traj;

void elhl_traj_config_default(elhl_traj_config *cfg);

/*
 * Ehrenfest (Hellmann-Feynman-Pulay) forces on every atom of one geometry
 * (Diabatic_Ehrenfest / Ehrenfest, diabatic-Ehren.f:36-150, :163-230).  For
 * each atom pair K < L closer than `cutoff` and each direction, dS(j in L,
 * i in K)/dR_K is the central difference of the S block rebuilt with atom K
 * displaced by +-delta (PULAY_OVERLAP, overlap_D.f:314-463), and
 *   F_K(L) = -sum_{j in L, i in K} dS_ji/dR_K * kernel(i, j),
 *   forces[a][xyz] = 2 * 1.602176565e-9 * (sum_{L > a} F_a(L) - sum_{K < a} F_K(a))  [N].
 * kernel: host N x N column-major (ld = N), the ehrenfestkernel2_gpu_ output
 * X o A - H' A.  coords: natoms x 3 Angstrom.  delta <= 0 selects the
 * reference's 1e-8 Angstrom, cutoff <= 0 its 12 Angstrom.  forces: natoms x 3.
 */
int elhl_ehrenfest_forces(const elhl_basis_desc *basis, const double *coords, const double *kernel, double delta,
                          double cutoff, double *forces);

/*
 * Extended-Hueckel Hamiltonian with environment fields (even_more_extended_Huckel
 * and Huckel_with_FIELDS, hamiltonians.f:69-264, the EnvField_ case): for AOs i
 * of atom a > b and j of atom b, closer than `cutoff` (<= 0: 12 Angstrom),
 *   h_ij = X_ij S_ij - [S_ij DP_1 + (mu_ij - (r0 - R_a) S_ij) . DP_2..4]  when |S_ij| > 1e-7,
 * r0 the midpoint of the atoms, h_ji = h_ij, h_ii = IP_i + V_shift_i, other entries 0.
 * S: host N x N (ld N); dp_ao: the AO dipole matrix DP_matrix_AO, host N x N x 3
 * column-major; dp4: the environment's potential and field per atom pair,
 * DP_4_matrix, host natoms x natoms x 4 column-major, entry (a, b) for a > b.
 * h: host N x N output.
 */
int elhl_huckel_with_fields(const elhl_basis_desc *basis, const double *coords, const double *S, const double *dp_ao,
                            const double *dp4, double cutoff, double *h);

/* Create a trajectory at the given coordinates (natoms*3, atom-major, Angstrom, host).
 * Builds S, h and H' on the device. */
int elhl_traj_create(const elhl_basis_desc *basis, const double *coords, const elhl_traj_config *cfg,
                     elhl_traj **out);
int elhl_traj_destroy(elhl_traj *tr);

/*
 * Initial states from fragment molecular orbitals (FMO_analysis / eigen_FMO /
 * projector('AO'), FMO.f:45-139, :260-350; wiring ElHl_Chebyshev.f:100-129).
 * For each particle the fragment's S_f and h_f are built on the device at the
 * current coordinates, H_f C = S_f C E is solved (cuSOLVER dsygvd), MO number
 * `electron_state` / `hole_state` (1-based, ascending energy) is embedded in the
 * full basis (zeros outside the fragment) as Psi_ket = C and Psi_bra = S C.
 * Eigenvector sign: the component of largest magnitude is made positive.
 */
int elhl_traj_init_fmo(elhl_traj *tr, int n_el_atoms, const int *el_atoms, int electron_state, int n_hl_atoms,
                       const int *hl_atoms, int hole_state);

/* Chebyshev trajectories: column c < nstates becomes fragment MO states[c]
 * (1-based) of the fragment `atoms`, embedded as in elhl_traj_init_fmo. */
int elhl_traj_init_fmo_states(elhl_traj *tr, int n_atoms, const int *atoms, int nstates, const int *states);

/* Set / get Psi (host, column-major N x nparticles: column 0 electron, 1 hole).
 * psi_bra may be NULL for the Chebyshev method (bra = S ket). */
int elhl_traj_set_psi(elhl_traj *tr, const elhl_zcomplex *psi_bra, const elhl_zcomplex *psi_ket);
int elhl_traj_get_psi(elhl_traj *tr, elhl_zcomplex *psi_bra, elhl_zcomplex *psi_ket);

/*
 * Advance `nsteps` nuclear steps (ElHl_Chebyshev, ElHl_Chebyshev.f:148-291).
 * coords: NULL = nuclei fixed (S, h, H' kept), else nsteps*natoms*3 host
 * coordinates, one set per step, rebuilt on the device before that step.
 * pops (host, may be NULL): nsteps x ncols x (nfrag+1) populations after each step.
 */
int elhl_traj_step(elhl_traj *tr, const double *coords, int nsteps, double *pops);

/* Same with device pointers (coords: nsteps*natoms*3 doubles, pops as above). */
int elhl_traj_step_device(elhl_traj *tr, const double *d_coords, int nsteps, double *d_pops);

/* Wavepacket energies per particle, E_p = sum_ij AO_bra_i h_ij AO_ket_j with
 * AO_bra = conj(S^-1 Psi_bra), AO_ket = Psi_ket (QuasiParticleEnergies,
 * ElHl_Chebyshev.f:329-371, evaluated with the Hueckel h).  E: [nparticles]. */
int elhl_traj_energies(elhl_traj *tr, elhl_zcomplex *E);

/*
 * Checkpoint and resume (Security_Copy_Cheb / Restart_State_Cheb,
 * backup.f:329-445).  elhl_traj_snapshot writes the trajectory's state to
 * `path` in the reference's layout -- a Fortran sequential unformatted file
 * with it, t, the basis size, the particle count and tags, per particle the
 * (DUAL_bra, DUAL_ket) and (AO_bra, AO_ket) pairs, and the Net_Charge record
 * -- followed by one record the reference does not read, holding what an exact
 * resume needs (tau continuation, norm targets, the Chebyshev interval and the
 * symmetrised columns).  elhl_traj_restore reads such a file into a trajectory
 * created with the same basis, configuration and coordinates (Psi_bra =
 * DUAL_ket, Psi_ket = AO_ket as in preprocess_from_restart,
 * ElHl_Chebyshev.f:396-397); the next steps then reproduce the uninterrupted
 * run bit for bit within one process.  A file written by the reference itself
 * (no trailing record) restores Psi, t and it, and the next step restarts at
 * tau_max.  ELHL_ERR_BAD_ARG for an unreadable or mismatched file.
 */
int elhl_traj_snapshot(elhl_traj *tr, const char *path);
int elhl_traj_restore(elhl_traj *tr, const char *path);

/* Copies of the device matrices (host, N x N, ld = N); any pointer may be NULL. */
int elhl_traj_get_matrices(elhl_traj *tr, double *S, double *h, double *Hp);

/* The Chebyshev propagator's current Cholesky factor L (S = L L^T, lower, zero
 * above the diagonal) and G = L^-1 (lower, zero above the diagonal); host,
 * N x N, ld = N; either pointer may be NULL.  ELHL_ERR_UNSUPPORTED on the
 * Taylor path. */
int elhl_traj_get_factor(elhl_traj *tr, double *L, double *G);

/* Counters of the last elhl_traj_step call. */
typedef struct {
    long long orders;     /* expansion orders executed, summed over particles */
    long long conv_calls; /* Taylor convergence attempts */
    long long substeps;   /* accepted sub-steps */
    double save_tau[2];   /* per particle */
    double t;             /* trajectory time, ps */
    int it;               /* reference step counter */
    int status;
    double prop_ms;       /* device time of the propagation kernels (CUDA events on the launch stream) */
    double rebuild_ms;    /* device time of the S, h, H' rebuilds */
    int prop_launches;    /* propagation kernel launches */
    int rebuild_count;    /* rebuilds */
    int tile_cols;        /* Chebyshev: complex columns per matrix pass chosen by the autotuner (0: GEMM regime) */
    int phases;           /* Chebyshev: grid phases per order (1 explicit H~, 3 implicit G h G^T) */
    double sh_ms;         /* moving nuclei: device time of the S, h build */
    double factor_ms;     /* ... of the Cholesky factorisation of S with G = L^-1 */
    double inverse_ms;    /* ... of the operator formed from them: H~ = G h G^T (ELHL_PREC_OZ64),
                             the zeroed upper triangles of L and G (implicit operator) */
    int cheb_retries;     /* Chebyshev steps redone on a widened spectral interval */
    double norm_drift;    /* Chebyshev: largest relative change of a column's squared norm in one step
                             (before renormalisation), over the call's accepted steps */
    double emin, emax;    /* Chebyshev: spectral interval of the current operator (eV): FP64 Lanczos
                             extremes with their residual bounds, widened by lanczos_guard */
} elhl_traj_stats;
int elhl_traj_get_stats(elhl_traj *tr, elhl_traj_stats *st);

/* ---- batches: many trajectories in one launch per nuclear step ---------- */
/* Batched Chebyshev propagation (config: method ELHL_METHOD_CHEBYSHEV, fixed
 * nuclei) of `ntraj` trajectories of any sizes: bases[i] / coords[i] describe
 * trajectory i.  Each nuclear step is ONE cooperative launch over all members'
 * expansion orders, followed by each member's read-out and populations.  No
 * counterpart in the reference, which propagates one trajectory per process. */
typedef struct elhl_batch elhl_batch;
int elhl_batch_create(int ntraj, const elhl_basis_desc *bases, const double *const *coords,
                      const elhl_traj_config *cfg, elhl_batch **out);
int elhl_batch_size(elhl_batch *b);
/* Member i as a trajectory handle (init_fmo / set_psi / get_psi / get_stats). */
elhl_traj *elhl_batch_member(elhl_batch *b, int i);
/* Free the members' set-up matrices (S, h, H~) once their initial states are set. */
int elhl_batch_compact(elhl_batch *b);
/* pops: nsteps x ntraj x 2 x (nfrag+1) host doubles, or NULL. */
int elhl_batch_step(elhl_batch *b, int nsteps, double *pops);
int elhl_batch_get_stats(elhl_batch *b, elhl_traj_stats *st);
int elhl_batch_destroy(elhl_batch *b);

/* ---- serving: continuous batching of propagation requests -------------- */
/* A request is one fixed-nuclei Chebyshev propagation: a system, its
 * coordinates, a step count and `nparticles` initial columns (fragment MOs
 * `states` of the fragment `frag_atoms`).  Everything is copied at submit.
 * Requests wait FIFO until their estimated device memory fits the HBM budget,
 * are set up on the device, join the running batch at the next step boundary
 * and leave it when done; elhl_server_step is one nuclear step of every
 * active request (one launch).  No counterpart in the reference. */
typedef struct {
    const elhl_basis_desc *basis;
    const double *coords;   /* natoms*3 */
    int nsteps;
    int nparticles;         /* complex columns, 1..64 */
    int n_frag_atoms;
    const int *frag_atoms;
    const int *states;      /* [nparticles], 1-based fragment MO indices */
} elhl_request;
typedef struct elhl_server elhl_server;
int elhl_server_create(double hbm_budget_bytes, const elhl_traj_config *cfg, elhl_server **out);
/* ELHL_ERR_OOM if the request can never fit the budget. */
int elhl_server_submit(elhl_server *sv, const elhl_request *req, long long *id);
int elhl_server_step(elhl_server *sv, int *n_active, int *n_pending);
/* ids of requests completed since the last poll */
int elhl_server_poll(elhl_server *sv, long long *ids, int max, int *n);
/* final populations (nparticles x (nfrag+1)), final kets (N x nparticles,
 * column-major) and times {submit, admit, done} (s, host steady clock); frees
 * the request; returns its status. */
int elhl_server_result(elhl_server *sv, long long id, double *pops, elhl_zcomplex *psi_ket, double *times);
/* Checkpoint of an admitted request (elhl_traj_snapshot's file layout; its it
 * and t count the server steps done), and a request that resumes from such a
 * file at admission: the trajectory is set up as for elhl_server_submit, its
 * state restored, and q->nsteps more steps run.  ELHL_ERR_BAD_ARG for a request
 * that is not active. */
int elhl_server_snapshot(elhl_server *sv, long long id, const char *path);
int elhl_server_submit_restart(elhl_server *sv, const elhl_request *q, const char *path, long long *id);
int elhl_server_destroy(elhl_server *sv);

/* Run all library work on the caller's CUDA stream (a cudaStream_t passed as
 * void*), e.g. to order it with the caller's own kernels or to time it with
 * events on that stream; NULL restores the library's own stream. */
int elhl_set_stream(void *stream);

/* Test hook for failure detection (no counterpart in the reference): the
 * grid-barrier wait limit of the Chebyshev propagation launches (limit_s <= 0
 * restores the default 5 s; at most 10 s) and, when exit_cta >= 0, one CTA of
 * the next propagation launch that leaves before its first grid barrier, so
 * that the other CTAs' waits run out and the call returns ELHL_ERR_TIMEOUT
 * with the device context intact.  No fault or hang is involved: every wait
 * is bounded. */
int elhl_debug_barrier(double limit_s, int exit_cta);

/* Kernels of this library launched so far in this process (each kernel node
 * of a replayed step graph counted; library calls such as cuBLAS not
 * counted): benchmarks read it before and after a timed region. */
long long elhl_kernel_launches(void);

/*
 * Allocation-free propagation of one particle (no counterpart in the
 * reference).  Same computation and thresholds as propagation_gpucaller_
 * (adaptive-tau Taylor, 1e-8), but for callers that cannot allocate device
 * memory -- a host whose pool allocator owns the device memory, code running
 * while a CUDA graph capture is in progress elsewhere, or code that must not
 * risk the device synchronisation cudaMalloc/cudaFree can trigger.  It calls
 * no cudaMalloc, cudaFree or allocating library routine: all scratch lives in
 * a fixed device array inside the library (about 0.9 MB).
 *   d_H         device, n x n column-major H', leading dimension ld >= n
 *   d_psi_bra/d_psi_ket  device, length n, propagated in place; left
 *               unchanged when the call returns an error status
 *   save_tau    host, receives the tau accepted by the first convergence
 *   stream      cudaStream_t as void* (NULL = legacy default stream)
 * Limit: n <= 4096 (larger n returns ELHL_ERR_BAD_ARG).  The call is
 * synchronous.  The array is device memory of the library's module: with
 * CUDA's lazy module loading the driver allocates it when that module is
 * first loaded on a device -- by gpu_init_ (and any other call that sets up
 * the library's context), or else by the first call of this function on that
 * device, which also looks up the array's address (cudaGetSymbolAddress) --
 * and the device holds it until the process exits.  Call gpu_init_ (or this
 * function once) before a pool allocator takes the device memory and before
 * any stream capture.  All calls share the array; calls that overlap on the
 * GPU race.
 */
int elhl_propagate_fixed_scratch(int n, const double *d_H, int ld, elhl_zcomplex *d_psi_bra,
                                 elhl_zcomplex *d_psi_ket, double t_init, double t_max, double tau,
                                 double *save_tau, void *stream);

/* Host-side mathematics of the Chebyshev method (no GPU needed).
 * elhl_bessel_j: J_0..J_kmax at beta (Miller backward recurrence).
 * elhl_chebyshev_coefficients: c_k, k = 0..*K, of exp(-i dt H / hbar) for a
 * spectrum in [emin, emax] (eV, dt in ps), truncated where |J_k| < tol; the
 * caller's arrays hold kcap + 1 values. */
int elhl_bessel_j(double beta, int kmax, double *J);
int elhl_chebyshev_coefficients(double dt, double emin, double emax, double tol, int kcap, double *cre,
                                double *cim, int *K);

/* Library / device information. */
int elhl_device_count(void);
int elhl_sm_count(void);

#ifdef __cplusplus
}
#endif
#endif
