/*
 * elhl_oracle.h -- CPU restatement of Dynemol's electron-hole propagation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA product
 * (libelhlprop.so) is compared against.  Only tests/, __graft_entry__.smoke()
 * and the CPU-baseline leg of bench.py may load it.  Nothing in the product
 * links, loads or calls it.
 *
 * Every routine cites the reference file:line whose arithmetic it restates.
 * Parity anchor: the reference ships no tests or golden vectors, so this
 * restatement is pinned against (1) the exact generalized-eigenbasis propagator
 * (ElHl_schroedinger.f:131-147 semantics, oracle/oracle.py), (2) closed-form STO
 * overlaps and numerical quadrature, and (3) conservation invariants.
 * Matrices are Fortran column-major, complex*16 is interleaved (re, im).
 */
#ifndef ELHL_ORACLE_H
#define ELHL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Per-AO descriptor arrays (Basis_Builder, structure.f:256-298). */
typedef struct {
    int nao;               /* number of atomic orbitals N */
    int natoms;
    const int *atom_ao0;   /* [natoms] first AO of atom (BasisPointer) */
    const int *atom_nao;   /* [natoms] AOs on atom (DOS) */
    const double *coord;   /* [natoms*3] x,y,z per atom (Angstrom), atom-major */
    const int *ao_n;       /* [nao] principal quantum number */
    const int *ao_l;       /* [nao] angular momentum */
    const int *ao_m;       /* [nao] real-harmonic m, -l..l */
    const int *ao_nzeta;   /* [nao] 1 or 2 */
    const double *ao_zeta; /* [nao*2] Angstrom^-1 */
    const double *ao_coef; /* [nao*2] */
    const double *ao_ip;   /* [nao] eV */
    const double *ao_kwh;  /* [nao] Wolfsberg-Helmholz k */
    const double *ao_vshift; /* [nao] eV */
} orc_basis;

/* Lined-up frame overlap <na la m | nb lb m>, m = 0..min(la,lb)  (SOLAP, overlap_D.f:701-962). */
int orc_solap(int na, int la, double za, int nb, int lb, double zb, double R, double *sol);

/* Dense overlap matrix S (BUILD_OVERLAP_MATRIX, overlap_D.f:144-311). Returns 0 or <0 on bad input. */
int orc_overlap(const orc_basis *b, double cutoff, double *S, int nthreads);

/* Extended-Hueckel H (Build_Huckel, ElHl_Chebyshev.f:296-323 with X_ij, hamiltonians.f:33-63). */
void orc_huckel(const orc_basis *b, const double *S, double *h);

/* Statistics of one Propagation call. */
typedef struct {
    long long gemv_terms;   /* expansion orders executed (each = one H'^T.bra and one H'.ket) */
    int conv_calls;         /* Convergence() invocations */
    int substeps;           /* accepted sub-steps */
    int status;             /* 0 ok, 1 = iteration cap hit (no convergence) */
} orc_prop_stats;

/*
 * Taylor propagation of one particle (Propagation/Convergence/coefficient,
 * Taylor.f:35-239).  Hp is N x N column-major, bra/ket length-N complex.
 * tau is read and modified as in the reference; save_tau is written.
 * tol / norm_tol are the reference's `error` / `norm_error` (Taylor.f:21-22,
 * 1e-8 there).  max_conv_calls bounds the otherwise unbounded tau retries.
 */
int orc_propagation(int N, const double *Hp, double *bra, double *ket,
                    double t_init, double t_max, double *tau, double *save_tau,
                    double tol, double norm_tol, int max_conv_calls, int nthreads,
                    orc_prop_stats *stats);

/* res = alpha * A^T x (trans=1) or alpha * A x (trans=0); A real N x N col-major, x/res complex. */
void orc_dzgemv(int trans, int N, const double *A, const double *x, const double *alpha,
                double *res, int nthreads);

/* pop[f] = Re sum_{i in f} conj(psi_ket_i) psi_bra_i, pop[nfrag] = total (pop_Slater, data_output.f:242-262). */
void orc_populations(int N, const int *ao_frag, int nfrag, const double *psi_bra,
                     const double *psi_ket, double *pop);

#ifdef __cplusplus
}
#endif
#endif
