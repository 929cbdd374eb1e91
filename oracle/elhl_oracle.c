/*
 * elhl_oracle.c -- CPU restatement of Dynemol's electron-hole propagation path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): loaded by tests/, smoke() and the
 * CPU-baseline leg of bench.py, never by the product library.
 *
 * Restated reference routines (paths relative to the Dynemol tree):
 *   constant tables ........ UTIL_OVERLAP            overlap_D.f:1194-1231
 *   lined-up overlaps ...... SOLAP                   overlap_D.f:701-962
 *   rotation (l <= 1) ...... ROTATIONOVERLAP / ROTAR overlap_D.f:520-583, 983-1051
 *   STO normalisation ...... GET_ANOR[_DIVISOR]      overlap_D.f:464-517
 *   overlap assembly ....... BUILD_OVERLAP_MATRIX    overlap_D.f:144-311
 *   Hueckel matrix ......... Build_Huckel + X_ij     ElHl_Chebyshev.f:296-323, hamiltonians.f:33-63
 *   Taylor propagator ...... Propagation / Convergence / coefficient / isConverged
 *                                                    Taylor.f:35-239, 290-303
 *   dzgemv semantics ....... bra_x_op / op_x_ket     Matrix_math.f:225-301
 *   populations ............ pop_Slater              data_output.f:242-262
 *
 * Only s and p shells (l <= 1) are supported, which covers the H/C/O single-zeta
 * EHT basis of the propagation workloads; other l return an error.
 */
#include "elhl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MXL 5
#define ORC_MXN 15
#define ORC_MXH (ORC_MXN + 3 * ORC_MXL) /* 30: index bound of the n tables */

/* ---- constant tables (UTIL_OVERLAP, overlap_D.f:1194-1231) ---------------- */
static double t_re[1001], t_reali[1001], t_fact[151], t_facti[151];
static int tables_ready = 0;

static void build_tables(void) {
    if (tables_ready) return;
    t_fact[0] = 1.0;
    t_facti[0] = 1.0;
    for (int i = 1; i <= 150; ++i) {
        t_fact[i] = t_fact[i - 1] * i;
        t_facti[i] = 1.0 / t_fact[i];
    }
    t_re[0] = 0.0;
    t_reali[0] = 0.0; /* the reference uses reali(0)=0 to zero the last auxk update */
    for (int i = 1; i <= 1000; ++i) {
        t_re[i] = t_re[i - 1] + 1.0;
        t_reali[i] = 1.0 / t_re[i];
    }
    tables_ready = 1;
}

/* util_m::fact -- real factorial by a product of dfloat(i) (util.f:22-36). */
static double real_fact(int n) {
    double f = 1.0;
    for (int i = 2; i <= n; ++i) f *= (double)i;
    return f;
}

static double ipow(double x, int e) {
    double r = 1.0;
    for (int i = 0; i < e; ++i) r *= x;
    return r;
}

/* ---- SOLAP (overlap_D.f:701-962) ------------------------------------------
 * Overlap integrals <na la m | nb lb m>, m = 0..min(la,lb), of unnormalised STOs
 * in the lined-up frame (A at origin, B on +z at distance R).  Starts from the
 * Fernandez-Rico 1F1 expansion of <n00|n'00> and climbs in l, l' and m by the
 * recurrences listed in the reference header (overlap_D.f:652-700). */
#define H1F1_ROWS (ORC_MXH + 2)
#define H1F1_COLS (2 * (ORC_MXH + 1) + 1)
#define SM (ORC_MXH + 1)

int orc_solap(int na, int la, double za, int nb, int lb, double zb, double R, double *sol) {
    build_tables();
    if (la < 0 || lb < 0 || la > ORC_MXL || lb > ORC_MXL || na < 1 || nb < 1) return -1;
    if (na + la + 2 * lb > ORC_MXH || nb + lb + 2 * la > ORC_MXH) return -1;

    static __thread double h1f1[H1F1_ROWS][H1F1_COLS];
    static __thread double smat[SM][SM], smataux[SM][SM], smatm[SM][SM];

    const double pi4 = 12.566370614359172953850573533118012;
    int nmin, nmax, npmin, npmax;
    double z, zp;
    const int a_is_big = (za >= zb);
    if (a_is_big) {
        nmin = na - la; nmax = na + la + lb + lb;
        npmin = nb - lb; npmax = nb + lb + la + la;
        z = za; zp = zb;
    } else {
        nmin = nb - lb; nmax = nb + lb + la + la;
        npmin = na - la; npmax = na + la + lb + lb;
        z = zb; zp = za;
    }
    const double expzR = exp(-z * R);

    /* 1F1[a, g, x] table: column g = ngmax from a series pair plus the three-term
     * recursion in a (upwards above ia, downwards below), then the remaining
     * columns g < ngmax by the contiguous relations (overlap_D.f:766-819). */
    const int ngmax = nmax + npmax + 2;
    const int namax = npmax + 1;
    const double arg = (z - zp) * R;
    const int iz = (int)z;
    int ia = (ngmax - iz) / 2;
    if (ia < 1) ia = 1;
    if (ia >= namax) ia = namax - 1;

    double auxa = arg * t_re[ia] * t_reali[ngmax];
    double f11a = 1.0;
    double auxb = arg * t_re[ia + 1] * t_reali[ngmax];
    double f11b = 1.0;
    /* The reference runs up to 1000 terms; the table index ngmax+i must stay
     * inside reali(0:1000), so the loop is bounded by that as well. */
    const int imax = 1000 - ngmax - 1;
    for (int i = 1; i <= imax; ++i) {
        f11a = f11a + auxa;
        f11b = f11b + auxb;
        auxa = auxa * t_re[ia + i] * arg * t_reali[ngmax + i] * t_reali[i + 1];
        auxb = auxb * t_re[ia + i + 1] * arg * t_reali[ngmax + i] * t_reali[i + 1];
        if (auxb < 1.0e-35 * f11b) break;
    }
    h1f1[ia][ngmax] = f11a;
    h1f1[ia + 1][ngmax] = f11b;

    double aux = arg - t_re[ngmax];
    for (int i = ia + 1; i <= namax - 1; ++i)
        h1f1[i + 1][ngmax] = ((aux + t_re[i + i]) * h1f1[i][ngmax] + t_re[ngmax - i] * h1f1[i - 1][ngmax]) * t_reali[i];
    for (int i = ia; i >= 2; --i)
        h1f1[i - 1][ngmax] = (t_re[i] * h1f1[i + 1][ngmax] - (aux + t_re[i + i]) * h1f1[i][ngmax]) * t_reali[ngmax - i];
    for (int j = ngmax - 1; j >= 2; --j) {
        h1f1[1][j] = (h1f1[2][j + 1] + t_re[j - 1] * h1f1[1][j + 1]) * t_reali[j];
        aux = arg * t_reali[j];
        const int itop = (namax - 1 < j - 2) ? namax - 1 : j - 2;
        for (int i = 1; i <= itop; ++i) h1f1[i + 1][j] = aux * h1f1[i + 1][j + 1] + h1f1[i][j];
    }

    /* basic integrals <N 0 0 | N' 0 0>, stored as smat[n_a][n_b] (overlap_D.f:823-879) */
    {
        const double zzpR = (z + zp) * R;
        const double zzpi = 1.0 / (z + zp);
        double zzpin = ipow(zzpi, nmin + npmin + 1);
        for (int n = nmin; n <= nmax; ++n) {
            double zzpinp = zzpin;
            for (int np = npmin; np <= npmax - n + nmin; ++np) {
                double auxk = t_fact[n + np] * zzpinp;
                double sumk = 0.0;
                for (int k = 0; k <= n + np; ++k) {
                    double sumj = 0.0;
                    const int jlo = (k - n > 0) ? k - n : 0;
                    const int jhi = (k < np) ? k : np;
                    for (int j = jlo; j <= jhi; ++j)
                        sumj = sumj + h1f1[j + 1][k + 2] * t_facti[n + j - k] * t_facti[np - j];
                    sumk = sumk + sumj * auxk;
                    auxk = auxk * zzpR * t_reali[n + np - k] * t_reali[k + 2];
                }
                const double v = pi4 * expzR * t_fact[n] * t_fact[np] * sumk;
                const int ra = a_is_big ? n : np, rb = a_is_big ? np : n;
                smat[ra][rb] = v;
                smataux[ra][rb] = v;
                smatm[ra][rb] = v;
                zzpinp = zzpinp * zzpi;
            }
            zzpin = zzpin * zzpi;
        }
    }

    /* climb in la, lb for each m, then step m (overlap_D.f:881-958) */
    nmin = na - la; nmax = na + la + lb + lb;
    npmin = nb - lb; npmax = nb + lb + la + la;
    const double Rinv = 1.0 / R;
    const double R2 = R * R;
    const double R4 = R2 * R2;
    double updltm0i = 0.5;
    const int mtop = (la < lb) ? la : lb;
    for (int m = 0; m <= mtop; ++m) {
        if (la > m) {
            for (int np = npmin; np <= npmax - 2; ++np) {
                double saux = smat[nmin][np];
                for (int n = nmin + 1; n <= nmax - 1 - np + npmin; ++n) {
                    const double sbux = t_re[m + m + 1] * 0.5 * Rinv *
                                        (smat[n + 1][np] + R2 * saux - smat[n - 1][np + 2]);
                    saux = smat[n][np];
                    smataux[n][np] = saux;
                    smat[n][np] = sbux;
                }
            }
            for (int ll = m + 1; ll <= la - 1; ++ll) {
                for (int np = npmin; np <= npmax - 2 * (ll + 1 - m); ++np) {
                    double saux = smat[nmin + ll - m][np];
                    for (int n = nmin + 1 + ll - m; n <= nmax - 1 - np + npmin - ll + m; ++n) {
                        const double sbux =
                            t_re[ll + ll + 1] * 0.5 * t_reali[ll - m + 1] * Rinv *
                                (smat[n + 1][np] + R2 * saux - smat[n - 1][np + 2]) -
                            t_re[ll + m] * t_reali[ll - m + 1] * smataux[n][np];
                        saux = smat[n][np];
                        smataux[n][np] = saux;
                        smat[n][np] = sbux;
                    }
                }
            }
        }
        if (lb > m) {
            for (int n = nmin + la - m; n <= nmax - la + m - 2; ++n) {
                double saux = smat[n][npmin];
                for (int np = npmin + 1; np <= npmax - 2 * (la - m) - n + nmin + la - m - 1; ++np) {
                    const double sbux = -t_re[m + m + 1] * 0.5 * Rinv *
                                        (smat[n][np + 1] + R2 * saux - smat[n + 2][np - 1]);
                    saux = smat[n][np];
                    smataux[n][np] = saux;
                    smat[n][np] = sbux;
                }
            }
            for (int ll = m + 1; ll <= lb - 1; ++ll) {
                for (int n = nmin + la - m; n <= nmax - la + m - 2 * (ll + 1 - m); ++n) {
                    double saux = smat[n][npmin + ll - m];
                    for (int np = npmin + 1 + ll - m;
                         np <= npmax - 2 * (la - m) - n + nmin + la - m - ll + m - 1; ++np) {
                        const double sbux =
                            -t_re[ll + ll + 1] * 0.5 * t_reali[ll - m + 1] * Rinv *
                                (smat[n][np + 1] + R2 * saux - smat[n + 2][np - 1]) -
                            t_re[ll + m] * t_reali[ll - m + 1] * smataux[n][np];
                        saux = smat[n][np];
                        smataux[n][np] = saux;
                        smat[n][np] = sbux;
                    }
                }
            }
        }
        sol[m] = smat[na][nb];
        if (m == mtop) break;

        nmin += 1; nmax -= 3; npmin += 1; npmax -= 3;
        aux = updltm0i * 0.25 * t_re[m + m + 1] * t_re[m + m + 1] * Rinv * Rinv;
        for (int n = nmin; n <= nmax; ++n)
            for (int np = npmin; np <= npmax - n + nmin; ++np)
                smataux[n][np] = aux * (2.0 * (smatm[n + 1][np + 1] + R2 * (smatm[n + 1][np - 1] + smatm[n - 1][np + 1])) -
                                        smatm[n + 3][np - 1] - smatm[n - 1][np + 3] - R4 * smatm[n - 1][np - 1]);
        for (int n = nmin; n <= nmax; ++n)
            for (int np = npmin; np <= npmax - n + nmin; ++np) {
                smat[n][np] = smataux[n][np];
                smatm[n][np] = smataux[n][np];
            }
        updltm0i = 1.0;
    }
    return 0;
}

/* ---- rotation matrices for l <= 1 (ROTAR, overlap_D.f:983-1051) ----------
 * rl[l][m+1][mp+1] = r(m, m'; l) with cos/sin(gamma) fixed to (1, 0) as in
 * ROTATIONOVERLAP (overlap_D.f:576-580). */
static void rotation_l1(double cosal, double sinal, double cosbet, double sinbet, double rl[2][3][3]) {
    const double root2 = 1.414213562373095; /* literal used by ROTAR */
    const double cosga = 1.0, singa = 0.0;
    memset(rl, 0, sizeof(double) * 2 * 9);
    rl[0][1][1] = 1.0;
    double d11 = (1.0 + cosbet) * 0.5;
    double d10 = -sinbet / root2;
    double d1m = (1.0 - cosbet) * 0.5;
    double d01 = -d10;
    double d00 = d11 - d1m;
    const double cosag = cosal * cosga - sinal * singa;
    const double cosamg = cosal * cosga + sinal * singa;
    const double sinag = sinal * cosga + cosal * singa;
    const double sinamg = sinal * cosga - cosal * singa;
#define RL1(m, mp) rl[1][(m) + 1][(mp) + 1]
    RL1(0, 0) = d00;
    RL1(1, 0) = root2 * d01 * cosal;
    RL1(-1, 0) = root2 * d01 * sinal;
    RL1(0, 1) = root2 * d10 * cosga;
    RL1(0, -1) = -root2 * d10 * singa;
    RL1(1, 1) = d11 * cosag - d1m * cosamg;
    RL1(1, -1) = -d11 * sinag - d1m * sinamg;
    RL1(-1, 1) = d11 * sinag - d1m * sinamg;
    RL1(-1, -1) = d11 * cosag + d1m * cosamg;
#undef RL1
}

/* GET_ANOR (overlap_D.f:496-517) */
static double get_anor(double expa, double expb, int na, int nb, int la, int lb, double aux) {
    const double PI = 4.0 * atan(1.0);
    double anor = ipow(expa * 2.0, na * 2 + 1);
    anor = anor * ipow(expb * 2.0, nb * 2 + 1);
    anor = anor * (la * 2 + 1.0);
    anor = anor * (lb * 2 + 1.0);
    anor = anor * aux;
    return sqrt(anor) / (4.0 * PI);
}

/* GET_ANOR_DIVISOR (overlap_D.f:464-478) */
static double get_anor_divisor(int la, int lb, int m) {
    double d = (la + m + 1.0) * (la - m) * (lb + m + 1.0) * (lb - m);
    return sqrt(d);
}

/* One atom pair (ia > ib): accumulate the S(a, b) block, a on ia, b on ib
 * (inner loop of BUILD_OVERLAP_MATRIX, overlap_D.f:228-291). */
static int pair_block(const orc_basis *b, int ia, int ib, double cutoff, double *S) {
    const int N = b->nao;
    const double xa = b->coord[3 * ia], ya = b->coord[3 * ia + 1], za = b->coord[3 * ia + 2];
    const double xb = b->coord[3 * ib], yb = b->coord[3 * ib + 1], zb = b->coord[3 * ib + 2];
    const double xab = xb - xa, yab = yb - ya, zab = zb - za;
    const double xy = sqrt(xab * xab + yab * yab);
    double sinal, cosal;
    if (xy > 1.0e-10) {
        sinal = yab / xy;
        cosal = xab / xy;
    } else {
        sinal = 0.0;
        cosal = 1.0;
    }
    const double Rab = sqrt(xab * xab + yab * yab + zab * zab);
    const double sinbet = xy / Rab;
    const double cosbet = zab / Rab;
    if (Rab > cutoff) return 0;
    double rl[2][3][3];
    rotation_l1(cosal, sinal, cosbet, sinbet, rl);

    for (int jb = 0; jb < b->atom_nao[ib]; ++jb) {
        for (int ja = 0; ja < b->atom_nao[ia]; ++ja) {
            const int bb = b->atom_ao0[ib] + jb;
            const int aa = b->atom_ao0[ia] + ja;
            const int nb = b->ao_n[bb], lb = b->ao_l[bb], mb = b->ao_m[bb];
            const int na = b->ao_n[aa], la = b->ao_l[aa], ma = b->ao_m[aa];
            if (la > 1 || lb > 1) return -2;
            const double aux = 1.0 / (real_fact(na + na) * real_fact(nb + nb));
            const int msup = (la < lb) ? la : lb;
            double solnorm[ORC_MXL + 1] = {0};
            for (int j = 0; j < b->ao_nzeta[bb]; ++j) {
                for (int i = 0; i < b->ao_nzeta[aa]; ++i) {
                    const double expb = b->ao_zeta[2 * bb + j];
                    const double expa = b->ao_zeta[2 * aa + i];
                    double solvec[ORC_MXL + 1];
                    if (orc_solap(na, la, expa, nb, lb, expb, Rab, solvec)) return -3;
                    double anor = get_anor(expa, expb, na, nb, la, lb, aux);
                    double part[ORC_MXL + 1];
                    for (int m = 0; m <= msup - 1; ++m) {
                        part[m] = solvec[m] * anor;
                        anor = anor / get_anor_divisor(la, lb, m);
                        if (m == 0) anor = anor + anor;
                    }
                    part[msup] = solvec[msup] * anor;
                    for (int k = 0; k <= msup; ++k)
                        solnorm[k] = solnorm[k] + b->ao_coef[2 * aa + i] * b->ao_coef[2 * bb + j] * part[k];
                }
            }
            double sux[ORC_MXL + 1];
            sux[0] = solnorm[0] * rl[la][ma + 1][1] * rl[lb][mb + 1][1];
            for (int k = 1; k <= msup; ++k)
                sux[k] = solnorm[k] * (rl[la][ma + 1][1 - k] * rl[lb][mb + 1][1 - k] +
                                       rl[la][ma + 1][1 + k] * rl[lb][mb + 1][1 + k]);
            double s = 0.0;
            for (int k = 0; k <= msup; ++k) s += sux[k];
            S[(size_t)bb * N + aa] += s; /* S(a,b), column-major */
        }
    }
    return 0;
}

int orc_overlap(const orc_basis *b, double cutoff, double *S, int nthreads) {
    build_tables();
    const int N = b->nao;
    memset(S, 0, sizeof(double) * (size_t)N * N);
    int err = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(| : err)
#endif
    for (int ib = 0; ib < b->natoms; ++ib)
        for (int ia = ib + 1; ia < b->natoms; ++ia) err |= (pair_block(b, ia, ib, cutoff, S) != 0);
    (void)nthreads;
    for (int i = 0; i < N; ++i) S[(size_t)i * N + i] = 1.0;
    /* upper triangle from the lower (overlap_D.f:309) */
    for (int i = 0; i < N; ++i)
        for (int j = i + 1; j < N; ++j) S[(size_t)j * N + i] = S[(size_t)i * N + j];
    return err ? -1 : 0;
}

/* X_ij (hamiltonians.f:33-63) */
static double x_ij(const orc_basis *b, int i, int j) {
    if (i == j) return b->ao_ip[i] + b->ao_vshift[i];
    const double c1 = b->ao_ip[i] - b->ao_ip[j];
    const double c2 = b->ao_ip[i] + b->ao_ip[j];
    const double c3 = (c1 / c2) * (c1 / c2);
    const double c4 = (b->ao_vshift[i] + b->ao_vshift[j]) * 0.5;
    const double kwh = (b->ao_kwh[i] + b->ao_kwh[j]) * 0.5;
    const double keff = kwh + c3 + c3 * c3 * (1.0 - kwh);
    return keff * c2 * 0.5 + c4;
}

void orc_huckel(const orc_basis *b, const double *S, double *h) {
    const int N = b->nao;
    for (int j = 0; j < N; ++j)
        for (int i = 0; i <= j; ++i) {
            const double v = x_ij(b, i, j) * S[(size_t)j * N + i];
            h[(size_t)j * N + i] = v;
            h[(size_t)i * N + j] = v;
        }
}

/* ---- dzgemv: real A times complex x, complex alpha (Matrix_math.f:225-301) */
void orc_dzgemv(int trans, int N, const double *A, const double *x, const double *alpha,
                double *res, int nthreads) {
    const double ar = alpha[0], ai = alpha[1];
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
    (void)nthreads;
    if (trans) {
        /* res_j = alpha * sum_i A(i,j) x_i : column dots */
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
        for (int j = 0; j < N; ++j) {
            const double *col = A + (size_t)j * N;
            double sr = 0.0, si = 0.0;
            for (int i = 0; i < N; ++i) {
                sr += col[i] * x[2 * i];
                si += col[i] * x[2 * i + 1];
            }
            res[2 * j] = ar * sr - ai * si;
            res[2 * j + 1] = ar * si + ai * sr;
        }
    } else {
        /* res_i = alpha * sum_j A(i,j) x_j : row blocks, contiguous column segments */
        const int RB = 256;
        const int nblk = (N + RB - 1) / RB;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
        for (int blk = 0; blk < nblk; ++blk) {
            const int i0 = blk * RB, i1 = (i0 + RB < N) ? i0 + RB : N;
            double accr[256], acci[256];
            for (int i = i0; i < i1; ++i) accr[i - i0] = acci[i - i0] = 0.0;
            for (int j = 0; j < N; ++j) {
                const double *col = A + (size_t)j * N;
                const double xr = x[2 * j], xi = x[2 * j + 1];
                for (int i = i0; i < i1; ++i) {
                    accr[i - i0] += col[i] * xr;
                    acci[i - i0] += col[i] * xi;
                }
            }
            for (int i = i0; i < i1; ++i) {
                const double sr = accr[i - i0], si = acci[i - i0];
                res[2 * i] = ar * sr - ai * si;
                res[2 * i + 1] = ar * si + ai * sr;
            }
        }
    }
}

/* ---- Taylor propagator (Taylor.f:35-239) ---------------------------------- */
#define ORDER 25
static const double H_BAR = 6.58264e-4; /* eV ps, constants_m.f:23 */

/* coefficient(tau, order): c1 = 1, c_k = -i c_{k-1} tau/(k-1) (Taylor.f:224-239); 0-based here */
static void coefficients(double tau, double *c /* [ORDER*2] */) {
    c[0] = 1.0;
    c[1] = 0.0;
    for (int k = 1; k < ORDER; ++k) {
        const double f = tau / k;
        /* -i * c * f */
        const double pr = c[2 * (k - 1)], pi = c[2 * (k - 1) + 1];
        const double qr = pi, qi = -pr; /* -i*(pr + i pi) = pi - i pr */
        c[2 * k] = qr * f;
        c[2 * k + 1] = qi * f;
    }
}

static void cdiv(const double *a, const double *b, double *q) {
    /* q = a / b (plain complex division; the ratio is a pure imaginary multiple of tau/k) */
    const double d = b[0] * b[0] + b[1] * b[1];
    q[0] = (a[0] * b[0] + a[1] * b[1]) / d;
    q[1] = (a[1] * b[0] - a[0] * b[1]) / d;
}

static double dotc_abs(int N, const double *x, const double *y) {
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < N; ++i) {
        /* conj(x) * y */
        sr += x[2 * i] * y[2 * i] + x[2 * i + 1] * y[2 * i + 1];
        si += x[2 * i] * y[2 * i + 1] - x[2 * i + 1] * y[2 * i];
    }
    return hypot(sr, si);
}

static int all_close(int N, const double *a, const double *b, double tol) {
    for (int i = 0; i < N; ++i)
        if (hypot(a[2 * i] - b[2 * i], a[2 * i + 1] - b[2 * i + 1]) > tol) return 0;
    return 1;
}

typedef struct {
    int N;
    const double *Hp;
    double *tb0, *tb1, *tk0, *tk1; /* previous / current term */
    double *ob, *nb, *ok_, *nk;    /* old / new partial sums */
    int nthreads;
    orc_prop_stats *st;
} orc_ws;

/* Convergence (Taylor.f:132-219).  Returns OK flag; writes k_ref and C. */
static int convergence(orc_ws *w, double *bra, double *ket, double *C, int *k_ref, double tau,
                       double norm_ref, double tol, double norm_tol) {
    const int N = w->N;
    const size_t vb = sizeof(double) * 2 * (size_t)N;
    w->st->conv_calls++;
    coefficients(tau, C);
    int k_max = ORDER; /* 1-based */
    for (int k = 2; k <= ORDER; ++k)
        if (hypot(C[2 * (k - 1)], C[2 * (k - 1) + 1]) < 1.0e-16) {
            k_max = k;
            break;
        }
    *k_ref = k_max;
    memcpy(w->tb0, bra, vb);
    memcpy(w->tk0, ket, vb);
    memcpy(w->ob, bra, vb);
    memcpy(w->ok_, ket, vb);
    double *pb = w->tb0, *pk = w->tk0, *cb = w->tb1, *ck = w->tk1;
    double *ob = w->ob, *okk = w->ok_, *nb = w->nb, *nk = w->nk;
    for (int k = 2; k <= k_max; ++k) {
        double r[2];
        cdiv(&C[2 * (k - 1)], &C[2 * (k - 2)], r);
        orc_dzgemv(1, N, w->Hp, pb, r, cb, w->nthreads);
        orc_dzgemv(0, N, w->Hp, pk, r, ck, w->nthreads);
        w->st->gemv_terms++;
        for (int i = 0; i < 2 * N; ++i) {
            nb[i] = ob[i] + cb[i];
            nk[i] = okk[i] + ck[i];
        }
        if (all_close(N, nb, ob, tol) && all_close(N, nk, okk, tol)) {
            const double nt = dotc_abs(N, nb, nk);
            if (fabs(nt - norm_ref) < norm_tol) {
                memcpy(bra, nb, vb);
                memcpy(ket, nk, vb);
                return 1;
            }
        }
        double *t;
        t = ob; ob = nb; nb = t;
        t = okk; okk = nk; nk = t;
        t = pb; pb = cb; cb = t;
        t = pk; pk = ck; ck = t;
    }
    return 0;
}

int orc_propagation(int N, const double *Hp, double *bra, double *ket,
                    double t_init, double t_max, double *tau, double *save_tau,
                    double tol, double norm_tol, int max_conv_calls, int nthreads,
                    orc_prop_stats *stats) {
    orc_prop_stats local = {0, 0, 0, 0};
    orc_prop_stats *st = stats ? stats : &local;
    memset(st, 0, sizeof(*st));
    const size_t vb = sizeof(double) * 2 * (size_t)N;
    double *mem = (double *)malloc(vb * 10);
    if (!mem) return -1;
    orc_ws w;
    w.N = N; w.Hp = Hp; w.nthreads = nthreads; w.st = st;
    w.tb0 = mem; w.tb1 = mem + 2 * N; w.tk0 = mem + 4 * N; w.tk1 = mem + 6 * N;
    w.ob = mem + 8 * N; w.nb = mem + 10 * N; w.ok_ = mem + 12 * N; w.nk = mem + 14 * N;
    double *sb = mem + 16 * N, *sk = mem + 18 * N; /* sub-step partial sums */
    double C[2 * ORDER];
    int k_ref = ORDER;

    const double norm_ref = dotc_abs(N, bra, ket);
    int ok = 0;
    for (;;) {
        if (st->conv_calls >= max_conv_calls) { st->status = 1; free(mem); return 1; }
        ok = convergence(&w, bra, ket, C, &k_ref, *tau, norm_ref, tol, norm_tol);
        if (ok) break;
        *tau = *tau * 0.9;
    }
    *save_tau = *tau;
    st->substeps++;
    double t = t_init + *tau * H_BAR;
    if (t_max - t < *tau * H_BAR) {
        *tau = (t_max - t) / H_BAR;
        coefficients(*tau, C);
    }
    while (t < t_max) {
        /* one sub-step of k_ref terms, no per-term test (Taylor.f:81-100) */
        memcpy(w.tb0, bra, vb);
        memcpy(w.tk0, ket, vb);
        memcpy(sb, bra, vb);
        memcpy(sk, ket, vb);
        double *pb = w.tb0, *pk = w.tk0, *cb = w.tb1, *ck = w.tk1;
        for (int k = 2; k <= k_ref; ++k) {
            double r[2];
            cdiv(&C[2 * (k - 1)], &C[2 * (k - 2)], r);
            orc_dzgemv(1, N, Hp, pb, r, cb, nthreads);
            orc_dzgemv(0, N, Hp, pk, r, ck, nthreads);
            st->gemv_terms++;
            for (int i = 0; i < 2 * N; ++i) {
                sb[i] = sb[i] + cb[i];
                sk[i] = sk[i] + ck[i];
            }
            double *tt;
            tt = pb; pb = cb; cb = tt;
            tt = pk; pk = ck; ck = tt;
        }
        const double nt = dotc_abs(N, sb, sk);
        if (fabs(nt - norm_ref) < norm_tol) {
            memcpy(bra, sb, vb);
            memcpy(ket, sk, vb);
        } else {
            ok = 0;
            while (!ok) {
                if (st->conv_calls >= max_conv_calls) { st->status = 1; free(mem); return 1; }
                *tau = *tau * 0.975;
                ok = convergence(&w, bra, ket, C, &k_ref, *tau, norm_ref, tol, norm_tol);
            }
        }
        st->substeps++;
        t = t + (*tau * H_BAR);
        if (t_max - t < *tau * H_BAR) {
            *tau = (t_max - t) / H_BAR;
            coefficients(*tau, C);
        }
    }
    free(mem);
    return 0;
}

void orc_populations(int N, const int *ao_frag, int nfrag, const double *psi_bra,
                     const double *psi_ket, double *pop) {
    for (int f = 0; f <= nfrag; ++f) pop[f] = 0.0;
    double tot = 0.0;
    for (int i = 0; i < N; ++i) {
        /* DUAL_bra = conj(Psi_ket), DUAL_ket = Psi_bra (ElHl_Chebyshev.f:270-271) */
        const double v = psi_ket[2 * i] * psi_bra[2 * i] + psi_ket[2 * i + 1] * psi_bra[2 * i + 1];
        if (ao_frag && ao_frag[i] >= 0 && ao_frag[i] < nfrag) pop[ao_frag[i]] += v;
        tot += v;
    }
    pop[nfrag] = tot;
}
