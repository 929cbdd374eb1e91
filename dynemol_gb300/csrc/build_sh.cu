// Device build of the STO overlap S and the extended-Hueckel h for one
// nuclear configuration.
//
// One thread per atom pair (ia >= ib).  Each thread writes its whole AO
// block of S and h and the transposed block, so every element of the two
// N x N matrices is written exactly once (no memset, no atomics).
//
//   lined-up overlaps ... SOLAP (overlap_D.f:701-962): Fernandez-Rico 1F1
//                         expansion of <n00|n'00>, then recurrences in l, l', m
//   rotation ............ ROTAR for l <= 1 (overlap_D.f:983-1027), gamma = 0
//   normalisation ....... GET_ANOR / GET_ANOR_DIVISOR (overlap_D.f:464-517)
//   assembly ............ BUILD_OVERLAP_MATRIX (overlap_D.f:228-291), diag 1
//   Hueckel ............. h_ij = X_ij S_ij, weighted Wolfsberg-Helmholz
//                         (hamiltonians.f:33-63, ElHl_Chebyshev.f:313-321)
//
// Supported basis: n <= 3, l <= 1, one or two zetas (the H/C/O EHT basis of
// the workloads).  re(i) = i is evaluated inline; 1/i, i! and 1/i! come from
// device tables holding the same IEEE values the reference tabulates.
#include "elhl_internal.cuh"

namespace elhl {
namespace {

constexpr int kMaxN = 3;
constexpr int kMaxL = 1;
constexpr int kNT = kMaxN + 3 * kMaxL + 1;  // n index bound: na + la + 2 lb <= 6 -> 7 entries
constexpr int kHR = kNT + 2;                // 1F1 rows (alpha up to namax + 1)
constexpr int kHC = 2 * kNT + 2;            // 1F1 columns (gamma up to ngmax)
constexpr int kMaxShell = 4;                // radial shells per atom handled per shell pair

// Constant tables (UTIL_OVERLAP, overlap_D.f:1194-1231): 1/i (0 at i = 0), i!
// and 1/i!.  Filled once per device by init_tables; FP64 division is slow on
// this part, so the inner loops read tables instead of dividing.
__device__ double g_reali[1001];
__device__ double g_fact[32];
__device__ double g_facti[32];

__global__ void init_tables_kernel() {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= 1000) g_reali[i] = (i == 0) ? 0.0 : 1.0 / (double)i;
    if (i == 0) {
        double f = 1.0;
        g_fact[0] = 1.0;
        g_facti[0] = 1.0;
        for (int k = 1; k < 32; ++k) {
            f = f * (double)k;
            g_fact[k] = f;
            g_facti[k] = 1.0 / f;
        }
    }
}

__device__ __forceinline__ double rcp_int(int i) { return __ldg(&g_reali[i]); }
__device__ __forceinline__ double dfact(int n) { return __ldg(&g_fact[n]); }
__device__ __forceinline__ double dfacti(int n) { return __ldg(&g_facti[n]); }

// 1F1[i, j, arg] for i = 1..namax and j = 2..ngmax, arg = (z - zp) R, as SOLAP
// builds it (overlap_D.f:766-819): column ngmax from the series pair at ia and
// ia + 1 and the three-term recursion in i, then the columns j < ngmax by the
// contiguous relations, downwards.  Entry [i][j] is filled for i <= min(namax, j - 1).
__device__ void h1f1_table(double z, double zp, double R, int ngmax, int namax, double (&h1f1)[kHR][kHC]) {
    const double arg = (z - zp) * R;
    int ia = (ngmax - (int)z) / 2;
    if (ia < 1) ia = 1;
    if (ia >= namax) ia = namax - 1;

    // 1F1[ia, ngmax, arg] and 1F1[ia+1, ngmax, arg] by their series
    double ta = arg * (double)ia * rcp_int(ngmax), fa = 1.0;
    double tb = arg * (double)(ia + 1) * rcp_int(ngmax), fb = 1.0;
    const int imax = 1000 - ngmax - 1;
    for (int i = 1; i <= imax; ++i) {
        fa = fa + ta;
        fb = fb + tb;
        ta = ta * (double)(ia + i) * arg * rcp_int(ngmax + i) * rcp_int(i + 1);
        tb = tb * (double)(ia + i + 1) * arg * rcp_int(ngmax + i) * rcp_int(i + 1);
        if (tb < 1.0e-35 * fb) break;
    }
    h1f1[ia][ngmax] = fa;
    h1f1[ia + 1][ngmax] = fb;
    double aux = arg - (double)ngmax;
    for (int i = ia + 1; i <= namax - 1; ++i)
        h1f1[i + 1][ngmax] = ((aux + (double)(i + i)) * h1f1[i][ngmax] + (double)(ngmax - i) * h1f1[i - 1][ngmax]) * rcp_int(i);
    for (int i = ia; i >= 2; --i)
        h1f1[i - 1][ngmax] = ((double)i * h1f1[i + 1][ngmax] - (aux + (double)(i + i)) * h1f1[i][ngmax]) * rcp_int(ngmax - i);
    for (int j = ngmax - 1; j >= 2; --j) {
        h1f1[1][j] = (h1f1[2][j + 1] + (double)(j - 1) * h1f1[1][j + 1]) * rcp_int(j);
        aux = arg * rcp_int(j);
        const int itop = min(namax - 1, j - 2);
        for (int i = 1; i <= itop; ++i) h1f1[i + 1][j] = aux * h1f1[i + 1][j + 1] + h1f1[i][j];
    }
}

// basic integral <N00|N'00> for the index n of the larger exponent z and np of
// the smaller zp (SOLAP's loop body, overlap_D.f:821-850); zpow[e] = (z + zp)^-e
// by repeated products, the same sequence SOLAP's running products take
__device__ double basic_integral(int n, int np, double z, double zp, double R, double expzR,
                                 const double (&h1f1)[kHR][kHC], const double *zpow) {
    const double pi4 = 12.566370614359172953850573533118012;
    const double zzpR = (z + zp) * R;
    double auxk = dfact(n + np) * zpow[n + np + 1];
    double sumk = 0.0;
    for (int k = 0; k <= n + np; ++k) {
        double sumj = 0.0;
        for (int j = max(0, k - n); j <= min(k, np); ++j)
            sumj = sumj + h1f1[j + 1][k + 2] * dfacti(n + j - k) * dfacti(np - j);
        sumk = sumk + sumj * auxk;
        auxk = auxk * zzpR * rcp_int(n + np - k) * rcp_int(k + 2);
    }
    return pi4 * expzR * dfact(n) * dfact(np) * sumk;
}

// index ranges of one lined-up overlap in the orientation of the basic integrals
// (n: the atom with the larger exponent, np: the other)
struct SolapRange {
    int nmin, nmax, npmin, npmax;
};
__device__ __forceinline__ SolapRange solap_range(int na, int la, int nb, int lb, bool a_big) {
    return a_big ? SolapRange{na - la, na + la + 2 * lb, nb - lb, nb + lb + 2 * la}
                 : SolapRange{nb - lb, nb + lb + 2 * la, na - la, na + la + 2 * lb};
}

// the l, l' and m recurrences of SOLAP (overlap_D.f:852-962) from the basic
// integrals base[n_a][n_b]: <na la m | nb lb m>, m = 0..min(la, lb)
__device__ void lined_up_from_base(int na, int la, int nb, int lb, double R, const double (&base)[kNT][kNT],
                                   double *sol) {
    double smat[kNT][kNT], saux_l[kNT][kNT], sbase[kNT][kNT];
    for (int i = 0; i < kNT; ++i)
        for (int j = 0; j < kNT; ++j) smat[i][j] = saux_l[i][j] = sbase[i][j] = base[i][j];
    int nmin = na - la, nmax = na + la + 2 * lb, npmin = nb - lb, npmax = nb + lb + 2 * la;
    const double Rinv = 1.0 / R, R2 = R * R, R4 = R2 * R2;
    double m0 = 0.5;
    const int mtop = min(la, lb);
    for (int m = 0; m <= mtop; ++m) {
        if (la > m) {  // raise l on A (l = m -> m+1; l <= 1 so no second rung)
            for (int np = npmin; np <= npmax - 2; ++np) {
                double prev = smat[nmin][np];
                for (int n = nmin + 1; n <= nmax - 1 - np + npmin; ++n) {
                    const double v = (double)(m + m + 1) * 0.5 * Rinv * (smat[n + 1][np] + R2 * prev - smat[n - 1][np + 2]);
                    prev = smat[n][np];
                    saux_l[n][np] = prev;
                    smat[n][np] = v;
                }
            }
        }
        if (lb > m) {  // raise l' on B
            for (int n = nmin + la - m; n <= nmax - la + m - 2; ++n) {
                double prev = smat[n][npmin];
                for (int np = npmin + 1; np <= npmax - 2 * (la - m) - n + nmin + la - m - 1; ++np) {
                    const double v = -(double)(m + m + 1) * 0.5 * Rinv * (smat[n][np + 1] + R2 * prev - smat[n + 2][np - 1]);
                    prev = smat[n][np];
                    saux_l[n][np] = prev;
                    smat[n][np] = v;
                }
            }
        }
        sol[m] = smat[na][nb];
        if (m == mtop) break;
        nmin += 1; nmax -= 3; npmin += 1; npmax -= 3;
        const double aux = m0 * 0.25 * (double)(m + m + 1) * (double)(m + m + 1) * Rinv * Rinv;
        for (int n = nmin; n <= nmax; ++n)
            for (int np = npmin; np <= npmax - n + nmin; ++np)
                saux_l[n][np] = aux * (2.0 * (sbase[n + 1][np + 1] + R2 * (sbase[n + 1][np - 1] + sbase[n - 1][np + 1])) -
                                       sbase[n + 3][np - 1] - sbase[n - 1][np + 3] - R4 * sbase[n - 1][np - 1]);
        for (int n = nmin; n <= nmax; ++n)
            for (int np = npmin; np <= npmax - n + nmin; ++np) {
                smat[n][np] = saux_l[n][np];
                sbase[n][np] = saux_l[n][np];
            }
        m0 = 1.0;
    }
}

__device__ __forceinline__ bool supported(int n, int l) { return n >= 1 && n <= kMaxN && l >= 0 && l <= kMaxL; }

// <na la m | nb lb m>, m = 0..min(la, lb), lined-up frame (SOLAP,
// overlap_D.f:701-962).  Returns false on quantum numbers outside the supported range.
__device__ bool lined_up_overlap(int na, int la, double za, int nb, int lb, double zb, double R,
                                 double *sol) {
    if (!supported(na, la) || !supported(nb, lb)) return false;
    double h1f1[kHR][kHC];
    double base[kNT][kNT] = {};
    const bool a_big = (za >= zb);
    const double z = a_big ? za : zb, zp = a_big ? zb : za;
    const SolapRange r = solap_range(na, la, nb, lb, a_big);
    h1f1_table(z, zp, R, r.nmax + r.npmax + 2, r.npmax + 1, h1f1);
    const double expzR = exp(-z * R), zzpi = 1.0 / (z + zp);
    double zpow[2 * kNT + 1];
    zpow[0] = 1.0;
    for (int e = 1; e <= 2 * kNT; ++e) zpow[e] = zpow[e - 1] * zzpi;
    for (int n = r.nmin; n <= r.nmax; ++n)
        for (int np = r.npmin; np <= r.npmax - n + r.nmin; ++np) {
            const double v = basic_integral(n, np, z, zp, R, expzR, h1f1, zpow);
            if (a_big) base[n][np] = v;
            else base[np][n] = v;
        }
    lined_up_from_base(na, la, nb, lb, R, base, sol);
    return true;
}

// Every shell pair of an atom pair whose shells all carry one exponent per atom
// (za for A, zb for B; the H/C/O EHT basis): the lined-up overlaps sol[p][q][m]
// from one 1F1 table, built at the largest (ngmax, namax) of the pairs, and one
// basic integral per (n, n') cell that some pair reads; each pair then runs only
// its own l, l' and m recurrences.  Per pair SOLAP rebuilds both (four times for
// the s/p shells of two C atoms), and they are most of the build's FP64
// instructions.  The shared table's columns below a pair's own ngmax come from
// the same downward relations started higher up, so values differ from the
// per-pair ones by rounding only.  Returns false on unsupported quantum numbers.
__device__ bool shared_lined_up(const int *na, const int *la, int nsa, double za, const int *nb, const int *lb,
                                int nsb, double zb, double R, double (*sol)[kMaxShell][kMaxL + 1]) {
    const bool a_big = (za >= zb);
    const double z = a_big ? za : zb, zp = a_big ? zb : za;
    int ngmax = 0, namax = 0;
    unsigned long long needl = 0;  // cells (n, np) of the basic integrals some pair reads: bit n * kNT + np
    for (int p = 0; p < nsa; ++p)
        for (int q = 0; q < nsb; ++q) {
            if (!supported(na[p], la[p]) || !supported(nb[q], lb[q])) return false;
            const SolapRange r = solap_range(na[p], la[p], nb[q], lb[q], a_big);
            ngmax = max(ngmax, r.nmax + r.npmax + 2);
            namax = max(namax, r.npmax + 1);
            for (int n = r.nmin; n <= r.nmax; ++n)
                for (int np = r.npmin; np <= r.npmax - n + r.nmin; ++np) needl |= 1ull << (n * kNT + np);
        }
    double h1f1[kHR][kHC];
    h1f1_table(z, zp, R, ngmax, namax, h1f1);
    const double expzR = exp(-z * R), zzpi = 1.0 / (z + zp);
    double zpow[2 * kNT + 1];
    zpow[0] = 1.0;
    for (int e = 1; e <= 2 * kNT; ++e) zpow[e] = zpow[e - 1] * zzpi;
    double base[kNT][kNT] = {};
    for (int n = 0; n < kNT; ++n)
        for (int np = 0; np < kNT; ++np) {
            if (!((needl >> (n * kNT + np)) & 1ull)) continue;
            const double v = basic_integral(n, np, z, zp, R, expzR, h1f1, zpow);
            if (a_big) base[n][np] = v;
            else base[np][n] = v;
        }
    for (int p = 0; p < nsa; ++p)
        for (int q = 0; q < nsb; ++q) lined_up_from_base(na[p], la[p], nb[q], lb[q], R, base, sol[p][q]);
    return true;
}

__device__ __forceinline__ double anor(double ea, double eb, int na, int nb, int la, int lb, double aux) {
    double a = 1.0;
    for (int e = 0; e < 2 * na + 1; ++e) a *= ea * 2.0;
    double b = 1.0;
    for (int e = 0; e < 2 * nb + 1; ++e) b *= eb * 2.0;
    double v = a * b;
    v = v * (la * 2 + 1.0);
    v = v * (lb * 2 + 1.0);
    v = v * aux;
    const double PI = 3.141592653589793;  // 4 atan(1), the nearest double to pi (GET_ANOR's PI)
    return sqrt(v) / (4.0 * PI);
}

__device__ __forceinline__ double x_ij(double ipi, double ipj, double vi, double vj, double ki, double kj) {
    const double c1 = ipi - ipj, c2 = ipi + ipj;
    const double c3 = (c1 / c2) * (c1 / c2);
    const double c4 = (vi + vj) * 0.5;
    const double k = (ki + kj) * 0.5;
    const double keff = k + c3 + c3 * c3 * (1.0 - k);
    return keff * c2 * 0.5 + c4;
}

// Shells of one atom: runs of consecutive AOs with the same n, l, zetas and
// coefficients (the m components of one radial function).  The lined-up
// overlaps depend on the shells only, so they are computed once per shell pair
// and the rotation is applied per AO pair.

__device__ bool same_radial(const DevBasis &b, int x, int y) {
    return b.ao_n[x] == b.ao_n[y] && b.ao_l[x] == b.ao_l[y] && b.ao_nzeta[x] == b.ao_nzeta[y] &&
           b.ao_zeta[2 * x] == b.ao_zeta[2 * y] && b.ao_zeta[2 * x + 1] == b.ao_zeta[2 * y + 1] &&
           b.ao_coef[2 * x] == b.ao_coef[2 * y] && b.ao_coef[2 * x + 1] == b.ao_coef[2 * y + 1];
}

// shell index of every AO of an atom (ao0, nao); returns the shell count, or
// -1 when the atom has more than kMaxShell shells.  first[s] = first AO of shell s.
__device__ int atom_shells(const DevBasis &b, int ao0, int nao, int *first, int *shell_of) {
    int ns = 0;
    for (int j = 0; j < nao; ++j) {
        if (j == 0 || !same_radial(b, ao0 + j, ao0 + j - 1)) {
            if (ns == kMaxShell) return -1;
            first[ns++] = ao0 + j;
        }
        shell_of[j] = ns - 1;
    }
    return ns;
}

// solnorm[m] += c_i c_j N_ij sol[m] for the zeta pair (i of aa, j of bb): the
// normalisation and contraction of BUILD_OVERLAP_MATRIX (overlap_D.f:228-280)
__device__ void add_normalised(const DevBasis &b, int aa, int bb, int i, int j, const double *sol, double *solnorm) {
    const int na = b.ao_n[aa], la = b.ao_l[aa];
    const int nb = b.ao_n[bb], lb = b.ao_l[bb];
    const double aux = 1.0 / (dfact(na + na) * dfact(nb + nb));
    const int msup = min(la, lb);
    const double eb = b.ao_zeta[2 * bb + j], ea = b.ao_zeta[2 * aa + i];
    double an = anor(ea, eb, na, nb, la, lb, aux);
    double part[kMaxL + 1];
    for (int m = 0; m <= msup - 1; ++m) {
        part[m] = sol[m] * an;
        an = an / sqrt((la + m + 1.0) * (la - m) * (lb + m + 1.0) * (lb - m));
        if (m == 0) an = an + an;
    }
    part[msup] = sol[msup] * an;
    const double cc = b.ao_coef[2 * aa + i] * b.ao_coef[2 * bb + j];
    for (int k = 0; k <= msup; ++k) solnorm[k] = solnorm[k] + cc * part[k];
}

// normalised, contracted lined-up overlaps <aa|bb>_m, m = 0..min(la, lb)
// (the SOLAP + GET_ANOR part of BUILD_OVERLAP_MATRIX, overlap_D.f:228-280)
__device__ void contracted_overlap(const DevBasis &b, int aa, int bb, double R, double *solnorm) {
    solnorm[0] = solnorm[1] = 0.0;
    for (int j = 0; j < b.ao_nzeta[bb]; ++j) {
        for (int i = 0; i < b.ao_nzeta[aa]; ++i) {
            double sol[kMaxL + 1];
            if (!lined_up_overlap(b.ao_n[aa], b.ao_l[aa], b.ao_zeta[2 * aa + i], b.ao_n[bb], b.ao_l[bb],
                                  b.ao_zeta[2 * bb + j], R, sol)) {
                sol[0] = sol[1] = __longlong_as_double(0x7ff8000000000000ULL);  // NaN marks unsupported
            }
            add_normalised(b, aa, bb, i, j, sol, solnorm);
        }
    }
}

// the single exponent carried by every shell (first AOs first[0..ns)) of an atom, if there is one
__device__ bool uniform_zeta(const DevBasis &b, const int *first, int ns, double *z) {
    const double z0 = b.ao_zeta[2 * first[0]];
    for (int s = 0; s < ns; ++s)
        if (b.ao_nzeta[first[s]] != 1 || b.ao_zeta[2 * first[s]] != z0) return false;
    *z = z0;
    return true;
}

// S block of atoms ia != ib for B - A = (xab, yab, zab) (Angstrom): calls
// out(ja, jb, s) for every AO pair (a0 + ja of ia, b0 + jb of ib); s = 0 beyond
// the cutoff.  ROTATIONOVERLAP (overlap_D.f:520-583, l <= 1), SOLAP + GET_ANOR
// once per shell pair, rotation to the molecular frame per AO pair
// (BUILD_OVERLAP_MATRIX, overlap_D.f:228-291).
template <typename Out>
__device__ void pair_overlap_block(const DevBasis &b, int ia, int ib, double xab, double yab, double zab,
                                   double cutoff, Out &&out) {
    const int a0 = b.atom_ao0[ia], na_ao = b.atom_nao[ia];
    const int b0 = b.atom_ao0[ib], nb_ao = b.atom_nao[ib];
    const double xy = sqrt(xab * xab + yab * yab);
    double sinal = 0.0, cosal = 1.0;
    if (xy > 1.0e-10) {
        sinal = yab / xy;
        cosal = xab / xy;
    }
    const double R = sqrt(xab * xab + yab * yab + zab * zab);
    const bool inside = !(R > cutoff);

    // rotation matrices r(m, m'; l) for l = 0, 1: rot[l][m+1][m'+1]
    double rot[2][3][3];
    if (inside) {
        const double sinbet = xy / R, cosbet = zab / R;
        const double root2 = 1.414213562373095;  // literal used by ROTAR
        const double d11 = (1.0 + cosbet) * 0.5, d10 = -sinbet / root2, d1m = (1.0 - cosbet) * 0.5;
        const double d01 = -d10, d00 = d11 - d1m;
        for (int l = 0; l < 2; ++l)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) rot[l][i][j] = 0.0;
        rot[0][1][1] = 1.0;
        rot[1][1][1] = d00;
        rot[1][2][1] = root2 * d01 * cosal;
        rot[1][0][1] = root2 * d01 * sinal;
        rot[1][1][2] = root2 * d10;
        rot[1][1][0] = -root2 * d10 * 0.0;
        rot[1][2][2] = d11 * cosal - d1m * cosal;
        rot[1][2][0] = -d11 * sinal - d1m * sinal;
        rot[1][0][2] = d11 * sinal - d1m * sinal;
        rot[1][0][0] = d11 * cosal + d1m * cosal;
    }

    // lined-up overlaps once per shell pair (per AO pair when an atom has more shells)
    int fa[kMaxShell], fb[kMaxShell], sha[16], shb[16];
    const int nsa = (inside && na_ao <= 16) ? atom_shells(b, a0, na_ao, fa, sha) : -1;
    const int nsb = (inside && nb_ao <= 16) ? atom_shells(b, b0, nb_ao, fb, shb) : -1;
    const bool shells = nsa > 0 && nsb > 0;
    double sn[kMaxShell][kMaxShell][kMaxL + 1];
    if (shells) {
        double za = 0.0, zb = 0.0;
        bool done = false;
        if (uniform_zeta(b, fa, nsa, &za) && uniform_zeta(b, fb, nsb, &zb)) {
            int nas[kMaxShell], las[kMaxShell], nbs[kMaxShell], lbs[kMaxShell];
            for (int p = 0; p < nsa; ++p) { nas[p] = b.ao_n[fa[p]]; las[p] = b.ao_l[fa[p]]; }
            for (int q = 0; q < nsb; ++q) { nbs[q] = b.ao_n[fb[q]]; lbs[q] = b.ao_l[fb[q]]; }
            double sol[kMaxShell][kMaxShell][kMaxL + 1];
            if (shared_lined_up(nas, las, nsa, za, nbs, lbs, nsb, zb, R, sol)) {
                for (int q = 0; q < nsb; ++q)
                    for (int p = 0; p < nsa; ++p) {
                        sn[p][q][0] = sn[p][q][1] = 0.0;
                        add_normalised(b, fa[p], fb[q], 0, 0, sol[p][q], sn[p][q]);
                    }
                done = true;
            }
        }
        if (!done)
            for (int q = 0; q < nsb; ++q)
                for (int p = 0; p < nsa; ++p) contracted_overlap(b, fa[p], fb[q], R, sn[p][q]);
    }

    for (int jb = 0; jb < nb_ao; ++jb) {
        const int bb = b0 + jb;
        for (int ja = 0; ja < na_ao; ++ja) {
            const int aa = a0 + ja;
            double s = 0.0;
            if (inside) {
                const int la = b.ao_l[aa], ma = b.ao_m[aa];
                const int lb = b.ao_l[bb], mb = b.ao_m[bb];
                const int msup = min(la, lb);
                double solnorm[kMaxL + 1];
                if (shells) {
                    solnorm[0] = sn[sha[ja]][shb[jb]][0];
                    solnorm[1] = sn[sha[ja]][shb[jb]][1];
                } else {
                    contracted_overlap(b, aa, bb, R, solnorm);
                }
                double sux0 = solnorm[0] * rot[la][ma + 1][1] * rot[lb][mb + 1][1];
                s = sux0;
                if (msup >= 1) {
                    const double sux1 = solnorm[1] * (rot[la][ma + 1][0] * rot[lb][mb + 1][0] +
                                                      rot[la][ma + 1][2] * rot[lb][mb + 1][2]);
                    s = s + sux1;
                }
            }
            out(ja, jb, s);
        }
    }
}

// One thread per atom pair.  Threads walk the pairs in b.atom_order (atoms
// grouped by kind), so that the lanes of a warp mostly take the same shell and
// zeta loops; each pair is computed as (ia, ib) with ia >= ib in the input order,
// the same arithmetic whatever the walk.
__global__ void build_sh_kernel(DevBasis b, const double *__restrict__ coords, double cutoff,
                                double *__restrict__ S, double *__restrict__ h, int ld) {
    const int py = blockIdx.y * blockDim.y + threadIdx.y;
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    if (py >= b.natoms || px >= b.natoms || px > py) return;
    int ia = b.atom_order ? b.atom_order[py] : py, ib = b.atom_order ? b.atom_order[px] : px;
    if (ib > ia) {
        const int t = ia;
        ia = ib;
        ib = t;
    }
    const int a0 = b.atom_ao0[ia], na_ao = b.atom_nao[ia];
    const int b0 = b.atom_ao0[ib], nb_ao = b.atom_nao[ib];

    if (ia == ib) {  // diagonal block: S = 1, h = IP + V_shift; same-atom off-diagonals 0
        for (int jb = 0; jb < nb_ao; ++jb)
            for (int ja = 0; ja < na_ao; ++ja) {
                const int r = a0 + ja, c = b0 + jb;
                const size_t o = (size_t)c * ld + r;
                S[o] = (r == c) ? 1.0 : 0.0;
                h[o] = (r == c) ? b.ao_ip[r] + b.ao_vshift[r] : 0.0;
            }
        return;
    }
    // B - A vector, lined-up frame (ROTATIONOVERLAP, overlap_D.f:558-574)
    const double xab = coords[3 * ib] - coords[3 * ia];
    const double yab = coords[3 * ib + 1] - coords[3 * ia + 1];
    const double zab = coords[3 * ib + 2] - coords[3 * ia + 2];
    pair_overlap_block(b, ia, ib, xab, yab, zab, cutoff, [&](int ja, int jb, double s) {
        const int aa = a0 + ja, bb = b0 + jb;
        const double hv = x_ij(b.ao_ip[aa], b.ao_ip[bb], b.ao_vshift[aa], b.ao_vshift[bb], b.ao_kwh[aa],
                               b.ao_kwh[bb]) * s;
        S[(size_t)bb * ld + aa] = s;
        S[(size_t)aa * ld + bb] = s;
        h[(size_t)bb * ld + aa] = hv;
        h[(size_t)aa * ld + bb] = hv;
    });
}

// Pulay (overlap-derivative) force terms of the Ehrenfest force
// (Ehrenfest, diabatic-Ehren.f:163-230): for every atom pair K < L with
// R_KL < cutoff and every direction, dS(j in L, i in K)/dR_K by central
// differences of the S block rebuilt with atom K displaced by +-delta
// (PULAY_OVERLAP, overlap_D.f:314-463), and
//   F[K][L][xyz] = -sum_{j in L} sum_{i in K} dS_ji/dR_K Kernel(i, j)
// (Kernel column-major, ld = ldk).  One thread per (L, K) pair; F is natoms x
// natoms x 3, written for K < L only.
constexpr int kMaxAoAtom = 16;

__global__ void pulay_pairs_kernel(DevBasis b, const double *__restrict__ coords, double cutoff, double delta,
                                   const double *__restrict__ kernel, int ldk, double *__restrict__ F) {
    const int L = blockIdx.y * blockDim.y + threadIdx.y;  // ia in PULAY_OVERLAP
    const int K = blockIdx.x * blockDim.x + threadIdx.x;  // the displaced site, ib
    if (L >= b.natoms || K >= L) return;
    const int nat = b.natoms;
    const double dx = coords[3 * K] - coords[3 * L], dy = coords[3 * K + 1] - coords[3 * L + 1],
                 dz = coords[3 * K + 2] - coords[3 * L + 2];
    const double R = sqrt(dx * dx + dy * dy + dz * dz);
    double f[3] = {0.0, 0.0, 0.0};
    const int a0 = b.atom_ao0[L], na = b.atom_nao[L], b0 = b.atom_ao0[K], nb = b.atom_nao[K];
    if (R < cutoff && na <= kMaxAoAtom && nb <= kMaxAoAtom) {
        double fwd[kMaxAoAtom * kMaxAoAtom];
        for (int xyz = 0; xyz < 3; ++xyz) {
            double pk[3] = {coords[3 * K], coords[3 * K + 1], coords[3 * K + 2]};
            pk[xyz] = coords[3 * K + xyz] + delta;
            pair_overlap_block(b, L, K, pk[0] - coords[3 * L], pk[1] - coords[3 * L + 1], pk[2] - coords[3 * L + 2],
                               cutoff, [&](int ja, int jb, double s) { fwd[ja * kMaxAoAtom + jb] = s; });
            pk[xyz] = coords[3 * K + xyz] - delta;
            double acc = 0.0;
            pair_overlap_block(b, L, K, pk[0] - coords[3 * L], pk[1] - coords[3 * L + 1], pk[2] - coords[3 * L + 2],
                               cutoff, [&](int ja, int jb, double s) {
                                   const double g = (fwd[ja * kMaxAoAtom + jb] - s) / (2.0 * delta);
                                   acc = acc - g * kernel[(size_t)(a0 + ja) * ldk + (b0 + jb)];
                               });
            f[xyz] = acc;
        }
    }
    for (int xyz = 0; xyz < 3; ++xyz) F[((size_t)K * nat + L) * 3 + xyz] = f[xyz];
}

// Extended-Hueckel Hamiltonian with environment fields (even_more_extended_Huckel
// and Huckel_with_FIELDS, hamiltonians.f:69-264), one thread per atom pair
// ia > ib closer than the cutoff: for i in ia, j in ib
//   h_ij = X_ij S_ij - [S_ij DP_1 + (mu_ij - (r0 - R_i) S_ij) . DP_2..4]   (|S_ij| > 1e-7)
// with r0 the midpoint of the two atoms, mu = dp_ao (the AO dipole matrix,
// N x N x 3, ld N) and DP the 4-vector (potential, field) of the pair, dp4
// (natoms x natoms x 4, entry (ia, ib)); h_ji = h_ij, h_ii = IP_i + V_shift_i.
// h must be zero on entry (blocks beyond the cutoff and same-atom off-diagonals stay 0).
__global__ void huckel_fields_kernel(DevBasis b, const double *__restrict__ coords, double cutoff,
                                     const double *__restrict__ S, int lds, const double *__restrict__ dp_ao,
                                     const double *__restrict__ dp4, double *__restrict__ h, int ldh) {
    const int ia = blockIdx.y * blockDim.y + threadIdx.y;
    const int ib = blockIdx.x * blockDim.x + threadIdx.x;
    const int nat = b.natoms, n = b.nao;
    if (ia >= nat || ib >= nat || ib > ia) return;
    const int a0 = b.atom_ao0[ia], na_ao = b.atom_nao[ia];
    const int b0 = b.atom_ao0[ib], nb_ao = b.atom_nao[ib];
    if (ia == ib) {
        for (int ja = 0; ja < na_ao; ++ja) h[(size_t)(a0 + ja) * ldh + a0 + ja] = b.ao_ip[a0 + ja] + b.ao_vshift[a0 + ja];
        return;
    }
    const double dx = coords[3 * ib] - coords[3 * ia], dy = coords[3 * ib + 1] - coords[3 * ia + 1],
                 dz = coords[3 * ib + 2] - coords[3 * ia + 2];
    if (sqrt(dx * dx + dy * dy + dz * dz) > cutoff) return;
    const double Ri[3] = {coords[3 * ia], coords[3 * ia + 1], coords[3 * ia + 2]};
    const double r0[3] = {(coords[3 * ia] + coords[3 * ib]) / 2.0, (coords[3 * ia + 1] + coords[3 * ib + 1]) / 2.0,
                          (coords[3 * ia + 2] + coords[3 * ib + 2]) / 2.0};
    const size_t nn = (size_t)nat * nat;
    const double DP[4] = {dp4[(size_t)ib * nat + ia], dp4[nn + (size_t)ib * nat + ia],
                          dp4[2 * nn + (size_t)ib * nat + ia], dp4[3 * nn + (size_t)ib * nat + ia]};
    const size_t n2 = (size_t)n * n;
    for (int jb = 0; jb < nb_ao; ++jb) {
        const int j = b0 + jb;
        for (int ja = 0; ja < na_ao; ++ja) {
            const int i = a0 + ja;
            const double sij = S[(size_t)j * lds + i];
            double v = x_ij(b.ao_ip[i], b.ao_ip[j], b.ao_vshift[i], b.ao_vshift[j], b.ao_kwh[i], b.ao_kwh[j]) * sij;
            if (fabs(sij) > 1.0e-7) {
                double vec[3];
                for (int c = 0; c < 3; ++c) vec[c] = dp_ao[c * n2 + (size_t)j * n + i] - (r0[c] - Ri[c]) * sij;
                v = v - (sij * DP[0] + (vec[0] * DP[1] + vec[1] * DP[2] + vec[2] * DP[3]));
            }
            h[(size_t)j * ldh + i] = v;
            h[(size_t)i * ldh + j] = v;
        }
    }
}

// force(a)[xyz] = scale * (sum_{L > a} F[a][L] - sum_{K < a} F[K][a]), fixed order
// (the atom(i)%Ehrenfest sum over F_snd, diabatic-Ehren.f:140-148 with 216-223)
__global__ void pulay_reduce_kernel(const double *__restrict__ F, int nat, double scale, double *__restrict__ force) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * nat) return;
    const int a = t / 3, xyz = t % 3;
    double s = 0.0;
    for (int q = 0; q < nat; ++q) {
        if (q > a) s = s + F[((size_t)a * nat + q) * 3 + xyz];
        else if (q < a) s = s - F[((size_t)q * nat + a) * 3 + xyz];
    }
    force[t] = scale * s;
}

}  // namespace

cudaError_t init_build_tables() {
    init_tables_kernel<<<(1001 + 255) / 256, 256>>>();
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e;
}

cudaError_t launch_pulay_forces(const DevBasis &b, const double *d_coords, double cutoff, double delta,
                                const double *d_kernel, int ldk, double *d_F, double scale, double *d_force,
                                cudaStream_t st) {
    if (b.natoms <= 0) return cudaSuccess;
    dim3 block(16, 8);
    dim3 grid((b.natoms + block.x - 1) / block.x, (b.natoms + block.y - 1) / block.y);
    pulay_pairs_kernel<<<grid, block, 0, st>>>(b, d_coords, cutoff, delta, d_kernel, ldk, d_F);
    count_launch();
    pulay_reduce_kernel<<<(3 * b.natoms + 127) / 128, 128, 0, st>>>(d_F, b.natoms, scale, d_force);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_huckel_fields(const DevBasis &b, const double *d_coords, double cutoff, const double *d_S, int lds,
                                 const double *d_dp_ao, const double *d_dp4, double *d_h, int ldh, cudaStream_t st) {
    if (b.natoms <= 0) return cudaSuccess;
    dim3 block(16, 8);
    dim3 grid((b.natoms + block.x - 1) / block.x, (b.natoms + block.y - 1) / block.y);
    huckel_fields_kernel<<<grid, block, 0, st>>>(b, d_coords, cutoff, d_S, lds, d_dp_ao, d_dp4, d_h, ldh);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_build_sh(const DevBasis &b, const double *d_coords, double cutoff, double *d_S,
                            double *d_h, int ld, cudaStream_t st) {
    if (b.natoms <= 0) return cudaSuccess;
    dim3 block(16, 8);
    dim3 grid((b.natoms + block.x - 1) / block.x, (b.natoms + block.y - 1) / block.y);
    build_sh_kernel<<<grid, block, 0, st>>>(b, d_coords, cutoff, d_S, d_h, ld);
    count_launch();
    return cudaGetLastError();
}

}  // namespace elhl
