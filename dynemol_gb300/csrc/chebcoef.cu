// Host-side FP64 mathematics of the Chebyshev propagator:
//   * Bessel J_k(beta), k = 0..kmax, by Miller's backward recurrence with the
//     normalisation J_0 + 2 sum_{k>=1} J_{2k} = 1 (our own implementation of
//     the textbook method, Abramowitz & Stegun 9.1.27 / 9.1.46);
//   * the expansion coefficients of exp(-i H dt / hbar) on the spectral
//     interval [emin, emax] (Tal-Ezer & Kosloff 1984):
//       exp(-i tau H) = exp(-i tau a) sum_k (2 - delta_k0) (-i)^k J_k(tau b) T_k((H - a)/b),
//     a = (emax + emin)/2, b = (emax - emin)/2, tau = dt / hbar;
//   * extreme eigenvalues of a symmetric tridiagonal matrix by Sturm-sequence
//     bisection (for the Lanczos spectral bounds).
#include <cmath>
#include <vector>

#include "elhl_internal.cuh"

namespace elhl {

int bessel_j_sequence(double beta, int kmax, double *J) {
    if (kmax < 0 || !(beta >= 0.0) || !std::isfinite(beta)) return ELHL_ERR_BAD_ARG;
    if (beta == 0.0) {
        for (int k = 0; k <= kmax; ++k) J[k] = (k == 0) ? 1.0 : 0.0;
        return ELHL_OK;
    }
    // start well above both kmax and beta; the recurrence is stable downwards
    const int start = 2 * ((std::max(kmax, (int)beta) + 30 + (int)std::sqrt(40.0 * std::max(beta, 1.0))) / 2 + 1);
    std::vector<double> t(start + 2, 0.0);
    double jp1 = 0.0, jk = 1.0e-300, norm = 0.0;
    t[start] = jk;
    for (int k = start; k >= 1; --k) {
        const double jm1 = (2.0 * k / beta) * jk - jp1;
        jp1 = jk;
        jk = jm1;
        t[k - 1] = jk;
        if (std::fabs(jk) > 1.0e250) {  // rescale to stay in range
            for (int q = k - 1; q <= start; ++q) t[q] *= 1.0e-250;
            jk *= 1.0e-250;
            jp1 *= 1.0e-250;
        }
    }
    norm = t[0];
    for (int k = 2; k <= start; k += 2) norm += 2.0 * t[k];
    for (int k = 0; k <= kmax; ++k) J[k] = (k <= start) ? t[k] / norm : 0.0;
    return ELHL_OK;
}

int chebyshev_coefficients(double dt, double emin, double emax, double tol, int kcap, std::vector<double> &cre,
                           std::vector<double> &cim, int *K_out) {
    if (!(emax > emin) || dt <= 0.0 || kcap < 2) return ELHL_ERR_BAD_ARG;
    const double tau = dt / kHbar;
    const double a = 0.5 * (emax + emin), b = 0.5 * (emax - emin);
    const double beta = tau * b;
    const int kmax = std::min(kcap, (int)(beta + 10.0 * std::cbrt(beta) + 60.0));
    std::vector<double> J(kmax + 1);
    if (int rc = bessel_j_sequence(beta, kmax, J.data())) return rc;
    // last order: beyond beta, |J_k| decays super-exponentially; stop once two
    // consecutive terms are below tol
    int K = kmax;
    for (int k = (int)beta + 1; k < kmax; ++k)
        if (std::fabs(J[k]) < tol && std::fabs(J[k + 1]) < tol) {
            K = k;
            break;
        }
    if (K >= kcap) return ELHL_ERR_UNSUPPORTED;
    cre.assign(K + 1, 0.0);
    cim.assign(K + 1, 0.0);
    const double pr = std::cos(-tau * a), pi = std::sin(-tau * a);  // exp(-i tau a)
    for (int k = 0; k <= K; ++k) {
        const double mag = (k == 0 ? 1.0 : 2.0) * J[k];
        // (-i)^k
        double ur = 0.0, ui = 0.0;
        switch (k & 3) {
            case 0: ur = 1.0; break;
            case 1: ui = -1.0; break;
            case 2: ur = -1.0; break;
            default: ui = 1.0; break;
        }
        cre[k] = mag * (ur * pr - ui * pi);
        cim[k] = mag * (ur * pi + ui * pr);
    }
    *K_out = K;
    return ELHL_OK;
}

// Number of eigenvalues of the symmetric tridiagonal (alpha, beta) below x.
static int sturm_count(const double *alpha, const double *beta, int n, double x) {
    int count = 0;
    double q = alpha[0] - x;
    if (q < 0) ++count;
    for (int i = 1; i < n; ++i) {
        const double d = (q != 0.0) ? q : 1.0e-300;
        q = alpha[i] - x - beta[i - 1] * beta[i - 1] / d;
        if (q < 0) ++count;
    }
    return count;
}

void tridiagonal_extremes(const double *alpha, const double *beta, int n, double *lo, double *hi) {
    double g0 = 1e300, g1 = -1e300;  // Gershgorin interval of the tridiagonal
    for (int i = 0; i < n; ++i) {
        const double r = (i > 0 ? std::fabs(beta[i - 1]) : 0.0) + (i < n - 1 ? std::fabs(beta[i]) : 0.0);
        g0 = std::min(g0, alpha[i] - r);
        g1 = std::max(g1, alpha[i] + r);
    }
    auto bisect = [&](int target) {  // smallest x with count(x) > target
        double a = g0 - 1.0, b = g1 + 1.0;
        for (int it = 0; it < 200 && b - a > 1e-13 * (std::fabs(a) + std::fabs(b) + 1.0); ++it) {
            const double m = 0.5 * (a + b);
            if (sturm_count(alpha, beta, n, m) > target) b = m; else a = m;
        }
        return 0.5 * (a + b);
    };
    *lo = bisect(0);
    *hi = bisect(n - 1);
}

// |last component| of the normalised eigenvector of the tridiagonal for the
// eigenvalue theta (two steps of inverse iteration with a tiny shift).  The
// Lanczos residual of that Ritz pair is beta_k * |s_k|.
double tridiagonal_last_component(const double *alpha, const double *beta, int n, double theta) {
    if (n == 1) return 1.0;
    double width = 0.0;
    for (int i = 0; i < n; ++i) width = std::max(width, std::fabs(alpha[i]));
    const double shift = theta + 1e-10 * (width + 1.0);
    std::vector<double> x(n, 1.0), c(n), d(n);
    for (int it = 0; it < 3; ++it) {
        // Thomas algorithm on (T - shift I) y = x
        double den = alpha[0] - shift;
        if (den == 0.0) den = 1e-300;
        c[0] = (n > 1 ? beta[0] : 0.0) / den;
        d[0] = x[0] / den;
        for (int i = 1; i < n; ++i) {
            den = (alpha[i] - shift) - beta[i - 1] * c[i - 1];
            if (den == 0.0) den = 1e-300;
            c[i] = (i < n - 1 ? beta[i] : 0.0) / den;
            d[i] = (x[i] - beta[i - 1] * d[i - 1]) / den;
        }
        x[n - 1] = d[n - 1];
        for (int i = n - 2; i >= 0; --i) x[i] = d[i] - c[i] * x[i + 1];
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
        nrm = std::sqrt(nrm);
        if (!(nrm > 0.0) || !std::isfinite(nrm)) return 1.0;
        for (int i = 0; i < n; ++i) x[i] /= nrm;
    }
    return std::fabs(x[n - 1]);
}

}  // namespace elhl

extern "C" int elhl_bessel_j(double beta, int kmax, double *J) {
    if (!J) return ELHL_ERR_BAD_ARG;
    return elhl::bessel_j_sequence(beta, kmax, J);
}

extern "C" int elhl_chebyshev_coefficients(double dt, double emin, double emax, double tol, int kcap,
                                           double *cre, double *cim, int *K) {
    if (!cre || !cim || !K) return ELHL_ERR_BAD_ARG;
    std::vector<double> r, i;
    int rc = elhl::chebyshev_coefficients(dt, emin, emax, tol, kcap, r, i, K);
    if (rc) return rc;
    for (int k = 0; k <= *K; ++k) {
        cre[k] = r[k];
        cim[k] = i[k];
    }
    return ELHL_OK;
}
