// Host-side FP64 plan numerics of the min-max interpolator.
//
// Per axis (N image points, K oversampled grid points, J neighbours):
//   * Kaiser-Bessel shape      src/_helper/helper.py:961-997
//   * KB Fourier transform     src/_helper/helper.py:1000-1012, in the closed
//     form J * sin(z)/z / I0(alpha) (z^2 = (pi J u)^2 - alpha^2), which is
//     what sqrt(2pi)(J/2) jv(1/2, z) / z^(1/2) / iv(0, alpha) reduces to.
//   * cosine-series fit        src/_helper/helper.py:910-958 (rank-truncated
//     least squares with the float32 cutoff of the reference's complex64
//     lstsq; coefficients rounded to float32).  Callers that hold the
//     reference's own coefficients pass them in instead (nufft_plan_set_alpha).
//   * scaling factor sn        src/_helper/helper.py:1015-1036 (real part)
//   * T = pinv(CSSC)           src/_helper/helper.py:1060-1083 (symmetric
//     Jacobi eigen-decomposition, scipy.linalg.pinv's default cutoff)
// Nothing here depends on the sample points; the per-point work runs on the
// GPU (points.cu).
#include "nufft_internal.cuh"

#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>

namespace nufft {

static double kb_shape(int J, double K_over_N) {
    static const double best[17] = {0, 0, 2.5, 2.27, 2.31, 2.34, 2.32, 2.32, 2.35,
                                    2.34, 2.34, 2.35, 2.34, 2.35, 2.35, 2.35, 2.33};
    if (K_over_N != 2.0) return 2.34 * J;
    if (J >= 2 && J <= 16) return J * best[J];
    // nearest tabulated J (only J == 1 reaches here)
    return J * best[2];
}

static double bessel_i0(double x) {
    // power series sum_k ((x/2)^2)^k / (k!)^2, converges for all x used here
    double q = 0.25 * x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 500; ++k) {
        term *= q / ((double)k * (double)k);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

static double kb_ft(double u, int J, double alpha) {
    double w = (M_PI * J * u) * (M_PI * J * u) - alpha * alpha;
    double s;
    if (w > 0) { double z = std::sqrt(w); s = std::sin(z) / z; }
    else if (w < 0) { double z = std::sqrt(-w); s = std::sinh(z) / z; }
    else s = 1.0;
    return J * s / bessel_i0(alpha);
}

static double sinc(double x) {
    if (x == 0.0) return 1.0;
    double px = M_PI * x;
    return std::sin(px) / px;
}

// Truncated least squares min ||A c - b|| (A rows x cols, row major) by a
// one-sided Jacobi SVD: singular values below rcond * s_max are dropped, as
// LAPACK xGELSD does.  With rcond = 2^-23 this restates the reference's
// numpy.linalg.lstsq(..., rcond=-1) in complex64, whose cutoff is the float32
// machine precision; the cosine basis is ill-conditioned (cond ~1e10), so the
// cutoff, not the arithmetic, decides the fitted coefficients.
static void lstsq_svd(const std::vector<double>& A, const std::vector<double>& b, int rows,
                      int cols, double rcond, std::vector<double>& c) {
    std::vector<double> U(A), V(cols * cols, 0.0);
    for (int i = 0; i < cols; ++i) V[i * cols + i] = 1.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < cols; ++p)
            for (int q = p + 1; q < cols; ++q) {
                double a = 0, bb = 0, g = 0;
                for (int i = 0; i < rows; ++i) {
                    double up = U[i * cols + p], uq = U[i * cols + q];
                    a += up * up; bb += uq * uq; g += up * uq;
                }
                if (a == 0 || bb == 0) continue;
                double rel = std::fabs(g) / std::sqrt(a * bb);
                off = std::max(off, rel);
                if (rel < 1e-15) continue;
                double zeta = (bb - a) / (2 * g);
                double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
                double cs = 1 / std::sqrt(1 + t * t), sn = cs * t;
                for (int i = 0; i < rows; ++i) {
                    double up = U[i * cols + p], uq = U[i * cols + q];
                    U[i * cols + p] = cs * up - sn * uq;
                    U[i * cols + q] = sn * up + cs * uq;
                }
                for (int i = 0; i < cols; ++i) {
                    double vp = V[i * cols + p], vq = V[i * cols + q];
                    V[i * cols + p] = cs * vp - sn * vq;
                    V[i * cols + q] = sn * vp + cs * vq;
                }
            }
        if (off < 1e-15) break;
    }
    std::vector<double> sv(cols);
    double smax = 0;
    for (int j = 0; j < cols; ++j) {
        double n2 = 0;
        for (int i = 0; i < rows; ++i) n2 += U[i * cols + j] * U[i * cols + j];
        sv[j] = std::sqrt(n2);
        smax = std::max(smax, sv[j]);
    }
    c.assign(cols, 0.0);
    for (int j = 0; j < cols; ++j) {
        if (!(sv[j] > rcond * smax)) continue;
        double d = 0;  // (u_j . b) / s_j with u_j = U[:, j] / s_j
        for (int i = 0; i < rows; ++i) d += U[i * cols + j] * b[i];
        d /= sv[j] * sv[j];
        for (int k = 0; k < cols; ++k) c[k] += d * V[k * cols + j];
    }
}

// pseudo-inverse of a symmetric n x n matrix by cyclic Jacobi rotations
static void pinv_sym(const std::vector<double>& S, int n, std::vector<double>& P) {
    std::vector<double> a(S), V(n * n, 0.0);
    for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += a[p * n + q] * a[p * n + q];
        if (off < 1e-300) break;
        for (int p = 0; p < n; ++p) {
            for (int q = p + 1; q < n; ++q) {
                double apq = a[p * n + q];
                if (std::fabs(apq) < 1e-300) continue;
                double app = a[p * n + p], aqq = a[q * n + q];
                double theta = (aqq - app) / (2 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
        }
    }
    double smax = 0;
    for (int i = 0; i < n; ++i) smax = std::max(smax, std::fabs(a[i * n + i]));
    double cut = smax * n * 2.220446049250313e-16;
    P.assign(n * n, 0.0);
    for (int e = 0; e < n; ++e) {
        double lam = a[e * n + e];
        if (std::fabs(lam) <= cut) continue;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) P[i * n + j] += V[i * n + e] * V[j * n + e] / lam;
    }
}

int axis_params(int N, int J, int K, AxisParams& ap) {
    if (N < 1 || J < 1 || K < 1 || J > NUFFT_MAXJ || N > K || J > K) return NUFFT_EINVAL;
    ap.N = N; ap.J = J; ap.K = K;
    const double Nmid = (N - 1.0) / 2.0;
    const int L = (N > 40) ? 13 : (int)std::ceil(N / 3.0);
    ap.L = L;
    const double gam = 2.0 * M_PI / K;
    std::vector<double> X(N * (L + 1)), rhs(N), coef;
    const double kba = kb_shape(J, (double)K / (double)N);
    for (int n = 0; n < N; ++n) {
        double nl = n - Nmid;
        rhs[n] = (J > 1) ? 1.0 / kb_ft(nl / K, J, kba) : 1.0;
        for (int l = 0; l <= L; ++l) X[n * (L + 1) + l] = std::cos(gam * nl * l);
    }
    for (int l = 0; l < NUFFT_NALPHA; ++l) ap.alpha[l] = 0.f;
    lstsq_svd(X, rhs, N, L + 1, 1.1920928955078125e-07, coef);
    if (J > 1) {
        ap.alpha[0] = (float)coef[0];
        for (int l = 1; l <= L; ++l) ap.alpha[l] = (float)coef[l] / 2.0f;
    } else {
        ap.alpha[0] = 1.0f;
    }
    return derive_axis(ap);
}

// sn and T of one axis from its (N, J, K, L, alpha).
int derive_axis(AxisParams& ap) {
    const int N = ap.N, J = ap.J, K = ap.K, L = ap.L;
    const double Nmid = (N - 1.0) / 2.0;
    const double gam = 2.0 * M_PI / K;
    // scaling factor: real part of sum_{l=-L..L} alpha_|l| exp(i gam (n - Nmid) l)
    ap.sn.assign(N, 0.0);
    for (int n = 0; n < N; ++n) {
        double s = ap.alpha[0];
        for (int l = 1; l <= L; ++l) s += 2.0 * (double)ap.alpha[l] * std::cos(gam * (n - Nmid) * l);
        ap.sn[n] = s;
    }
    // CSSC and its pseudo-inverse
    const double ratio = (double)K / (double)N;
    std::vector<double> cssc(J * J, 0.0);
    for (int l1 = -L; l1 <= L; ++l1)
        for (int l2 = -L; l2 <= L; ++l2) {
            double a12 = (double)(ap.alpha[std::abs(l1)] * ap.alpha[std::abs(l2)]);
            for (int j1 = 0; j1 < J; ++j1)
                for (int j2 = 0; j2 < J; ++j2)
                    cssc[j1 * J + j2] += a12 * sinc(((j2 - j1) + (double)(l1 - l2)) / ratio);
        }
    pinv_sym(cssc, J, ap.T);
    return NUFFT_OK;
}

}  // namespace nufft

extern "C" int nufft_axis_params(int N, int J, int K, const float* alpha_in, int L_in,
                                 float* alpha_out, int* L_out, double* sn_out, double* T_out) {
    nufft::AxisParams ap;
    int st = nufft::axis_params(N, J, K, ap);
    if (st != NUFFT_OK) {
        nufft::set_error("nufft_axis_params: need 1 <= J <= 16, N <= K, J <= K");
        return st;
    }
    if (alpha_in) {
        if (L_in < 0 || L_in > NUFFT_MAXL) {
            nufft::set_error("nufft_axis_params: L must be in 0..14");
            return NUFFT_EINVAL;
        }
        ap.L = L_in;
        for (int l = 0; l < NUFFT_NALPHA; ++l) ap.alpha[l] = (l <= L_in) ? alpha_in[l] : 0.f;
        nufft::derive_axis(ap);
    }
    if (alpha_out) std::memcpy(alpha_out, ap.alpha, sizeof(ap.alpha));
    if (L_out) *L_out = ap.L;
    if (sn_out) std::memcpy(sn_out, ap.sn.data(), sizeof(double) * N);
    if (T_out) std::memcpy(T_out, ap.T.data(), sizeof(double) * J * J);
    return NUFFT_OK;
}
