// gx_scf.cuh -- SCF basis-function expansion on the device (FP64).
//
// Same expansion as gala's scf_potential_helper / scf_gradient_helper /
// scf_density_helper (src/gala/potential/scf/src/bfe.cpp:16-189) and
// phi_nl / rho_nl / sph_grad_phi_nlm (bfe_helper.cpp:14-90), with gala's
// coefficient packing p = [G, nmax, lmax, M, r_s, S[n][l][m], T[n][l][m]].
//
// gala calls GSL once per (n, l, m) term.  Here every special function is
// produced by its three-term recurrence once per point and reused:
//   Gegenbauer  n C_n^a = 2 x (n + a - 1) C_{n-1}^a - (n + 2a - 2) C_{n-2}^a
//   Legendre    (l - m) P_l^m = x (2l - 1) P_{l-1}^m - (l + m - 1) P_{l-2}^m,
//               P_m^m = (-1)^m (2m - 1)!! (1 - x^2)^{m/2}   (Condon-Shortley, as GSL)
//   sphPlm      sqrt((2l + 1)/(4 pi) (l - m)!/(l + m)!) P_l^m
// The terms are summed l-major instead of n-major, so results agree with the
// term-by-term form to rounding (checked against the oracle in the tests).
#pragma once

#include "gx_device.cuh"

namespace gx {

constexpr int SCF_MAX_N = 24;   // nmax + 1
constexpr int SCF_MAX_L = 16;   // lmax + 1

__device__ __forceinline__ double scf_fact(int k) {
    double f = 1.0;
    for (int i = 2; i <= k; i++) f *= i;
    return f;
}

// P_l^m(X) for all m <= l of one l, given the values of l-1 and l-2 (running
// recurrence in l).  Arrays are indexed by m.
__device__ __forceinline__ void scf_legendre_step(int l, double X, double sintheta_pos,
                                                  const double *Pm1, const double *Pm2, double *P) {
    // diagonal P_l^l = -(2l-1) sqrt(1-X^2) P_{l-1}^{l-1}
    for (int m = 0; m <= l; m++) {
        if (m == l) {
            P[m] = (l == 0) ? 1.0 : -(2.0 * l - 1.0) * sintheta_pos * Pm1[l - 1];
        } else if (m == l - 1) {
            P[m] = X * (2.0 * m + 1.0) * Pm1[m];
        } else {
            P[m] = (X * (2.0 * l - 1.0) * Pm1[m] - (l + m - 1.0) * Pm2[m]) / (double)(l - m);
        }
    }
}

// kind 0: value, 1: gradient (accumulated into g), 2: density.
template <int KIND>
__device__ __forceinline__ double scf_eval(const double *p, const double *q, double *g) {
    const double SQRT_FOURPI = 3.544907701811031;
    const double PI = 3.14159265358979323846;
    const double G = p[0];
    const int nmax = (int)p[1];
    const int lmax = (int)p[2];
    const double M = p[3];
    const double r_s = p[4];
    const int ncoef = (nmax + 1) * (lmax + 1) * (lmax + 1);
    const double *Snlm = p + 5;
    const double *Tnlm = p + 5 + ncoef;

    const double r = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    const double s = r / r_s;
    const double X = q[2] / r;
    const double phi = atan2(q[1], q[0]);
    const double sintheta = sqrt(1 - X * X);
    const double xi = (s - 1) / (s + 1);

    double cosmphi[SCF_MAX_L], sinmphi[SCF_MAX_L];
    for (int m = 0; m <= lmax; m++) sincos(m * phi, &sinmphi[m], &cosmphi[m]);

    double Pl[SCF_MAX_L], Pl1[SCF_MAX_L], Pl2[SCF_MAX_L];
    for (int m = 0; m < SCF_MAX_L; m++) { Pl[m] = 0.; Pl1[m] = 0.; Pl2[m] = 0.; }
    double acc0 = 0., acc1 = 0., acc2 = 0.;

    for (int l = 0; l <= lmax; l++) {
        // Legendre P_l^m (this l) and keep P_{l-1}^m for dY/dtheta
        for (int m = 0; m < l; m++) { Pl2[m] = Pl1[m]; Pl1[m] = Pl[m]; }
        scf_legendre_step(l, X, sintheta, Pl1, Pl2, Pl);

        const double a1 = 2 * l + 1.5, a2 = 2 * l + 2.5;
        const double pow_s_l = pow(s, (double)l);
        const double pow_s_lm1 = pow(s, (double)(l - 1));
        double Cn_m2 = 0., Cn_m1 = 0., Cn = 1.;       // C_n^{a1}
        double Dn_m2 = 0., Dn_m1 = 0., Dn = 1.;       // C_{n-1}^{a2} (Dn is C_{n-1})
        for (int n = 0; n <= nmax; n++) {
            // advance Gegenbauer recurrences to index n (C) and n-1 (D)
            if (n == 0) { Cn = 1.; }
            else if (n == 1) { Cn_m1 = 1.; Cn = 2. * a1 * xi; }
            else {
                Cn_m2 = Cn_m1; Cn_m1 = Cn;
                Cn = (2. * xi * (n + a1 - 1.) * Cn_m1 - (n + 2. * a1 - 2.) * Cn_m2) / n;
            }
            const int nd = n - 1;
            if (nd == 0) { Dn = 1.; }
            else if (nd == 1) { Dn_m1 = 1.; Dn = 2. * a2 * xi; }
            else if (nd > 1) {
                Dn_m2 = Dn_m1; Dn_m1 = Dn;
                Dn = (2. * xi * (nd + a2 - 1.) * Dn_m1 - (nd + 2. * a2 - 2.) * Dn_m2) / nd;
            }

            double radial, dradial = 0.;
            if (KIND == 2) {
                const double Knl = 0.5 * n * (n + 4 * l + 3) + (l + 1) * (2 * l + 1);
                radial = SQRT_FOURPI * (Knl / (2 * PI) * pow_s_l / (s * pow(1 + s, 2.0 * l + 3)) * Cn);
            } else {
                radial = -SQRT_FOURPI * pow_s_l * pow(1 + s, -2.0 * l - 1) * Cn;
                if (KIND == 1) {
                    if (n == 0)
                        dradial = SQRT_FOURPI * pow_s_lm1 * pow(1 + s, -3.0 - 2 * l) * (1 + s) * (l * (-1 + s) + s);
                    else
                        dradial = SQRT_FOURPI * pow_s_lm1 * pow(1 + s, -3.0 - 2 * l) *
                                  (-2 * (3 + 4 * l) * s * Dn + (1 + s) * (l * (-1 + s) + s) * Cn);
                }
            }

            for (int m = 0; m <= l; m++) {
                const int i = m + (lmax + 1) * (l + (lmax + 1) * n);
                const double S = Snlm[i], T = Tnlm[i];
                if ((S == 0.) & (T == 0.)) continue;
                const double norm = sqrt((double)(2 * l + 1) / (4.0 * PI) * scf_fact(l - m) / scf_fact(l + m));
                const double Ylm = norm * Pl[m];
                const double tmp = (S * cosmphi[m] + T * sinmphi[m]);
                if (KIND != 1) {
                    acc0 += radial * Ylm * tmp;
                } else {
                    double dYlm_dtheta = 0.;
                    if (l > 0) {
                        const double Pl1m = (m <= l - 1) ? Pl1[m] : 0.;
                        const double A = sqrt((double)(2 * l + 1)) / SQRT_FOURPI * sqrt(scf_fact(l - m) / scf_fact(l + m));
                        dYlm_dtheta = A / sintheta * (l * X * Pl[m] - (l + m) * Pl1m);
                    }
                    acc0 += dradial * Ylm * tmp;
                    acc1 += dYlm_dtheta * radial / s * tmp;
                    acc2 += ((m == 0) ? 0. : (double)m) * Ylm * radial * (T * cosmphi[m] - S * sinmphi[m]) /
                            (s * sintheta);
                }
            }
        }
    }

    if (KIND == 0) return acc0 * G * M / r_s;
    if (KIND == 2) return acc0 * M / (r_s * r_s * r_s);
    double cosphi, sinphi;
    sincos(phi, &sinphi, &cosphi);
    const double gx_ = sintheta * cosphi * acc0 + X * cosphi * acc1 - sinphi * acc2;
    const double gy_ = sintheta * sinphi * acc0 + X * sinphi * acc1 + cosphi * acc2;
    const double gz_ = X * acc0 - sintheta * acc1;
    g[0] += gx_ * G * M / (r_s * r_s);
    g[1] += gy_ * G * M / (r_s * r_s);
    g[2] += gz_ * G * M / (r_s * r_s);
    return 0.;
}

static __device__ __noinline__ double scf_value_dev(const double *p, const double *q) { return scf_eval<0>(p, q, nullptr); }
static __device__ __noinline__ void scf_gradient_dev(const double *p, const double *q, double *g) { scf_eval<1>(p, q, g); }
static __device__ __noinline__ double scf_density_dev(const double *p, const double *q) { return scf_eval<2>(p, q, nullptr); }

}  // namespace gx
