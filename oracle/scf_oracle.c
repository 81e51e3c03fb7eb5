/*
 * ORACLE (test infrastructure only): CPU restatement of gala's SCF expansion.
 * See scf_oracle.h for the special functions and how this file is pinned.
 * Loop structure and accumulation order follow scf_potential_helper
 * (bfe.cpp:72-115), scf_gradient_helper (:117-189), scf_density_helper
 * (:16-56) and sph_grad_phi_nlm / phi_nl / rho_nl (bfe_helper.cpp:14-90).
 */
#include <math.h>
#include <string.h>

#include "scf_oracle.h"

#define SQRT_FOURPI 3.544907701811031

double orc_gegenpoly(int n, double a, double x) {
    if (n < 0) return 0.0;
    if (n == 0) return 1.0;
    double cm2 = 1.0, cm1 = 2.0 * a * x;
    for (int k = 2; k <= n; k++) {
        const double ck = (2.0 * x * (k + a - 1.0) * cm1 - (k + 2.0 * a - 2.0) * cm2) / k;
        cm2 = cm1;
        cm1 = ck;
    }
    return cm1;
}

double orc_legendre_Plm(int l, int m, double x) {
    if (m < 0 || m > l) return 0.0;
    /* P_m^m with the Condon-Shortley phase */
    double pmm = 1.0;
    if (m > 0) {
        const double somx2 = sqrt((1.0 - x) * (1.0 + x));
        double fact = 1.0;
        for (int i = 1; i <= m; i++) {
            pmm *= -fact * somx2;
            fact += 2.0;
        }
    }
    if (l == m) return pmm;
    double pmmp1 = x * (2 * m + 1) * pmm;
    if (l == m + 1) return pmmp1;
    double pll = 0.0;
    for (int ll = m + 2; ll <= l; ll++) {
        pll = (x * (2 * ll - 1) * pmmp1 - (ll + m - 1) * pmm) / (ll - m);
        pmm = pmmp1;
        pmmp1 = pll;
    }
    return pll;
}

static double factorial(int k) {
    double f = 1.0;
    for (int i = 2; i <= k; i++) f *= i;
    return f;
}

double orc_legendre_sphPlm(int l, int m, double x) {
    if (m < 0 || m > l) return 0.0;
    const double norm = sqrt((2 * l + 1) / (4.0 * M_PI) * factorial(l - m) / factorial(l + m));
    return norm * orc_legendre_Plm(l, m, x);
}

/* phi_nl (bfe_helper.cpp:24-26) */
static double phi_nl(double s, int n, int l) {
    return -SQRT_FOURPI * pow(s, l) * pow(1 + s, -2 * l - 1) * orc_gegenpoly(n, 2 * l + 1.5, (s - 1) / (s + 1));
}

/* rho_nl (bfe_helper.cpp:14-19) */
static double rho_nl(double s, int n, int l) {
    const double Knl = 0.5 * n * (n + 4 * l + 3) + (l + 1) * (2 * l + 1);
    const double RR = Knl / (2 * M_PI) * pow(s, l) / (s * pow(1 + s, 2 * l + 3)) *
                      orc_gegenpoly(n, 2 * l + 1.5, (s - 1) / (s + 1));
    return SQRT_FOURPI * RR;
}

/* sph_grad_phi_nlm (bfe_helper.cpp:31-90) */
static void sph_grad_phi_nlm(double s, double X, int n, int l, int m, double *sphgrad) {
    const double sintheta = sqrt(1 - X * X);
    const double Phi_nl = phi_nl(s, n, l);
    const double Ylm = orc_legendre_sphPlm(l, m, X);
    const double Plm = (m <= l) ? orc_legendre_Plm(l, m, X) : 0.;
    double dPhinl_dr;
    if (n == 0) {
        dPhinl_dr = SQRT_FOURPI * pow(s, -1 + l) * pow(1 + s, -3 - 2 * l) * (1 + s) * (l * (-1 + s) + s);
    } else {
        dPhinl_dr = (SQRT_FOURPI * pow(s, -1 + l) * pow(1 + s, -3 - 2 * l) *
                     (-2 * (3 + 4 * l) * s * orc_gegenpoly(-1 + n, 2.5 + 2 * l, (-1 + s) / (1 + s)) +
                      (1 + s) * (l * (-1 + s) + s) * orc_gegenpoly(n, 1.5 + 2 * l, (-1 + s) / (1 + s))));
    }
    dPhinl_dr *= Ylm;
    double dYlm_dtheta;
    if (l == 0) {
        dYlm_dtheta = 0.;
    } else {
        const double Pl1m = (m <= (l - 1)) ? orc_legendre_Plm(l - 1, m, X) : 0.;
        double A;
        if (l == m)
            A = sqrt(2 * l + 1) / SQRT_FOURPI * sqrt(1. / factorial(l + m));
        else
            A = sqrt(2 * l + 1) / SQRT_FOURPI * sqrt(factorial(l - m) / factorial(l + m));
        dYlm_dtheta = A / sintheta * (l * X * Plm - (l + m) * Pl1m);
    }
    const double dPhi_dtheta = dYlm_dtheta * Phi_nl / s;
    double dPhi_dphi = (m == 0) ? 0. : (double)m;
    dPhi_dphi *= Ylm * Phi_nl;
    sphgrad[0] = dPhinl_dr;
    sphgrad[1] = dPhi_dtheta;
    sphgrad[2] = dPhi_dphi;
}

#define SCF_UNPACK                                             \
    const double G = p[0];                                     \
    const int nmax = (int)p[1];                                \
    const int lmax = (int)p[2];                                \
    const double M = p[3];                                     \
    const double r_s = p[4];                                   \
    const int ncoef = (nmax + 1) * (lmax + 1) * (lmax + 1);    \
    const double *Snlm = p + 5;                                \
    const double *Tnlm = p + 5 + ncoef;                        \
    (void)G; (void)M

/* scf_value -> scf_potential_helper (bfe.cpp:72-115, 191-227) */
double orc_scf_value(const double *p, const double *q) {
    SCF_UNPACK;
    double cosmphi[64], sinmphi[64];
    const double r = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    const double s = r / r_s;
    const double X = q[2] / r;
    const double phi = atan2(q[1], q[0]);
    double val = 0.;
    for (int m = 0; m < lmax + 1; m++) {
        cosmphi[m] = cos(m * phi);
        sinmphi[m] = sin(m * phi);
    }
    for (int n = 0; n < nmax + 1; n++)
        for (int l = 0; l < lmax + 1; l++)
            for (int m = 0; m < lmax + 1; m++) {
                if (m > l) continue;
                const int i = m + (lmax + 1) * (l + (lmax + 1) * n);
                if ((Snlm[i] == 0.) & (Tnlm[i] == 0.)) continue;
                val += phi_nl(s, n, l) * orc_legendre_sphPlm(l, m, X) *
                       (Snlm[i] * cosmphi[m] + Tnlm[i] * sinmphi[m]);
            }
    val *= G * M / r_s;
    return val;
}

/* scf_gradient -> scf_gradient_helper (bfe.cpp:117-189, 229-259); accumulates. */
void orc_scf_gradient(const double *p, const double *q, double *g) {
    SCF_UNPACK;
    double cosmphi[64], sinmphi[64], tmp_grad[3], tmp_grad2[3];
    const double r = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    const double s = r / r_s;
    const double X = q[2] / r;
    const double phi = atan2(q[1], q[0]);
    const double sintheta = sqrt(1 - X * X);
    const double cosphi = cos(phi);
    const double sinphi = sin(phi);
    for (int m = 0; m < lmax + 1; m++) {
        cosmphi[m] = cos(m * phi);
        sinmphi[m] = sin(m * phi);
    }
    tmp_grad2[0] = 0.;
    tmp_grad2[1] = 0.;
    tmp_grad2[2] = 0.;
    for (int n = 0; n < nmax + 1; n++)
        for (int l = 0; l < lmax + 1; l++)
            for (int m = 0; m < lmax + 1; m++) {
                if (m > l) continue;
                const int i = m + (lmax + 1) * (l + (lmax + 1) * n);
                const double tmp = (Snlm[i] * cosmphi[m] + Tnlm[i] * sinmphi[m]);
                if ((Snlm[i] == 0.) & (Tnlm[i] == 0.)) continue;
                sph_grad_phi_nlm(s, X, n, l, m, tmp_grad);
                tmp_grad2[0] += tmp_grad[0] * tmp;
                tmp_grad2[1] += tmp_grad[1] * tmp;
                tmp_grad2[2] += tmp_grad[2] * (Tnlm[i] * cosmphi[m] - Snlm[i] * sinmphi[m]) / (s * sintheta);
            }
    tmp_grad[0] = tmp_grad2[0];
    tmp_grad[1] = tmp_grad2[1];
    tmp_grad[2] = tmp_grad2[2];
    tmp_grad2[0] = sintheta * cosphi * tmp_grad[0] + X * cosphi * tmp_grad[1] - sinphi * tmp_grad[2];
    tmp_grad2[1] = sintheta * sinphi * tmp_grad[0] + X * sinphi * tmp_grad[1] + cosphi * tmp_grad[2];
    tmp_grad2[2] = X * tmp_grad[0] - sintheta * tmp_grad[1];
    g[0] += tmp_grad2[0] * G * M / (r_s * r_s);
    g[1] += tmp_grad2[1] * G * M / (r_s * r_s);
    g[2] += tmp_grad2[2] * G * M / (r_s * r_s);
}

/* scf_density -> scf_density_helper (bfe.cpp:16-56) */
double orc_scf_density(const double *p, const double *q) {
    SCF_UNPACK;
    double cosmphi[64], sinmphi[64];
    const double r = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    const double s = r / r_s;
    const double X = q[2] / r;
    const double phi = atan2(q[1], q[0]);
    double dens = 0.;
    for (int m = 0; m < lmax + 1; m++) {
        cosmphi[m] = cos(m * phi);
        sinmphi[m] = sin(m * phi);
    }
    for (int n = 0; n < nmax + 1; n++)
        for (int l = 0; l < lmax + 1; l++)
            for (int m = 0; m < lmax + 1; m++) {
                if (m > l) continue;
                const int i = m + (lmax + 1) * (l + (lmax + 1) * n);
                if ((Snlm[i] == 0.) & (Tnlm[i] == 0.)) continue;
                dens += rho_nl(s, n, l) * orc_legendre_sphPlm(l, m, X) *
                        (Snlm[i] * cosmphi[m] + Tnlm[i] * sinmphi[m]);
            }
    dens *= M / (r_s * r_s * r_s);
    return dens;
}
