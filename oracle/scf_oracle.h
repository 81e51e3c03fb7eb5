/*
 * ORACLE (test infrastructure only): CPU restatement of gala's SCF basis-function
 * expansion (src/gala/potential/scf/src/bfe.cpp, bfe_helper.cpp).
 *
 * gala evaluates the special functions with GSL (gsl_sf_gegenpoly_n,
 * gsl_sf_legendre_Plm, gsl_sf_legendre_sphPlm, gsl_sf_gamma; call sites
 * bfe_helper.cpp:17-25, 42-74).  GSL is a third-party dependency that is not part
 * of the gala sources (version unpinned: CI installs the distribution's
 * libgsl-dev).  Here those functions are written from their published
 * definitions and three-term recurrences:
 *   Gegenbauer  C_n^a(x):  C_0 = 1, C_1 = 2 a x,
 *               n C_n = 2 x (n + a - 1) C_{n-1} - (n + 2a - 2) C_{n-2}
 *               (Abramowitz & Stegun 22.7.3)
 *   Legendre    P_m^m = (-1)^m (2m-1)!! (1-x^2)^{m/2}  (Condon-Shortley phase, as GSL),
 *               P_{m+1}^m = x (2m+1) P_m^m,
 *               (l-m) P_l^m = x (2l-1) P_{l-1}^m - (l+m-1) P_{l-2}^m   (A&S 8.5.3)
 *   sphPlm      sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!) P_l^m(x)
 *   Gamma       (k-1)! for the positive integer arguments used here.
 * Parity of this restatement is pinned against the original Fortran SCF code's
 * potential and acceleration at 32768 positions for five coefficient sets (gala's
 * tests/potential/scf/data, test_accp_fortran.py), at rtol 1e-6.
 *
 * Parameter packing is gala's: p = [G, nmax, lmax, M, r_s, S(nmax+1, lmax+1, lmax+1),
 * T(nmax+1, lmax+1, lmax+1)] (bfe.cpp:191-259), index m + (lmax+1)(l + (lmax+1) n).
 */
#ifndef ORC_SCF_ORACLE_H
#define ORC_SCF_ORACLE_H
double orc_scf_value(const double *p, const double *q);
void orc_scf_gradient(const double *p, const double *q, double *g);
double orc_scf_density(const double *p, const double *q);
double orc_gegenpoly(int n, double a, double x);
double orc_legendre_Plm(int l, int m, double x);
double orc_legendre_sphPlm(int l, int m, double x);
#endif
