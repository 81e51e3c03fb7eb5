/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A plain-C restatement of gala's orbit-integration hot path, used only by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the
 * checker of the CUDA library.  Nothing in gala_gb300/ links, imports or calls
 * this file.
 *
 * Every function follows one gala function (file:line inside the gala project)
 * and keeps its floating-point expression order, so that with a build that
 * forbids contraction and reassociation (-O2 -ffp-contract=off) it reproduces
 * gala's arithmetic operation by operation:
 *
 *   potentials     src/gala/potential/potential/builtin/builtin_potentials.cpp
 *   composition    src/gala/potential/potential/src/cpotential.cpp:137-287
 *   frames         src/gala/potential/frame/builtin/builtin_frames.cpp:8-112
 *   hamiltonian    src/gala/potential/hamiltonian/src/chamiltonian.cpp:7-57
 *   leapfrog       src/gala/integrate/cyintegrators/leapfrog.pyx:24-121
 *   ruth4          src/gala/integrate/cyintegrators/ruth4.pyx:24-113
 *   dop853         src/gala/integrate/cyintegrators/dopri/dop853.cpp:18-904 and
 *                  src/gala/integrate/cyintegrators/dop853.pyx:90-250
 *
 * The same source is also built with gala's own flags (-Ofast) as the CPU
 * baseline that bench.py times on the host cores; both builds are made by
 * oracle/Makefile.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/gala_gb300.h"
#include "dop853_tableau.h"
#include "scf_oracle.h"

/* ------------------------------------------------------------------------- */
/* Single-component potentials (builtin_potentials.cpp)                       */
/* ------------------------------------------------------------------------- */

static double norm3_sq(const double *q) { return q[0] * q[0] + q[1] * q[1] + q[2] * q[2]; }

/* kepler_value :58-64, hernquist_value :211-219, plummer_value :292-300,
 * miyamotonagai_value :1287-1296, sphericalnfw_value :819-833,
 * flattenednfw_value :925-942, triaxialnfw_value :1028-1049, scf_value
 * (src/gala/potential/scf/src/bfe.cpp:191-227). */
static double comp_value(int type, const double *p, const double *q) {
    switch (type) {
    case GX_POT_NULL:
        return 0.;
    case GX_POT_KEPLER:
        return -p[0] * p[1] / sqrt(norm3_sq(q));
    case GX_POT_HERNQUIST: {
        const double r = sqrt(norm3_sq(q));
        return -p[0] * p[1] / (r + p[2]);
    }
    case GX_POT_PLUMMER: {
        const double r2 = norm3_sq(q);
        return -p[0] * p[1] / sqrt(r2 + p[2] * p[2]);
    }
    case GX_POT_MIYAMOTONAGAI: {
        const double zd = (p[2] + sqrt(q[2] * q[2] + p[3] * p[3]));
        return -p[0] * p[1] / sqrt(q[0] * q[0] + q[1] * q[1] + zd * zd);
    }
    case GX_POT_SPHERICALNFW: {
        const double v_h2 = -p[0] * p[1] / p[2];
        const double u = sqrt(norm3_sq(q)) / p[2];
        if (u == 0) return v_h2;
        return v_h2 * log(1 + u) / u;
    }
    case GX_POT_FLATTENEDNFW: {
        const double v_h2 = -p[0] * p[1] / p[2];
        const double u = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] / (p[5] * p[5])) / p[2];
        if (u == 0) return v_h2;
        return v_h2 * log(1 + u) / u;
    }
    case GX_POT_TRIAXIALNFW: {
        const double v_h2 = -p[0] * p[1] / p[2];
        const double u = sqrt(q[0] * q[0] / (p[3] * p[3]) + q[1] * q[1] / (p[4] * p[4]) +
                              q[2] * q[2] / (p[5] * p[5])) / p[2];
        if (u == 0) return v_h2;
        return v_h2 * log(1 + u) / u;
    }
    case GX_POT_SCF:
        return orc_scf_value(p, q);
    default:
        return NAN;
    }
}

/* *_gradient_single: kepler :66-76, hernquist :221-233, plummer :302-314,
 * miyamotonagai :1298-1312, sphericalnfw :835-850, flattenednfw :944-962,
 * triaxialnfw :1051-1072.  One point (x, y, z); accumulates into (gx, gy, gz).
 * Written as inline functions so that the loops over points below vectorise
 * as gala's gradientv loops do (vectorization.h): same per-point arithmetic. */
static inline void grad_kepler(const double *p, double x, double y, double z, double *gx, double *gy, double *gz) {
    const double fac = p[0] * p[1] / pow(sqrt(x * x + y * y + z * z), 3);
    *gx = *gx + fac * x;
    *gy = *gy + fac * y;
    *gz = *gz + fac * z;
}
static inline void grad_hernquist(const double *p, double x, double y, double z, double *gx, double *gy,
                                  double *gz) {
    const double r = sqrt(x * x + y * y + z * z);
    const double fac = p[0] * p[1] / ((r + p[2]) * (r + p[2]) * r);
    *gx = *gx + fac * x;
    *gy = *gy + fac * y;
    *gz = *gz + fac * z;
}
static inline void grad_plummer(const double *p, double x, double y, double z, double *gx, double *gy, double *gz) {
    const double R2b = x * x + y * y + z * z + p[2] * p[2];
    const double fac = p[0] * p[1] / sqrt(R2b) / R2b;
    *gx = *gx + fac * x;
    *gy = *gy + fac * y;
    *gz = *gz + fac * z;
}
static inline void grad_mn(const double *p, double x, double y, double z, double *gx, double *gy, double *gz) {
    const double sqrtz = sqrt(z * z + p[3] * p[3]);
    const double zd = p[2] + sqrtz;
    const double fac = p[0] * p[1] * pow(x * x + y * y + zd * zd, -1.5);
    *gx = *gx + fac * x;
    *gy = *gy + fac * y;
    *gz = *gz + fac * z * (1. + p[2] / sqrtz);
}
static inline void grad_snfw(const double *p, double x, double y, double z, double *gx, double *gy, double *gz) {
    const double v_h2 = p[0] * p[1] / p[2];
    const double u = sqrt(x * x + y * y + z * z) / p[2];
    const double fac = v_h2 / (u * u * u) / (p[2] * p[2]) * (log(1 + u) - u / (1 + u));
    *gx = *gx + fac * x;
    *gy = *gy + fac * y;
    *gz = *gz + fac * z;
}
static inline void grad_fnfw(const double *p, double x, double y, double z, double *gx, double *gy, double *gz) {
    const double v_h2 = p[0] * p[1] / p[2];
    const double u = sqrt(x * x + y * y + z * z / (p[5] * p[5])) / p[2];
    const double fac = v_h2 / (u * u * u) / (p[2] * p[2]) * (log(1 + u) - u / (1 + u));
    *gx = *gx + fac * x;
    *gy = *gy + fac * y;
    *gz = *gz + fac * z / (p[5] * p[5]);
}
static inline void grad_tnfw(const double *p, double x, double y, double z, double *gx, double *gy, double *gz) {
    const double v_h2 = p[0] * p[1] / p[2];
    const double u = sqrt(x * x / (p[3] * p[3]) + y * y / (p[4] * p[4]) + z * z / (p[5] * p[5])) / p[2];
    const double fac = v_h2 / (u * u * u) / (p[2] * p[2]) * (log(1 + u) - u / (1 + u));
    *gx = *gx + fac * x / (p[3] * p[3]);
    *gy = *gy + fac * y / (p[4] * p[4]);
    *gz = *gz + fac * z / (p[5] * p[5]);
}

/* One point of one component (scf_gradient: bfe.cpp:229-259).  Accumulates into g. */
static void comp_gradient(int type, const double *p, const double *q, double *g) {
    switch (type) {
    case GX_POT_NULL: return;
    case GX_POT_KEPLER: grad_kepler(p, q[0], q[1], q[2], &g[0], &g[1], &g[2]); return;
    case GX_POT_HERNQUIST: grad_hernquist(p, q[0], q[1], q[2], &g[0], &g[1], &g[2]); return;
    case GX_POT_PLUMMER: grad_plummer(p, q[0], q[1], q[2], &g[0], &g[1], &g[2]); return;
    case GX_POT_MIYAMOTONAGAI: grad_mn(p, q[0], q[1], q[2], &g[0], &g[1], &g[2]); return;
    case GX_POT_SPHERICALNFW: grad_snfw(p, q[0], q[1], q[2], &g[0], &g[1], &g[2]); return;
    case GX_POT_FLATTENEDNFW: grad_fnfw(p, q[0], q[1], q[2], &g[0], &g[1], &g[2]); return;
    case GX_POT_TRIAXIALNFW: grad_tnfw(p, q[0], q[1], q[2], &g[0], &g[1], &g[2]); return;
    case GX_POT_SCF: orc_scf_gradient(p, q, g); return;
    default: g[0] = NAN; g[1] = NAN; g[2] = NAN; return;
    }
}

/* One component over N points, SoA q[3, N], accumulated into g[3, N]: the
 * gradientv loop of vectorization.h (one pass per component). */
#define GX_POINT_LOOP(FN)                                                                  \
    for (size_t i = 0; i < N; i++) {                                                       \
        double a = gx[i], b = gy[i], c = gz[i];                                            \
        FN(p, qx[i], qy[i], qz[i], &a, &b, &c);                                            \
        gx[i] = a;                                                                         \
        gy[i] = b;                                                                         \
        gz[i] = c;                                                                         \
    }
static void comp_gradient_n(int type, const double *p, size_t N, const double *restrict q, double *restrict g) {
    const double *restrict qx = q, *restrict qy = q + N, *restrict qz = q + 2 * N;
    double *restrict gx = g, *restrict gy = g + N, *restrict gz = g + 2 * N;
    switch (type) {
    case GX_POT_NULL: return;
    case GX_POT_KEPLER: GX_POINT_LOOP(grad_kepler) return;
    case GX_POT_HERNQUIST: GX_POINT_LOOP(grad_hernquist) return;
    case GX_POT_PLUMMER: GX_POINT_LOOP(grad_plummer) return;
    case GX_POT_MIYAMOTONAGAI: GX_POINT_LOOP(grad_mn) return;
    case GX_POT_SPHERICALNFW: GX_POINT_LOOP(grad_snfw) return;
    case GX_POT_FLATTENEDNFW: GX_POINT_LOOP(grad_fnfw) return;
    case GX_POT_TRIAXIALNFW: GX_POINT_LOOP(grad_tnfw) return;
    default:
        for (size_t i = 0; i < N; i++) {
            double qi[3] = {qx[i], qy[i], qz[i]}, gi[3] = {gx[i], gy[i], gz[i]};
            comp_gradient(type, p, qi, gi);
            gx[i] = gi[0];
            gy[i] = gi[1];
            gz[i] = gi[2];
        }
        return;
    }
}
#undef GX_POINT_LOOP

/* kepler_density :78-88, hernquist_density :235-244, plummer_density :316-324,
 * miyamotonagai_density :1314-1332, sphericalnfw_density :852-864,
 * scf_density (bfe.cpp).  Flattened/triaxial NFW have no density in gala
 * (nan_density is installed, cybuiltin.pyx), nor do we. */
static double comp_density(int type, const double *p, const double *q) {
    switch (type) {
    case GX_POT_NULL:
        return 0.;
    case GX_POT_KEPLER:
        return (norm3_sq(q) == 0.) ? INFINITY : 0.;
    case GX_POT_HERNQUIST: {
        const double r = sqrt(norm3_sq(q));
        const double rho0 = p[1] / (2 * M_PI * p[2] * p[2] * p[2]);
        return rho0 / ((r / p[2]) * pow(1 + r / p[2], 3));
    }
    case GX_POT_PLUMMER: {
        const double r2 = norm3_sq(q);
        return 3 * p[1] / (4 * M_PI * p[2] * p[2] * p[2]) * pow(1 + r2 / (p[2] * p[2]), -2.5);
    }
    case GX_POT_MIYAMOTONAGAI: {
        const double M = p[1], a = p[2], b = p[3];
        const double R2 = q[0] * q[0] + q[1] * q[1];
        const double sqrt_zb = sqrt(q[2] * q[2] + b * b);
        const double numer = (b * b * M / (4 * M_PI)) * (a * R2 + (a + 3 * sqrt_zb) * (a + sqrt_zb) * (a + sqrt_zb));
        const double denom = pow(R2 + (a + sqrt_zb) * (a + sqrt_zb), 2.5) * sqrt_zb * sqrt_zb * sqrt_zb;
        return numer / denom;
    }
    case GX_POT_SPHERICALNFW: {
        const double v_h2 = p[0] * p[1] / p[2];
        const double r = sqrt(norm3_sq(q));
        const double rho0 = v_h2 / (4 * M_PI * p[0] * p[2] * p[2]);
        return rho0 / ((r / p[2]) * pow(1 + r / p[2], 2));
    }
    case GX_POT_SCF:
        return orc_scf_density(p, q);
    default:
        return NAN;
    }
}

/* ------------------------------------------------------------------------- */
/* Composition with shift/rotate (cpotential.cpp:137-287)                      */
/* ------------------------------------------------------------------------- */

/* apply_shift_rotate (:137-149) followed by apply_rotate with q_out = 0 (:80-100):
 * q' = R (q - q0), each row summed left to right starting from 0. */
static void shift_rotate(const gx_component *c, const double *q, double *qt) {
    const double *R = c->R;
    const double x = q[0] - c->q0[0], y = q[1] - c->q0[1], z = q[2] - c->q0[2];
    qt[0] = 0. + R[0] * x + R[1] * y + R[2] * z;
    qt[1] = 0. + R[3] * x + R[4] * y + R[5] * z;
    qt[2] = 0. + R[6] * x + R[7] * y + R[8] * z;
}

/* apply_rotate_T with transpose = 1 (:103-134): g = R^T g'. */
static void rotate_back(const gx_component *c, const double *gt, double *g) {
    const double *R = c->R;
    g[0] = R[0] * gt[0] + R[3] * gt[1] + R[6] * gt[2];
    g[1] = R[1] * gt[0] + R[4] * gt[1] + R[7] * gt[2];
    g[2] = R[2] * gt[0] + R[5] * gt[1] + R[8] * gt[2];
}

/* The shift/rotate path of apply_shift_rotate_N (:152-167) rotates (q - q0) in
 * place without the leading 0 term; for finite inputs 0 + a == a, so both forms
 * give the same bits except for the sign of an exact zero. */

/* c_potential (:170-189) */
double orc_potential(const gx_potential *pot, double t, const double *q) {
    (void)t;
    double v = 0;
    for (int i = 0; i < pot->n_components; i++) {
        const gx_component *c = &pot->components[i];
        const double *p = pot->params + c->param_offset;
        if (c->do_shift_rotate == 0) {
            v = v + comp_value(c->type, p, q);
        } else {
            double qt[3];
            shift_rotate(c, q, qt);
            v = v + comp_value(c->type, p, qt);
        }
    }
    return v;
}

/* c_density (:192-211) */
double orc_density(const gx_potential *pot, double t, const double *q) {
    (void)t;
    double v = 0;
    for (int i = 0; i < pot->n_components; i++) {
        const gx_component *c = &pot->components[i];
        const double *p = pot->params + c->param_offset;
        if (c->do_shift_rotate == 0) {
            v = v + comp_density(c->type, p, q);
        } else {
            double qt[3];
            shift_rotate(c, q, qt);
            v = v + comp_density(c->type, p, qt);
        }
    }
    return v;
}

/* c_gradient for one point (:214-287): zero, then accumulate components in
 * order; a shifted/rotated component is evaluated into a zeroed temporary,
 * rotated back and added. */
static void gradient_point(const gx_potential *pot, const double *q, double *g) {
    g[0] = 0.; g[1] = 0.; g[2] = 0.;
    for (int i = 0; i < pot->n_components; i++) {
        const gx_component *c = &pot->components[i];
        const double *p = pot->params + c->param_offset;
        if (c->do_shift_rotate == 0) {
            comp_gradient(c->type, p, q, g);
        } else {
            double qt[3], gt[3] = {0., 0., 0.}, gr[3];
            const double *R = c->R;
            const double x = q[0] - c->q0[0], y = q[1] - c->q0[1], z = q[2] - c->q0[2];
            qt[0] = R[0] * x + R[1] * y + R[2] * z;
            qt[1] = R[3] * x + R[4] * y + R[5] * z;
            qt[2] = R[6] * x + R[7] * y + R[8] * z;
            comp_gradient(c->type, p, qt, gt);
            rotate_back(c, gt, gr);
            g[0] += gr[0];
            g[1] += gr[1];
            g[2] += gr[2];
        }
    }
}

/* c_gradient over N points, SoA q[3, N] -> grad[3, N] (overwritten): zero,
 * then component by component over all points (:214-287).  A shifted/rotated
 * component is evaluated on transformed points into a zeroed temporary, its
 * gradients rotated back and added, in blocks of points. */
void orc_gradient(const gx_potential *pot, size_t N, double t, const double *q, double *grad) {
    (void)t;
    enum { BLK = 256 };
    for (size_t i = 0; i < 3 * N; i++) grad[i] = 0.;
    for (int ci = 0; ci < pot->n_components; ci++) {
        const gx_component *c = &pot->components[ci];
        const double *p = pot->params + c->param_offset;
        if (c->do_shift_rotate == 0) {
            comp_gradient_n(c->type, p, N, q, grad);
            continue;
        }
        for (size_t lo = 0; lo < N; lo += BLK) {
            const size_t m = (N - lo < BLK) ? N - lo : BLK;
            double qt[3 * BLK], gt[3 * BLK];
            for (size_t i = 0; i < m; i++) {
                const double x = q[lo + i] - c->q0[0], y = q[N + lo + i] - c->q0[1], z = q[2 * N + lo + i] - c->q0[2];
                const double *R = c->R;
                qt[i] = R[0] * x + R[1] * y + R[2] * z;
                qt[m + i] = R[3] * x + R[4] * y + R[5] * z;
                qt[2 * m + i] = R[6] * x + R[7] * y + R[8] * z;
                gt[i] = 0.;
                gt[m + i] = 0.;
                gt[2 * m + i] = 0.;
            }
            comp_gradient_n(c->type, p, m, qt, gt);
            for (size_t i = 0; i < m; i++) {
                const double g1[3] = {gt[i], gt[m + i], gt[2 * m + i]};
                double gr[3];
                rotate_back(c, g1, gr);
                grad[lo + i] += gr[0];
                grad[N + lo + i] += gr[1];
                grad[2 * N + lo + i] += gr[2];
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Frames and Hamiltonian (builtin_frames.cpp, chamiltonian.cpp)             */
/* ------------------------------------------------------------------------- */

/* static_frame_hamiltonian (:8-16) / constant_rotating_frame_3d_hamiltonian (:78-94) */
static double frame_energy(const gx_frame *fr, const double *w) {
    if (fr == NULL || fr->type == GX_FRAME_STATIC) {
        double E = 0.;
        for (int i = 0; i < 3; i++) E += w[i + 3] * w[i + 3];
        return 0.5 * E;
    } else {
        const double *O = fr->params;
        double E = 0.;
        for (int i = 0; i < 3; i++) E += 0.5 * w[i + 3] * w[i + 3];
        const double Lx = w[1] * w[5] - w[2] * w[4];
        const double Ly = -w[0] * w[5] + w[2] * w[3];
        const double Lz = w[0] * w[4] - w[1] * w[3];
        return E - (O[0] * Lx + O[1] * Ly + O[2] * Lz);
    }
}

/* Hamiltonian.energy (src/gala/potential/hamiltonian/chamiltonian.pyx:83-86, 107-128):
 * potential energy through c_potential (shift/rotate aware) plus the frame's
 * energy (CFrameWrapper.energy, src/gala/potential/frame/cframe.pyx:29-45). */
double orc_hamiltonian_value(const gx_potential *pot, const gx_frame *fr, double t, const double *w) {
    return orc_potential(pot, t, w) + frame_energy(fr, w);
}

/* Fwrapper_T -> hamiltonian_gradient_T (chamiltonian.cpp:38-57) for one point
 * whose potential gradient g is already known: f[3:6] = g, the frame gradient
 * fills f[0:3] (and for the rotating frame adds Omega x p to f[3:6],
 * builtin_frames.cpp:96-112), then the momentum half is negated. */
static void rhs_from_gradient(const gx_frame *fr, const double *w, const double *g, double *f) {
    if (fr == NULL || fr->type == GX_FRAME_STATIC) {
        f[0] = w[3];
        f[1] = w[4];
        f[2] = w[5];
        f[3] = g[0];
        f[4] = g[1];
        f[5] = g[2];
    } else {
        const double *O = fr->params;
        double Cx = O[1] * w[2] - O[2] * w[1];
        double Cy = -O[0] * w[2] + O[2] * w[0];
        double Cz = O[0] * w[1] - O[1] * w[0];
        f[0] = 0. + w[3] - Cx;
        f[1] = 0. + w[4] - Cy;
        f[2] = 0. + w[5] - Cz;
        Cx = O[1] * w[5] - O[2] * w[4];
        Cy = -O[0] * w[5] + O[2] * w[3];
        Cz = O[0] * w[4] - O[1] * w[3];
        f[3] = g[0] + Cx;
        f[4] = g[1] + Cy;
        f[5] = g[2] + Cz;
    }
    f[3] *= -1;
    f[4] *= -1;
    f[5] *= -1;
}

static void rhs_point(const gx_potential *pot, const gx_frame *fr, const double *w, double *f) {
    double g[3];
    gradient_point(pot, w, g);
    rhs_from_gradient(fr, w, g, f);
}

/* hamiltonian_gradient_T over SoA w[6, N] -> f[6, N]: c_gradient over all N
 * positions first (written into the momentum half, as gala does), then the
 * frame part and the negation point by point. */
void orc_hamiltonian_gradient(const gx_potential *pot, const gx_frame *fr, size_t N, double t,
                              const double *w, double *f) {
    orc_gradient(pot, N, t, w, f + 3 * N);
    for (size_t i = 0; i < N; i++) {
        double wi[6], fi[6];
        const double g[3] = {f[3 * N + i], f[4 * N + i], f[5 * N + i]};
        for (int k = 0; k < 6; k++) wi[k] = w[k * N + i];
        rhs_from_gradient(fr, wi, g, fi);
        for (int k = 0; k < 6; k++) f[k * N + i] = fi[k];
    }
}

/* ------------------------------------------------------------------------- */
/* Parallel-for over index ranges (pthreads), used to spread independent      */
/* orbits (leapfrog/ruth4) or batches (dop853) over host cores.               */
/* ------------------------------------------------------------------------- */
typedef void (*range_fn)(void *ctx, int64_t lo, int64_t hi);
typedef struct {
    range_fn fn;
    void *ctx;
    int64_t n, chunk;
    int64_t next;
    pthread_mutex_t mu;
} pool_t;

static void *pool_worker(void *arg) {
    pool_t *P = (pool_t *)arg;
    for (;;) {
        pthread_mutex_lock(&P->mu);
        int64_t lo = P->next;
        P->next += P->chunk;
        pthread_mutex_unlock(&P->mu);
        if (lo >= P->n) break;
        int64_t hi = lo + P->chunk < P->n ? lo + P->chunk : P->n;
        P->fn(P->ctx, lo, hi);
    }
    return NULL;
}

static void parallel_for(int nthreads, int64_t n, int64_t chunk, range_fn fn, void *ctx) {
    if (nthreads <= 1 || n <= chunk) {
        fn(ctx, 0, n);
        return;
    }
    pool_t P;
    P.fn = fn;
    P.ctx = ctx;
    P.n = n;
    P.chunk = chunk;
    P.next = 0;
    pthread_mutex_init(&P.mu, NULL);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    int started = 0;
    if (th)
        while (started < nthreads - 1 && pthread_create(&th[started], NULL, pool_worker, &P) == 0) started++;
    pool_worker(&P); /* the caller is the last worker, so the work ends even without threads */
    for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&P.mu);
}

/* ------------------------------------------------------------------------- */
/* Leapfrog (leapfrog.pyx:24-121) and Ruth4 (ruth4.pyx:24-113)                 */
/* ------------------------------------------------------------------------- */
typedef struct {
    const gx_potential *pot;
    const double *w0, *t;
    int64_t n, ntimes;
    int save_all, method;
    double *w_out;
} fixed_ctx;

/* One chunk of orbits [lo, hi) advanced exactly like gala advances its whole
 * (6, n) array: the per-orbit arithmetic does not depend on the other orbits,
 * so chunking changes no bits. */
static void fixed_chunk(void *vctx, int64_t lo, int64_t hi) {
    fixed_ctx *C = (fixed_ctx *)vctx;
    const int64_t n = C->n, ntimes = C->ntimes, m = hi - lo;
    const double dt = C->t[1] - C->t[0];
    double *x = (double *)malloc(sizeof(double) * 6 * (size_t)m);
    double *vh = (double *)malloc(sizeof(double) * 3 * (size_t)m);
    double *grad = (double *)malloc(sizeof(double) * 3 * (size_t)m);
    for (int k = 0; k < 6; k++)
        for (int64_t i = 0; i < m; i++) x[k * m + i] = C->w0[k * n + lo + i];
    if (C->save_all)
        for (int k = 0; k < 6; k++)
            for (int64_t i = 0; i < m; i++) C->w_out[(k * ntimes + 0) * n + lo + i] = x[k * m + i];

    if (C->method == 0) {
        /* c_init_velocity (:24-32) */
        orc_gradient(C->pot, (size_t)m, C->t[0], x, grad);
        for (int k = 0; k < 3; k++)
            for (int64_t i = 0; i < m; i++) vh[k * m + i] = x[(3 + k) * m + i] - grad[k * m + i] * dt / 2.;
        for (int64_t j = 1; j < ntimes; j++) {
            /* c_leapfrog_step (:35-51) */
            for (int k = 0; k < 3; k++)
                for (int64_t i = 0; i < m; i++) x[k * m + i] = x[k * m + i] + vh[k * m + i] * dt;
            orc_gradient(C->pot, (size_t)m, C->t[j], x, grad);
            for (int k = 0; k < 3; k++)
                for (int64_t i = 0; i < m; i++) {
                    x[(3 + k) * m + i] = vh[k * m + i] - grad[k * m + i] * dt / 2.;
                    vh[k * m + i] = vh[k * m + i] - grad[k * m + i] * dt;
                }
            if (C->save_all)
                for (int k = 0; k < 6; k++)
                    for (int64_t i = 0; i < m; i++) C->w_out[(k * ntimes + j) * n + lo + i] = x[k * m + i];
        }
    } else {
        /* coefficients (ruth4.pyx:65-78) */
        const double two_13 = pow(2., 1. / 3.);
        const double cs[4] = {1. / (2. * (2. - two_13)), (1. - two_13) / (2. * (2. - two_13)),
                              (1. - two_13) / (2. * (2. - two_13)), 1. / (2. * (2. - two_13))};
        const double ds[4] = {0., 1. / (2. - two_13), -two_13 / (2. - two_13), 1. / (2. - two_13)};
        for (int64_t j = 1; j < ntimes; j++) {
            /* c_ruth4_step (:24-35) */
            for (int s = 0; s < 4; s++) {
                orc_gradient(C->pot, (size_t)m, C->t[j], x, grad);
                for (int k = 0; k < 3; k++)
                    for (int64_t i = 0; i < m; i++) {
                        x[(3 + k) * m + i] = x[(3 + k) * m + i] - ds[s] * grad[k * m + i] * dt;
                        x[k * m + i] = x[k * m + i] + cs[s] * x[(3 + k) * m + i] * dt;
                    }
            }
            if (C->save_all)
                for (int k = 0; k < 6; k++)
                    for (int64_t i = 0; i < m; i++) C->w_out[(k * ntimes + j) * n + lo + i] = x[k * m + i];
        }
    }
    if (!C->save_all)
        for (int k = 0; k < 6; k++)
            for (int64_t i = 0; i < m; i++) C->w_out[k * n + lo + i] = x[k * m + i];
    free(x);
    free(vh);
    free(grad);
}

/* leapfrog_integrate_hamiltonian / ruth4_integrate_hamiltonian.
 * w0 (6, n); w_out (6, ntimes, n) if save_all else (6, n).  method 0 =
 * leapfrog, 1 = ruth4.  Orbits are spread over nthreads in chunks. */
int orc_fixed_integrate(const gx_potential *pot, int method, const double *w0, int64_t n,
                        const double *t, int64_t ntimes, int save_all, double *w_out, int nthreads) {
    if (ntimes < 2 || n < 0) return -1;
    fixed_ctx C = {pot, w0, t, n, ntimes, save_all, method, w_out};
    int64_t chunk = 256;
    if (nthreads > 1 && n / nthreads < chunk) chunk = (n + nthreads - 1) / nthreads;
    if (chunk < 1) chunk = 1;
    parallel_for(nthreads, n, chunk, fixed_chunk, &C);
    return 0;
}

/* Many orbits of uneven length, step and integrator, each integrated the way
 * gala integrates one orbit with its own time grid: integrate_orbit(w0_i,
 * dt=dt_i, n_steps=n_i) builds t = cumsum([0, dt_i, ..., dt_i]) (timespec.py:
 * 98-102) and runs leapfrog_integrate_hamiltonian or ruth4_integrate_hamiltonian
 * on the (6, 1) array (leapfrog.pyx:99-116, ruth4.pyx:98-108).  w_out (6, n)
 * receives the final states.  Orbits are spread over nthreads. */
typedef struct {
    const gx_potential *pot;
    const double *w0, *dt;
    const int64_t *nsteps;
    const int32_t *method;
    int64_t n;
    double *w_out;
} batch_fixed_ctx;

static void batch_fixed_chunk(void *vctx, int64_t lo, int64_t hi) {
    batch_fixed_ctx *B = (batch_fixed_ctx *)vctx;
    for (int64_t i = lo; i < hi; i++) {
        double w0[6], w1[6];
        for (int k = 0; k < 6; k++) w0[k] = B->w0[k * B->n + i];
        const int64_t ns = B->nsteps[i];
        if (ns <= 0) {
            for (int k = 0; k < 6; k++) B->w_out[k * B->n + i] = w0[k];
            continue;
        }
        double *t = (double *)malloc(sizeof(double) * (size_t)(ns + 1));
        if (!t) continue;
        double acc = 0.0;
        t[0] = 0.0;
        for (int64_t j = 1; j <= ns; j++) {
            acc += B->dt[i];
            t[j] = acc;
        }
        fixed_ctx C = {B->pot, w0, t, 1, ns + 1, 0, B->method[i] ? 1 : 0, w1};
        fixed_chunk(&C, 0, 1);
        for (int k = 0; k < 6; k++) B->w_out[k * B->n + i] = w1[k];
        free(t);
    }
}

int orc_batch_fixed(const gx_potential *pot, const double *w0, int64_t n, const int64_t *nsteps,
                    const double *dt, const int32_t *method, double *w_out, int nthreads) {
    if (n < 0) return -1;
    batch_fixed_ctx B = {pot, w0, dt, nsteps, method, n, w_out};
    int64_t chunk = 16;
    if (nthreads > 1 && n / nthreads < chunk) chunk = (n + nthreads - 1) / nthreads;
    if (chunk < 1) chunk = 1;
    parallel_for(nthreads, n, chunk, batch_fixed_chunk, &B);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* DOP853 (dop853.cpp)                                                        */
/* ------------------------------------------------------------------------- */
static double sign_d(double a, double b) { return (b < 0.0) ? -fabs(a) : fabs(a); }
static double min_d(double a, double b) { return (a < b) ? a : b; }
static double max_d(double a, double b) { return (a > b) ? a : b; }

/* Right-hand side of a DOP853 system: f = F(y) for the system's state y. */
typedef struct {
    void (*fn)(const void *ctx, const double *y, double *f);
    const void *ctx;
} rhs_t;

/* Fwrapper_T on a batch held as y[6 * nb] in SoA order (component k of orbit j
 * at k * nb + j), as dop853_helper lays it out (dop853.pyx:135-136, 157-182). */
static void batch_rhs(const gx_potential *pot, const gx_frame *fr, int nb, const double *y, double *f) {
    orc_hamiltonian_gradient(pot, fr, (size_t)nb, 0.0, y, f);
}

typedef struct {
    const gx_potential *pot;
    const gx_frame *fr;
    int nb;
} batch_ctx;

static void batch_rhs_cb(const void *vctx, const double *y, double *f) {
    const batch_ctx *c = (const batch_ctx *)vctx;
    batch_rhs(c->pot, c->fr, c->nb, y, f);
}

/* hinit (:18-86), scalar tolerances. */
static double orc_hinit(rhs_t R, int n, double x, const double *y,
                        double posneg, const double *f0, double *f1, double *yy1, int iord,
                        double hmax, double atoli, double rtoli) {
    double dnf = 0.0, dny = 0.0, sk, sqr, h, h1, der2, der12;
    for (int i = 0; i < n; i++) {
        sk = atoli + rtoli * fabs(y[i]);
        sqr = f0[i] / sk;
        dnf += sqr * sqr;
        sqr = y[i] / sk;
        dny += sqr * sqr;
    }
    if ((dnf <= 1.0E-10) || (dny <= 1.0E-10))
        h = 1.0E-6;
    else
        h = sqrt(dny / dnf) * 0.01;
    h = min_d(h, hmax);
    h = sign_d(h, posneg);
    for (int i = 0; i < n; i++) yy1[i] = y[i] + h * f0[i];
    R.fn(R.ctx, yy1, f1);
    (void)x;
    der2 = 0.0;
    for (int i = 0; i < n; i++) {
        sk = atoli + rtoli * fabs(y[i]);
        sqr = (f1[i] - f0[i]) / sk;
        der2 += sqr * sqr;
    }
    der2 = sqrt(der2) / h;
    der12 = max_d(fabs(der2), sqrt(dnf));
    if (der12 <= 1.0E-15)
        h1 = max_d(1.0E-6, fabs(h) * 1.0E-3);
    else
        h1 = pow(0.01 / der12, 1.0 / (double)iord);
    h = min_d(100.0 * fabs(h), min_d(h1, hmax));
    return sign_d(h, posneg);
}

/* One dop853() call (dopcor :89-650 with the front-end defaults of :653-866)
 * on a system of n components with right-hand side R.
 *   y       : (n) in/out state
 *   out     : if non-NULL, dense output (n_out, n) at t[0], t[stride], ... up to
 *             t[ntimes-1] (xend); x starts at t[0]
 *   x0,xend : used instead of t[0], t[ntimes-1] when out is NULL and t is NULL
 *   uround  : gala passes np.finfo(float).eps from dop853_helper and 0 (the
 *             front-end default 2.3e-16) from dop853_step
 *   stats   : if non-NULL, {nfcn, nstep, naccpt, nrejct}
 * Returns gala's idid: 1 on success, -2 / -3 / -4 on failure. */
static int orc_dop853_core(rhs_t R, int n, double *y, const double *t, int64_t ntimes, double x0, double xend_in,
                           double h0, double atol, double rtol, int64_t nmax, double dt_max, int64_t nstiff,
                           double uround, int64_t out_stride, double *out, long *stats) {
    double x = t ? t[0] : x0;
    const double xend = t ? t[ntimes - 1] : xend_in;
    double h = h0;
    double hmax = dt_max;
    const double safe = 0.9, fac1 = 0.333, fac2 = 6.0, beta = 0.0;
    if (!nmax) nmax = 1000000;
    if (!nstiff) nstiff = 1000;
    else if (nstiff < 0) nstiff = nmax + 10;
    if (uround == 0.0) uround = 2.3E-16;
    if (hmax == 0.0) hmax = xend - x;

    double *work = (double *)malloc(sizeof(double) * (size_t)n * 19);
    double *yy1 = work, *k1 = work + n, *k2 = work + 2 * n, *k3 = work + 3 * n, *k4 = work + 4 * n;
    double *k5 = work + 5 * n, *k6 = work + 6 * n, *k7 = work + 7 * n, *k8 = work + 8 * n;
    double *k9 = work + 9 * n, *k10 = work + 10 * n;
    double *rc1 = work + 11 * n, *rc2 = work + 12 * n, *rc3 = work + 13 * n, *rc4 = work + 14 * n;
    double *rc5 = work + 15 * n, *rc6 = work + 16 * n, *rc7 = work + 17 * n, *rc8 = work + 18 * n;

    double facold = 1.0E-4;
    const double expo1 = 1.0 / 8.0 - beta * 0.2;
    const double facc1 = 1.0 / fac1, facc2 = 1.0 / fac2;
    const double posneg = sign_d(1.0, xend - x);
    const double atoli = atol, rtoli = rtol;
    int last = 0, reject = 0, iasti = 0, nonsti = 0, idid = 0;
    double hlamb = 0.0, xold = x, hout = 0.0;
    long nfcn = 0, nstep = 0, naccpt = 0, nrejct = 0;
    int64_t out_idx = 0; /* index into t of the next output time */
    int64_t out_slot = 0;

    R.fn(R.ctx, y, k1);
    hmax = fabs(hmax);
    const int iord = 8;
    if (h == 0.0) h = orc_hinit(R, n, x, y, posneg, k1, k2, k3, iord, hmax, atoli, rtoli);
    nfcn += 2;

    for (;;) {
        if (nstep > nmax) { idid = -2; break; }
        if (0.1 * fabs(h) <= fabs(x) * uround) { idid = -3; break; }
        if ((x + 1.01 * h - xend) * posneg > 0.0) {
            h = xend - x;
            last = 1;
        }
        xold = x;
        hout = h;
        nstep++;

        for (int i = 0; i < n; i++) yy1[i] = y[i] + h * a21 * k1[i];
        R.fn(R.ctx, yy1, k2);
        for (int i = 0; i < n; i++) yy1[i] = y[i] + h * (a31 * k1[i] + a32 * k2[i]);
        R.fn(R.ctx, yy1, k3);
        for (int i = 0; i < n; i++) yy1[i] = y[i] + h * (a41 * k1[i] + a43 * k3[i]);
        R.fn(R.ctx, yy1, k4);
        for (int i = 0; i < n; i++) yy1[i] = y[i] + h * (a51 * k1[i] + a53 * k3[i] + a54 * k4[i]);
        R.fn(R.ctx, yy1, k5);
        for (int i = 0; i < n; i++) yy1[i] = y[i] + h * (a61 * k1[i] + a64 * k4[i] + a65 * k5[i]);
        R.fn(R.ctx, yy1, k6);
        for (int i = 0; i < n; i++)
            yy1[i] = y[i] + h * (a71 * k1[i] + a74 * k4[i] + a75 * k5[i] + a76 * k6[i]);
        R.fn(R.ctx, yy1, k7);
        for (int i = 0; i < n; i++)
            yy1[i] = y[i] + h * (a81 * k1[i] + a84 * k4[i] + a85 * k5[i] + a86 * k6[i] + a87 * k7[i]);
        R.fn(R.ctx, yy1, k8);
        for (int i = 0; i < n; i++)
            yy1[i] = y[i] + h * (a91 * k1[i] + a94 * k4[i] + a95 * k5[i] + a96 * k6[i] + a97 * k7[i] +
                                 a98 * k8[i]);
        R.fn(R.ctx, yy1, k9);
        for (int i = 0; i < n; i++)
            yy1[i] = y[i] + h * (a101 * k1[i] + a104 * k4[i] + a105 * k5[i] + a106 * k6[i] +
                                 a107 * k7[i] + a108 * k8[i] + a109 * k9[i]);
        R.fn(R.ctx, yy1, k10);
        for (int i = 0; i < n; i++)
            yy1[i] = y[i] + h * (a111 * k1[i] + a114 * k4[i] + a115 * k5[i] + a116 * k6[i] +
                                 a117 * k7[i] + a118 * k8[i] + a119 * k9[i] + a1110 * k10[i]);
        R.fn(R.ctx, yy1, k2);
        const double xph = x + h;
        for (int i = 0; i < n; i++)
            yy1[i] = y[i] + h * (a121 * k1[i] + a124 * k4[i] + a125 * k5[i] + a126 * k6[i] +
                                 a127 * k7[i] + a128 * k8[i] + a129 * k9[i] + a1210 * k10[i] +
                                 a1211 * k2[i]);
        R.fn(R.ctx, yy1, k3);
        nfcn += 11;
        for (int i = 0; i < n; i++) {
            k4[i] = b1 * k1[i] + b6 * k6[i] + b7 * k7[i] + b8 * k8[i] + b9 * k9[i] + b10 * k10[i] +
                    b11 * k2[i] + b12 * k3[i];
            k5[i] = y[i] + h * k4[i];
        }

        /* error estimation, scalar tolerances (:416-444) */
        double err = 0.0, err2 = 0.0, sk, erri, sqr;
        for (int i = 0; i < n; i++) {
            sk = atoli + rtoli * max_d(fabs(y[i]), fabs(k5[i]));
            erri = k4[i] - bhh1 * k1[i] - bhh2 * k9[i] - bhh3 * k3[i];
            sqr = erri / sk;
            err2 += sqr * sqr;
            erri = er1 * k1[i] + er6 * k6[i] + er7 * k7[i] + er8 * k8[i] + er9 * k9[i] + er10 * k10[i] +
                   er11 * k2[i] + er12 * k3[i];
            sqr = erri / sk;
            err += sqr * sqr;
        }
        double deno = err + 0.01 * err2;
        if (deno <= 0.0) deno = 1.0;
        err = fabs(h) * err * sqrt(1.0 / (deno * (double)n));

        /* step-size factor (:446-452) */
        const double fac11 = pow(err, expo1);
        double fac = fac11 / pow(facold, beta);
        fac = max_d(facc2, min_d(facc1, fac / safe));
        double hnew = h / fac;

        if (err <= 1.0) {
            facold = max_d(err, 1.0E-4);
            naccpt++;
            R.fn(R.ctx, k5, k4);
            nfcn++;

            /* stiffness detection (:463-486); gala returns -4 on the first
             * detection because the `return -4` sits outside the iasti == 15 test */
            if (!(naccpt % nstiff) || (iasti > 0)) {
                double stnum = 0.0, stden = 0.0;
                for (int i = 0; i < n; i++) {
                    sqr = k4[i] - k3[i];
                    stnum += sqr * sqr;
                    sqr = k5[i] - yy1[i];
                    stden += sqr * sqr;
                }
                if (stden > 0.0) hlamb = h * sqrt(stnum / stden);
                if (hlamb > 6.1) {
                    nonsti = 0;
                    iasti++;
                    idid = -4;
                    break;
                } else {
                    nonsti++;
                    if (nonsti == 6) iasti = 0;
                }
            }

            if (out) {
                /* dense output coefficients (:492-582) */
                for (int i = 0; i < n; i++) {
                    rc1[i] = y[i];
                    const double ydiff = k5[i] - y[i];
                    rc2[i] = ydiff;
                    const double bspl = h * k1[i] - ydiff;
                    rc3[i] = bspl;
                    rc4[i] = ydiff - h * k4[i] - bspl;
                    rc5[i] = d41 * k1[i] + d46 * k6[i] + d47 * k7[i] + d48 * k8[i] + d49 * k9[i] +
                             d410 * k10[i] + d411 * k2[i] + d412 * k3[i];
                    rc6[i] = d51 * k1[i] + d56 * k6[i] + d57 * k7[i] + d58 * k8[i] + d59 * k9[i] +
                             d510 * k10[i] + d511 * k2[i] + d512 * k3[i];
                    rc7[i] = d61 * k1[i] + d66 * k6[i] + d67 * k7[i] + d68 * k8[i] + d69 * k9[i] +
                             d610 * k10[i] + d611 * k2[i] + d612 * k3[i];
                    rc8[i] = d71 * k1[i] + d76 * k6[i] + d77 * k7[i] + d78 * k8[i] + d79 * k9[i] +
                             d710 * k10[i] + d711 * k2[i] + d712 * k3[i];
                }
                for (int i = 0; i < n; i++)
                    yy1[i] = y[i] + h * (a141 * k1[i] + a147 * k7[i] + a148 * k8[i] + a149 * k9[i] +
                                         a1410 * k10[i] + a1411 * k2[i] + a1412 * k3[i] + a1413 * k4[i]);
                R.fn(R.ctx, yy1, k10);
                for (int i = 0; i < n; i++)
                    yy1[i] = y[i] + h * (a151 * k1[i] + a156 * k6[i] + a157 * k7[i] + a158 * k8[i] +
                                         a1511 * k2[i] + a1512 * k3[i] + a1513 * k4[i] + a1514 * k10[i]);
                R.fn(R.ctx, yy1, k2);
                for (int i = 0; i < n; i++)
                    yy1[i] = y[i] + h * (a161 * k1[i] + a166 * k6[i] + a167 * k7[i] + a168 * k8[i] +
                                         a169 * k9[i] + a1613 * k4[i] + a1614 * k10[i] + a1615 * k2[i]);
                R.fn(R.ctx, yy1, k3);
                nfcn += 3;
                for (int i = 0; i < n; i++) {
                    rc5[i] = h * (rc5[i] + d413 * k4[i] + d414 * k10[i] + d415 * k2[i] + d416 * k3[i]);
                    rc6[i] = h * (rc6[i] + d513 * k4[i] + d514 * k10[i] + d515 * k2[i] + d516 * k3[i]);
                    rc7[i] = h * (rc7[i] + d613 * k4[i] + d614 * k10[i] + d615 * k2[i] + d616 * k3[i]);
                    rc8[i] = h * (rc8[i] + d713 * k4[i] + d714 * k10[i] + d715 * k2[i] + d716 * k3[i]);
                }

                /* fill every output time inside [xold, xold + hout] (:584-612)
                 * with contd8_threadsafe (:869-904) */
                const double x0 = xold, x1 = x0 + hout;
                while (out_idx < ntimes) {
                    const double t_out = t[out_idx];
                    if ((x0 <= t_out && t_out <= x1) || (x1 <= t_out && t_out <= x0)) {
                        if (out_idx % out_stride == 0) {
                            const double s = (t_out - xold) / hout;
                            const double s1 = 1.0 - s;
                            double *o = out + (size_t)out_slot * (size_t)n;
                            for (int i = 0; i < n; i++)
                                o[i] = rc1[i] +
                                       s * (rc2[i] +
                                            s1 * (rc3[i] +
                                                  s * (rc4[i] + s1 * (rc5[i] + s * (rc6[i] + s1 * (rc7[i] + s * rc8[i]))))));
                            out_slot++;
                        }
                        out_idx++;
                    } else {
                        break;
                    }
                }
            }

            memcpy(k1, k4, (size_t)n * sizeof(double));
            memcpy(y, k5, (size_t)n * sizeof(double));
            x = xph;
            if (last) { idid = 1; break; }
            if (fabs(hnew) > hmax) hnew = posneg * hmax;
            if (reject) hnew = posneg * min_d(fabs(hnew), fabs(h));
            reject = 0;
        } else {
            hnew = h / min_d(facc1, fac11 / safe);
            reject = 1;
            if (naccpt >= 1) nrejct = nrejct + 1;
            last = 0;
        }
        h = hnew;
    }
    (void)nonsti;
    if (stats) {
        stats[0] = nfcn;
        stats[1] = nstep;
        stats[2] = naccpt;
        stats[3] = nrejct;
    }
    free(work);
    return idid;
}

/* dop853_helper's call of dop853() on one batch (dop853.pyx:157-182):
 * uround = np.finfo(float).eps, h0 = t[1] - t[0], dense output on t. */
int orc_dop853_batch(const gx_potential *pot, const gx_frame *fr, int nb, double *y,
                     const double *t, int64_t ntimes, double atol, double rtol, int64_t nmax,
                     double dt_max, int64_t nstiff, int64_t out_stride, double *out, long *stats) {
    batch_ctx c = {pot, fr, nb};
    rhs_t R = {batch_rhs_cb, &c};
    return orc_dop853_core(R, 6 * nb, y, t, ntimes, 0., 0., t[1] - t[0], atol, rtol, nmax, dt_max, nstiff,
                           2.220446049250313e-16, out_stride, out, stats);
}

typedef struct {
    const gx_potential *pot;
    const gx_frame *fr;
    const double *w0, *t;
    int64_t n, ntimes, nmax, nstiff, out_stride, n_out;
    double atol, rtol, dt_max;
    int save_all, nbatch;
    double *w_out;
    int32_t *status;
    long *stats; /* per batch {nfcn, nstep, naccpt, nrejct} or NULL */
} dop_ctx;

static void dop_chunk(void *vctx, int64_t blo, int64_t bhi) {
    dop_ctx *C = (dop_ctx *)vctx;
    const int64_t n = C->n;
    for (int64_t b = blo; b < bhi; b++) {
        const int64_t i0 = b * C->nbatch;
        const int nb = (int)((i0 + C->nbatch <= n) ? C->nbatch : n - i0);
        double *y = (double *)malloc(sizeof(double) * 6 * (size_t)nb);
        for (int k = 0; k < 6; k++)
            for (int j = 0; j < nb; j++) y[k * nb + j] = C->w0[k * n + i0 + j];
        double *out = NULL;
        if (C->save_all) out = (double *)malloc(sizeof(double) * 6 * (size_t)nb * (size_t)C->n_out);
        int res = orc_dop853_batch(C->pot, C->fr, nb, y, C->t, C->ntimes, C->atol, C->rtol, C->nmax,
                                   C->dt_max, C->nstiff, C->out_stride, out,
                                   C->stats ? C->stats + 4 * b : NULL);
        C->status[b] = res;
        if (C->save_all) {
            /* (n_out, 6, nb) -> (6, n_out, N) (dop853.pyx:187-193, 242-243) */
            for (int64_t s = 0; s < C->n_out; s++)
                for (int k = 0; k < 6; k++)
                    for (int j = 0; j < nb; j++)
                        C->w_out[(k * C->n_out + s) * n + i0 + j] = out[(s * 6 + k) * nb + j];
            free(out);
        } else {
            for (int k = 0; k < 6; k++)
                for (int j = 0; j < nb; j++) C->w_out[k * n + i0 + j] = y[k * nb + j];
        }
        free(y);
    }
}

/* dop853_integrate_hamiltonian (dop853.pyx:196-250): batches of nbatch orbits,
 * one dop853() call each; batches are spread over nthreads. */
int orc_dop853_integrate(const gx_potential *pot, const gx_frame *fr, const double *w0, int64_t n,
                         const double *t, int64_t ntimes, double atol, double rtol, int64_t nmax,
                         double dt_max, int64_t nstiff, int save_all, int nbatch, int64_t out_stride,
                         double *w_out, int32_t *status, long *stats, int nthreads) {
    if (ntimes < 2 || nbatch < 1 || out_stride < 1) return -1;
    dop_ctx C;
    C.pot = pot;
    C.fr = fr;
    C.w0 = w0;
    C.t = t;
    C.n = n;
    C.ntimes = ntimes;
    C.nmax = nmax;
    C.nstiff = nstiff;
    C.out_stride = out_stride;
    C.n_out = (ntimes - 1) / out_stride + 1;
    C.atol = atol;
    C.rtol = rtol;
    C.dt_max = dt_max;
    C.save_all = save_all;
    C.nbatch = nbatch;
    C.w_out = w_out;
    C.status = status;
    C.stats = stats;
    const int64_t nbatches = (n + nbatch - 1) / nbatch;
    parallel_for(nthreads, nbatches, 1, dop_chunk, &C);
    return 0;
}

/* Batched potential evaluation helpers for the tests: q (3, N) SoA. */
void orc_potential_value_n(const gx_potential *pot, double t, const double *q, int64_t N, double *out) {
    for (int64_t i = 0; i < N; i++) {
        double qi[3] = {q[i], q[N + i], q[2 * N + i]};
        out[i] = orc_potential(pot, t, qi);
    }
}

void orc_potential_density_n(const gx_potential *pot, double t, const double *q, int64_t N, double *out) {
    for (int64_t i = 0; i < N; i++) {
        double qi[3] = {q[i], q[N + i], q[2 * N + i]};
        out[i] = orc_density(pot, t, qi);
    }
}

void orc_hamiltonian_value_n(const gx_potential *pot, const gx_frame *fr, double t, const double *w,
                             int64_t N, double *out) {
    for (int64_t i = 0; i < N; i++) {
        double wi[6];
        for (int k = 0; k < 6; k++) wi[k] = w[k * N + i];
        out[i] = orc_hamiltonian_value(pot, fr, t, wi);
    }
}

/* ------------------------------------------------------------------------- */
/* Direct n-body systems and mock streams                                    */
/* (dop853.cpp:990-1006, cpotential.cpp:346-415, nbody.pyx:30-115,           */
/*  mockstream.pyx:176-303, dop853.pyx:27-75)                                */
/* ------------------------------------------------------------------------- */

/* Gradient of a body's potential, shifted to the body's position q0: the
 * body's CPotential with do_shift_rotate = 1 and q0 pointing at the body
 * (cpotential.cpp:402-405), R the identity, evaluated by c_gradient (:214-287). */
static void body_gradient(const gx_body *b, const double *q0, const double *q, double *g) {
    gx_component c;
    memset(&c, 0, sizeof(c));
    c.type = b->type;
    c.n_params = b->n_params;
    c.param_offset = 0;
    c.do_shift_rotate = 1;
    for (int k = 0; k < 3; k++) c.q0[k] = q0[k];
    c.R[0] = c.R[4] = c.R[8] = 1.;
    gx_potential bp;
    memset(&bp, 0, sizeof(bp));
    bp.n_components = 1;
    bp.n_dim = 3;
    bp.components = &c;
    bp.params = b->params;
    gradient_point(&bp, q, g);
}

typedef struct {
    const gx_potential *pot;
    const gx_frame *fr;
    int norbits, nbody;
    const gx_body *bodies; /* nbody entries */
} nbody_ctx;

/* Fwrapper_direct_nbody (dop853.cpp:990-1006): hamiltonian_gradient for every
 * body of the AoS state y[6 * norbits], then c_nbody_acceleration
 * (cpotential.cpp:389-415): every non-null massive body j pulls every other
 * body i, acc[6 i + 3 + k] += -f2[k]. */
static void nbody_rhs_cb(const void *vctx, const double *y, double *f) {
    const nbody_ctx *C = (const nbody_ctx *)vctx;
    for (int i = 0; i < C->norbits; i++) rhs_point(C->pot, C->fr, y + 6 * i, f + 6 * i);
    for (int j = 0; j < C->nbody; j++) {
        const gx_body *b = &C->bodies[j];
        if (b->type == GX_POT_NULL) continue;
        for (int i = 0; i < C->norbits; i++) {
            if (i == j) continue;
            double f2[3];
            body_gradient(b, y + 6 * j, y + 6 * i, f2);
            for (int k = 0; k < 3; k++) f[6 * i + 3 + k] += -f2[k];
        }
    }
}

/* direct_nbody_dop853 (nbody.pyx:30-115) -> dop853_helper (dop853.pyx:90-193)
 * on one system of nparticles bodies, the first nbody of them massive:
 * w0 (nparticles, 6); w_out (ntimes, nparticles, 6) if save_all else
 * (nparticles, 6).  uround = eps, h0 = t[1] - t[0], nstiff as given (gala
 * passes -1). */
int orc_nbody_dop853(const gx_potential *pot, const gx_frame *fr, int nparticles, int nbody,
                     const gx_body *bodies, const double *w0, const double *t, int64_t ntimes,
                     double atol, double rtol, int64_t nmax, double dt_max, int64_t nstiff,
                     int save_all, double *w_out, long *stats) {
    if (ntimes < 2 || nparticles < 1 || nbody < 0 || nbody > nparticles) return -1;
    nbody_ctx C = {pot, fr, nparticles, nbody, bodies};
    rhs_t R = {nbody_rhs_cb, &C};
    const int n = 6 * nparticles;
    double *y = (double *)malloc(sizeof(double) * (size_t)n);
    memcpy(y, w0, sizeof(double) * (size_t)n);
    int res = orc_dop853_core(R, n, y, t, ntimes, 0., 0., t[1] - t[0], atol, rtol, nmax, dt_max, nstiff,
                              2.220446049250313e-16, 1, save_all ? w_out : NULL, stats);
    if (!save_all) memcpy(w_out, y, sizeof(double) * (size_t)n);
    free(y);
    return res;
}

/* dop853_step (dop853.pyx:27-75) on one release system: the state w
 * (nsys, 6) from t1 to t2 with h0 = dt0, uround 0 (-> 2.3e-16), hmax 0,
 * nstiff 1 (the literal in dop853_step, whatever the caller passes), no output. */
static int orc_dop853_step_system(const gx_potential *pot, const gx_frame *fr, int nsys, int nbody,
                                  const gx_body *bodies, double *w, double t1, double t2, double dt0,
                                  double atol, double rtol, int64_t nmax, long *stats) {
    nbody_ctx C = {pot, fr, nsys, nbody, bodies};
    rhs_t R = {nbody_rhs_cb, &C};
    return orc_dop853_core(R, 6 * nsys, w, NULL, 0, t1, t2, dt0, atol, rtol, nmax, 0.0, 1, 0.0, 1, NULL,
                           stats);
}

/* mockstream_dop853 (mockstream.pyx:176-303) for one progenitor system:
 *   nbody_w0  (nbodies, 6)   massive bodies (progenitor first) at time[0]
 *   time      (ntimes)       release-time grid; dt0 = time[1] - time[0]
 *   stream_w0 (ntot, 6)      released particles, grouped by release time
 *   stream_t1 (ntimes), nstream (ntimes)
 * First the bodies are integrated over `time` with dense output (dop853_helper,
 * nstiff as given), then every release i with nstream[i] > 0 integrates
 * [bodies at time[i], its particles] from stream_t1[i] to tfinal.
 * Outputs: nbody_w_final (nbodies, 6) = the bodies after the last release
 * system, stream_w_final (ntot, 6), status (ntimes): gala's idid per release,
 * 0 where nothing was released. */
int orc_mockstream_dop853(const gx_potential *pot, const gx_frame *fr, int nbodies, const gx_body *bodies,
                          const double *nbody_w0, const double *time, int64_t ntimes, const double *stream_w0,
                          const double *stream_t1, double tfinal, const int32_t *nstream, double atol,
                          double rtol, int64_t nmax, double dt_max, int64_t nstiff, double *nbody_w_final,
                          double *stream_w_final, int32_t *status) {
    if (ntimes < 2 || nbodies < 1) return -1;
    int maxn = 0;
    for (int64_t i = 0; i < ntimes; i++) maxn = nstream[i] > maxn ? nstream[i] : maxn;
    double *nbody_w = (double *)malloc(sizeof(double) * (size_t)ntimes * 6 * (size_t)nbodies);
    int res = orc_nbody_dop853(pot, fr, nbodies, nbodies, bodies, nbody_w0, time, ntimes, atol, rtol, nmax,
                               dt_max, nstiff, 1, nbody_w, NULL);
    if (res < 0) {
        free(nbody_w);
        return res;
    }
    const double dt0 = time[1] - time[0];
    double *w_tmp = (double *)malloc(sizeof(double) * 6 * (size_t)(nbodies + maxn));
    int64_t n = 0;
    for (int64_t i = 0; i < ntimes; i++) {
        status[i] = 0;
        if (nstream[i] == 0) continue;
        memcpy(w_tmp, nbody_w + (size_t)i * 6 * (size_t)nbodies, sizeof(double) * 6 * (size_t)nbodies);
        memcpy(w_tmp + 6 * nbodies, stream_w0 + 6 * n, sizeof(double) * 6 * (size_t)nstream[i]);
        status[i] = orc_dop853_step_system(pot, fr, nbodies + nstream[i], nbodies, bodies, w_tmp, stream_t1[i],
                                           tfinal, dt0, atol, rtol, nmax, NULL);
        memcpy(stream_w_final + 6 * n, w_tmp + 6 * nbodies, sizeof(double) * 6 * (size_t)nstream[i]);
        memcpy(nbody_w_final, w_tmp, sizeof(double) * 6 * (size_t)nbodies);
        n += nstream[i];
    }
    free(w_tmp);
    free(nbody_w);
    return 0;
}

/* mockstream_dop853_animate (mockstream.pyx:306-440) for one progenitor system:
 *   nbody_w0  (nbodies, 6)  the bodies at t[0]
 *   t         (ntimes)      the whole orbit grid; h0 = t[1] - t[0]
 *   stream_w0 (ntot, 6)     released particles in release order
 *   nstream   (ntimes)      particles released at t[i] (zeros allowed)
 * The state holds every body and particle from the start; interval i
 * (t[i-1] -> t[i]) steps the first nbodies + n of them as one dop853_step
 * system (nstiff 1), n being the particles released at t[0..i-1], and
 * n += nstream[i] follows the interval (:402-411).  Snapshots (:393-421):
 *   snap   (noutput, nbodies + ntot, 6)  the state at t[0] and after every
 *          interval i with i % output_every == 0 or i == ntimes - 1; members
 *          not yet released are NaN (the HDF5 datasets' fill value)
 *   snap_t (noutput)
 * w_final (nbodies + ntot, 6) is the last state, status (ntimes) the idid of
 * every interval (status[0] = 1), stats (4) the summed counters or NULL.
 * Returns the number of snapshots, or -1 on bad arguments. */
static void anim_snapshot(double *dst, const double *w, int64_t live, int64_t all) {
    for (int64_t k = 0; k < 6 * all; k++) dst[k] = (k < 6 * live) ? w[k] : NAN;
}

int orc_mockstream_dop853_animate(const gx_potential *pot, const gx_frame *fr, int nbodies, const gx_body *bodies,
                                  const double *nbody_w0, const double *t, int64_t ntimes, const double *stream_w0,
                                  const int32_t *nstream, int64_t output_every, double atol, double rtol,
                                  int64_t nmax, double *snap, double *snap_t, double *w_final, int32_t *status,
                                  long *stats) {
    if (ntimes < 2 || nbodies < 1 || output_every < 1) return -1;
    int64_t ntot = 0;
    for (int64_t i = 0; i < ntimes; i++) {
        if (nstream[i] < 0) return -1;
        ntot += nstream[i];
    }
    const int64_t all = nbodies + ntot;
    double *w = w_final;
    memcpy(w, nbody_w0, sizeof(double) * 6 * (size_t)nbodies);
    memcpy(w + 6 * nbodies, stream_w0, sizeof(double) * 6 * (size_t)ntot);
    const double dt0 = t[1] - t[0];
    int64_t n = nstream[0], j = 0;
    anim_snapshot(snap, w, nbodies + n, all);
    snap_t[j++] = t[0];
    status[0] = 1;
    if (stats)
        for (int k = 0; k < 4; k++) stats[k] = 0;
    for (int64_t i = 1; i < ntimes; i++) {
        long st[4] = {0, 0, 0, 0};
        status[i] = orc_dop853_step_system(pot, fr, (int)(nbodies + n), nbodies, bodies, w, t[i - 1], t[i], dt0,
                                           atol, rtol, nmax, st);
        if (stats)
            for (int k = 0; k < 4; k++) stats[k] += st[k];
        n += nstream[i];
        if (i % output_every == 0 || i == ntimes - 1) {
            anim_snapshot(snap + (size_t)j * 6 * (size_t)all, w, nbodies + n, all);
            snap_t[j++] = t[i];
        }
    }
    return (int)j;
}

/* Release systems of many independent streams that share one release grid,
 * the layout of the GPU library's mock-stream entry point:
 *   bodies    (n_streams, nbodies)
 *   nbody_w   (n_streams, n_release, nbodies, 6)  bodies at each release time
 *   stream_w0 (n_streams, ntot, 6), particles of release i at offset
 *             sum(nstream[:i])
 * System id = i * n_streams + s; systems [sys_lo, sys_hi) are integrated
 * (release systems with nstream[i] == 0 are skipped, status 0).
 * stats (n_streams * n_release, 4) may be NULL. */
typedef struct {
    const gx_potential *pot;
    const gx_frame *fr;
    int64_t n_streams, n_release, ntot;
    int nbodies;
    const gx_body *bodies;
    const double *nbody_w, *release_t, *stream_w0;
    const int32_t *nstream;
    const int64_t *offset;
    double t_final, dt0, atol, rtol;
    int64_t nmax;
    double *stream_w_out, *nbody_w_out;
    int32_t *status;
    long *stats;
    int64_t last_release;
    int64_t sys_base; /* ranges handed to ms_chunk are relative to this id */
} ms_ctx;

static void ms_chunk(void *vctx, int64_t lo, int64_t hi) {
    const ms_ctx *C = (const ms_ctx *)vctx;
    int maxn = 0;
    for (int64_t i = 0; i < C->n_release; i++) maxn = C->nstream[i] > maxn ? C->nstream[i] : maxn;
    const int nb = C->nbodies;
    double *w = (double *)malloc(sizeof(double) * 6 * (size_t)(nb + maxn));
    for (int64_t sys = C->sys_base + lo; sys < C->sys_base + hi; sys++) {
        const int64_t i = sys / C->n_streams, s = sys % C->n_streams;
        const int np = C->nstream[i];
        if (np == 0) {
            C->status[s * C->n_release + i] = 0;
            continue;
        }
        memcpy(w, C->nbody_w + ((size_t)(s * C->n_release + i)) * 6 * (size_t)nb, sizeof(double) * 6 * (size_t)nb);
        memcpy(w + 6 * nb, C->stream_w0 + ((size_t)(s * C->ntot + C->offset[i])) * 6, sizeof(double) * 6 * (size_t)np);
        long st[4];
        C->status[s * C->n_release + i] = orc_dop853_step_system(C->pot, C->fr, nb + np, nb, C->bodies + s * nb, w,
                                                                 C->release_t[i], C->t_final, C->dt0, C->atol,
                                                                 C->rtol, C->nmax, st);
        if (C->stats)
            for (int k = 0; k < 4; k++) C->stats[(s * C->n_release + i) * 4 + k] = st[k];
        memcpy(C->stream_w_out + ((size_t)(s * C->ntot + C->offset[i])) * 6, w + 6 * nb, sizeof(double) * 6 * (size_t)np);
        if (i == C->last_release && C->nbody_w_out)
            memcpy(C->nbody_w_out + (size_t)s * 6 * (size_t)nb, w, sizeof(double) * 6 * (size_t)nb);
    }
    free(w);
}

int orc_mockstream_systems(const gx_potential *pot, const gx_frame *fr, int64_t n_streams, int nbodies,
                           const gx_body *bodies, const double *nbody_w, int64_t n_release, const double *release_t,
                           const int32_t *nstream, const double *stream_w0, double t_final, double dt0, double atol,
                           double rtol, int64_t nmax, double *stream_w_out, double *nbody_w_out, int32_t *status,
                           long *stats, int64_t sys_lo, int64_t sys_hi, int nthreads) {
    if (n_streams < 1 || n_release < 1 || nbodies < 1) return -1;
    int64_t *offset = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n_release + 1));
    offset[0] = 0;
    int64_t last = -1;
    for (int64_t i = 0; i < n_release; i++) {
        offset[i + 1] = offset[i] + nstream[i];
        if (nstream[i] > 0) last = i;
    }
    if (sys_hi > n_streams * n_release) sys_hi = n_streams * n_release;
    ms_ctx C = {pot, fr, n_streams, n_release, offset[n_release], nbodies, bodies, nbody_w, release_t, stream_w0,
                nstream, offset, t_final, dt0, atol, rtol, nmax, stream_w_out, nbody_w_out, status, stats, last,
                sys_lo};
    if (sys_lo < sys_hi) parallel_for(nthreads, sys_hi - sys_lo, 16, ms_chunk, &C);
    free(offset);
    return 0;
}

/* c_d2_dr2 (cpotential.cpp:346-371): second radial difference of Phi with the
 * fixed step h = 1e-2, at N points q (N, 3). */
void orc_d2_dr2_n(const gx_potential *pot, double t, const double *q, int64_t N, double *out) {
    for (int64_t n = 0; n < N; n++) {
        const double *qp = q + 3 * n;
        double eps[3], r2 = 0;
        for (int j = 0; j < 3; j++) r2 = r2 + qp[j] * qp[j];
        const double h = 1E-2;
        const double r = sqrt(r2);
        for (int j = 0; j < 3; j++) eps[j] = qp[j] + h * qp[j] / r;
        double d2 = orc_potential(pot, t, eps);
        d2 = d2 - 2. * orc_potential(pot, t, qp);
        for (int j = 0; j < 3; j++) eps[j] = qp[j] - h * qp[j] / r;
        d2 = d2 + orc_potential(pot, t, eps);
        out[n] = d2 / (h * h);
    }
}

/* FardalStreamDF._sample (df.pyx:363-457) for one progenitor orbit, with
 * get_rj_vj_R (:61-92), transform_from_sat (:94-106) and _coord.pyx's cross /
 * norm / apply_3matrix.  Same layout as the GPU sampler:
 *   prog_w (ntimes, row_stride) x, v first; prog_m (ntimes); t (ntimes)
 *   offset (ntimes + 1) first particle row per time (trailing rows first)
 *   draws (n_particles, 4) the normal draws kx, kz, kvt, kvz
 *   w_out (n_particles, 6) */
void orc_stream_sample(const gx_potential *pot, int64_t ntimes, const double *prog_w, int64_t row_stride,
                       const double *prog_m, const double *t, const int64_t *offset, int kind, int ndraw,
                       const double *draws, double G, int lead, int trail, int gala_modified, double *w_out);

void orc_fardal_sample(const gx_potential *pot, int64_t ntimes, const double *prog_w, int64_t row_stride,
                       const double *prog_m, const double *t, const int64_t *offset, const double *draws, double G,
                       int lead, int trail, int gala_modified, double *w_out) {
    orc_stream_sample(pot, ntimes, prog_w, row_stride, prog_m, t, offset, 0, 4, draws, G, lead, trail, gala_modified,
                      w_out);
}

/* Release placement of the stream DFs in the satellite frame, per particle.
 * kind 0, FardalStreamDF (df.pyx:410-450): draws kx, kz, kvt, kvz;
 * kind 1, LagrangeCloudStreamDF (df.pyx:515-552): position (+-rj, 0, 0), velocity
 *   the three draws (normal(0, v_disp) each, drawn by the caller);
 * kind 2, ChenStreamDF (df.pyx:614-700): the six draws of multivariate_normal
 *   (r, phi, theta, v, alpha, beta; degrees), Dr = r rj, Dv = v sqrt(2 G m / Dr),
 *   the leading tail adds pi to phi and alpha. */
static void orc_release_offsets(int kind, int gala_modified, const double *d, int lead_tail, double rj, double vj,
                                double G, double m, double *tx, double *tv) {
    const double sr = lead_tail == 0 ? rj : -rj, sv = lead_tail == 0 ? vj : -vj;
    tx[0] = tx[1] = tx[2] = 0.;
    tv[0] = tv[1] = tv[2] = 0.;
    if (kind == 0) {
        const double kx = d[0];
        tx[0] = kx * sr;
        tx[2] = d[1] * sr;
        tv[1] = d[2] * sv;
        if (gala_modified) tv[1] *= kx;
        tv[2] = d[3] * sv;
    } else if (kind == 1) {
        tx[0] = sr;
        tv[0] = d[0];
        tv[1] = d[1];
        tv[2] = d[2];
    } else {
        const double pi = 3.14159265358979323846;
        const double Dr = d[0] * rj;
        const double Dv = d[3] * sqrt(2 * G * m / Dr);
        double p1 = d[1] * (pi / 180), p2 = d[2] * (pi / 180), p4 = d[4] * (pi / 180), p5 = d[5] * (pi / 180);
        if (lead_tail == 1) {
            p1 = p1 + pi;
            p4 = p4 + pi;
        }
        tx[0] = Dr * cos(p2) * cos(p1);
        tx[1] = Dr * cos(p2) * sin(p1);
        tx[2] = Dr * sin(p2);
        tv[0] = Dv * cos(p5) * cos(p4);
        tv[1] = Dv * cos(p5) * sin(p4);
        tv[2] = Dv * sin(p5);
    }
}

void orc_stream_sample(const gx_potential *pot, int64_t ntimes, const double *prog_w, int64_t row_stride,
                       const double *prog_m, const double *t, const int64_t *offset, int kind, int ndraw,
                       const double *draws, double G, int lead, int trail, int gala_modified, double *w_out) {
    const int ntail = lead + trail;
    for (int64_t i = 0; i < ntimes; i++) {
        const int64_t o0 = offset[i], o1 = offset[i + 1];
        if (o1 == o0 || ntail == 0) continue;
        const int64_t np_ = (o1 - o0) / ntail;
        const double *px = prog_w + i * row_stride, *pv = px + 3;
        const double m = prog_m[i];
        double dist = 0.;
        for (int k = 0; k < 3; k++) dist += px[k] * px[k];
        dist = sqrt(dist);
        double L[3];
        L[0] = px[1] * pv[2] - px[2] * pv[1];
        L[1] = -px[0] * pv[2] + px[2] * pv[0];
        L[2] = px[0] * pv[1] - px[1] * pv[0];
        double Lnorm = 0.;
        for (int k = 0; k < 3; k++) Lnorm += L[k] * L[k];
        Lnorm = sqrt(Lnorm);
        double R[3][3];
        for (int k = 0; k < 3; k++) {
            R[0][k] = px[k] / dist;
            R[2][k] = L[k] / Lnorm;
        }
        const double Om = Lnorm / (dist * dist);
        double d2r;
        orc_d2_dr2_n(pot, t[i], px, 1, &d2r);
        const double rj = pow(G * m / (Om * Om - d2r), 1 / 3.);
        const double vj = Om * rj;
        R[1][0] = R[0][1] * R[2][2] - R[0][2] * R[2][1];
        R[1][1] = -R[0][0] * R[2][2] + R[0][2] * R[2][0];
        R[1][2] = R[0][0] * R[2][1] - R[0][1] * R[2][0];
        for (int k = 0; k < 3; k++) R[1][k] = -R[1][k];
        int64_t row = o0;
        for (int tail = 0; tail < 2; tail++) {
            if (tail == 0 && !trail) continue;
            if (tail == 1 && !lead) continue;
            for (int64_t k = 0; k < np_; k++, row++) {
                double tx[3], tv[3];
                orc_release_offsets(kind, gala_modified, draws + row * ndraw, tail, rj, vj, G, m, tx, tv);
                double *o = w_out + row * 6;
                for (int n = 0; n < 3; n++) {
                    o[n] = R[0][n] * tx[0] + R[1][n] * tx[1] + R[2][n] * tx[2];
                    o[3 + n] = R[0][n] * tv[0] + R[1][n] * tv[1] + R[2][n] * tv[2];
                }
                for (int n = 0; n < 3; n++) {
                    o[n] += px[n];
                    o[3 + n] += pv[n];
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Leapfrog n-body and mock streams (leapfrog.pyx:126-255,                   */
/* cpotential.cpp:418-442, mockstream.pyx:442-610)                           */
/* ------------------------------------------------------------------------- */

/* c_nbody_gradient_symplectic (cpotential.cpp:418-442): grad += the gradient of
 * every non-null massive body j != self, shifted to body j's current position
 * x_nbody[6 j]. */
static void nbody_gradient_symplectic(const gx_body *bodies, int nbody, int self, const double *x_nbody,
                                      const double *x, double *grad) {
    for (int j = 0; j < nbody; j++) {
        if (bodies[j].type == GX_POT_NULL || j == self) continue;
        double f2[3];
        body_gradient(&bodies[j], x_nbody + 6 * j, x, f2);
        for (int k = 0; k < 3; k++) grad[k] += f2[k];
    }
}

/* c_init_velocity_nbody (leapfrog.pyx:126-138) for body i of the AoS state w. */
static void lf_init_nbody(const gx_potential *pot, const gx_body *bodies, int nbody, double *w, int i, double dt,
                          double *v_half) {
    double grad[3];
    gradient_point(pot, w + 6 * i, grad);
    nbody_gradient_symplectic(bodies, nbody, i, w, w + 6 * i, grad);
    for (int k = 0; k < 3; k++) v_half[3 * i + k] = w[6 * i + 3 + k] - grad[k] * dt / 2.;
}

/* c_leapfrog_step_nbody (leapfrog.pyx:140-158) for body i: drift, gradient with
 * the other bodies' CURRENT positions, kick. */
static void lf_step_nbody(const gx_potential *pot, const gx_body *bodies, int nbody, double *w, int i, double dt,
                          double *v_half) {
    double *x = w + 6 * i, *v = x + 3, *vh = v_half + 3 * i;
    for (int k = 0; k < 3; k++) x[k] = x[k] + vh[k] * dt;
    double grad[3];
    gradient_point(pot, x, grad);
    nbody_gradient_symplectic(bodies, nbody, i, w, x, grad);
    for (int k = 0; k < 3; k++) {
        v[k] = vh[k] - grad[k] * dt / 2.;
        vh[k] = vh[k] - grad[k] * dt;
    }
}

/* leapfrog_integrate_nbody (leapfrog.pyx:161-255) on one system of n bodies,
 * the first nbody massive: w0 (n, 6); w_out (ntimes, n, 6) if save_all else (n, 6). */
int orc_leapfrog_nbody(const gx_potential *pot, int n, int nbody, const gx_body *bodies, const double *w0,
                       const double *t, int64_t ntimes, int save_all, double *w_out) {
    if (ntimes < 2 || n < 1 || nbody < 0 || nbody > n) return -1;
    const double dt = t[1] - t[0];
    double *w = (double *)malloc(sizeof(double) * 6 * (size_t)n);
    double *vh = (double *)calloc(3 * (size_t)n, sizeof(double));
    memcpy(w, w0, sizeof(double) * 6 * (size_t)n);
    if (save_all) memcpy(w_out, w0, sizeof(double) * 6 * (size_t)n);
    for (int i = 0; i < n; i++) lf_init_nbody(pot, bodies, nbody, w, i, dt, vh);
    for (int64_t j = 1; j < ntimes; j++) {
        for (int i = 0; i < n; i++) lf_step_nbody(pot, bodies, nbody, w, i, dt, vh);
        if (save_all) memcpy(w_out + (size_t)j * 6 * (size_t)n, w, sizeof(double) * 6 * (size_t)n);
    }
    if (!save_all) memcpy(w_out, w, sizeof(double) * 6 * (size_t)n);
    free(w);
    free(vh);
    return 0;
}

/* The release systems of mockstream_leapfrog (mockstream.pyx:548-593) for many
 * streams sharing one release grid, the layout of orc_mockstream_systems:
 * nbody_w (S, n_release, nb, 6) bodies at each release time; each system takes
 * n_steps = (int)((t_final - release_t[i]) / dt + 0.5) steps of dt. */
typedef struct {
    const gx_potential *pot;
    int64_t n_streams, n_release, ntot;
    int nbodies;
    const gx_body *bodies;
    const double *nbody_w, *release_t, *stream_w0;
    const int32_t *nstream;
    const int64_t *offset;
    double t_final, dt;
    double *stream_w_out, *nbody_w_out;
    int64_t last_release, sys_base;
} mslf_ctx;

static void mslf_chunk(void *vctx, int64_t lo, int64_t hi) {
    const mslf_ctx *C = (const mslf_ctx *)vctx;
    int maxn = 0;
    for (int64_t i = 0; i < C->n_release; i++) maxn = C->nstream[i] > maxn ? C->nstream[i] : maxn;
    const int nb = C->nbodies;
    double *w = (double *)malloc(sizeof(double) * 6 * (size_t)(nb + maxn));
    double *vh = (double *)malloc(sizeof(double) * 3 * (size_t)(nb + maxn));
    for (int64_t sys = C->sys_base + lo; sys < C->sys_base + hi; sys++) {
        const int64_t i = sys / C->n_streams, s = sys % C->n_streams;
        const int np = C->nstream[i];
        if (np == 0) continue;
        const int nsys = nb + np;
        const gx_body *bod = C->bodies + s * nb;
        memcpy(w, C->nbody_w + ((size_t)(s * C->n_release + i)) * 6 * (size_t)nb, sizeof(double) * 6 * (size_t)nb);
        memcpy(w + 6 * nb, C->stream_w0 + ((size_t)(s * C->ntot + C->offset[i])) * 6, sizeof(double) * 6 * (size_t)np);
        for (int j = 0; j < nsys; j++) lf_init_nbody(C->pot, bod, nb, w, j, C->dt, vh);
        const int n_steps = (int)((C->t_final - C->release_t[i]) / C->dt + 0.5);
        for (int j = 0; j < n_steps; j++)
            for (int k = 0; k < nsys; k++) lf_step_nbody(C->pot, bod, nb, w, k, C->dt, vh);
        memcpy(C->stream_w_out + ((size_t)(s * C->ntot + C->offset[i])) * 6, w + 6 * nb, sizeof(double) * 6 * (size_t)np);
        if (i == C->last_release && C->nbody_w_out)
            memcpy(C->nbody_w_out + (size_t)s * 6 * (size_t)nb, w, sizeof(double) * 6 * (size_t)nb);
    }
    free(w);
    free(vh);
}

int orc_mockstream_leapfrog_systems(const gx_potential *pot, int64_t n_streams, int nbodies, const gx_body *bodies,
                                    const double *nbody_w, int64_t n_release, const double *release_t,
                                    const int32_t *nstream, const double *stream_w0, double t_final, double dt,
                                    double *stream_w_out, double *nbody_w_out, int64_t sys_lo, int64_t sys_hi,
                                    int nthreads) {
    if (n_streams < 1 || n_release < 1 || nbodies < 1 || dt == 0.0) return -1;
    int64_t *offset = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n_release + 1));
    offset[0] = 0;
    int64_t last = -1;
    for (int64_t i = 0; i < n_release; i++) {
        offset[i + 1] = offset[i] + nstream[i];
        if (nstream[i] > 0) last = i;
    }
    if (sys_hi > n_streams * n_release) sys_hi = n_streams * n_release;
    mslf_ctx C = {pot, n_streams, n_release, offset[n_release], nbodies, bodies, nbody_w, release_t, stream_w0,
                  nstream, offset, t_final, dt, stream_w_out, nbody_w_out, last, sys_lo};
    if (sys_lo < sys_hi) parallel_for(nthreads, sys_hi - sys_lo, 16, mslf_chunk, &C);
    free(offset);
    return 0;
}

/* mockstream_leapfrog (mockstream.pyx:442-610) for one progenitor system:
 * the bodies are integrated over full_time (leapfrog_integrate_nbody), taken at
 * each spawn time by index (int)((stream_t1[i] - full_time[0]) / dt + 0.5),
 * then every release system is integrated to tfinal. */
int orc_mockstream_leapfrog(const gx_potential *pot, int nbodies, const gx_body *bodies, const double *nbody_w0,
                            const double *full_time, int64_t nfull, const double *stream_w0, const double *stream_t1,
                            int64_t ntimes, double tfinal, const int32_t *nstream, double *nbody_w_final,
                            double *stream_w_final) {
    if (nfull < 2 || nbodies < 1) return -1;
    const double dt = full_time[1] - full_time[0];
    double *traj = (double *)malloc(sizeof(double) * (size_t)nfull * 6 * (size_t)nbodies);
    orc_leapfrog_nbody(pot, nbodies, nbodies, bodies, nbody_w0, full_time, nfull, 1, traj);
    double *nbody_w = (double *)malloc(sizeof(double) * (size_t)ntimes * 6 * (size_t)nbodies);
    for (int64_t i = 0; i < ntimes; i++) {
        const int idx = (int)((stream_t1[i] - full_time[0]) / dt + 0.5);
        memcpy(nbody_w + (size_t)i * 6 * (size_t)nbodies, traj + (size_t)idx * 6 * (size_t)nbodies,
               sizeof(double) * 6 * (size_t)nbodies);
    }
    int64_t total = 0;
    for (int64_t i = 0; i < ntimes; i++) total += nstream[i];
    double *nb_out = (double *)malloc(sizeof(double) * 6 * (size_t)nbodies);
    int rc = orc_mockstream_leapfrog_systems(pot, 1, nbodies, bodies, nbody_w, ntimes, stream_t1, nstream, stream_w0,
                                             tfinal, dt, stream_w_final, nb_out, 0, ntimes, 1);
    memcpy(nbody_w_final, nb_out, sizeof(double) * 6 * (size_t)nbodies);
    (void)total;
    free(nb_out);
    free(nbody_w);
    free(traj);
    return rc;
}
