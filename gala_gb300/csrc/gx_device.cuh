// gx_device.cuh -- device-side potential, frame and Hamiltonian evaluation.
//
// Every evaluation function is instantiated twice: SCF = false for potentials
// made only of closed-form components (all state stays in registers) and
// SCF = true when an SCF component is present (the SCF series is an
// out-of-line call, which forces the caller's small arrays into local memory).
//
// The potential is handed to every kernel BY VALUE (DevPot below, a few KB of
// kernel parameters that sit in the constant bank): component type tags,
// shift/rotate data and up to GX_MAX_INLINE_PARAMS packed parameters.  Large
// parameter blocks (SCF coefficients) stay in global memory behind `pdev`.
//
// Every FP64 expression below keeps gala's evaluation order (the cited
// *_gradient_single / *_value functions of
// src/gala/potential/potential/builtin/builtin_potentials.cpp); the FP64
// translation units are compiled with -fmad=false so that no multiply-add is
// contracted, which makes the results operation-for-operation those of gala's
// C code built without contraction.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gala_gb300.h"

namespace gx {

struct DevComp {
    int32_t type;
    int32_t do_sr;
    int32_t poff;     // offset of this component's [G, ...] in DevPot::p (inline) or pdev
    int32_t inl;      // 1: parameters are in DevPot::p; 0: in pdev (SCF)
    double q0[3];
    double R[9];
    // Constants derived from the parameters on the host (for the forms of
    // gx_fast64.cuh): dc[0] = G m; Plummer, Miyamoto-Nagai: dc[1] = b^2;
    // NFW: dc[1] = 1 / r_s, dc[2..4] = 1 / a^2, 1 / b^2, 1 / c^2 (1 where the
    // shape has no such axis).
    double dc[5];
};

struct DevPot {
    int32_t ncomp;
    int32_t n_inline;
    int32_t has_scf;      // selects the SCF = true instantiation on the host
    int32_t pad;
    const double *pdev;   // device copy of the packed parameters (may be null)
    const DevComp *cdev;  // component table in device memory (more than
                          // GX_MAX_COMPONENTS components), else null
    DevComp c[GX_MAX_COMPONENTS];
    double p[GX_MAX_INLINE_PARAMS];
};

// A large composite seen through its device table: the same members as DevPot
// (c, p, pdev, ncomp), so the component evaluators below serve both; every
// table component reads its parameters from the device copy (inl == 0).
struct TabPot {
    int32_t ncomp;
    const DevComp *c;
    const double *p;
    const double *pdev;
};

__device__ __forceinline__ TabPot table_view(const DevPot &pot) { return TabPot{pot.ncomp, pot.cdev, pot.pdev, pot.pdev}; }

struct DevFrame {
    int32_t type;   // gx_frame_type
    int32_t pad;
    double O[3];
};

// ---------------------------------------------------------------------------
// SCF (src/gala/potential/scf/src/bfe.cpp:114-259, bfe_helper.cpp:14-90).
// Implemented in gx_scf.cuh; declared here so the component switch can call it.
// ---------------------------------------------------------------------------
static __device__ double scf_value_dev(const double *p, const double *q);
static __device__ void scf_gradient_dev(const double *p, const double *q, double *g);
static __device__ double scf_density_dev(const double *p, const double *q);

__device__ __forceinline__ double norm3_sq(const double *q) {
    return q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
}

// Powers in the gradients.  gala calls pow(x, -1.5) (Miyamoto-Nagai) and
// pow(r, 3.0) (Kepler).  The FP64 pow of CUDA runs an extended-precision log
// and exp, a hundred-odd instructions on the FP64 pipe, whose rate on this part
// is 1/64 of FP32.  1 / (x sqrt(x)) is correctly rounded in each of its three
// operations (within 1.5 ulp of x^-1.5) and r r r within 1 ulp of r^3: the
// accuracy class of pow itself, which does not round like the host's pow
// either.  Edge values match pow: 0 -> inf, inf -> 0, NaN -> NaN.
__device__ __forceinline__ double pow_m1p5(double x) { return 1.0 / (x * sqrt(x)); }
__device__ __forceinline__ double cube(double r) { return r * r * r; }

// Parameters of component ci as a plain pointer: inline ones are read from the
// kernel-parameter copy, SCF blocks from global memory.
#define GX_PARAM(pot, ci, k) ((pot).c[ci].inl ? (pot).p[(pot).c[ci].poff + (k)] : (pot).pdev[(pot).c[ci].poff + (k)])

// Value of one component at q (kepler_value :58-64, hernquist_value :211-219,
// plummer_value :292-300, miyamotonagai_value :1287-1296, sphericalnfw_value
// :819-833, flattenednfw_value :925-942, triaxialnfw_value :1028-1049).
template <bool SCF, typename PV>
__device__ __forceinline__ double comp_value(const PV &pot, int ci, const double *q) {
    const int type = pot.c[ci].type;
#define P(k) GX_PARAM(pot, ci, k)
    switch (type) {
    case GX_POT_NULL:
        return 0.;
    case GX_POT_KEPLER:
        return -P(0) * P(1) / sqrt(norm3_sq(q));
    case GX_POT_HERNQUIST: {
        const double r = sqrt(norm3_sq(q));
        return -P(0) * P(1) / (r + P(2));
    }
    case GX_POT_PLUMMER: {
        const double r2 = norm3_sq(q);
        return -P(0) * P(1) / sqrt(r2 + P(2) * P(2));
    }
    case GX_POT_MIYAMOTONAGAI: {
        const double zd = (P(2) + sqrt(q[2] * q[2] + P(3) * P(3)));
        return -P(0) * P(1) / sqrt(q[0] * q[0] + q[1] * q[1] + zd * zd);
    }
    case GX_POT_SPHERICALNFW: {
        const double v_h2 = -P(0) * P(1) / P(2);
        const double u = sqrt(norm3_sq(q)) / P(2);
        if (u == 0) return v_h2;
        return v_h2 * log(1 + u) / u;
    }
    case GX_POT_FLATTENEDNFW: {
        const double v_h2 = -P(0) * P(1) / P(2);
        const double u = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] / (P(5) * P(5))) / P(2);
        if (u == 0) return v_h2;
        return v_h2 * log(1 + u) / u;
    }
    case GX_POT_TRIAXIALNFW: {
        const double v_h2 = -P(0) * P(1) / P(2);
        const double u = sqrt(q[0] * q[0] / (P(3) * P(3)) + q[1] * q[1] / (P(4) * P(4)) +
                              q[2] * q[2] / (P(5) * P(5))) / P(2);
        if (u == 0) return v_h2;
        return v_h2 * log(1 + u) / u;
    }
    case GX_POT_SCF:
        if constexpr (SCF) return scf_value_dev(pot.pdev + pot.c[ci].poff, q);
        return __longlong_as_double(0x7ff8000000000000LL);
    default:
        return __longlong_as_double(0x7ff8000000000000LL);
    }
#undef P
}

// Gradient of one component, accumulated into g (kepler :66-76, hernquist
// :221-233, plummer :302-314, miyamotonagai :1298-1312, sphericalnfw :835-850,
// flattenednfw :944-962, triaxialnfw :1051-1072).
template <bool SCF, typename PV>
__device__ __forceinline__ void comp_gradient(const PV &pot, int ci, const double *q, double *g) {
    const int type = pot.c[ci].type;
#define P(k) GX_PARAM(pot, ci, k)
    double fac;
    switch (type) {
    case GX_POT_NULL:
        return;
    case GX_POT_KEPLER:
        fac = P(0) * P(1) / cube(sqrt(norm3_sq(q)));
        break;
    case GX_POT_HERNQUIST: {
        const double r = sqrt(norm3_sq(q));
        fac = P(0) * P(1) / ((r + P(2)) * (r + P(2)) * r);
        break;
    }
    case GX_POT_PLUMMER: {
        const double R2b = norm3_sq(q) + P(2) * P(2);
        fac = P(0) * P(1) / sqrt(R2b) / R2b;
        break;
    }
    case GX_POT_MIYAMOTONAGAI: {
        const double sqrtz = sqrt(q[2] * q[2] + P(3) * P(3));
        const double zd = P(2) + sqrtz;
        fac = P(0) * P(1) * pow_m1p5(q[0] * q[0] + q[1] * q[1] + zd * zd);
        g[0] = g[0] + fac * q[0];
        g[1] = g[1] + fac * q[1];
        g[2] = g[2] + fac * q[2] * (1. + P(2) / sqrtz);
        return;
    }
    case GX_POT_SPHERICALNFW: {
        const double v_h2 = P(0) * P(1) / P(2);
        const double u = sqrt(norm3_sq(q)) / P(2);
        fac = v_h2 / (u * u * u) / (P(2) * P(2)) * (log(1 + u) - u / (1 + u));
        break;
    }
    case GX_POT_FLATTENEDNFW: {
        const double v_h2 = P(0) * P(1) / P(2);
        const double u = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] / (P(5) * P(5))) / P(2);
        fac = v_h2 / (u * u * u) / (P(2) * P(2)) * (log(1 + u) - u / (1 + u));
        g[0] = g[0] + fac * q[0];
        g[1] = g[1] + fac * q[1];
        g[2] = g[2] + fac * q[2] / (P(5) * P(5));
        return;
    }
    case GX_POT_TRIAXIALNFW: {
        const double v_h2 = P(0) * P(1) / P(2);
        const double u = sqrt(q[0] * q[0] / (P(3) * P(3)) + q[1] * q[1] / (P(4) * P(4)) +
                              q[2] * q[2] / (P(5) * P(5))) / P(2);
        fac = v_h2 / (u * u * u) / (P(2) * P(2)) * (log(1 + u) - u / (1 + u));
        g[0] = g[0] + fac * q[0] / (P(3) * P(3));
        g[1] = g[1] + fac * q[1] / (P(4) * P(4));
        g[2] = g[2] + fac * q[2] / (P(5) * P(5));
        return;
    }
    case GX_POT_SCF:
        if constexpr (SCF) {
            scf_gradient_dev(pot.pdev + pot.c[ci].poff, q, g);
            return;
        }
        fac = __longlong_as_double(0x7ff8000000000000LL);
        break;
    default: {
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        g[0] = nan; g[1] = nan; g[2] = nan;
        return;
    }
    }
    g[0] = g[0] + fac * q[0];
    g[1] = g[1] + fac * q[1];
    g[2] = g[2] + fac * q[2];
#undef P
}

// Density of one component (kepler_density :78-88, hernquist_density :235-244,
// plummer_density :316-324, miyamotonagai_density :1314-1332,
// sphericalnfw_density :852-864).  Flattened/triaxial NFW have no density in
// gala (nan_density).
template <bool SCF, typename PV>
__device__ __forceinline__ double comp_density(const PV &pot, int ci, const double *q) {
    const int type = pot.c[ci].type;
    const double PI = 3.14159265358979323846;
#define P(k) GX_PARAM(pot, ci, k)
    switch (type) {
    case GX_POT_NULL:
        return 0.;
    case GX_POT_KEPLER:
        return (norm3_sq(q) == 0.) ? __longlong_as_double(0x7ff0000000000000LL) : 0.;
    case GX_POT_HERNQUIST: {
        const double r = sqrt(norm3_sq(q));
        const double rho0 = P(1) / (2 * PI * P(2) * P(2) * P(2));
        return rho0 / ((r / P(2)) * pow(1 + r / P(2), 3.0));
    }
    case GX_POT_PLUMMER: {
        const double r2 = norm3_sq(q);
        return 3 * P(1) / (4 * PI * P(2) * P(2) * P(2)) * pow(1 + r2 / (P(2) * P(2)), -2.5);
    }
    case GX_POT_MIYAMOTONAGAI: {
        const double M = P(1), a = P(2), b = P(3);
        const double R2 = q[0] * q[0] + q[1] * q[1];
        const double sqrt_zb = sqrt(q[2] * q[2] + b * b);
        const double numer = (b * b * M / (4 * PI)) * (a * R2 + (a + 3 * sqrt_zb) * (a + sqrt_zb) * (a + sqrt_zb));
        const double denom = pow(R2 + (a + sqrt_zb) * (a + sqrt_zb), 2.5) * sqrt_zb * sqrt_zb * sqrt_zb;
        return numer / denom;
    }
    case GX_POT_SPHERICALNFW: {
        const double v_h2 = P(0) * P(1) / P(2);
        const double r = sqrt(norm3_sq(q));
        const double rho0 = v_h2 / (4 * PI * P(0) * P(2) * P(2));
        return rho0 / ((r / P(2)) * pow(1 + r / P(2), 2.0));
    }
    case GX_POT_SCF:
        if constexpr (SCF) return scf_density_dev(pot.pdev + pot.c[ci].poff, q);
        return __longlong_as_double(0x7ff8000000000000LL);
    default:
        return __longlong_as_double(0x7ff8000000000000LL);
    }
#undef P
}

// q' = R (q - q0) (apply_shift_rotate_N, cpotential.cpp:152-167).
__device__ __forceinline__ void shift_rotate(const DevComp &c, const double *q, double *qt) {
    const double x = q[0] - c.q0[0], y = q[1] - c.q0[1], z = q[2] - c.q0[2];
    qt[0] = c.R[0] * x + c.R[1] * y + c.R[2] * z;
    qt[1] = c.R[3] * x + c.R[4] * y + c.R[5] * z;
    qt[2] = c.R[6] * x + c.R[7] * y + c.R[8] * z;
}

// c_potential (cpotential.cpp:170-189).  The shifted path of gala builds q'
// as 0 + R0 x + ...; for finite values that equals R0 x + ..., bit for bit.
template <bool SCF, typename PV>
__device__ __forceinline__ double potential_value_t(const PV &pot, const double *q) {
    double v = 0;
    for (int i = 0; i < pot.ncomp; i++) {
        if (pot.c[i].do_sr == 0) {
            v = v + comp_value<SCF>(pot, i, q);
        } else {
            double qt[3];
            shift_rotate(pot.c[i], q, qt);
            v = v + comp_value<SCF>(pot, i, qt);
        }
    }
    return v;
}

// c_density (cpotential.cpp:192-211).
template <bool SCF, typename PV>
__device__ __forceinline__ double potential_density_t(const PV &pot, const double *q) {
    double v = 0;
    for (int i = 0; i < pot.ncomp; i++) {
        if (pot.c[i].do_sr == 0) {
            v = v + comp_density<SCF>(pot, i, q);
        } else {
            double qt[3];
            shift_rotate(pot.c[i], q, qt);
            v = v + comp_density<SCF>(pot, i, qt);
        }
    }
    return v;
}

// c_gradient at one point (cpotential.cpp:214-287): zero, accumulate each
// component in order; shifted/rotated components go through a zeroed
// temporary, are rotated back with R^T (apply_rotate_T, :103-134) and added.
template <bool SCF, typename PV>
__device__ __forceinline__ void potential_gradient_t(const PV &pot, const double *q, double *g) {
    g[0] = 0.; g[1] = 0.; g[2] = 0.;
    for (int i = 0; i < pot.ncomp; i++) {
        if (pot.c[i].do_sr == 0) {
            comp_gradient<SCF>(pot, i, q, g);
        } else {
            const DevComp &c = pot.c[i];
            double qt[3], gt[3] = {0., 0., 0.};
            shift_rotate(c, q, qt);
            comp_gradient<SCF>(pot, i, qt, gt);
            g[0] += c.R[0] * gt[0] + c.R[3] * gt[1] + c.R[6] * gt[2];
            g[1] += c.R[1] * gt[0] + c.R[4] * gt[1] + c.R[7] * gt[2];
            g[2] += c.R[2] * gt[0] + c.R[5] * gt[1] + c.R[8] * gt[2];
        }
    }
}

// The descriptor's components: the by-value array, or the device table of a
// large composite (the branch is uniform over the grid).
template <bool SCF>
__device__ __forceinline__ double potential_value(const DevPot &pot, const double *q) {
    if (pot.cdev) return potential_value_t<SCF>(table_view(pot), q);
    return potential_value_t<SCF>(pot, q);
}
template <bool SCF>
__device__ __forceinline__ double potential_density(const DevPot &pot, const double *q) {
    if (pot.cdev) return potential_density_t<SCF>(table_view(pot), q);
    return potential_density_t<SCF>(pot, q);
}
template <bool SCF>
__device__ __forceinline__ void potential_gradient(const DevPot &pot, const double *q, double *g) {
    if (pot.cdev) {
        potential_gradient_t<SCF>(table_view(pot), q, g);
        return;
    }
    potential_gradient_t<SCF>(pot, q, g);
}

// Frame energy: static_frame_hamiltonian (builtin_frames.cpp:8-16) or
// constant_rotating_frame_3d_hamiltonian (:78-94).
__device__ __forceinline__ double frame_energy(const DevFrame &fr, const double *w) {
    if (fr.type == GX_FRAME_STATIC) {
        double E = 0.;
        for (int i = 0; i < 3; i++) E += w[i + 3] * w[i + 3];
        return 0.5 * E;
    }
    double E = 0.;
    for (int i = 0; i < 3; i++) E += 0.5 * w[i + 3] * w[i + 3];
    const double Lx = w[1] * w[5] - w[2] * w[4];
    const double Ly = -w[0] * w[5] + w[2] * w[3];
    const double Lz = w[0] * w[4] - w[1] * w[3];
    return E - (fr.O[0] * Lx + fr.O[1] * Ly + fr.O[2] * Lz);
}

// Hamilton's equations at one point, Fwrapper_T -> hamiltonian_gradient_T
// (chamiltonian.cpp:38-57) with the frame gradient of builtin_frames.cpp:18-24
// (static) or :96-112 (rotating); the momentum half is multiplied by -1.
template <bool SCF>
__device__ __forceinline__ void hamiltonian_rhs(const DevPot &pot, const DevFrame &fr, const double *w, double *f) {
    double g[3];
    potential_gradient<SCF>(pot, w, g);
    if (fr.type == GX_FRAME_STATIC) {
        f[0] = w[3];
        f[1] = w[4];
        f[2] = w[5];
        f[3] = g[0] * -1;
        f[4] = g[1] * -1;
        f[5] = g[2] * -1;
    } else {
        const double *O = fr.O;
        double Cx = O[1] * w[2] - O[2] * w[1];
        double Cy = -O[0] * w[2] + O[2] * w[0];
        double Cz = O[0] * w[1] - O[1] * w[0];
        f[0] = 0. + w[3] - Cx;
        f[1] = 0. + w[4] - Cy;
        f[2] = 0. + w[5] - Cz;
        Cx = O[1] * w[5] - O[2] * w[4];
        Cy = -O[0] * w[5] + O[2] * w[3];
        Cz = O[0] * w[4] - O[1] * w[3];
        f[3] = (g[0] + Cx) * -1;
        f[4] = (g[1] + Cy) * -1;
        f[5] = (g[2] + Cz) * -1;
    }
}

// Out-of-line entry points for the integrator kernels.  A kernel calls the
// potential many times per step (up to 16 for DOP853); calling one compiled
// copy instead of inlining every call keeps code size and compile time small.
// Arguments and results are passed by value so they stay in registers.
struct V3 {
    double v[3];
};
struct V6 {
    double v[6];
};

template <bool SCF>
__device__ __noinline__ V3 gradient_call(const DevPot &pot, V3 q) {
    V3 g;
    potential_gradient<SCF>(pot, q.v, g.v);
    return g;
}

template <bool SCF>
__device__ __noinline__ V6 rhs_call(const DevPot &pot, const DevFrame &fr, V6 w) {
    V6 f;
    hamiltonian_rhs<SCF>(pot, fr, w.v, f.v);
    return f;
}

}  // namespace gx
