// gx_body.cuh -- the force of one massive body of an n-body system (FP64).
#pragma once

#include "gx_device.cuh"

namespace gx {

// Gradient of a body's potential at d = q - q0 (q0 = the body's position).
// gala evaluates the body's CPotential with do_shift_rotate = 1 and R = I
// (c_gradient, cpotential.cpp:214-287): q' = I d, g' = 0 + fac q', g = I^T g';
// multiplying by the identity changes no finite value, so it is left out.
// Component formulas: builtin_potentials.cpp (kepler :66-76, hernquist :221-233,
// plummer :302-314, miyamotonagai :1298-1312, sphericalnfw :835-850).
__device__ __forceinline__ void body_gradient(int type, const double *__restrict__ P, double x, double y, double z,
                                              double *g) {
    const double G = __ldg(P + 0), m = __ldg(P + 1);
    double fac;
    switch (type) {
    case GX_POT_KEPLER:
        fac = G * m / cube(sqrt(x * x + y * y + z * z));
        break;
    case GX_POT_HERNQUIST: {
        const double c = __ldg(P + 2);
        const double r = sqrt(x * x + y * y + z * z);
        fac = G * m / ((r + c) * (r + c) * r);
        break;
    }
    case GX_POT_PLUMMER: {
        const double b = __ldg(P + 2);
        const double R2b = x * x + y * y + z * z + b * b;
        fac = G * m / sqrt(R2b) / R2b;
        break;
    }
    case GX_POT_MIYAMOTONAGAI: {
        const double a = __ldg(P + 2), b = __ldg(P + 3);
        const double sqrtz = sqrt(z * z + b * b);
        const double zd = a + sqrtz;
        fac = G * m * pow_m1p5(x * x + y * y + zd * zd);
        g[0] = 0. + fac * x;
        g[1] = 0. + fac * y;
        g[2] = 0. + fac * z * (1. + a / sqrtz);
        return;
    }
    case GX_POT_SPHERICALNFW: {
        const double rs = __ldg(P + 2);
        const double v_h2 = G * m / rs;
        const double u = sqrt(x * x + y * y + z * z) / rs;
        fac = v_h2 / (u * u * u) / (rs * rs) * (log(1 + u) - u / (1 + u));
        break;
    }
    default: {  // a type without a GPU body formula poisons the result
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        g[0] = nan; g[1] = nan; g[2] = nan;
        return;
    }
    }
    g[0] = 0. + fac * x;
    g[1] = 0. + fac * y;
    g[2] = 0. + fac * z;
}

// Out-of-line form for kernels that call it many times per step.
static __device__ __noinline__ V3 body_gradient_call(int type, const double *__restrict__ P, double x, double y, double z) {
    V3 g;
    body_gradient(type, P, x, y, z, g.v);
    return g;
}

}  // namespace gx
