// gx_fp32.cuh -- FP32 force evaluation for the compensated integrators.
//
// The closed-form potentials of gx_device.cuh, evaluated in FP32 with the
// special-function units: 1/sqrt via rsqrt, reciprocals via the fast
// reciprocal, and the NFW radial factor f(u) = ln(1+u) - u/(1+u) computed
// without cancellation (for u < 1 as the positive series in w = u/(1+u):
// f = sum_{k>=2} w^k / k; for u >= 1 directly).  Relative force error is a
// few FP32 ulps; the integrators accumulate positions and velocities in
// compensated (Kahan) form so that FP32 rounding of the state does not build up.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gala_gb300.h"

namespace gx {

struct DevCompF {
    int32_t type;
    int32_t do_sr;
    float p[6];    // type-specific constants, see pack_potential_f32
    float q0[3];
    float R[9];
};

struct DevPotF {
    int32_t ncomp;
    int32_t pad;
    DevCompF c[GX_MAX_COMPONENTS];
};

__device__ __forceinline__ float frcp(float x) { return __frcp_rn(x); }

// f(u)/u^3 for the NFW force, u = r / r_s.
__device__ __forceinline__ float nfw_f_over_u3(float u) {
    if (u < 1.0f) {
        const float w = u * frcp(1.0f + u);
        // sum_{k=2}^{25} w^k / k, Horner in w (w <= 1/2: truncation < 2^-25 relative)
        float s = 1.0f / 25.0f;
#pragma unroll
        for (int k = 24; k >= 2; k--) s = fmaf(s, w, 1.0f / (float)k);
        // f = w^2 * s ; w^2 / u^3 = 1 / (u (1+u)^2)
        const float opu = 1.0f + u;
        return s * frcp(u * opu * opu);
    }
    const float f = log1pf(u) - u * frcp(1.0f + u);
    return f * frcp(u * u * u);
}

// Gradient of one component (accumulated into g), FP32.
__device__ __forceinline__ void comp_gradient_f(const DevCompF &c, const float *q, float *g) {
    const float *p = c.p;
    switch (c.type) {
    case GX_POT_KEPLER: {  // p = {G m}
        const float ri = rsqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
        const float fac = p[0] * ri * ri * ri;
        g[0] += fac * q[0]; g[1] += fac * q[1]; g[2] += fac * q[2];
        return;
    }
    case GX_POT_HERNQUIST: {  // p = {G m, c}
        const float r2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        const float ri = rsqrtf(r2);
        const float r = r2 * ri;
        const float rc = r + p[1];
        const float fac = p[0] * ri * frcp(rc * rc);
        g[0] += fac * q[0]; g[1] += fac * q[1]; g[2] += fac * q[2];
        return;
    }
    case GX_POT_PLUMMER: {  // p = {G m, b^2}
        const float ri = rsqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + p[1]);
        const float fac = p[0] * ri * ri * ri;
        g[0] += fac * q[0]; g[1] += fac * q[1]; g[2] += fac * q[2];
        return;
    }
    case GX_POT_MIYAMOTONAGAI: {  // p = {G m, a, b^2}
        const float szi = rsqrtf(q[2] * q[2] + p[2]);
        const float sz = (q[2] * q[2] + p[2]) * szi;
        const float zd = p[1] + sz;
        const float ti = rsqrtf(q[0] * q[0] + q[1] * q[1] + zd * zd);
        const float fac = p[0] * ti * ti * ti;
        g[0] += fac * q[0]; g[1] += fac * q[1]; g[2] += fac * q[2] * (1.0f + p[1] * szi);
        return;
    }
    case GX_POT_SPHERICALNFW: {  // p = {G m / r_s^3, 1 / r_s}
        const float r2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        const float u = r2 * rsqrtf(r2) * p[1];
        const float fac = p[0] * nfw_f_over_u3(u);
        g[0] += fac * q[0]; g[1] += fac * q[1]; g[2] += fac * q[2];
        return;
    }
    case GX_POT_FLATTENEDNFW: {  // p = {G m / r_s^3, 1 / r_s, 1 / c^2}
        const float r2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] * p[2];
        const float u = r2 * rsqrtf(r2) * p[1];
        const float fac = p[0] * nfw_f_over_u3(u);
        g[0] += fac * q[0]; g[1] += fac * q[1]; g[2] += fac * q[2] * p[2];
        return;
    }
    case GX_POT_TRIAXIALNFW: {  // p = {G m / r_s^3, 1 / r_s, 1/a^2, 1/b^2, 1/c^2}
        const float r2 = q[0] * q[0] * p[2] + q[1] * q[1] * p[3] + q[2] * q[2] * p[4];
        const float u = r2 * rsqrtf(r2) * p[1];
        const float fac = p[0] * nfw_f_over_u3(u);
        g[0] += fac * q[0] * p[2]; g[1] += fac * q[1] * p[3]; g[2] += fac * q[2] * p[4];
        return;
    }
    default:
        return;  // GX_POT_NULL
    }
}

__device__ __forceinline__ void potential_gradient_f(const DevPotF &pot, const float *q, float *g) {
    g[0] = 0.f; g[1] = 0.f; g[2] = 0.f;
    for (int i = 0; i < pot.ncomp; i++) {
        const DevCompF &c = pot.c[i];
        if (!c.do_sr) {
            comp_gradient_f(c, q, g);
        } else {
            const float x = q[0] - c.q0[0], y = q[1] - c.q0[1], z = q[2] - c.q0[2];
            const float qt[3] = {c.R[0] * x + c.R[1] * y + c.R[2] * z, c.R[3] * x + c.R[4] * y + c.R[5] * z,
                                 c.R[6] * x + c.R[7] * y + c.R[8] * z};
            float gt[3] = {0.f, 0.f, 0.f};
            comp_gradient_f(c, qt, gt);
            g[0] += c.R[0] * gt[0] + c.R[3] * gt[1] + c.R[6] * gt[2];
            g[1] += c.R[1] * gt[0] + c.R[4] * gt[1] + c.R[7] * gt[2];
            g[2] += c.R[2] * gt[0] + c.R[5] * gt[1] + c.R[8] * gt[2];
        }
    }
}

// Compensated (Kahan) accumulation s += d with running compensation c.
__device__ __forceinline__ void kahan_add(float &s, float &c, float d) {
    const float y = __fsub_rn(d, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

}  // namespace gx
