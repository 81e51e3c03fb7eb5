// gx_body_f32.cuh -- FP32 pieces shared by the FP32-stage DOP853 systems of
// mock streams (gx_nbody_fp32.cu, gx_nbody_wide_fp32.cu): the force of one
// massive body and the double-float state arithmetic.
#pragma once

#include "gx_fp32.cuh"

namespace gx {

// The FP32 constants of one body's potential (pack_potential_f32's packing);
// a body is an unrotated single component, so three constants suffice.
struct BodyF {
    int32_t type;
    float p[3];
};

__device__ __forceinline__ void body_consts_f32(const gx_body *b, BodyF &c) {
    const int type = __ldg(&b->type);
    const double G = __ldg(b->params + 0), m = __ldg(b->params + 1);
    const double p2 = __ldg(b->params + 2), p3 = __ldg(b->params + 3);
    c.type = type;
    c.p[0] = c.p[1] = c.p[2] = 0.f;
    switch (type) {
    case GX_POT_KEPLER: c.p[0] = (float)(G * m); break;
    case GX_POT_HERNQUIST: c.p[0] = (float)(G * m); c.p[1] = (float)p2; break;
    case GX_POT_PLUMMER: c.p[0] = (float)(G * m); c.p[1] = (float)(p2 * p2); break;
    case GX_POT_MIYAMOTONAGAI: c.p[0] = (float)(G * m); c.p[1] = (float)p2; c.p[2] = (float)(p3 * p3); break;
    case GX_POT_SPHERICALNFW: c.p[0] = (float)(G * m / (p2 * p2 * p2)); c.p[1] = (float)(1.0 / p2); c.p[2] = (float)p2; break;
    default: c.type = GX_POT_NULL; break;
    }
}

// Gradient of a body's potential at separation d, accumulated into g.
__device__ __forceinline__ void body_grad_f32(const BodyF &c, const float *d, float *g) {
    switch (c.type) {
    case GX_POT_KEPLER: comp_grad_t<GX_POT_KEPLER>(c.p, d, g); return;
    case GX_POT_HERNQUIST: comp_grad_t<GX_POT_HERNQUIST>(c.p, d, g); return;
    case GX_POT_PLUMMER: comp_grad_t<GX_POT_PLUMMER>(c.p, d, g); return;
    case GX_POT_MIYAMOTONAGAI: comp_grad_t<GX_POT_MIYAMOTONAGAI>(c.p, d, g); return;
    case GX_POT_SPHERICALNFW: comp_grad_t<GX_POT_SPHERICALNFW>(c.p, d, g); return;
    default: return;
    }
}

__device__ __forceinline__ void two_sum32(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (hi, lo) <- (yh, yl) + h k as a double-float, with the FMA residue of h k.
__device__ __forceinline__ void df_axpy32(float yh, float yl, float h, float k, float &hi, float &lo) {
    const float d = __fmul_rn(h, k);
    const float dr = __fmaf_rn(h, k, -d);
    float s, e;
    two_sum32(yh, d, s, e);
    const float l = __fadd_rn(yl, __fadd_rn(e, dr));
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

__device__ __forceinline__ float ex2_approx32(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

}  // namespace gx
