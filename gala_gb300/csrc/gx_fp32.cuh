// gx_fp32.cuh -- FP32 force evaluation for the compensated integrators.
//
// The closed-form potentials of gx_device.cuh, evaluated in FP32 on the
// special-function unit: 1/sqrt, reciprocal and log2 are single approximate
// MUFU instructions (relative error a few 1e-8), and the NFW radial factor
// f(u)/u^3, f(u) = ln(1+u) - u/(1+u), is a polynomial on either side of u = 1
// (nfw_fac) with no cancellation.
// The integrators accumulate positions and velocities in compensated (Kahan)
// form, so FP32 rounding of the state does not build up; the force error (a
// few FP32 ulps) acts like a slightly perturbed potential.
//
// Each component type has a compile-time evaluator (comp_grad_t<TYPE>); a
// potential whose component list is known at compile time (PotSig below) is
// evaluated with no per-component branching, which lets the compiler overlap
// the independent component evaluations.  Any other list goes through the
// run-time switch.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gala_gb300.h"
#include "gx_nfw_poly.cuh"

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

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float lg2_approx(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// p0 f(u) / u^3 for the NFW force, f(u) = ln(1 + u) - u / (1 + u), u = s / r_s
// for the (scaled) radius s, from s^2, 1/s, p0, 1/r_s and r_s.  Both forms below
// are computed and the right one selected (lanes on either side of u = 1 do not
// run two branches one after the other), and no special-function instruction
// waits on another: log2(u^2) issues beside rsqrt(s^2), so the factor is one
// MUFU latency and a depth-4 polynomial away from s^2.
//   inside  (u < 1):  f / u^3 = H(u) / (2 u),       H(u) = 2 f(u) / u^2
//   outside (u >= 1): f / u^3 = (ln u + K(w)) w^3,  K(w) = ln(1 + w) - 1 / (1 + w), w = 1 / u
// H and K are degree-10 polynomials in 2u - 1 and 2w - 1 (gx_nfw_poly.cuh); the
// only subtraction that cancels, ln u + K(w) at u ~ 1.3, loses under one bit.
__device__ __forceinline__ float nfw_fac(float p0, float irs, float rs, float s2, float si) {
    const float x = fmaf(s2, si * (2.0f * irs), -1.0f);   // 2u - 1
    const float y = fmaf(si, 2.0f * rs, -1.0f);           // 2w - 1
    const float lg = lg2_approx(s2 * (irs * irs));        // log2(u^2)
    const float w = si * rs;
    const float inner = nfw_poly_h(x) * (si * (0.5f * rs * p0));
    const float outer = fmaf(lg, 0.34657359027997264f, nfw_poly_k(y)) * ((p0 * w) * (w * w));  // ln u = log2(u^2) ln2 / 2
    return x < 1.0f ? inner : outer;
}

// Components whose force is fac(r) q (centred, spherical): Kepler, Hernquist,
// Plummer, spherical NFW.
template <int T>
inline constexpr bool spherical_t =
    T == GX_POT_KEPLER || T == GX_POT_HERNQUIST || T == GX_POT_PLUMMER || T == GX_POT_SPHERICALNFW;

// fac(r) of a spherical component of compile-time type T, from r^2 and 1/r.
template <int T>
__device__ __forceinline__ float comp_fac_t(const float *p, float r2, float ri) {
    if constexpr (T == GX_POT_KEPLER) {  // p = {G m}
        return (p[0] * ri) * (ri * ri);
    } else if constexpr (T == GX_POT_HERNQUIST) {  // p = {G m, c}
        const float irc = rcp_approx(fmaf(r2, ri, p[1]));
        return (p[0] * ri) * (irc * irc);
    } else if constexpr (T == GX_POT_PLUMMER) {  // p = {G m, b^2}
        const float rb = rsqrt_approx(r2 + p[1]);
        return (p[0] * rb) * (rb * rb);
    } else {  // spherical NFW, p = {G m / r_s^3, 1 / r_s, r_s}
        return nfw_fac(p[0], p[1], p[2], r2, ri);
    }
}

// Gradient of one component of compile-time type T, written to v.
template <int T>
__device__ __forceinline__ void comp_vec_t(const float *p, const float *q, float *v) {
    if constexpr (spherical_t<T>) {
        const float r2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        const float fac = comp_fac_t<T>(p, r2, rsqrt_approx(r2));
        v[0] = fac * q[0]; v[1] = fac * q[1]; v[2] = fac * q[2];
    } else if constexpr (T == GX_POT_MIYAMOTONAGAI) {  // p = {G m, a, b^2}
        const float z2b = fmaf(q[2], q[2], p[2]);
        const float szi = rsqrt_approx(z2b);
        const float zd = fmaf(z2b, szi, p[1]);
        const float ti = rsqrt_approx(fmaf(zd, zd, q[0] * q[0] + q[1] * q[1]));
        const float fac = (p[0] * ti) * (ti * ti);
        v[0] = fac * q[0]; v[1] = fac * q[1]; v[2] = fac * q[2] * fmaf(p[1], szi, 1.0f);
    } else if constexpr (T == GX_POT_FLATTENEDNFW) {  // p = {G m / r_s^3, 1 / r_s, r_s, 1 / c^2}
        const float s2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] * p[3];
        const float fac = nfw_fac(p[0], p[1], p[2], s2, rsqrt_approx(s2));
        v[0] = fac * q[0]; v[1] = fac * q[1]; v[2] = fac * q[2] * p[3];
    } else if constexpr (T == GX_POT_TRIAXIALNFW) {  // p = {G m / r_s^3, 1 / r_s, r_s, 1/a^2, 1/b^2, 1/c^2}
        const float s2 = q[0] * q[0] * p[3] + q[1] * q[1] * p[4] + q[2] * q[2] * p[5];
        const float fac = nfw_fac(p[0], p[1], p[2], s2, rsqrt_approx(s2));
        v[0] = fac * q[0] * p[3]; v[1] = fac * q[1] * p[4]; v[2] = fac * q[2] * p[5];
    } else {  // GX_POT_NULL
        v[0] = 0.f; v[1] = 0.f; v[2] = 0.f;
    }
}

// Gradient of one component of compile-time type T, accumulated into g.
template <int T>
__device__ __forceinline__ void comp_grad_t(const float *p, const float *q, float *g) {
    float v[3];
    comp_vec_t<T>(p, q, v);
    g[0] += v[0]; g[1] += v[1]; g[2] += v[2];
}

// Run-time dispatch on the component type.
__device__ __forceinline__ void comp_gradient_f(const DevCompF &c, const float *q, float *g) {
    switch (c.type) {
    case GX_POT_KEPLER: comp_grad_t<GX_POT_KEPLER>(c.p, q, g); return;
    case GX_POT_HERNQUIST: comp_grad_t<GX_POT_HERNQUIST>(c.p, q, g); return;
    case GX_POT_PLUMMER: comp_grad_t<GX_POT_PLUMMER>(c.p, q, g); return;
    case GX_POT_MIYAMOTONAGAI: comp_grad_t<GX_POT_MIYAMOTONAGAI>(c.p, q, g); return;
    case GX_POT_SPHERICALNFW: comp_grad_t<GX_POT_SPHERICALNFW>(c.p, q, g); return;
    case GX_POT_FLATTENEDNFW: comp_grad_t<GX_POT_FLATTENEDNFW>(c.p, q, g); return;
    case GX_POT_TRIAXIALNFW: comp_grad_t<GX_POT_TRIAXIALNFW>(c.p, q, g); return;
    default: return;  // GX_POT_NULL
    }
}

__device__ __forceinline__ void comp_gradient_sr(const DevCompF &c, const float *q, float *g) {
    if (!c.do_sr) {
        comp_gradient_f(c, q, g);
        return;
    }
    const float x = q[0] - c.q0[0], y = q[1] - c.q0[1], z = q[2] - c.q0[2];
    const float qt[3] = {c.R[0] * x + c.R[1] * y + c.R[2] * z, c.R[3] * x + c.R[4] * y + c.R[5] * z,
                         c.R[6] * x + c.R[7] * y + c.R[8] * z};
    float gt[3] = {0.f, 0.f, 0.f};
    comp_gradient_f(c, qt, gt);
    g[0] += c.R[0] * gt[0] + c.R[3] * gt[1] + c.R[6] * gt[2];
    g[1] += c.R[1] * gt[0] + c.R[4] * gt[1] + c.R[7] * gt[2];
    g[2] += c.R[2] * gt[0] + c.R[5] * gt[1] + c.R[8] * gt[2];
}

// Component lists known at compile time (-1 = no component).  SIG_GENERIC
// means: use the run-time loop over pot.ncomp components.
template <int T0, int T1, int T2, int T3>
struct PotSig {
    static constexpr bool generic = (T0 == -2);
};
using SigGeneric = PotSig<-2, -1, -1, -1>;

template <typename S>
struct SigTypes;
template <int T0, int T1, int T2, int T3>
struct SigTypes<PotSig<T0, T1, T2, T3>> {
    static constexpr int t0 = T0, t1 = T1, t2 = T2, t3 = T3;
};

// One component of a compile-time list: a spherical one adds its factor to fs,
// any other its gradient to gm (the flags say whether fs / gm hold a term yet;
// they are compile-time constants after inlining, so no 0 + x is issued).
template <int T>
__device__ __forceinline__ void sig_term(const float *p, const float *q, float r2, float ri, float &fs, bool &has_fs,
                                         float *gm, bool &has_gm) {
    if constexpr (T < 0) {
        return;
    } else if constexpr (spherical_t<T>) {
        const float f = comp_fac_t<T>(p, r2, ri);
        fs = has_fs ? fs + f : f;
        has_fs = true;
    } else {
        float v[3];
        comp_vec_t<T>(p, q, v);
        for (int k = 0; k < 3; k++) gm[k] = has_gm ? gm[k] + v[k] : v[k];
        has_gm = true;
    }
}

// Gradient of the whole potential at q.  A compile-time list shares r^2 and
// 1/r among its spherical components and multiplies the sum of their factors
// by q once: g = (sum fac) q + (the other components' gradients).
template <typename S>
__device__ __forceinline__ void potential_gradient_f(const DevPotF &pot, const float *q, float *g) {
    if constexpr (S::generic) {
        g[0] = 0.f; g[1] = 0.f; g[2] = 0.f;
        for (int i = 0; i < pot.ncomp; i++) comp_gradient_sr(pot.c[i], q, g);
    } else {
        using T = SigTypes<S>;
        const float r2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        const float ri = rsqrt_approx(r2);
        float fs = 0.f, gm[3] = {0.f, 0.f, 0.f};
        bool has_fs = false, has_gm = false;
        sig_term<T::t0>(pot.c[0].p, q, r2, ri, fs, has_fs, gm, has_gm);
        sig_term<T::t1>(pot.c[1].p, q, r2, ri, fs, has_fs, gm, has_gm);
        sig_term<T::t2>(pot.c[2].p, q, r2, ri, fs, has_fs, gm, has_gm);
        sig_term<T::t3>(pot.c[3].p, q, r2, ri, fs, has_fs, gm, has_gm);
        for (int k = 0; k < 3; k++) g[k] = has_fs ? (has_gm ? fmaf(fs, q[k], gm[k]) : fs * q[k]) : gm[k];
    }
}

// Compensated accumulation into the pair (s, c), whose value is s + c (the
// convention of the FP64 split hi = (float)x, lo = (float)(x - hi), of the
// drift increments h (vh + vl) and of the output hi + lo): the increment d and
// the carried low part are added to s, and the rounding error of that addition
// (Fast2Sum, exact while |s| >= |d + c|) becomes the new low part.
__device__ __forceinline__ void kahan_add(float &s, float &c, float d) {
    const float y = __fadd_rn(d, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(y, __fsub_rn(t, s));
    s = t;
}

// Kick (vh, vl) += dh g, compensated, with the product fused into the addition
// of the carried low part.
__device__ __forceinline__ void kick(float &vh, float &vl, float dh, float g) {
    const float a = fmaf(dh, g, vl);
    const float t = __fadd_rn(vh, a);
    vl = __fsub_rn(a, __fsub_rn(t, vh));
    vh = t;
}

// The kick above followed by the drift (xh, xl) += ch v: the drift increment
// ch (vh + (vl + dh g)) is formed from the velocity before its compensated
// addition, so the drift does not wait for it (a shorter dependent chain per
// sub-step than kick, then drift from the new pair).
__device__ __forceinline__ void kick_drift(float &xh, float &xl, float &vh, float &vl, float dh, float g, float ch) {
    const float a = fmaf(dh, g, vl);
    const float d = fmaf(ch, vh, ch * a);
    const float t = __fadd_rn(vh, a);
    vl = __fsub_rn(a, __fsub_rn(t, vh));
    vh = t;
    kahan_add(xh, xl, d);
}

}  // namespace gx
