// gx_fast64.cuh -- the FP64 force in instructions the FP64 pipe can afford.
//
// On this part the FP64 pipe retires one warp instruction per ~64 cycles of a
// sub-partition, and the library forms of the special operations are long
// sequences on it: sqrt and a/b cost 8 FP64-pipe instructions each, 1/x 5,
// log ~30, pow ~84 (measured with ncu instruction counters).  The adaptive
// DOP853 kernel, which evaluates the force 12 to 16 times a step and cannot be
// bit-identical to gala anyway (its step control runs pow), uses the forms
// below instead of gala's literal expressions; the fixed-step integrators and
// the potential evaluation entry points keep gala's operation order.
//
//   * sqrt and 1/x from an FP32 seed (rsqrtf / __frcp_rn of the double rounded
//     to 23 mantissa bits, built with integer operations: no F2F conversion,
//     which also runs on the FP64 pipe) and two Newton steps: 5 and 4 FP64
//     instructions, within about an ulp (the seed's relative error ~3e-7 is
//     cubed or squared twice); outside the FP32 normal range the library
//     operations are used;
//   * every a/b becomes a * (1/b) and products and sums are fused (fma);
//   * gala's formulas are rearranged algebraically where that removes an
//     operation (the NFW factor v_h^2 / u^3 / r_s^2 is G m / r^3, etc.);
//   * ln is table-driven (log_f below, ~14 instructions instead of ~30).
// The results differ from gala's expressions by a few ulp per evaluation; the
// integrated orbits are checked against the oracle at 1e-12 relative.
#pragma once

#include "gx_device.cuh"
#include "gx_log_table.cuh"

namespace gx {
namespace fast {

// FP32 approximation (23 mantissa bits, truncated, sign kept) of x whose high
// word is hi; valid when the exponent is in the FP32 normal range.
__device__ __forceinline__ float f32_of(unsigned hi, unsigned lo) {
    return __uint_as_float((hi & 0x80000000u) | ((((hi & 0x7fffffffu) - (896u << 20)) << 3) | (lo >> 29)));
}
// The double with the value of the FP32 number of bits fb (normal, any sign);
// *half receives half of it.
__device__ __forceinline__ double f64_of(unsigned fb, double *half) {
    const int hi = (int)((fb & 0x80000000u) | ((((fb >> 23) & 0xffu) + 896u) << 20) | ((fb >> 3) & 0xfffffu));
    const int lo = (int)(fb << 29);
    if (half) *half = __hiloint2double(hi - (1 << 20), lo);
    return __hiloint2double(hi, lo);
}
// |exponent| small enough that x, 1/x and 1/sqrt(x) are FP32 normal numbers
__device__ __forceinline__ bool f32_safe(unsigned hi) {
    const unsigned e = (hi >> 20) & 0x7ffu;
    return e >= 1023u - 120u && e <= 1023u + 120u;
}

// sqrt(u), u >= 0: Heron steps r += (u - r^2) / (2 sqrt(u)) with the slope
// taken from the seed.
__device__ __forceinline__ double sqrt_f(double u) {
    const unsigned hi = (unsigned)__double2hiint(u), lo = (unsigned)__double2loint(u);
    if (!f32_safe(hi) || (int)hi < 0) return sqrt(u);
    double h;
    const double y = f64_of(__float_as_uint(rsqrtf(f32_of(hi, lo))), &h);
    double r = u * y;
    r = fma(fma(-r, r, u), h, r);
    return fma(fma(-r, r, u), h, r);
}

// 1/x: Newton steps y += y (1 - x y).
__device__ __forceinline__ double rcp_f(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    if (!f32_safe(hi)) return 1.0 / x;
    double y = f64_of(__float_as_uint(__frcp_rn(f32_of(hi, lo))), nullptr);
    y = fma(y, fma(-x, y, 1.0), y);
    return fma(y, fma(-x, y, 1.0), y);
}

// ln x, Tang's table-driven method (P. T. P. Tang, ACM TOMS 16, 1990): x = 2^k m
// with m in [1, 2), c_j = 1 + j/64 the nearest table point (j = 0..64), f = m - c_j
// (exact), r = f / c_j as f * (1 / c_j), and ln x = k ln 2 + ln c_j + ln(1 + r)
// with |r| <= 1/128 and ln(1 + r) from its Taylor series through r^9 (truncation
// below 2^-60 relative).  ln c_j and ln 2 come in high and low parts
// (gx_log_table.cuh, from 60-digit arithmetic).  About an ulp; 14 FP64-pipe
// instructions against ~30 for the library log.  Zero, negative, subnormal,
// infinite and NaN arguments go to the library.
__device__ __forceinline__ double log_f(double x) {
    const int hi = __double2hiint(x), lo = __double2loint(x);
    if (hi < 0x00100000 || hi >= 0x7ff00000) return log(x);
    const int k = (hi >> 20) - 1023;
    const int mant = hi & 0x000fffff;
    const int j = (mant + (1 << 13)) >> 14;  // nearest multiple of 1/64
    const double m = __hiloint2double(0x3ff00000 | mant, lo);
    const double c = __hiloint2double(0x3ff00000 + (j << 14), 0);
    const double r = (m - c) * __ldg(&LOG_TAB[j][0]);
    // ln(1 + r) = r (1 - r/2 + r^2/3 - ... + r^8/9)
    double p = 1.0 / 9;
    p = fma(p, r, -1.0 / 8);
    p = fma(p, r, 1.0 / 7);
    p = fma(p, r, -1.0 / 6);
    p = fma(p, r, 1.0 / 5);
    p = fma(p, r, -1.0 / 4);
    p = fma(p, r, 1.0 / 3);
    p = fma(p, r, -0.5);
    const double l1r = fma(p * r, r, r);
    // k as a double from its bits (2^52 + 2^31 + k, minus the offset)
    const double kd = __hiloint2double(0x43300000, (int)(0x80000000u ^ (unsigned)k)) - 4503601774854144.0;
    const double lo_part = fma(kd, LN2_LO, __ldg(&LOG_TAB[j][2]) + l1r);
    return fma(kd, LN2_HI, __ldg(&LOG_TAB[j][1])) + lo_part;
}

__device__ __forceinline__ double norm3_sq_f(const double *q) { return fma(q[0], q[0], fma(q[1], q[1], q[2] * q[2])); }

// Gradient of one component accumulated into g; the same cases and gala
// references as comp_gradient in gx_device.cuh.
template <bool SCF, typename PV>
__device__ __forceinline__ void comp_gradient_f(const PV &pot, int ci, const double *q, double *g) {
    const DevComp &C = pot.c[ci];
    const int type = C.type;
#define P(k) GX_PARAM(pot, ci, k)
    double fac;
    switch (type) {
    case GX_POT_NULL:
        return;
    case GX_POT_KEPLER: {
        const double r = sqrt_f(norm3_sq_f(q));
        fac = C.dc[0] * rcp_f(r * r * r);
        break;
    }
    case GX_POT_HERNQUIST: {
        const double r = sqrt_f(norm3_sq_f(q));
        const double rc = r + P(2);
        fac = C.dc[0] * rcp_f(rc * rc * r);
        break;
    }
    case GX_POT_PLUMMER: {
        const double R2b = norm3_sq_f(q) + C.dc[1];
        fac = C.dc[0] * rcp_f(R2b * sqrt_f(R2b));
        break;
    }
    case GX_POT_MIYAMOTONAGAI: {
        const double sqrtz = sqrt_f(fma(q[2], q[2], C.dc[1]));
        const double zd = P(2) + sqrtz;
        const double W = fma(q[0], q[0], fma(q[1], q[1], zd * zd));
        fac = C.dc[0] * rcp_f(W * sqrt_f(W));
        g[0] = fma(fac, q[0], g[0]);
        g[1] = fma(fac, q[1], g[1]);
        g[2] = fma(fac * q[2], fma(P(2), rcp_f(sqrtz), 1.), g[2]);
        return;
    }
    case GX_POT_SPHERICALNFW:
    case GX_POT_FLATTENEDNFW:
    case GX_POT_TRIAXIALNFW: {
        // gala: v_h^2 / u^3 / r_s^2 (log(1 + u) - u / (1 + u)) with v_h^2 = G m / r_s
        // and u = m_r / r_s, m_r the (scaled) radius: G m / m_r^3 (...)
        const bool sph = type == GX_POT_SPHERICALNFW;
        const double mr2 = sph ? norm3_sq_f(q)
                               : fma(q[0] * q[0], C.dc[2], fma(q[1] * q[1], C.dc[3], q[2] * q[2] * C.dc[4]));
        const double mr = sqrt_f(mr2);
        const double u = mr * C.dc[1];
        const double mr3 = mr2 * mr, u1 = 1. + u;
        const double R = rcp_f(mr3 * u1);  // 1 / (m_r^3 (1 + u))
        fac = C.dc[0] * (u1 * R) * fma(-u, mr3 * R, log_f(u1));
        if (sph) break;
        g[0] = fma(fac * C.dc[2], q[0], g[0]);
        g[1] = fma(fac * C.dc[3], q[1], g[1]);
        g[2] = fma(fac * C.dc[4], q[2], g[2]);
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
    g[0] = fma(fac, q[0], g[0]);
    g[1] = fma(fac, q[1], g[1]);
    g[2] = fma(fac, q[2], g[2]);
#undef P
}

template <bool SCF, typename PV>
__device__ __forceinline__ void potential_gradient_ft(const PV &pot, const double *q, double *g) {
    g[0] = 0.; g[1] = 0.; g[2] = 0.;
    for (int i = 0; i < pot.ncomp; i++) {
        if (pot.c[i].do_sr == 0) {
            comp_gradient_f<SCF>(pot, i, q, g);
        } else {
            const DevComp &c = pot.c[i];
            double qt[3], gt[3] = {0., 0., 0.};
            shift_rotate(c, q, qt);
            comp_gradient_f<SCF>(pot, i, qt, gt);
            g[0] += fma(c.R[0], gt[0], fma(c.R[3], gt[1], c.R[6] * gt[2]));
            g[1] += fma(c.R[1], gt[0], fma(c.R[4], gt[1], c.R[7] * gt[2]));
            g[2] += fma(c.R[2], gt[0], fma(c.R[5], gt[1], c.R[8] * gt[2]));
        }
    }
}

// A large composite (device component table) takes gala's own expressions: the
// lean forms' ulp-level differences, summed over hundreds of components, would
// exceed the 1e-12 orbit parity that DOP853 holds with a few components.
template <bool SCF>
__device__ __forceinline__ void potential_gradient_f(const DevPot &pot, const double *q, double *g) {
    if (pot.cdev) {
        potential_gradient_t<SCF>(table_view(pot), q, g);
        return;
    }
    potential_gradient_ft<SCF>(pot, q, g);
}

// Hamilton's equations (hamiltonian_rhs in gx_device.cuh) with the fast force.
template <bool SCF>
__device__ __noinline__ V6 rhs_call_f(const DevPot &pot, const DevFrame &fr, V6 w) {
    double g[3];
    potential_gradient_f<SCF>(pot, w.v, g);
    V6 f;
    if (fr.type == GX_FRAME_STATIC) {
        f.v[0] = w.v[3];
        f.v[1] = w.v[4];
        f.v[2] = w.v[5];
        f.v[3] = -g[0];
        f.v[4] = -g[1];
        f.v[5] = -g[2];
    } else {
        const double *O = fr.O;
        f.v[0] = w.v[3] - fma(O[1], w.v[2], -O[2] * w.v[1]);
        f.v[1] = w.v[4] - fma(-O[0], w.v[2], O[2] * w.v[0]);
        f.v[2] = w.v[5] - fma(O[0], w.v[1], -O[1] * w.v[0]);
        f.v[3] = -(g[0] + fma(O[1], w.v[5], -O[2] * w.v[4]));
        f.v[4] = -(g[1] + fma(-O[0], w.v[5], O[2] * w.v[3]));
        f.v[5] = -(g[2] + fma(O[0], w.v[4], -O[1] * w.v[3]));
    }
    return f;
}

}  // namespace fast
}  // namespace gx
