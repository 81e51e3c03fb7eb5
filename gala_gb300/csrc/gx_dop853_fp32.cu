// gx_dop853_fp32.cu -- DOP853 with FP32 stages and forces, FP64 step control.
//
// The same Dormand-Prince 8(5,3) method as gala's dopcor (dopri/dop853.cpp:
// 89-650) with per-orbit step control (gala's dop853_helper with nbatch = 1:
// every orbit is its own 6-component system), arranged for the GB300's 64:1
// FP32:FP64 throughput:
//   * the twelve stages, the FSAL evaluation, the dense-output stages and the
//     forces are FP32 (the force on the special-function unit, gx_fp32.cuh);
//   * the state is a double-float pair (hi + lo, both FP32) advanced with an
//     exact two-sum, and the product h * k contributes its exact FMA residue,
//     so rounding of the state does not accumulate over 1e4-1e5 steps;
//   * FP64 is kept for the time accumulator x, the step size h, the error
//     norm's final combination err = |h| err sqrt(1 / (deno n)) (:441-444, in
//     the equivalent form h^2 err^2 <= deno n for accept/reject) and the step
//     limits; h is kept FP32-representable (except on the final step to xend)
//     so the FP32 stages and the FP64 clock use the same step;
//   * dense output (contd8, :869-904) is evaluated as an FP32 increment over
//     the double-float state at the start of the step, stored as FP64.
// One thread integrates one orbit; threads take orbits from a queue counter
// one at a time, in the caller's order (orbits of similar cost next to each
// other keep the lanes of a warp busy together), so a thread that finishes its
// orbit starts the next while the rest of its warp keeps stepping.  Every loop
// is bounded by nmax.
#include "gx_host.h"
#include "gx_fp32.cuh"
#include "gx_scf.cuh"
#include "gx_dop853_tableau.cuh"

namespace gx {

int pack_potential_f32(const gx_potential *pot, DevPotF *out);

struct Dop32Args {
    double atol, rtol, dt_max;
    int64_t nmax, nstiff, ntimes, out_stride, n_out, n;
    int32_t save_all, pad;
    float O[3];   // rotating-frame angular velocity (ROT kernels)
    float pad2;
    const int32_t *cancel;  // host cancel flag (mapped memory) or nullptr
};

// s + e = a + b exactly (Knuth's two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (hi, lo) <- (yh, yl) + h * k as a double-float, with the exact residue of
// the FP32 product h * k.
__device__ __forceinline__ void df_axpy(float yh, float yl, float h, float k, float &hi, float &lo) {
    const float d = __fmul_rn(h, k);
    const float dr = __fmaf_rn(h, k, -d);
    float s, e;
    two_sum(yh, d, s, e);
    const float l = __fadd_rn(yl, __fadd_rn(e, dr));
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

__device__ __forceinline__ void split_d(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

__device__ __forceinline__ float ex2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Hamiltonian right-hand side in FP32: static frame, or constant rotation O
// (builtin_frames.cpp:73-112).
template <typename S, bool ROT>
__device__ __forceinline__ void rhs32(const DevPotF &pot, const float *O, const float *w, float *f) {
    float g[3];
    potential_gradient_f<S>(pot, w, g);
    if constexpr (!ROT) {
        f[0] = w[3]; f[1] = w[4]; f[2] = w[5];
        f[3] = -g[0]; f[4] = -g[1]; f[5] = -g[2];
    } else {
        f[0] = w[3] - (O[1] * w[2] - O[2] * w[1]);
        f[1] = w[4] - (-O[0] * w[2] + O[2] * w[0]);
        f[2] = w[5] - (O[0] * w[1] - O[1] * w[0]);
        f[3] = -(g[0] + (O[1] * w[5] - O[2] * w[4]));
        f[4] = -(g[1] + (-O[0] * w[5] + O[2] * w[3]));
        f[5] = -(g[2] + (O[0] * w[4] - O[1] * w[3]));
    }
}

#define F32(c) ((float)(dop::c))

// Four CTAs per SM (128 registers) for the compiled potential signatures, three
// for the run-time component loop, which needs more registers.
template <typename S, bool ROT>
__global__ void __launch_bounds__(128, S::generic ? 3 : 4)
dop853_fp32_kernel(const __grid_constant__ DevPotF pot, const Dop32Args A, const double *__restrict__ w0,
                   const double *__restrict__ t, const int32_t *__restrict__ order, double *__restrict__ out,
                   int32_t *__restrict__ status, int64_t *__restrict__ stats, int32_t *__restrict__ counter) {
    const int64_t n = A.n;
    const double x0 = t[0], xend = t[A.ntimes - 1];
    const double posneg = (xend - x0 < 0.0) ? -1.0 : 1.0;
    double hmax = (A.dt_max == 0.0) ? xend - x0 : A.dt_max;
    hmax = fabs(hmax);
    const float hmaxf = (float)hmax;
    const int64_t nmax = A.nmax ? A.nmax : 1000000;
    const int64_t nstiff = A.nstiff == 0 ? 1000 : (A.nstiff < 0 ? nmax + 10 : A.nstiff);
    const float atol = (float)A.atol, rtol = (float)A.rtol;
    const double uround = 2.220446049250313e-16;
    const float safe = 0.9f, facc1 = 1.0f / 0.333f, facc2 = 1.0f / 6.0f;
    const float *O = A.O;

    float yh[6], yl[6], k1[6], k2[6], k3[6], k4[6], k5[6], k5l[6], k6[6], k7[6], k8[6], k9[6], k10[6], yy1[6];
    double x = 0.0, h = 0.0;
    float hlamb = 0.f;
    int last = 0, reject = 0, iasti = 0, nonsti = 0, idid = 0;
    int64_t nfcn = 0, nstep = 0, naccpt = 0, nrejct = 0, out_idx = 0, out_slot = 0;
    int64_t i = 0;
    bool need = true;

    for (;;) {
        if (need) {
            if (cancel_requested(A.cancel)) break;  // no further orbit once cancelled
            const int64_t k = atomicAdd(counter, 1);
            if (k >= n) break;
            i = order ? (int64_t)order[k] : k;
            // an order entry outside [0, n) is skipped (and recorded in the debug build)
            if (!GX_DBG_CHECK(i >= 0 && i < n, DBG_ORDER, i, n)) continue;
            need = false;
            for (int c = 0; c < 6; c++) split_d(w0[c * n + i], yh[c], yl[c]);
            x = x0;
            h = t[1] - t[0];
            last = reject = iasti = nonsti = idid = 0;
            hlamb = 0.f;
            nfcn = nstep = naccpt = nrejct = 0;
            out_idx = out_slot = 0;
            if (A.save_all) {
                // t[0] is the first output time: the initial state, exactly
                for (int c = 0; c < 6; c++) __stcs(&out[(int64_t)c * A.n_out * n + i], w0[c * n + i]);
                out_idx = out_slot = 1;
            }
            rhs32<S, ROT>(pot, O, yh, k1);
            if (h == 0.0) {
                // hinit (dop853.cpp:18-86) on this orbit's 6 components
                float dnf = 0.f, dny = 0.f;
                for (int c = 0; c < 6; c++) {
                    const float isk = rcp_approx(fmaf(rtol, fabsf(yh[c]), atol));
                    dnf = fmaf(k1[c] * isk, k1[c] * isk, dnf);
                    dny = fmaf(yh[c] * isk, yh[c] * isk, dny);
                }
                double hh = ((dnf <= 1.0E-10f) || (dny <= 1.0E-10f)) ? 1.0E-6 : sqrt((double)dny / dnf) * 0.01;
                hh = fmin(hh, hmax);
                hh = posneg * fabs(hh);
                const float hhf = (float)hh;
                for (int c = 0; c < 6; c++) yy1[c] = fmaf(hhf, k1[c], yh[c]);
                rhs32<S, ROT>(pot, O, yy1, k2);
                float der2 = 0.f;
                for (int c = 0; c < 6; c++) {
                    const float isk = rcp_approx(fmaf(rtol, fabsf(yh[c]), atol));
                    const float sq = (k2[c] - k1[c]) * isk;
                    der2 = fmaf(sq, sq, der2);
                }
                const double d2 = sqrt((double)der2) / fabs(hh);
                const double der12 = fmax(fabs(d2), sqrt((double)dnf));
                const double h1 = (der12 <= 1.0E-15) ? fmax(1.0E-6, fabs(hh) * 1.0E-3) : pow(0.01 / der12, 1.0 / 8.0);
                hh = fmin(100.0 * fabs(hh), fmin(h1, hmax));
                h = posneg * hh;
            }
            h = (double)(float)h;
            nfcn += 2;
        }

        // ---------------------------------------------------------------- step
        bool done = false;
        if (nstep > nmax || !(fabsf((float)h) <= 3.0e38f)) {
            idid = -2;
            done = true;
        } else if (0.1 * fabs(h) <= fabs(x) * uround) {
            idid = -3;
            done = true;
        } else {
            if ((x + 1.01 * h - xend) * posneg > 0.0) {
                h = xend - x;
                last = 1;
            }
            const double xold = x, hout = h;
            nstep++;
            const float hf = (float)h;

            // the twelve stages (dop853.cpp:368-414): FP32 sums of h a_ij k_j
            // added to the double-float state; the forces see the FP32 sum
#define GX_STAGE(dst, expr)                                                    \
    for (int c = 0; c < 6; c++) yy1[c] = __fadd_rn(yh[c], __fmaf_rn(hf, (expr), yl[c])); \
    rhs32<S, ROT>(pot, O, yy1, dst)
            GX_STAGE(k2, F32(a21) * k1[c]);
            GX_STAGE(k3, fmaf(F32(a32), k2[c], F32(a31) * k1[c]));
            GX_STAGE(k4, fmaf(F32(a43), k3[c], F32(a41) * k1[c]));
            GX_STAGE(k5, fmaf(F32(a54), k4[c], fmaf(F32(a53), k3[c], F32(a51) * k1[c])));
            GX_STAGE(k6, fmaf(F32(a65), k5[c], fmaf(F32(a64), k4[c], F32(a61) * k1[c])));
            GX_STAGE(k7, fmaf(F32(a76), k6[c], fmaf(F32(a75), k5[c], fmaf(F32(a74), k4[c], F32(a71) * k1[c]))));
            GX_STAGE(k8, fmaf(F32(a87), k7[c], fmaf(F32(a86), k6[c], fmaf(F32(a85), k5[c],
                         fmaf(F32(a84), k4[c], F32(a81) * k1[c])))));
            GX_STAGE(k9, fmaf(F32(a98), k8[c], fmaf(F32(a97), k7[c], fmaf(F32(a96), k6[c], fmaf(F32(a95), k5[c],
                         fmaf(F32(a94), k4[c], F32(a91) * k1[c]))))));
            GX_STAGE(k10, fmaf(F32(a109), k9[c], fmaf(F32(a108), k8[c], fmaf(F32(a107), k7[c],
                          fmaf(F32(a106), k6[c], fmaf(F32(a105), k5[c], fmaf(F32(a104), k4[c],
                          F32(a101) * k1[c])))))));
            GX_STAGE(k2, fmaf(F32(a1110), k10[c], fmaf(F32(a119), k9[c], fmaf(F32(a118), k8[c],
                         fmaf(F32(a117), k7[c], fmaf(F32(a116), k6[c], fmaf(F32(a115), k5[c],
                         fmaf(F32(a114), k4[c], F32(a111) * k1[c]))))))));
            GX_STAGE(k3, fmaf(F32(a1211), k2[c], fmaf(F32(a1210), k10[c], fmaf(F32(a129), k9[c],
                         fmaf(F32(a128), k8[c], fmaf(F32(a127), k7[c], fmaf(F32(a126), k6[c],
                         fmaf(F32(a125), k5[c], fmaf(F32(a124), k4[c], F32(a121) * k1[c])))))))));
            nfcn += 11;
            // 8th-order solution: k4 = sum b_i k_i, (k5, k5l) = y + h k4
            for (int c = 0; c < 6; c++) {
                k4[c] = fmaf(F32(b12), k3[c], fmaf(F32(b11), k2[c], fmaf(F32(b10), k10[c], fmaf(F32(b9), k9[c],
                        fmaf(F32(b8), k8[c], fmaf(F32(b7), k7[c], fmaf(F32(b6), k6[c], F32(b1) * k1[c])))))));
                df_axpy(yh[c], yl[c], hf, k4[c], k5[c], k5l[c]);
            }

            // error estimation (:416-444): per-component terms in FP32, the
            // norm's combination and the accept test in FP64
            float e1 = 0.f, e2 = 0.f;
            for (int c = 0; c < 6; c++) {
                const float isk = rcp_approx(fmaf(rtol, fmaxf(fabsf(yh[c]), fabsf(k5[c])), atol));
                float erri = k4[c] - F32(bhh1) * k1[c] - F32(bhh2) * k9[c] - F32(bhh3) * k3[c];
                float sq = erri * isk;
                e2 = fmaf(sq, sq, e2);
                erri = fmaf(F32(er12), k3[c], fmaf(F32(er11), k2[c], fmaf(F32(er10), k10[c], fmaf(F32(er9), k9[c],
                       fmaf(F32(er8), k8[c], fmaf(F32(er7), k7[c], fmaf(F32(er6), k6[c], F32(er1) * k1[c])))))));
                sq = erri * isk;
                e1 = fmaf(sq, sq, e1);
            }
            double deno = fma(0.01, (double)e2, (double)e1);
            if (deno <= 0.0) deno = 1.0;
            // err = |h| e1 / sqrt(deno n), n = 6: accept iff err^2 = h^2 e1^2 / (deno n) <= 1
            const double he = h * (double)e1;
            const bool acc = fma(he, he, -6.0 * deno) <= 0.0;
            // fac11 = err^(1/8) = (err^2)^(1/16) and the new step: step-size
            // factors, FP32 (h stays FP32-representable)
            float denof = fmaf(0.01f, e2, e1);
            if (denof <= 0.f) denof = 1.f;
            const float hef = hf * e1;
            const float ratio = hef * hef * rcp_approx(6.0f * denof);
            const float fac11 = ex2_approx(lg2_approx(ratio) * 0.0625f);
            const float fac = fmaxf(facc2, fminf(facc1, fac11 / safe));
            float hnew = hf * rcp_approx(fac);

            if (acc) {
                naccpt++;
                rhs32<S, ROT>(pot, O, k5, k4);   // FSAL: f at the new state
                nfcn++;
                // stiffness detection (:463-486); the first detection returns -4.
                // gala estimates h |df/dy| from the last stage point and the new
                // state, which agree to the local error: below FP32 resolution, so
                // in FP32 that quotient is rounding noise.  The same estimate is
                // formed here over the whole step, from f and y at its two ends
                // (the difference of the double-float states is exact enough).
                if (!(naccpt % nstiff) || iasti > 0) {
                    float stnum = 0.f, stden = 0.f;
                    for (int c = 0; c < 6; c++) {
                        float d = k4[c] - k1[c];
                        stnum = fmaf(d, d, stnum);
                        d = __fsub_rn(k5[c], yh[c]) + __fsub_rn(k5l[c], yl[c]);
                        stden = fmaf(d, d, stden);
                    }
                    if (stden > 0.f) hlamb = hf * sqrtf(stnum / stden);
                    if (hlamb > 6.1f) {
                        nonsti = 0;
                        iasti++;
                        idid = -4;
                        done = true;
                    } else {
                        nonsti++;
                        if (nonsti == 6) iasti = 0;
                    }
                }
            }
            if (acc && !done) {
                // output times inside [xold, xold + hout] (:584-612); every
                // out_stride-th is stored, from the dense-output polynomial
                int64_t out_end = out_idx, first_kept = 0;
                if (A.save_all) {
                    const double xa = xold, xb = xold + hout;
                    while (out_end < A.ntimes) {
                        const double to = t[out_end];
                        if (!((xa <= to && to <= xb) || (xb <= to && to <= xa))) break;
                        out_end++;
                    }
                    first_kept = (out_idx + A.out_stride - 1) / A.out_stride * A.out_stride;
                }
                if (A.save_all && first_kept < out_end) {
                    float r5[6], r6[6], r7[6], r8[6];
#define GX_D8(p, c)                                                                                           \
    fmaf(F32(p##12), k3[c], fmaf(F32(p##11), k2[c], fmaf(F32(p##10), k10[c], fmaf(F32(p##9), k9[c],           \
         fmaf(F32(p##8), k8[c], fmaf(F32(p##7), k7[c], fmaf(F32(p##6), k6[c], F32(p##1) * k1[c])))))))
                    for (int c = 0; c < 6; c++) {
                        r5[c] = GX_D8(d4, c);
                        r6[c] = GX_D8(d5, c);
                        r7[c] = GX_D8(d6, c);
                        r8[c] = GX_D8(d7, c);
                    }
#undef GX_D8
                    GX_STAGE(k10, fmaf(F32(a1413), k4[c], fmaf(F32(a1412), k3[c], fmaf(F32(a1411), k2[c],
                                  fmaf(F32(a1410), k10[c], fmaf(F32(a149), k9[c], fmaf(F32(a148), k8[c],
                                  fmaf(F32(a147), k7[c], F32(a141) * k1[c]))))))));
                    GX_STAGE(k2, fmaf(F32(a1514), k10[c], fmaf(F32(a1513), k4[c], fmaf(F32(a1512), k3[c],
                                 fmaf(F32(a1511), k2[c], fmaf(F32(a158), k8[c], fmaf(F32(a157), k7[c],
                                 fmaf(F32(a156), k6[c], F32(a151) * k1[c]))))))));
                    GX_STAGE(k3, fmaf(F32(a1615), k2[c], fmaf(F32(a1614), k10[c], fmaf(F32(a1613), k4[c],
                                 fmaf(F32(a169), k9[c], fmaf(F32(a168), k8[c], fmaf(F32(a167), k7[c],
                                 fmaf(F32(a166), k6[c], F32(a161) * k1[c]))))))));
                    nfcn += 3;
                    float r2[6], r3[6], r4[6];
                    for (int c = 0; c < 6; c++) {
                        r5[c] = hf * fmaf(F32(d416), k3[c], fmaf(F32(d415), k2[c], fmaf(F32(d414), k10[c],
                                     fmaf(F32(d413), k4[c], r5[c]))));
                        r6[c] = hf * fmaf(F32(d516), k3[c], fmaf(F32(d515), k2[c], fmaf(F32(d514), k10[c],
                                     fmaf(F32(d513), k4[c], r6[c]))));
                        r7[c] = hf * fmaf(F32(d616), k3[c], fmaf(F32(d615), k2[c], fmaf(F32(d614), k10[c],
                                     fmaf(F32(d613), k4[c], r7[c]))));
                        r8[c] = hf * fmaf(F32(d716), k3[c], fmaf(F32(d715), k2[c], fmaf(F32(d714), k10[c],
                                     fmaf(F32(d713), k4[c], r8[c]))));
                        // ydiff = y_new - y_old from the double-float pairs
                        const float ydiff = __fsub_rn(k5[c], yh[c]) + __fsub_rn(k5l[c], yl[c]);
                        r2[c] = ydiff;
                        const float bspl = fmaf(hf, k1[c], -ydiff);
                        r3[c] = bspl;
                        r4[c] = fmaf(-hf, k4[c], ydiff) - bspl;
                    }
                    const float ihout = rcp_approx((float)hout);
                    for (int64_t oi = first_kept; oi < out_end; oi += A.out_stride) {
                        const float s = (float)(t[oi] - xold) * ihout;
                        const float s1 = 1.0f - s;
                        for (int c = 0; c < 6; c++) {
                            const float inc =
                                s * fmaf(s1, fmaf(s, fmaf(s1, fmaf(s, fmaf(s1, fmaf(s, r8[c], r7[c]), r6[c]), r5[c]),
                                                     r4[c]), r3[c]), r2[c]);
                            const double v = (double)yh[c] + ((double)yl[c] + (double)inc);
                            __stcs(&out[((int64_t)c * A.n_out + out_slot) * n + i], v);
                        }
                        out_slot++;
                    }
                }
                out_idx = out_end;
                for (int c = 0; c < 6; c++) {
                    k1[c] = k4[c];
                    yh[c] = k5[c];
                    yl[c] = k5l[c];
                }
                x = xold + hout;
                if (last) {
                    idid = 1;
                    done = true;
                } else {
                    if (fabsf(hnew) > hmaxf) hnew = copysignf(hmaxf, hf);
                    if (reject) hnew = copysignf(fminf(fabsf(hnew), fabsf(hf)), hf);
                    reject = 0;
                }
            } else if (!acc) {
                hnew = hf * rcp_approx(fminf(facc1, fac11 / safe));
                reject = 1;
                if (naccpt >= 1) nrejct++;
                last = 0;
            }
            if (!done) h = (double)hnew;
        }
#undef GX_STAGE

        if (done) {
            if (!A.save_all)
                for (int c = 0; c < 6; c++) out[c * n + i] = (double)yh[c] + (double)yl[c];
            status[i] = idid;
            GX_DBG_DONE(i, nstep);
            if (stats) {
                stats[4 * i + 0] = nfcn;
                stats[4 * i + 1] = nstep;
                stats[4 * i + 2] = naccpt;
                stats[4 * i + 3] = nrejct;
            }
            need = true;
        }
    }
}
#undef F32

template <typename S, bool ROT>
static int launch_one(const DevPotF &dp, const Dop32Args &A, const double *w0, const double *t, const int32_t *order,
                      double *out, int32_t *status, int64_t *stats, int32_t *counter, cudaStream_t st) {
    constexpr int block = 128;
    int sms = 0, dev = 0, occ = 0;
    GX_CUDA_TRY(cudaGetDevice(&dev));
    GX_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dop853_fp32_kernel<S, ROT>, block, 0));
    // one resident wave of threads; each thread takes orbits from the queue
    const int64_t want = (A.n + block - 1) / block;
    const int64_t cap = (int64_t)sms * (occ > 0 ? occ : 1);
    const unsigned grid = (unsigned)(want < cap ? want : cap);
    dop853_fp32_kernel<S, ROT><<<grid, block, 0, st>>>(dp, A, w0, t, order, out, status, stats, counter);
    return check_launch("dop853_fp32");
}

static int launch_dop853_fp32(const DevPotF &dp, bool rotating, const Dop32Args &A, const double *w0,
                              const double *t, const int32_t *order, double *out, int32_t *status, int64_t *stats,
                              int32_t *counter, cudaStream_t st) {
    auto is = [&](int a, int b, int c, int d) {
        const int want_t[4] = {a, b, c, d};
        int nc = 0;
        for (int k = 0; k < 4; k++) nc += want_t[k] >= 0;
        if (dp.ncomp != nc) return false;
        for (int k = 0; k < nc; k++)
            if (dp.c[k].type != want_t[k] || dp.c[k].do_sr) return false;
        return true;
    };
    constexpr int H = GX_POT_HERNQUIST, MN = GX_POT_MIYAMOTONAGAI, NFW = GX_POT_SPHERICALNFW, P = GX_POT_PLUMMER;
    if (rotating) return launch_one<SigGeneric, true>(dp, A, w0, t, order, out, status, stats, counter, st);
    if (is(H, H, MN, NFW))
        return launch_one<PotSig<H, H, MN, NFW>, false>(dp, A, w0, t, order, out, status, stats, counter, st);
    if (is(H, -1, -1, -1))
        return launch_one<PotSig<H, -1, -1, -1>, false>(dp, A, w0, t, order, out, status, stats, counter, st);
    if (is(P, -1, -1, -1))
        return launch_one<PotSig<P, -1, -1, -1>, false>(dp, A, w0, t, order, out, status, stats, counter, st);
    return launch_one<SigGeneric, false>(dp, A, w0, t, order, out, status, stats, counter, st);
}

}  // namespace gx

extern "C" int gx_dop853_fp32(const gx_potential *pot, const gx_frame *frame, const double *w0, int64_t n,
                              const double *t, int64_t ntimes, double atol, double rtol, int64_t nmax,
                              double dt_max, int64_t nstiff, int32_t save_all, int64_t out_stride,
                              const int32_t *order, double *w_out, int32_t *status, int64_t *stats,
                              int32_t *queue_counter, void *stream) {
    gx::DevPotF dp;
    int rc = gx::pack_potential_f32(pot, &dp);
    if (rc) return rc;
    gx::DevFrame df;
    rc = gx::pack_frame(frame, &df);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0 && n < (int64_t)INT32_MAX, "n out of range");
    GX_CHECK_ARG(ntimes >= 2, "ntimes must be >= 2 (got %lld)", (long long)ntimes);
    GX_CHECK_ARG(out_stride >= 1, "out_stride must be >= 1");
    GX_CHECK_ARG(nmax >= 0, "nmax must be >= 0 (0 = gala's default 1e6)");
    GX_CHECK_ARG(atol >= 0 && rtol >= 0, "tolerances must be non-negative");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(w0 && t && w_out && status && queue_counter, "NULL array");
    gx::Dop32Args A;
    memset(&A, 0, sizeof(A));
    A.atol = atol;
    A.rtol = rtol;
    A.dt_max = dt_max;
    A.nmax = nmax;
    A.nstiff = nstiff;
    A.ntimes = ntimes;
    A.out_stride = out_stride;
    A.n_out = (ntimes - 1) / out_stride + 1;
    A.n = n;
    A.save_all = save_all ? 1 : 0;
    const bool rotating = df.type != GX_FRAME_STATIC;
    for (int k = 0; k < 3; k++) A.O[k] = (float)df.O[k];
    A.cancel = gx::cancel_flag();
    cudaStream_t st = gx::as_stream(stream);
    GX_CUDA_TRY(cudaMemsetAsync(queue_counter, 0, sizeof(int32_t), st));
    return gx::launch_dop853_fp32(dp, rotating, A, w0, t, order, w_out, status, stats, queue_counter, st);
}
