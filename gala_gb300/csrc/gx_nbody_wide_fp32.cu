// gx_nbody_wide_fp32.cu -- the animate mode of mock streams with FP32 stages and
// forces and FP64 step control (the FP32 form of gx_mockstream_dop853_animate).
//
// The computation is mockstream_dop853_animate's (src/gala/dynamics/mockstream/
// mockstream.pyx:306-440): per stream one system of the bodies and every
// particle released so far, stepped interval by interval over the orbit grid by
// dop853_step (dop853.pyx:27-75 -> dopcor, dopri/dop853.cpp:89-650), growing
// after each interval.  GPU mapping as gx_nbody_wide.cu (one CTA per stream,
// the state in device scratch, two passes per stage, fixed-order CTA sums);
// arithmetic as gx_nbody_fp32.cu:
//   * stages, forces (external and the bodies' pulls) and stage sums in FP32;
//   * the state a double-float pair; a stage argument is the state's high part
//     plus an FP32 offset (low part + h * sum a_ij k_j), and a particle-body
//     separation is (hi_p - hi_b) + (offset_p - offset_b);
//   * FP64 for the time, the step size (kept FP32-representable), the error
//     norm's combination (accept iff h^2 E1^2 <= deno n, E1 and E2 summed in
//     FP64 from FP32 partials) and accept/reject;
//   * stiffness after every accepted step (dop853_step's nstiff = 1) estimated
//     over the whole step, as in the other FP32 forms.
// Not bit-compatible with gala; tolerances below ~1e-8 relative only shrink the
// steps.  Static frames only.
#include "gx_host.h"
#include "gx_body_f32.cuh"
#include "gx_fp32.cuh"
#include "gx_dop853_tableau.cuh"

namespace gx {

int pack_potential_f32(const gx_potential *pot, DevPotF *out);

constexpr int AF_THREADS = 256;
constexpr int AF_MAXNB = 32;  // massive bodies per system

// FP32 scratch arrays per stream, each 6 x M: the state (hi, lo), the stage
// derivatives, the new state's low part and the stage-argument offsets.
enum { F_YH = 0, F_YL, F_K1, F_K2, F_K3, F_K4, F_K5, F_K5L, F_K6, F_K7, F_K8, F_K9, F_K10, F_OFF, F_NARR };

struct AnimF32Args {
    int32_t nbody;
    int64_t n_streams, ntimes, n_particles, M;  // M = nbody + n_particles members per stream
    const gx_body *bodies;     // (n_streams, nbody)
    const double *nbody_w0;    // (n_streams, nbody, 6) at t[0]
    const double *t;           // (ntimes)
    const int32_t *nstream;    // (ntimes), summing to n_particles
    const double *stream_w0;   // (n_streams, n_particles, 6) in release order
    int64_t output_every, n_output;
    double dt0, atol, rtol;
    int64_t nmax;
    float *scratch;            // n_streams x F_NARR x 6 x M floats
    double *snap;              // (n_streams, 6, n_output, M) or NULL
    double *w_out;             // (n_streams, M, 6)
    int32_t *status;           // (n_streams, ntimes)
    int64_t *stats;            // (n_streams, 4) or NULL
    const int32_t *cancel;     // host cancel flag (mapped memory) or nullptr
};

// The step controller's decisions, made by thread 0 and read by every thread
// after a barrier: the FP64 control (time, step size, error-norm combination,
// accept / reject, stiffness) runs once per step on one thread -- on GB300 a
// warp instruction of the FP64 pipe costs the same whether one lane or all are
// active, so the CTA's other warps issue none.
struct Ctl {
    double h;
    float hf;
    int go;    // take the step
    int acc;   // the step was accepted
    int stop;  // the call ends after this step
    int idid;
};

// Deterministic CTA sums of two FP32 partials: each thread's partials over its
// members in order, an FP32 warp butterfly, then thread 0 adds the warps' sums
// in order in FP64 (only thread 0 receives them).
__device__ __forceinline__ void cta_sum2_f(float a, float b, double &sa, double &sb, float *redf) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
        redf[wid] = a;
        redf[32 + wid] = b;
    }
    __syncthreads();
    sa = 0.;
    sb = 0.;
    if (threadIdx.x == 0)
        for (int w = 0; w < nw; w++) {
            sa += (double)redf[w];
            sb += (double)redf[32 + w];
        }
}

// Fwrapper_direct_nbody (dop853.cpp:990-1006) in FP32 for member m, its
// argument given as (hi, off): Hamilton's equations in the external potential
// at hi + off, then the pull of every non-null massive body j != m at the
// separation (hi_m - hi_j) + (off_m - off_j).
template <typename S>
__device__ __forceinline__ void af_rhs(const DevPotF &pot, const BodyF *bc, int nbody, const float *__restrict__ hi,
                                       const float *__restrict__ off, int64_t M, int m, float *__restrict__ kout) {
    float w[6], g[3];
#pragma unroll
    for (int c = 0; c < 6; c++) w[c] = hi[c * M + m] + off[c * M + m];
    potential_gradient_f<S>(pot, w, g);
    for (int j = 0; j < nbody; j++) {
        if (j == m || bc[j].type == GX_POT_NULL) continue;
        const float d[3] = {(hi[m] - hi[j]) + (off[m] - off[j]),
                            (hi[M + m] - hi[M + j]) + (off[M + m] - off[M + j]),
                            (hi[2 * M + m] - hi[2 * M + j]) + (off[2 * M + m] - off[2 * M + j])};
        body_grad_f32(bc[j], d, g);
    }
    kout[m] = w[3];
    kout[M + m] = w[4];
    kout[2 * M + m] = w[5];
    kout[3 * M + m] = -g[0];
    kout[4 * M + m] = -g[1];
    kout[5 * M + m] = -g[2];
}

#define F32(c) ((float)(dop::c))

// One dop853_step call in the FP32 form on the first nmem members, from x to
// xend with the initial step dt0, run by the whole CTA, the controller on
// thread 0.  Adds {nfcn, nstep, naccpt, nrejct} to thread 0's ctr; returns
// gala's idid (the same on every thread).
template <typename S>
__device__ __forceinline__ int wide_dop853_f32(const DevPotF &pot, const BodyF *bc, int nbody, int nmem, int64_t M,
                                               float *const *Ar, float *redf, Ctl &ctl, double x, const double xend,
                                               const double dt0, const float atol, const float rtol,
                                               const int64_t nmax_in, int64_t *ctr) {
    const int tid = threadIdx.x, nt = blockDim.x;
    __syncthreads();
    for (int m = tid; m < nmem; m += nt) af_rhs<S>(pot, bc, nbody, Ar[F_YH], Ar[F_YL], M, m, Ar[F_K1]);

    // controller state (meaningful on thread 0)
    const double uround = 2.3E-16;
    const int64_t nmax = nmax_in ? nmax_in : 1000000;
    const double hmax = fabs(xend - x);
    const double posneg = (xend - x < 0.0) ? -1.0 : 1.0;
    const float safe = 0.9f, facc1 = 1.0f / 0.333f, facc2 = 1.0f / 6.0f;
    double h = (double)(float)dt0, xold = x;
    float hlamb = 0.f, hnew = 0.f, fac11 = 1.f;
    int last = 0, reject = 0, nonsti = 0;
    int64_t nfcn = 2, nstep = 0, naccpt = 0, nrejct = 0;

#define FSTAGE(dst, expr)                                                                            \
    for (int m = tid; m < nmem; m += nt)                                                             \
        for (int c = 0; c < 6; c++) {                                                                \
            const int64_t o = c * M + m;                                                             \
            Ar[F_OFF][o] = __fmaf_rn(hf, (expr), Ar[F_YL][o]);                                       \
        }                                                                                            \
    __syncthreads();                                                                                 \
    for (int m = tid; m < nmem; m += nt) af_rhs<S>(pot, bc, nbody, Ar[F_YH], Ar[F_OFF], M, m, Ar[dst]); \
    __syncthreads()
#define K(a) Ar[a][o]

    for (;;) {
        if (tid == 0) {
            ctl.go = 1;
            if (nstep > nmax || !(fabsf((float)h) <= 3.0e38f)) {
                ctl.idid = -2;  // a NaN step never recovers: gala's -2 after nmax rejections, at once
                ctl.go = 0;
            } else if (0.1 * fabs(h) <= fabs(x) * uround) {
                ctl.idid = -3;
                ctl.go = 0;
            } else {
                if ((x + 1.01 * h - xend) * posneg > 0.0) {
                    h = xend - x;
                    last = 1;
                }
                xold = x;
                nstep++;
                ctl.h = h;
                ctl.hf = (float)h;
            }
        }
        __syncthreads();
        if (!ctl.go) break;
        const float hf = ctl.hf;
        // the twelve stages (dop853.cpp:368-414) with FP32 stage sums
        FSTAGE(F_K2, F32(a21) * K(F_K1));
        FSTAGE(F_K3, fmaf(F32(a32), K(F_K2), F32(a31) * K(F_K1)));
        FSTAGE(F_K4, fmaf(F32(a43), K(F_K3), F32(a41) * K(F_K1)));
        FSTAGE(F_K5, fmaf(F32(a54), K(F_K4), fmaf(F32(a53), K(F_K3), F32(a51) * K(F_K1))));
        FSTAGE(F_K6, fmaf(F32(a65), K(F_K5), fmaf(F32(a64), K(F_K4), F32(a61) * K(F_K1))));
        FSTAGE(F_K7, fmaf(F32(a76), K(F_K6), fmaf(F32(a75), K(F_K5), fmaf(F32(a74), K(F_K4), F32(a71) * K(F_K1)))));
        FSTAGE(F_K8, fmaf(F32(a87), K(F_K7), fmaf(F32(a86), K(F_K6), fmaf(F32(a85), K(F_K5),
                     fmaf(F32(a84), K(F_K4), F32(a81) * K(F_K1))))));
        FSTAGE(F_K9, fmaf(F32(a98), K(F_K8), fmaf(F32(a97), K(F_K7), fmaf(F32(a96), K(F_K6), fmaf(F32(a95), K(F_K5),
                     fmaf(F32(a94), K(F_K4), F32(a91) * K(F_K1)))))));
        FSTAGE(F_K10, fmaf(F32(a109), K(F_K9), fmaf(F32(a108), K(F_K8), fmaf(F32(a107), K(F_K7),
                      fmaf(F32(a106), K(F_K6), fmaf(F32(a105), K(F_K5), fmaf(F32(a104), K(F_K4),
                      F32(a101) * K(F_K1))))))));
        FSTAGE(F_K2, fmaf(F32(a1110), K(F_K10), fmaf(F32(a119), K(F_K9), fmaf(F32(a118), K(F_K8),
                     fmaf(F32(a117), K(F_K7), fmaf(F32(a116), K(F_K6), fmaf(F32(a115), K(F_K5),
                     fmaf(F32(a114), K(F_K4), F32(a111) * K(F_K1)))))))));
        FSTAGE(F_K3, fmaf(F32(a1211), K(F_K2), fmaf(F32(a1210), K(F_K10), fmaf(F32(a129), K(F_K9),
                     fmaf(F32(a128), K(F_K8), fmaf(F32(a127), K(F_K7), fmaf(F32(a126), K(F_K6),
                     fmaf(F32(a125), K(F_K5), fmaf(F32(a124), K(F_K4), F32(a121) * K(F_K1))))))))));
        // 8th-order solution (k4), new state (k5, k5l) and error terms (:416-444)
        float e1 = 0.f, e2 = 0.f;
        for (int m = tid; m < nmem; m += nt)
            for (int c = 0; c < 6; c++) {
                const int64_t o = c * M + m;
                const float k4 = fmaf(F32(b12), K(F_K3), fmaf(F32(b11), K(F_K2), fmaf(F32(b10), K(F_K10),
                                 fmaf(F32(b9), K(F_K9), fmaf(F32(b8), K(F_K8), fmaf(F32(b7), K(F_K7),
                                 fmaf(F32(b6), K(F_K6), F32(b1) * K(F_K1))))))));
                float k5, k5l;
                df_axpy32(K(F_YH), K(F_YL), hf, k4, k5, k5l);
                const float isk = rcp_approx(fmaf(rtol, fmaxf(fabsf(K(F_YH)), fabsf(k5)), atol));
                float erri = k4 - F32(bhh1) * K(F_K1) - F32(bhh2) * K(F_K9) - F32(bhh3) * K(F_K3);
                float sq = erri * isk;
                e2 = fmaf(sq, sq, e2);
                erri = fmaf(F32(er12), K(F_K3), fmaf(F32(er11), K(F_K2), fmaf(F32(er10), K(F_K10),
                       fmaf(F32(er9), K(F_K9), fmaf(F32(er8), K(F_K8), fmaf(F32(er7), K(F_K7),
                       fmaf(F32(er6), K(F_K6), F32(er1) * K(F_K1))))))));
                sq = erri * isk;
                e1 = fmaf(sq, sq, e1);
                K(F_K4) = k4;
                K(F_K5) = k5;
                K(F_K5L) = k5l;
            }
        double E1, E2;
        cta_sum2_f(e1, e2, E1, E2, redf);
        if (tid == 0) {
            nfcn += 11;
            // err = |h| E1 / sqrt(deno n), n = 6 nmem: accept iff h^2 E1^2 <= deno n
            double deno = fma(0.01, E2, E1);
            if (deno <= 0.0) deno = 1.0;
            const double he = h * E1;
            ctl.acc = fma(he, he, -(double)(6 * nmem) * deno) <= 0.0;
            const float ratio = (float)(he * he / ((double)(6 * nmem) * deno));
            fac11 = ex2_approx32(lg2_approx(ratio) * 0.0625f);  // err^(1/8) = ratio^(1/16)
            const float fac = fmaxf(facc2, fminf(facc1, fac11 / safe));
            hnew = hf * rcp_approx(fac);
        }
        __syncthreads();
        if (ctl.acc) {
            // FSAL: k4 = f(new state); the stiffness estimate over the whole step
            for (int m = tid; m < nmem; m += nt) af_rhs<S>(pot, bc, nbody, Ar[F_K5], Ar[F_K5L], M, m, Ar[F_K4]);
            __syncthreads();
            float tn = 0.f, td = 0.f;
            for (int m = tid; m < nmem; m += nt)
                for (int c = 0; c < 6; c++) {
                    const int64_t o = c * M + m;
                    float d = K(F_K4) - K(F_K1);
                    tn = fmaf(d, d, tn);
                    d = __fsub_rn(K(F_K5), K(F_YH)) + __fsub_rn(K(F_K5L), K(F_YL));
                    td = fmaf(d, d, td);
                }
            double stnum, stden;
            cta_sum2_f(tn, td, stnum, stden, redf);
            if (tid == 0) {
                naccpt++;
                nfcn++;
                if (stden > 0.0) hlamb = hf * (float)sqrt(stnum / stden);
                ctl.stop = 0;
                if (hlamb > 6.1f) {
                    nonsti = 0;
                    ctl.idid = -4;
                    ctl.stop = 1;
                } else {
                    nonsti++;
                    x = xold + h;
                    if (last) {
                        ctl.idid = 1;
                        ctl.stop = 1;
                    } else {
                        if (fabsf(hnew) > (float)hmax) hnew = copysignf((float)hmax, hf);
                        if (reject) hnew = copysignf(fminf(fabsf(hnew), fabsf(hf)), hf);
                        reject = 0;
                        h = (double)hnew;
                    }
                }
            }
            __syncthreads();
            if (ctl.idid == -4 && ctl.stop) break;  // stiff: the state stays that of the last step
            for (int m = tid; m < nmem; m += nt)
                for (int c = 0; c < 6; c++) {
                    const int64_t o = c * M + m;
                    K(F_K1) = K(F_K4);
                    K(F_YH) = K(F_K5);
                    K(F_YL) = K(F_K5L);
                }
            if (ctl.stop) break;
            __syncthreads();
        } else if (tid == 0) {
            hnew = hf * rcp_approx(fminf(facc1, fac11 / safe));
            reject = 1;
            if (naccpt >= 1) nrejct++;
            last = 0;
            h = (double)hnew;
        }
    }
#undef K
#undef FSTAGE
    (void)nonsti;
    __syncthreads();
    const int idid = ctl.idid;
    if (tid == 0) {
        ctr[0] += nfcn;
        ctr[1] += nstep;
        ctr[2] += naccpt;
        ctr[3] += nrejct;
    }
    __syncthreads();
    return idid;
}

template <typename S>
__global__ void __launch_bounds__(AF_THREADS, 1)
animate_f32_kernel(const __grid_constant__ DevPotF pot, const __grid_constant__ AnimF32Args A) {
    __shared__ float redf[64];
    __shared__ Ctl ctl;
    __shared__ BodyF bc[AF_MAXNB];
    const int64_t s = blockIdx.x;
    if (s >= A.n_streams) return;
    const int64_t M = A.M;
    const int nbody = A.nbody;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid < nbody) body_consts_f32(A.bodies + s * nbody + tid, bc[tid]);
    float *base = A.scratch + s * (int64_t)F_NARR * 6 * M;
    float *Ar[F_NARR];
#pragma unroll
    for (int a = 0; a < F_NARR; a++) Ar[a] = base + (int64_t)a * 6 * M;
    // the state at t[0] as double-float pairs: bodies, then every particle
    for (int m = tid; m < M; m += nt) {
        const double *src = (m < nbody) ? A.nbody_w0 + (s * nbody + m) * 6
                                        : A.stream_w0 + (s * A.n_particles + (m - nbody)) * 6;
#pragma unroll
        for (int c = 0; c < 6; c++) {
            const double v = src[c];
            const float hi = (float)v;
            Ar[F_YH][c * M + m] = hi;
            Ar[F_YL][c * M + m] = (float)(v - (double)hi);
        }
    }
    __syncthreads();
    const double qnan = __longlong_as_double(0x7ff8000000000000LL);
    // members beyond the released ones are NaN in a snapshot (the HDF5 fill value)
    auto snapshot = [&](int64_t j, int64_t live) {
        if (!A.snap) return;
        for (int m = tid; m < M; m += nt)
#pragma unroll
            for (int c = 0; c < 6; c++)
                A.snap[((s * 6 + c) * A.n_output + j) * M + m] =
                    (m < live) ? (double)Ar[F_YH][c * M + m] + (double)Ar[F_YL][c * M + m] : qnan;
    };
    // the particles released so far, kept within [0, n_particles] whatever the
    // counts say; an interval whose count breaks the bound reports -1
    auto grow = [&](int64_t n, int64_t i, int &bad) {
        const int64_t k = A.nstream[i];
        bad = (k < 0 || n + k > A.n_particles);
        if (bad && tid == 0) (void)GX_DBG_CHECK(false, DBG_COUNT, i, A.ntimes);
        return bad ? (k < 0 ? n : A.n_particles) : n + k;
    };
    int bad = 0;
    int64_t n = grow(0, 0, bad), j = 0;
    snapshot(j++, nbody + n);
    int64_t ctr[4] = {0, 0, 0, 0};
    if (tid == 0) A.status[s * A.ntimes] = bad ? -1 : 1;
    for (int64_t i = 1; i < A.ntimes; i++) {
        // after cancellation the stream stops between intervals (one reader, CTA-uniform)
        if (__syncthreads_or(tid == 0 && cancel_requested(A.cancel))) {
            for (int64_t k = i + tid; k < A.ntimes; k += nt) A.status[s * A.ntimes + k] = 0;
            while (j < A.n_output) snapshot(j++, 0);  // snapshots not reached: all NaN
            break;
        }
        const int idid = wide_dop853_f32<S>(pot, bc, nbody, (int)(nbody + n), M, Ar, redf, ctl, A.t[i - 1],
                                            A.t[i], A.dt0, (float)A.atol, (float)A.rtol, A.nmax, ctr);
        n = grow(n, i, bad);
        if (tid == 0) A.status[s * A.ntimes + i] = bad ? -1 : idid;
        if (i % A.output_every == 0 || i == A.ntimes - 1) snapshot(j++, nbody + n);
    }
    __syncthreads();
    for (int m = tid; m < M; m += nt)
#pragma unroll
        for (int c = 0; c < 6; c++)
            A.w_out[(s * M + m) * 6 + c] = (double)Ar[F_YH][c * M + m] + (double)Ar[F_YL][c * M + m];
    if (tid == 0 && A.stats)
        for (int q = 0; q < 4; q++) A.stats[4 * s + q] = ctr[q];
}
#undef F32

}  // namespace gx

extern "C" int64_t gx_mockstream_wide_scratch_bytes(int64_t n_systems, int32_t max_members);
extern "C" int64_t gx_mockstream_animate_snapshots(int64_t ntimes, int64_t output_every);

extern "C" int gx_mockstream_dop853_animate_fp32(const gx_potential *pot, int64_t n_streams, int32_t nbody,
                                                 const gx_body *bodies, const double *nbody_w0, int64_t ntimes,
                                                 const double *t, double dt0, const int32_t *nstream,
                                                 const double *stream_w0, int64_t n_particles, int64_t output_every,
                                                 double atol, double rtol, int64_t nmax, double *scratch,
                                                 int64_t scratch_bytes, double *snap, double *w_out, int32_t *status,
                                                 int64_t *stats, void *stream) {
    gx::DevPotF dp;
    int rc = gx::pack_potential_f32(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(n_streams >= 1 && n_particles >= 0, "bad size");
    GX_CHECK_ARG(ntimes >= 2, "the time grid needs at least two points");
    GX_CHECK_ARG(nbody >= 1 && nbody <= gx::AF_MAXNB, "nbody must be in [1, %d] (the progenitor first)",
                 gx::AF_MAXNB);
    GX_CHECK_ARG(output_every >= 1, "output_every must be >= 1");
    GX_CHECK_ARG(nmax >= 0, "nmax must be >= 0 (0 = gala's default 1e6)");
    GX_CHECK_ARG(atol >= 0 && rtol >= 0, "tolerances must be non-negative");
    GX_CHECK_ARG(bodies && nbody_w0 && t && nstream && (stream_w0 || n_particles == 0) && scratch && w_out &&
                     status,
                 "NULL array");
    GX_CHECK_ARG(n_streams <= (int64_t)INT32_MAX && nbody + n_particles <= (int64_t)INT32_MAX, "too large");
    GX_CHECK_ARG(dt0 != 0.0, "dt0 (t[1] - t[0], gala's h0) must be non-zero");
    const int64_t M = nbody + n_particles;
    // the FP64 form's scratch size covers the FP32 arrays
    const int64_t need = gx_mockstream_wide_scratch_bytes(n_streams, (int32_t)M);
    GX_CHECK_ARG(scratch_bytes >= need, "scratch of %lld bytes, %lld needed", (long long)scratch_bytes,
                 (long long)need);
    static_assert(gx::F_NARR * sizeof(float) <= 12 * sizeof(double), "FP32 scratch must fit the FP64 size");
    gx::AnimF32Args A;
    memset(&A, 0, sizeof(A));
    A.nbody = nbody;
    A.n_streams = n_streams;
    A.ntimes = ntimes;
    A.n_particles = n_particles;
    A.M = M;
    A.bodies = bodies;
    A.nbody_w0 = nbody_w0;
    A.t = t;
    A.nstream = nstream;
    A.stream_w0 = stream_w0;
    A.output_every = output_every;
    A.n_output = gx_mockstream_animate_snapshots(ntimes, output_every);
    A.dt0 = dt0;
    A.atol = atol;
    A.rtol = rtol;
    A.nmax = nmax;
    A.scratch = reinterpret_cast<float *>(scratch);
    A.snap = snap;
    A.w_out = w_out;
    A.status = status;
    A.stats = stats;
    A.cancel = gx::cancel_flag();
    cudaStream_t st = gx::as_stream(stream);
    const bool mw = dp.ncomp == 4 && dp.c[0].type == GX_POT_HERNQUIST && dp.c[1].type == GX_POT_HERNQUIST &&
                    dp.c[2].type == GX_POT_MIYAMOTONAGAI && dp.c[3].type == GX_POT_SPHERICALNFW &&
                    !(dp.c[0].do_sr | dp.c[1].do_sr | dp.c[2].do_sr | dp.c[3].do_sr);
    using namespace gx;
    if (mw)
        animate_f32_kernel<PotSig<GX_POT_HERNQUIST, GX_POT_HERNQUIST, GX_POT_MIYAMOTONAGAI, GX_POT_SPHERICALNFW>>
            <<<(unsigned)n_streams, AF_THREADS, 0, st>>>(dp, A);
    else
        animate_f32_kernel<SigGeneric><<<(unsigned)n_streams, AF_THREADS, 0, st>>>(dp, A);
    return check_launch("mockstream_dop853_animate_fp32");
}
