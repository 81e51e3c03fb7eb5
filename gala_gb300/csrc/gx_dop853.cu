// gx_dop853.cu -- FP64 DOP853 with gala's batch semantics, one CTA per batch.
//
// gala integrates `nbatch` orbits (default 100) as ONE ODE system of size
// n = 6 * nb: one shared step size, one RMS error norm over all 6 * nb
// components, one accept/reject decision, one dense-output grid
// (dop853.pyx:228-245 -> dop853_helper :90-193 -> dopcor, dopri/dop853.cpp:89-650).
// Here a batch is a group of consecutive threads of a CTA -- two batches per CTA
// when that fills the warps better (100 orbits alone leave 28 idle lanes), the
// two stepping in lock-step -- and each thread owns one orbit's six components:
//   * the twelve stages, FSAL evaluation and the three dense-output stages are
//     evaluated per thread in registers with gala's expression order;
//   * the error norms (err, err2) and the stiffness sums (stnum, stden) are
//     per-batch sums: a fixed-order warp butterfly plus an ordered sum over
//     warps, so the step-size sequence is deterministic run to run;
//   * every scalar of the step-size controller (x, h, facold, reject, last,
//     naccpt, ...) is computed identically by all threads of a batch from the
//     same sums, so control flow is uniform inside a batch; every thread of
//     the CTA takes part in each step's two reductions, and a CTA leaves its
//     loop when none of its batches is stepping;
//   * dense output (contd8_threadsafe, :869-904) is written directly into the
//     (6, n_out, N) result for every requested time inside [xold, xold + h].
// The loop is bounded by nmax like gala's; no thread ever waits on another CTA.
#include "gx_host.h"
#include "gx_scf.cuh"
#include "gx_dop853_tableau.cuh"
#include "gx_fast64.cuh"

namespace gx {

struct DopArgs {
    double atol, rtol, dt_max;
    int64_t nmax, nstiff;
    int64_t ntimes, out_stride, n_out;
    int32_t save_all, nbatch;
    const int32_t *cancel;  // host cancel flag (mapped memory) or nullptr
};

constexpr int DOP_MAX_WARPS = 32;

// Deterministic sums of two values over each batch of the CTA (BPC batches;
// bl is the caller's batch): a fixed-order warp butterfly, with the lanes of
// the other batch contributing zeros, then an ordered sum over warps.  Every
// thread of a batch returns the same bits.
template <int BPC>
__device__ __forceinline__ void block_sum2(double &a, double &b, double *red, int bl) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    double v[2 * BPC];
#pragma unroll
    for (int q = 0; q < BPC; q++) {
        v[q] = (bl == q) ? a : 0.0;
        v[BPC + q] = (bl == q) ? b : 0.0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int q = 0; q < 2 * BPC; q++) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 2 * BPC; q++) red[q * DOP_MAX_WARPS + wid] = v[q];
    __syncthreads();
    double sa = 0., sb = 0.;
    for (int w = 0; w < nw; w++) {
        sa += red[bl * DOP_MAX_WARPS + w];
        sb += red[(BPC + bl) * DOP_MAX_WARPS + w];
    }
    __syncthreads();
    a = sa;
    b = sb;
}

__device__ __forceinline__ double sign_d(double a, double b) { return (b < 0.0) ? -fabs(a) : fabs(a); }
__device__ __forceinline__ double min_d(double a, double b) { return (a < b) ? a : b; }
__device__ __forceinline__ double max_d(double a, double b) { return (a > b) ? a : b; }

#define RHS(yin, kout)                                                   \
    do {                                                                 \
        if (active) {                                                    \
            V6 a_;                                                       \
            for (int c_ = 0; c_ < 6; c_++) a_.v[c_] = yin[c_];           \
            const V6 r_ = fast::rhs_call_f<SCF>(pot, fr, a_);            \
            for (int c_ = 0; c_ < 6; c_++) kout[c_] = r_.v[c_];          \
        } else {                                                         \
            for (int c_ = 0; c_ < 6; c_++) kout[c_] = 0.;                \
        }                                                                \
    } while (0)

template <int MAXT, bool SCF, int BPC>
__global__ void __launch_bounds__(MAXT, 1)
dop853_kernel(const __grid_constant__ DevPot pot, const __grid_constant__ DevFrame fr, DopArgs A,
              const double *__restrict__ w0, int64_t n, const double *__restrict__ t, double *__restrict__ out,
              int32_t *__restrict__ status,
              int64_t *__restrict__ stats) {
    using namespace dop;
    __shared__ double red[4 * DOP_MAX_WARPS];
    // a CTA that starts after cancellation integrates nothing (one reader, CTA-uniform)
    if (__syncthreads_or(threadIdx.x == 0 && cancel_requested(A.cancel))) return;

    // BPC batches per CTA, batch bl on threads [bl * nbatch, (bl + 1) * nbatch)
    const int nbs = A.nbatch;
    const int bl = (BPC == 1) ? 0 : min((int)threadIdx.x / nbs, BPC - 1);
    const int j = threadIdx.x - bl * nbs;  // lane within the batch
    const int64_t b = (int64_t)blockIdx.x * BPC + bl;
    const int64_t nbt = (n + nbs - 1) / nbs;
    const bool batch_ok = b < nbt && j < nbs;
    const int64_t i0 = b * nbs;
    const int nb = batch_ok ? (int)((i0 + nbs <= n) ? nbs : n - i0) : 0;
    const bool active = batch_ok && j < nb;
    const int nsys = 6 * nb;

    double y[6], k1[6], k2[6], k3[6], k4[6], k5[6], k6[6], k7[6], k8[6], k9[6], k10[6], yy1[6];
    for (int c = 0; c < 6; c++) y[c] = active ? w0[c * n + i0 + j] : 0.;

    // dop853() front-end defaults with dop853_helper's arguments (dop853.pyx:157-182)
    double x = t[0];
    const double xend = t[A.ntimes - 1];
    double h = t[1] - t[0];
    double hmax = A.dt_max;
    const double uround = 2.220446049250313e-16;
    const double safe = 0.9, fac1 = 0.333, fac2 = 6.0;  // and beta = 0
    int64_t nmax = A.nmax, nstiff = A.nstiff;
    if (!nmax) nmax = 1000000;
    if (!nstiff) nstiff = 1000;
    else if (nstiff < 0) nstiff = nmax + 10;
    if (hmax == 0.0) hmax = xend - x;

    double facold = 1.0E-4;
    const double facc1 = 1.0 / fac1, facc2 = 1.0 / fac2;
    const double posneg = sign_d(1.0, xend - x);
    const double atoli = A.atol, rtoli = A.rtol;
    int last = 0, reject = 0, iasti = 0, nonsti = 0, idid = 0;
    double hlamb = 0.0;
    int64_t nfcn = 0, nstep = 0, naccpt = 0, nrejct = 0;
    int64_t out_idx = 0, out_slot = 0;

    RHS(y, k1);
    hmax = fabs(hmax);
    if (h == 0.0) {
        // hinit (dop853.cpp:18-86), scalar tolerances, CTA-wide norms
        double dnf = 0.0, dny = 0.0;
        for (int c = 0; c < 6; c++) {
            const double sk = atoli + rtoli * fabs(y[c]);
            double sqr = k1[c] / sk;
            dnf += active ? sqr * sqr : 0.;
            sqr = y[c] / sk;
            dny += active ? sqr * sqr : 0.;
        }
        block_sum2<BPC>(dnf, dny, red, bl);
        double hh = ((dnf <= 1.0E-10) || (dny <= 1.0E-10)) ? 1.0E-6 : sqrt(dny / dnf) * 0.01;
        hh = min_d(hh, hmax);
        hh = sign_d(hh, posneg);
        for (int c = 0; c < 6; c++) yy1[c] = y[c] + hh * k1[c];
        RHS(yy1, k2);
        double der2 = 0.0, unused = 0.0;
        for (int c = 0; c < 6; c++) {
            const double sk = atoli + rtoli * fabs(y[c]);
            const double sqr = (k2[c] - k1[c]) / sk;
            der2 += active ? sqr * sqr : 0.;
        }
        block_sum2<BPC>(der2, unused, red, bl);
        der2 = sqrt(der2) / hh;
        const double der12 = max_d(fabs(der2), sqrt(dnf));
        const double h1 = (der12 <= 1.0E-15) ? max_d(1.0E-6, fabs(hh) * 1.0E-3) : pow(0.01 / der12, 1.0 / 8.0);
        hh = min_d(100.0 * fabs(hh), min_d(h1, hmax));
        h = sign_d(hh, posneg);
    }
    nfcn += 2;

    bool done = !batch_ok;
    double xold = 0.0, hout = 0.0, xph = 0.0;
    for (;;) {
        // the batches of a CTA step in lock-step: every thread takes part in the
        // two CTA reductions of each step, and the loop ends when no batch of
        // the CTA is stepping any more
        if (!__syncthreads_or(done ? 0 : 1)) break;
        bool stepping = !done;
        if (stepping && nstep > nmax) {
            idid = -2;
            done = true;
            stepping = false;
        }
        if (stepping && 0.1 * fabs(h) <= fabs(x) * uround) {
            idid = -3;
            done = true;
            stepping = false;
        }
        if (stepping) {
            if ((x + 1.01 * h - xend) * posneg > 0.0) {
                h = xend - x;
                last = 1;
            }
            xold = x;
            hout = h;
            nstep++;

            // the twelve stages (dop853.cpp:368-414)
            // stage sums as fused multiply-add chains in gala's term order
            for (int c = 0; c < 6; c++) yy1[c] = fma(h * a21, k1[c], y[c]);
            RHS(yy1, k2);
            for (int c = 0; c < 6; c++) yy1[c] = fma(h, fma(a32, k2[c], a31 * k1[c]), y[c]);
            RHS(yy1, k3);
            for (int c = 0; c < 6; c++) yy1[c] = fma(h, fma(a43, k3[c], a41 * k1[c]), y[c]);
            RHS(yy1, k4);
            for (int c = 0; c < 6; c++) yy1[c] = fma(h, fma(a54, k4[c], fma(a53, k3[c], a51 * k1[c])), y[c]);
            RHS(yy1, k5);
            for (int c = 0; c < 6; c++) yy1[c] = fma(h, fma(a65, k5[c], fma(a64, k4[c], a61 * k1[c])), y[c]);
            RHS(yy1, k6);
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a76, k6[c], fma(a75, k5[c], fma(a74, k4[c], a71 * k1[c]))), y[c]);
            RHS(yy1, k7);
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a87, k7[c], fma(a86, k6[c], fma(a85, k5[c], fma(a84, k4[c], a81 * k1[c])))), y[c]);
            RHS(yy1, k8);
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a98, k8[c], fma(a97, k7[c], fma(a96, k6[c], fma(a95, k5[c], fma(a94, k4[c],
                                                                                                    a91 * k1[c]))))),
                             y[c]);
            RHS(yy1, k9);
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a109, k9[c], fma(a108, k8[c], fma(a107, k7[c], fma(a106, k6[c], fma(a105, k5[c],
                                    fma(a104, k4[c], a101 * k1[c])))))), y[c]);
            RHS(yy1, k10);
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a1110, k10[c], fma(a119, k9[c], fma(a118, k8[c], fma(a117, k7[c], fma(a116, k6[c],
                                    fma(a115, k5[c], fma(a114, k4[c], a111 * k1[c]))))))), y[c]);
            RHS(yy1, k2);
            xph = x + h;
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a1211, k2[c], fma(a1210, k10[c], fma(a129, k9[c], fma(a128, k8[c], fma(a127, k7[c],
                                    fma(a126, k6[c], fma(a125, k5[c], fma(a124, k4[c], a121 * k1[c])))))))), y[c]);
            RHS(yy1, k3);
            nfcn += 11;
            for (int c = 0; c < 6; c++) {
                k4[c] = fma(b12, k3[c], fma(b11, k2[c], fma(b10, k10[c], fma(b9, k9[c], fma(b8, k8[c], fma(b7, k7[c],
                            fma(b6, k6[c], b1 * k1[c])))))));
                k5[c] = fma(h, k4[c], y[c]);
            }
        }

        // error estimation (:416-444), summed over each batch
        double err = 0.0, err2 = 0.0;
        if (stepping && active) {
            for (int c = 0; c < 6; c++) {
                const double isk = fast::rcp_f(fma(rtoli, fmax(fabs(y[c]), fabs(k5[c])), atoli));
                double erri = fma(-bhh3, k3[c], fma(-bhh2, k9[c], fma(-bhh1, k1[c], k4[c])));
                double sqr = erri * isk;
                err2 = fma(sqr, sqr, err2);
                erri = fma(er12, k3[c], fma(er11, k2[c], fma(er10, k10[c], fma(er9, k9[c], fma(er8, k8[c],
                           fma(er7, k7[c], fma(er6, k6[c], er1 * k1[c])))))));
                sqr = erri * isk;
                err = fma(sqr, sqr, err);
            }
        }
        block_sum2<BPC>(err, err2, red, bl);
        double hnew = h, fac11 = 1.0;
        bool acc = false;
        if (stepping) {
            double deno = err + 0.01 * err2;
            if (deno <= 0.0) deno = 1.0;
            err = fabs(h) * err * sqrt(1.0 / (deno * (double)nsys));
            // computation of hnew (:446-452); gala's pow(err, expo1) with expo1 = 1/8
            // (beta = 0) as three square roots instead of pow's ~84 FP64-pipe instructions
            fac11 = sqrt(sqrt(sqrt(err)));
            double fac = fac11;  // gala divides by pow(facold, beta) == 1 for its beta = 0
            fac = max_d(facc2, min_d(facc1, fac / safe));
            hnew = h / fac;
            acc = err <= 1.0;
            if (acc) {
                facold = max_d(err, 1.0E-4);
                naccpt++;
                RHS(k5, k4);
                nfcn++;
            }
        }

        // stiffness detection (:463-486); like gala, the first detection returns -4.
        // The sums are formed every step (zero where no test is due) so that all
        // batches of the CTA share the barrier.
        const bool stiff_due = stepping && acc && (!(naccpt % nstiff) || (iasti > 0));
        double stnum = 0.0, stden = 0.0;
        if (stiff_due && active) {
            for (int c = 0; c < 6; c++) {
                double sqr = k4[c] - k3[c];
                stnum += sqr * sqr;
                sqr = k5[c] - yy1[c];
                stden += sqr * sqr;
            }
        }
        block_sum2<BPC>(stnum, stden, red, bl);
        if (stiff_due) {
            if (stden > 0.0) hlamb = h * sqrt(stnum / stden);
            if (hlamb > 6.1) {
                nonsti = 0;
                iasti++;
                idid = -4;
                done = true;
                stepping = false;
            } else {
                nonsti++;
                if (nonsti == 6) iasti = 0;
            }
        }

        if (stepping && acc) {
            // Output times inside [xold, xold + hout] (:584-612): [out_idx, out_end).
            // Only every out_stride-th time is stored; the three dense-output stages
            // are evaluated only for a step that holds a stored time (their results
            // feed nothing else: the next step starts from k4 = f(k5) and recomputes
            // every other stage), so the trajectory is unchanged.
            int64_t out_end = out_idx, first_kept = 0;
            if (A.save_all) {
                const double x0 = xold, x1 = x0 + hout;
                while (out_end < A.ntimes) {
                    const double t_out = t[out_end];
                    if (!((x0 <= t_out && t_out <= x1) || (x1 <= t_out && t_out <= x0))) break;
                    out_end++;
                }
                first_kept = (out_idx + A.out_stride - 1) / A.out_stride * A.out_stride;
            }
            if (A.save_all && first_kept < out_end) {
                // dense output preparation (:492-582)
                double r5[6], r6[6], r7[6], r8[6];
#define GX_D8(p, k1_, k6_, k7_, k8_, k9_, k10_, k2_, k3_)                                                      \
    fma(p##12, k3_, fma(p##11, k2_, fma(p##10, k10_, fma(p##9, k9_, fma(p##8, k8_, fma(p##7, k7_,              \
        fma(p##6, k6_, p##1 * k1_)))))))
                for (int c = 0; c < 6; c++) {
                    r5[c] = GX_D8(d4, k1[c], k6[c], k7[c], k8[c], k9[c], k10[c], k2[c], k3[c]);
                    r6[c] = GX_D8(d5, k1[c], k6[c], k7[c], k8[c], k9[c], k10[c], k2[c], k3[c]);
                    r7[c] = GX_D8(d6, k1[c], k6[c], k7[c], k8[c], k9[c], k10[c], k2[c], k3[c]);
                    r8[c] = GX_D8(d7, k1[c], k6[c], k7[c], k8[c], k9[c], k10[c], k2[c], k3[c]);
                }
#undef GX_D8
                for (int c = 0; c < 6; c++)
                    yy1[c] = fma(h, fma(a1413, k4[c], fma(a1412, k3[c], fma(a1411, k2[c], fma(a1410, k10[c],
                                 fma(a149, k9[c], fma(a148, k8[c], fma(a147, k7[c], a141 * k1[c]))))))), y[c]);
                RHS(yy1, k10);
                for (int c = 0; c < 6; c++)
                    yy1[c] = fma(h, fma(a1514, k10[c], fma(a1513, k4[c], fma(a1512, k3[c], fma(a1511, k2[c],
                                 fma(a158, k8[c], fma(a157, k7[c], fma(a156, k6[c], a151 * k1[c]))))))), y[c]);
                RHS(yy1, k2);
                for (int c = 0; c < 6; c++)
                    yy1[c] = fma(h, fma(a1615, k2[c], fma(a1614, k10[c], fma(a1613, k4[c], fma(a169, k9[c],
                                 fma(a168, k8[c], fma(a167, k7[c], fma(a166, k6[c], a161 * k1[c]))))))), y[c]);
                RHS(yy1, k3);
                nfcn += 3;
                double r1[6], r2[6], r3[6], r4[6];
                for (int c = 0; c < 6; c++) {
                    r5[c] = h * fma(d416, k3[c], fma(d415, k2[c], fma(d414, k10[c], fma(d413, k4[c], r5[c]))));
                    r6[c] = h * fma(d516, k3[c], fma(d515, k2[c], fma(d514, k10[c], fma(d513, k4[c], r6[c]))));
                    r7[c] = h * fma(d616, k3[c], fma(d615, k2[c], fma(d614, k10[c], fma(d613, k4[c], r7[c]))));
                    r8[c] = h * fma(d716, k3[c], fma(d715, k2[c], fma(d714, k10[c], fma(d713, k4[c], r8[c]))));
                    r1[c] = y[c];
                    const double ydiff = k5[c] - y[c];
                    r2[c] = ydiff;
                    const double bspl = fma(h, k1[c], -ydiff);
                    r3[c] = bspl;
                    r4[c] = fma(-h, k4[c], ydiff) - bspl;
                }

                for (int64_t oi = first_kept; oi < out_end; oi += A.out_stride) {
                    const double s = (t[oi] - xold) / hout;
                    const double s1 = 1.0 - s;
                    if (active) {
                        for (int c = 0; c < 6; c++) {
                            const double v =
                                fma(s, fma(s1, fma(s, fma(s1, fma(s, fma(s1, fma(s, r8[c], r7[c]), r6[c]), r5[c]),
                                                          r4[c]), r3[c]), r2[c]), r1[c]);
                            __stcs(&out[((int64_t)c * A.n_out + out_slot) * n + i0 + j], v);
                        }
                    }
                    out_slot++;
                }
            }
            out_idx = out_end;


            for (int c = 0; c < 6; c++) {
                k1[c] = k4[c];
                y[c] = k5[c];
            }
            x = xph;
            if (last) {
                idid = 1;
                done = true;
            } else {
                if (fabs(hnew) > hmax) hnew = posneg * hmax;
                if (reject) hnew = posneg * min_d(fabs(hnew), fabs(h));
                reject = 0;
            }
        } else if (stepping) {
            hnew = h / min_d(facc1, fac11 / safe);
            reject = 1;
            if (naccpt >= 1) nrejct = nrejct + 1;
            last = 0;
        }
        if (stepping && !done) h = hnew;
    }
    (void)nonsti;

    if (!A.save_all && active)
        for (int c = 0; c < 6; c++) out[c * n + i0 + j] = y[c];
    if (j == 0 && batch_ok) {
        status[b] = idid;
        if (stats) {
            stats[4 * b + 0] = nfcn;
            stats[4 * b + 1] = nstep;
            stats[4 * b + 2] = naccpt;
            stats[4 * b + 3] = nrejct;
        }
    }
}
#undef RHS

}  // namespace gx

extern "C" int gx_dop853_integrate_hamiltonian(const gx_potential *pot, const gx_frame *frame, const double *w0,
                                               int64_t n, const double *t, int64_t ntimes, double atol,
                                               double rtol, int64_t nmax, double dt_max, int64_t nstiff,
                                               int32_t save_all, int32_t nbatch, int64_t out_stride,
                                               double *w_out, int32_t *status, int64_t *stats, void *stream) {
    gx::DevPot dp;
    gx::DevFrame df;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    rc = gx::pack_frame(frame, &df);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0, "n < 0");
    GX_CHECK_ARG(ntimes >= 2, "ntimes must be >= 2 (got %lld)", (long long)ntimes);
    GX_CHECK_ARG(nbatch >= 1 && nbatch <= 1024, "nbatch must be in [1, 1024] (got %d)", nbatch);
    GX_CHECK_ARG(out_stride >= 1, "out_stride must be >= 1");
    GX_CHECK_ARG(nmax >= 0, "nmax must be >= 0 (0 = gala's default 1e6)");
    GX_CHECK_ARG(atol >= 0 && rtol >= 0, "tolerances must be non-negative");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(w0 && t && w_out && status, "NULL array");
    gx::DopArgs A;
    memset(&A, 0, sizeof(A));
    A.cancel = gx::cancel_flag();
    A.atol = atol;
    A.rtol = rtol;
    A.dt_max = dt_max;
    A.nmax = nmax;
    A.nstiff = nstiff;
    A.ntimes = ntimes;
    A.out_stride = out_stride;
    A.n_out = (ntimes - 1) / out_stride + 1;
    A.save_all = save_all ? 1 : 0;
    A.nbatch = nbatch;
    const int64_t nbatches = (n + nbatch - 1) / nbatch;
    cudaStream_t st = gx::as_stream(stream);
    // Two batches share a CTA when that fills the warps better (a 100-orbit batch
    // alone leaves 28 lanes of its fourth warp idle, and the FP64 pipe costs a
    // warp instruction whatever its mask); they step in lock-step.
    const int t1 = ((nbatch + 31) / 32) * 32, t2 = ((2 * nbatch + 31) / 32) * 32;
    const bool pair = !dp.has_scf && t2 <= 256 && t2 < 2 * t1;
    const int threads = pair ? t2 : t1;
    const unsigned grid = (unsigned)(pair ? (nbatches + 1) / 2 : nbatches);
    if (pair)
        gx::dop853_kernel<256, false, 2><<<grid, threads, 0, st>>>(dp, df, A, w0, n, t, w_out, status, stats);
    else if (threads <= 256 && !dp.has_scf)
        gx::dop853_kernel<256, false, 1><<<grid, threads, 0, st>>>(dp, df, A, w0, n, t, w_out, status, stats);
    else if (threads <= 256)
        gx::dop853_kernel<256, true, 1><<<grid, threads, 0, st>>>(dp, df, A, w0, n, t, w_out, status, stats);
    else if (!dp.has_scf)
        gx::dop853_kernel<1024, false, 1><<<grid, threads, 0, st>>>(dp, df, A, w0, n, t, w_out, status, stats);
    else
        gx::dop853_kernel<1024, true, 1><<<grid, threads, 0, st>>>(dp, df, A, w0, n, t, w_out, status, stats);
    return gx::check_launch("dop853");
}

namespace gx {
__global__ void selfcheck_fast64_kernel(const double *__restrict__ x, int64_t n, double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    out[i] = fast::log_f(v);
    out[n + i] = log(v);
    out[2 * n + i] = fast::sqrt_f(v);
    out[3 * n + i] = fast::rcp_f(v);
}
}  // namespace gx

extern "C" int gx_selfcheck_fast64(const double *x, int64_t n, double *out, void *stream) {
    GX_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(x && out, "NULL array");
    gx::selfcheck_fast64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, gx::as_stream(stream)>>>(x, n, out);
    return gx::check_launch("selfcheck_fast64");
}
