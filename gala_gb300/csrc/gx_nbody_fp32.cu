// gx_nbody_fp32.cu -- mock-stream release systems by DOP853 with FP32 stages and
// forces and FP64 step control (the FP32 form of gx_mockstream_dop853).
//
// The same systems as mockstream_dop853 (src/gala/dynamics/mockstream/
// mockstream.pyx:176-303): for every release time one dop853_step problem
// (dop853.pyx:27-75 -> dopcor, dopri/dop853.cpp:89-650) over the massive bodies
// at that time and the particles released then, one step size per system.
// GPU mapping as gx_nbody.cu: a system is a group of consecutive lanes, one
// lane per body or particle, groups taking systems from a queue.  Arithmetic as
// gx_dop853_fp32.cu:
//   * stages, forces (external and the bodies' pulls) and stage sums in FP32;
//   * the state a double-float pair; a stage argument is carried as the state's
//     high part plus an FP32 offset (low part + h * sum a_ij k_j), so the
//     particle-body separations, ~1e-3 of the positions, keep their accuracy:
//     d = (hi_p - hi_b) + (offset_p - offset_b);
//   * FP64 for the time, the step size (kept FP32-representable), the error
//     norm's combination err = |h| err sqrt(1 / (deno n)) as the test
//     h^2 err^2 <= deno n, and accept/reject;
//   * stiffness every accepted step (mockstream's nstiff = 1) estimated over
//     the whole step (f and y at its two ends), as in gx_dop853_fp32.cu: gala's
//     estimate from the last stage point is below FP32 resolution.
// Not bit-compatible with gala; accuracy is that of FP32 forces, and tolerances
// below ~1e-8 relative only shrink the steps.
#include "gx_host.h"
#include "gx_body_f32.cuh"
#include "gx_fp32.cuh"
#include "gx_scf.cuh"
#include "gx_dop853_tableau.cuh"

namespace gx {

int pack_potential_f32(const gx_potential *pot, DevPotF *out);

constexpr int MS32_MAXNB = 4;  // massive bodies per system

struct Ms32Args {
    int32_t gs;     // lanes per group
    int32_t nbody;  // massive bodies per system (the first lanes)
    int64_t n_sys, n_streams, n_release, n_particles;
    const gx_body *bodies;    // (n_streams, nbody)
    const double *nbody_w;    // (n_streams, n_release, nbody, 6)
    const double *release_t;  // (n_release)
    const int64_t *offset;    // (n_release + 1)
    const double *stream_w0;  // (n_streams, n_particles, 6)
    double t_final, dt0, atol, rtol;
    int64_t nmax;
    double *stream_w_out, *nbody_w_out;
    int32_t *status;
    int64_t *stats;
    unsigned long long *counter;
    const int32_t *cancel;  // host cancel flag (mapped memory) or nullptr
};

// Sums of two values over the lanes of a group, lane by lane in member order;
// every lane of the group gets the same bits.
__device__ __forceinline__ void group_sum2(unsigned mask, int gs, int base, int member, bool in_sys, float ta,
                                           float tb, float &sa, float &sb) {
    float a = 0.f, b = 0.f;
    for (int m = 0; m < gs; m++) {
        if (member == m && in_sys) {
            a += ta;
            b += tb;
        }
        a = __shfl_sync(mask, a, base + m);
        b = __shfl_sync(mask, b, base + m);
    }
    sa = a;
    sb = b;
}

// Fwrapper_direct_nbody (dop853.cpp:990-1006) in FP32 for the lane's member,
// its argument given as (hi, off): Hamilton's equations in the external
// potential at hi + off, then the pull of every non-null massive body j != the
// lane at the separation (hi - hi_j) + (off - off_j).
template <typename S>
__device__ __forceinline__ void ms_rhs(const DevPotF &pot, unsigned mask, int base, int member, int nmem, int nbody,
                                       const BodyF (&bc)[MS32_MAXNB], const float *hi, const float *off,
                                       float *f) {
    float w[6], g[3];
#pragma unroll
    for (int c = 0; c < 6; c++) w[c] = hi[c] + off[c];
    potential_gradient_f<S>(pot, w, g);
#pragma unroll
    for (int j = 0; j < MS32_MAXNB; j++) {
        if (j >= nbody) break;
        float hj[3], oj[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            hj[k] = __shfl_sync(mask, hi[k], base + j);
            oj[k] = __shfl_sync(mask, off[k], base + j);
        }
        if (member != j && member < nmem && bc[j].type != GX_POT_NULL) {
            const float d[3] = {(hi[0] - hj[0]) + (off[0] - oj[0]), (hi[1] - hj[1]) + (off[1] - oj[1]),
                                (hi[2] - hj[2]) + (off[2] - oj[2])};
            body_grad_f32(bc[j], d, g);
        }
    }
    f[0] = w[3];
    f[1] = w[4];
    f[2] = w[5];
    f[3] = -g[0];
    f[4] = -g[1];
    f[5] = -g[2];
}

#define F32(c) ((float)(dop::c))

template <typename S>
__global__ void __launch_bounds__(128) ms_dop853_fp32_kernel(const __grid_constant__ DevPotF pot,
                                                             const __grid_constant__ Ms32Args A) {
    const int lane = threadIdx.x & 31;
    const int gs = A.gs;
    const int grp = lane / gs;
    const int member = lane - grp * gs;
    const int base = grp * gs;
    const bool lane_ok = grp < 32 / gs;
    const unsigned gmask = lane_ok ? (((gs == 32) ? 0xffffffffu : ((1u << gs) - 1u)) << base) : 0u;
    const float atol = (float)A.atol, rtol = (float)A.rtol;
    const double uround = 2.3E-16;
    const float safe = 0.9f, facc1 = 1.0f / 0.333f, facc2 = 1.0f / 6.0f;
    const int nbody = A.nbody;

    BodyF bc[MS32_MAXNB];
    float yh[6], yl[6], k1[6], k2[6], k3[6], k4[6], k5[6], k5l[6], k6[6], k7[6], k8[6], k9[6], k10[6], off[6];
    int64_t si = 0, ss = 0;
    int nmem = 0;
    double x = 0., xend = 0., h = 0., hmax = 0., posneg = 1.;
    float hlamb = 0.f;
    int64_t nmax = 0, nfcn = 0, nstep = 0, naccpt = 0, nrejct = 0;
    int last = 0, reject = 0, iasti = 0, nonsti = 0, idid = 0;
    bool have = false, done = !lane_ok;

#define MRHS(mask_, hi_, off_, out_) ms_rhs<S>(pot, (mask_), base, member, nmem, nbody, bc, (hi_), (off_), (out_))

    for (;;) {
        // -- a group without a system takes the next one ------------------------
        if (!have && !done) {
            for (;;) {
                // a cancelled launch takes no further system (member 0 decides for the group)
                unsigned long long id = ~0ull;
                if (member == 0 && !cancel_requested(A.cancel)) id = atomicAdd(A.counter, 1ull);
                id = __shfl_sync(gmask, id, base);
                if (id >= (unsigned long long)A.n_sys) {
                    done = true;
                    break;
                }
                const int64_t sys = (int64_t)id;
                si = sys / A.n_streams;
                ss = sys - si * A.n_streams;
                const int64_t o0 = A.offset[si], o1 = A.offset[si + 1];
                // nothing released at this time (gala skips it), or an offset table
                // inconsistent with the particle array (rejected, no access)
                const bool bad = o1 < o0 || o0 < 0 || o1 > A.n_particles || o1 - o0 > gs - nbody;
                if (o1 == o0 || bad) {
                    if (member == 0) {
                        (void)GX_DBG_CHECK(!bad, DBG_OFFSET, si, A.n_release);
                        A.status[ss * A.n_release + si] = bad ? -1 : 0;
                        if (A.stats)
                            for (int k = 0; k < 4; k++) A.stats[(ss * A.n_release + si) * 4 + k] = 0;
                    }
                    continue;
                }
                nmem = nbody + (int)(o1 - o0);
#pragma unroll
                for (int j = 0; j < MS32_MAXNB; j++) {
                    if (j < nbody) body_consts_f32(A.bodies + ss * nbody + j, bc[j]);
                    else bc[j].type = GX_POT_NULL;
                }
                const double *src = nullptr;
                if (member < nbody) src = A.nbody_w + ((ss * A.n_release + si) * nbody + member) * 6;
                else if (member < nmem) src = A.stream_w0 + (ss * A.n_particles + o0 + (member - nbody)) * 6;
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    const double v = src ? src[c] : 0.;
                    yh[c] = (float)v;
                    yl[c] = (float)(v - (double)yh[c]);
                }
                // dop853_step's dop853() arguments (dop853.pyx:46-72)
                x = A.release_t[si];
                xend = A.t_final;
                h = (double)(float)A.dt0;
                hmax = fabs(xend - x);
                posneg = (xend - x < 0.0) ? -1.0 : 1.0;
                nmax = A.nmax ? A.nmax : 1000000;
                hlamb = 0.f;
                last = reject = iasti = nonsti = idid = 0;
                nfcn = 2;
                nstep = naccpt = nrejct = 0;
                have = true;
                break;
            }
            if (have) {
                const unsigned im = __ballot_sync(gmask, true);
                MRHS(im, yh, yl, k1);
            }
        }
        const unsigned act = __ballot_sync(0xffffffffu, have);
        if (act == 0u) break;
        if (!have) continue;
        const bool in_sys = member < nmem;

        bool fin = false;
        if (nstep > nmax || !(fabsf((float)h) <= 3.0e38f)) {
            idid = -2;  // a NaN step never recovers: gala's -2 after nmax rejections, at once
            fin = true;
        } else if (0.1 * fabs(h) <= fabs(x) * uround) {
            idid = -3;
            fin = true;
        }
        const unsigned am = __ballot_sync(act, !fin);
        if (!fin) {
            if ((x + 1.01 * h - xend) * posneg > 0.0) {
                h = xend - x;
                last = 1;
            }
            const double xold = x;
            nstep++;
            const float hf = (float)h;
            // the twelve stages (dop853.cpp:368-414): the argument is carried as
            // (yh, off) with off = yl + h sum a_ij k_j in FP32
#define MSTAGE(dst, expr)                                                          \
    for (int c = 0; c < 6; c++) off[c] = __fmaf_rn(hf, (expr), yl[c]);            \
    MRHS(am, yh, off, dst)
            MSTAGE(k2, F32(a21) * k1[c]);
            MSTAGE(k3, fmaf(F32(a32), k2[c], F32(a31) * k1[c]));
            MSTAGE(k4, fmaf(F32(a43), k3[c], F32(a41) * k1[c]));
            MSTAGE(k5, fmaf(F32(a54), k4[c], fmaf(F32(a53), k3[c], F32(a51) * k1[c])));
            MSTAGE(k6, fmaf(F32(a65), k5[c], fmaf(F32(a64), k4[c], F32(a61) * k1[c])));
            MSTAGE(k7, fmaf(F32(a76), k6[c], fmaf(F32(a75), k5[c], fmaf(F32(a74), k4[c], F32(a71) * k1[c]))));
            MSTAGE(k8, fmaf(F32(a87), k7[c], fmaf(F32(a86), k6[c], fmaf(F32(a85), k5[c],
                       fmaf(F32(a84), k4[c], F32(a81) * k1[c])))));
            MSTAGE(k9, fmaf(F32(a98), k8[c], fmaf(F32(a97), k7[c], fmaf(F32(a96), k6[c], fmaf(F32(a95), k5[c],
                       fmaf(F32(a94), k4[c], F32(a91) * k1[c]))))));
            MSTAGE(k10, fmaf(F32(a109), k9[c], fmaf(F32(a108), k8[c], fmaf(F32(a107), k7[c],
                        fmaf(F32(a106), k6[c], fmaf(F32(a105), k5[c], fmaf(F32(a104), k4[c],
                        F32(a101) * k1[c])))))));
            MSTAGE(k2, fmaf(F32(a1110), k10[c], fmaf(F32(a119), k9[c], fmaf(F32(a118), k8[c],
                       fmaf(F32(a117), k7[c], fmaf(F32(a116), k6[c], fmaf(F32(a115), k5[c],
                       fmaf(F32(a114), k4[c], F32(a111) * k1[c]))))))));
            MSTAGE(k3, fmaf(F32(a1211), k2[c], fmaf(F32(a1210), k10[c], fmaf(F32(a129), k9[c],
                       fmaf(F32(a128), k8[c], fmaf(F32(a127), k7[c], fmaf(F32(a126), k6[c],
                       fmaf(F32(a125), k5[c], fmaf(F32(a124), k4[c], F32(a121) * k1[c])))))))));
#undef MSTAGE
            nfcn += 11;
            float e1 = 0.f, e2 = 0.f;
#pragma unroll
            for (int c = 0; c < 6; c++) {
                k4[c] = fmaf(F32(b12), k3[c], fmaf(F32(b11), k2[c], fmaf(F32(b10), k10[c], fmaf(F32(b9), k9[c],
                        fmaf(F32(b8), k8[c], fmaf(F32(b7), k7[c], fmaf(F32(b6), k6[c], F32(b1) * k1[c])))))));
                df_axpy32(yh[c], yl[c], hf, k4[c], k5[c], k5l[c]);
                const float isk = rcp_approx(fmaf(rtol, fmaxf(fabsf(yh[c]), fabsf(k5[c])), atol));
                float erri = k4[c] - F32(bhh1) * k1[c] - F32(bhh2) * k9[c] - F32(bhh3) * k3[c];
                float sq = erri * isk;
                e2 = fmaf(sq, sq, e2);
                erri = fmaf(F32(er12), k3[c], fmaf(F32(er11), k2[c], fmaf(F32(er10), k10[c], fmaf(F32(er9), k9[c],
                       fmaf(F32(er8), k8[c], fmaf(F32(er7), k7[c], fmaf(F32(er6), k6[c], F32(er1) * k1[c])))))));
                sq = erri * isk;
                e1 = fmaf(sq, sq, e1);
            }
            float E1, E2;
            group_sum2(am, gs, base, member, in_sys, in_sys ? e1 : 0.f, in_sys ? e2 : 0.f, E1, E2);
            // err = |h| E1 / sqrt(deno n), n = 6 nmem: accept iff h^2 E1^2 <= deno n
            double deno = fma(0.01, (double)E2, (double)E1);
            if (deno <= 0.0) deno = 1.0;
            const double he = h * (double)E1;
            const bool acc = fma(he, he, -(double)(6 * nmem) * deno) <= 0.0;
            float denof = fmaf(0.01f, E2, E1);
            if (denof <= 0.f) denof = 1.f;
            const float hef = hf * E1;
            const float ratio = hef * hef * rcp_approx((float)(6 * nmem) * denof);
            const float fac11 = ex2_approx32(lg2_approx(ratio) * 0.0625f);
            const float fac = fmaxf(facc2, fminf(facc1, fac11 / safe));
            float hnew = hf * rcp_approx(fac);

            // FSAL derivative at the new state (k5, k5l), evaluated by every
            // group of the warp; a rejected group does not use it
            MRHS(am, k5, k5l, k4);
            bool stiff = false;
            if (acc) {
                naccpt++;
                nfcn++;
            }
            // stiffness (nstiff = 1: every accepted step), over the whole step
            {
                float tn = 0.f, td = 0.f;
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    float d = k4[c] - k1[c];
                    tn = fmaf(d, d, tn);
                    d = __fsub_rn(k5[c], yh[c]) + __fsub_rn(k5l[c], yl[c]);
                    td = fmaf(d, d, td);
                }
                float stnum, stden;
                group_sum2(am, gs, base, member, in_sys, in_sys ? tn : 0.f, in_sys ? td : 0.f, stnum, stden);
                if (acc) {
                    if (stden > 0.f) hlamb = hf * sqrtf(stnum / stden);
                    if (hlamb > 6.1f) {
                        nonsti = 0;
                        iasti++;
                        idid = -4;
                        stiff = true;
                    } else {
                        nonsti++;
                        if (nonsti == 6) iasti = 0;
                    }
                }
            }
            if (acc && !stiff) {
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    k1[c] = k4[c];
                    yh[c] = k5[c];
                    yl[c] = k5l[c];
                }
                x = xold + h;
                if (last) {
                    idid = 1;
                } else {
                    if (fabsf(hnew) > (float)hmax) hnew = copysignf((float)hmax, hf);
                    if (reject) hnew = copysignf(fminf(fabsf(hnew), fabsf(hf)), hf);
                    reject = 0;
                }
            } else if (!acc) {
                hnew = hf * rcp_approx(fminf(facc1, fac11 / safe));
                reject = 1;
                if (naccpt >= 1) nrejct++;
                last = 0;
            }
            if (idid == 0) h = (double)hnew;
        }

        // -- a finished system writes its results --------------------------------
        if (idid != 0) {
            const int64_t o0 = A.offset[si];
            if (member >= nbody && member < nmem) {
                double *o = A.stream_w_out + (ss * A.n_particles + o0 + (member - nbody)) * 6;
#pragma unroll
                for (int c = 0; c < 6; c++) o[c] = (double)yh[c] + (double)yl[c];
            }
            if (member < nbody && A.nbody_w_out && A.offset[si + 1] == A.offset[A.n_release]) {
                double *o = A.nbody_w_out + (ss * nbody + member) * 6;
#pragma unroll
                for (int c = 0; c < 6; c++) o[c] = (double)yh[c] + (double)yl[c];
            }
            if (member == 0) {
                const int64_t k = ss * A.n_release + si;
                A.status[k] = idid;
                if (A.stats) {
                    A.stats[4 * k + 0] = nfcn;
                    A.stats[4 * k + 1] = nstep;
                    A.stats[4 * k + 2] = naccpt;
                    A.stats[4 * k + 3] = nrejct;
                }
            }
            have = false;
        }
    }
#undef MRHS
    (void)nonsti;
}
#undef F32

template <typename S>
static int launch_ms32(const DevPotF &dp, const Ms32Args &A, cudaStream_t st) {
    int dev = 0, sms = 0, per_sm = 0;
    GX_CUDA_TRY(cudaGetDevice(&dev));
    GX_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ms_dop853_fp32_kernel<S>, 128, 0));
    if (per_sm < 1) per_sm = 1;
    const int64_t groups_per_block = 4 * (32 / A.gs);
    int64_t need = (A.n_sys + groups_per_block - 1) / groups_per_block;
    int64_t grid = (int64_t)sms * per_sm;
    if (need < grid) grid = need;
    if (grid < 1) grid = 1;
    GX_CUDA_TRY(cudaMemsetAsync(A.counter, 0, sizeof(unsigned long long), st));
    ms_dop853_fp32_kernel<S><<<(unsigned)grid, 128, 0, st>>>(dp, A);
    return check_launch("mockstream_dop853_fp32");
}

}  // namespace gx

extern "C" int gx_mockstream_dop853_fp32(const gx_potential *pot, int64_t n_streams, int32_t nbody,
                                         const gx_body *bodies, const double *nbody_w, int64_t n_release,
                                         const double *release_t, const int64_t *release_offset,
                                         int32_t max_per_release, const double *stream_w0, int64_t n_particles,
                                         double t_final, double dt0, double atol, double rtol, int64_t nmax,
                                         double *stream_w_out, double *nbody_w_out, int32_t *status,
                                         int64_t *stats, int64_t *queue_counter, void *stream) {
    gx::DevPotF dp;
    int rc = gx::pack_potential_f32(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(n_streams >= 0 && n_release >= 0 && n_particles >= 0, "negative size");
    GX_CHECK_ARG(nbody >= 1 && nbody <= gx::MS32_MAXNB, "nbody must be in [1, %d] (the progenitor first)",
                 gx::MS32_MAXNB);
    GX_CHECK_ARG(max_per_release >= 0 && nbody + max_per_release <= 32,
                 "nbody + max_per_release must be <= 32 (got %d + %d)", nbody, max_per_release);
    GX_CHECK_ARG(nmax >= 0, "nmax must be >= 0 (0 = gala's default 1e6)");
    GX_CHECK_ARG(atol >= 0 && rtol >= 0, "tolerances must be non-negative");
    GX_CHECK_ARG(dt0 != 0.0, "dt0 must be non-zero");
    if (n_streams == 0 || n_release == 0) return GX_OK;
    GX_CHECK_ARG(bodies && nbody_w && release_t && release_offset && status && queue_counter, "NULL array");
    GX_CHECK_ARG(n_particles == 0 || (stream_w0 && stream_w_out), "NULL particle array");
    gx::Ms32Args A;
    memset(&A, 0, sizeof(A));
    A.gs = nbody + max_per_release;
    A.nbody = nbody;
    A.n_sys = n_streams * n_release;
    A.n_streams = n_streams;
    A.n_release = n_release;
    A.n_particles = n_particles;
    A.bodies = bodies;
    A.nbody_w = nbody_w;
    A.release_t = release_t;
    A.offset = release_offset;
    A.stream_w0 = stream_w0;
    A.t_final = t_final;
    A.dt0 = dt0;
    A.atol = atol;
    A.rtol = rtol;
    A.nmax = nmax;
    A.stream_w_out = stream_w_out;
    A.nbody_w_out = nbody_w_out;
    A.status = status;
    A.stats = stats;
    A.counter = reinterpret_cast<unsigned long long *>(queue_counter);
    A.cancel = gx::cancel_flag();
    cudaStream_t st = gx::as_stream(stream);
    const bool mw = dp.ncomp == 4 && dp.c[0].type == GX_POT_HERNQUIST && dp.c[1].type == GX_POT_HERNQUIST &&
                    dp.c[2].type == GX_POT_MIYAMOTONAGAI && dp.c[3].type == GX_POT_SPHERICALNFW &&
                    !(dp.c[0].do_sr | dp.c[1].do_sr | dp.c[2].do_sr | dp.c[3].do_sr);
    using namespace gx;
    if (mw)
        return launch_ms32<PotSig<GX_POT_HERNQUIST, GX_POT_HERNQUIST, GX_POT_MIYAMOTONAGAI, GX_POT_SPHERICALNFW>>(dp, A,
                                                                                                              st);
    return launch_ms32<SigGeneric>(dp, A, st);
}
