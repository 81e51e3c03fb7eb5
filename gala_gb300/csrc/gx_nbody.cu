// gx_nbody.cu -- FP64 DOP853 for many small direct n-body systems, and the
// Fardal release sampler of mock streams.
//
// Two gala paths integrate many small, independent ODE systems of a few bodies:
//   * DirectNBody.integrate_orbit with DOPRI853 (src/gala/dynamics/nbody/core.py:
//     166-260 -> direct_nbody_dop853, nbody.pyx:30-115 -> dop853_helper,
//     dop853.pyx:90-193) on one system of massive bodies (+ test particles);
//   * mockstream_dop853 (src/gala/dynamics/mockstream/mockstream.pyx:176-303):
//     for every release time one dop853_step call (dop853.pyx:27-75) on
//     [massive bodies at that time, the particles released then], from the
//     release time to the final time.
// Every system is ONE DOP853 problem (dopcor, dopri/dop853.cpp:89-650) over its
// 6 * nsys components in gala's AoS order (body 0: x..vz, body 1, ...): one step
// size, one error norm, one accept/reject and stiffness test.  The right-hand
// side is Fwrapper_direct_nbody (dop853.cpp:990-1006): Hamilton's equations in
// the external potential for every body, then c_nbody_acceleration
// (cpotential.cpp:389-415): every non-null massive body j pulls every other
// body with its own potential shifted to body j's position.
//
// GPU mapping: a system is a GROUP of `gs` consecutive lanes of a warp, one
// lane per body (32 / gs groups per warp).
//   * Stage algebra runs per lane on its six components, in gala's term order
//     as fused multiply-add chains, with the external force and the step
//     controller in the FP64-pipe-lean forms of gx_fast64.cuh (this unit is
//     compiled with -fmad=false: only the explicit fma calls fuse).
//   * The n-body force broadcasts body j's position to the group with warp
//     shuffles; each other lane adds -grad of body j's potential, j ascending.
//   * The error norms and the stiffness sums are SEQUENTIAL sums in gala's
//     component order: the running sum travels lane to lane (shuffle), each lane
//     adding its six terms, so every norm sums in gala's order.
//   * Groups take systems from a global counter, longest first; a group that
//     finishes takes the next system at once, so a warp never idles on its
//     slowest system.  Every loop is bounded by nmax like gala's.
#include "gx_host.h"
#include "gx_scf.cuh"
#include "gx_dop853_tableau.cuh"
#include "gx_body.cuh"
#include "gx_fast64.cuh"

static_assert(sizeof(gx_body) == 64, "gx_body layout");

namespace gx {

constexpr int NB_THREADS = 128;

struct NbArgs {
    int32_t gs;             // lanes per group (largest system)
    int32_t nbody;          // massive bodies per system (the first lanes)
    int64_t n_sys;          // systems in the queue
    const gx_body *bodies;  // (n_streams or n_sys, nbody)
    double atol, rtol;
    int64_t nmax;
    // direct n-body systems
    int32_t nparticles;
    int32_t save_all;
    const double *w0;       // (n_sys, nparticles, 6)
    const double *t;
    int64_t ntimes, out_stride, n_out, nstiff;
    double dt_max;
    double *w_out;
    // release systems of mock streams
    int64_t n_streams, n_release, n_particles;
    const double *nbody_w;  // (n_streams, n_release, nbody, 6)
    const double *release_t;
    const int64_t *offset;  // (n_release + 1)
    const double *stream_w0;
    double t_final, dt0;
    double *stream_w_out, *nbody_w_out;
    // outputs
    int32_t *status;
    int64_t *stats;
    unsigned long long *counter;
    const int32_t *cancel;  // host cancel flag (mapped memory) or nullptr
};

__device__ __forceinline__ double nb_sign(double a, double b) { return (b < 0.0) ? -fabs(a) : fabs(a); }
__device__ __forceinline__ double nb_min(double a, double b) { return (a < b) ? a : b; }
__device__ __forceinline__ double nb_max(double a, double b) { return (a > b) ? a : b; }

// Fwrapper_direct_nbody for the lane's body: Hamilton's equations in the
// external potential, then the pull of every non-null massive body j != self.
// Out of line (one compiled copy for the fifteen call sites of a step); the
// state travels by value so it stays in registers.
template <bool SCF>
__device__ __noinline__ V6 group_rhs_call(const DevPot &pot, const DevFrame &fr, unsigned mask, int base, int member,
                                          int nmem, int nbody, const gx_body *__restrict__ bod, V6 yin) {
    V6 k = fast::rhs_call_f<SCF>(pot, fr, yin);
    for (int j = 0; j < nbody; j++) {
        const double q0x = __shfl_sync(mask, yin.v[0], base + j);
        const double q0y = __shfl_sync(mask, yin.v[1], base + j);
        const double q0z = __shfl_sync(mask, yin.v[2], base + j);
        const int type = __ldg(&bod[j].type);
        if (member != j && member < nmem && type != GX_POT_NULL) {
            double f2[3];
            body_gradient(type, bod[j].params, yin.v[0] - q0x, yin.v[1] - q0y, yin.v[2] - q0z, f2);
            k.v[3] += -f2[0];
            k.v[4] += -f2[1];
            k.v[5] += -f2[2];
        }
    }
    return k;
}

template <bool SCF>
__device__ __forceinline__ void group_rhs(const DevPot &pot, const DevFrame &fr, unsigned mask, int base, int member,
                                          int nmem, int nbody, const gx_body *__restrict__ bod, const double *yin,
                                          double *kout) {
    V6 a;
#pragma unroll
    for (int c = 0; c < 6; c++) a.v[c] = yin[c];
    const V6 r = group_rhs_call<SCF>(pot, fr, mask, base, member, nmem, nbody, bod, a);
#pragma unroll
    for (int c = 0; c < 6; c++) kout[c] = r.v[c];
}

// Sequential sums of two per-component series over the whole system, in gala's
// order: lane m adds its six terms to the running sums of lanes 0..m-1.
__device__ __forceinline__ void chain_sum2(unsigned mask, int gs, int base, int member, bool in_sys,
                                           const double *ta, const double *tb, double &sa, double &sb) {
    double a = 0.0, b = 0.0;
    for (int m = 0; m < gs; m++) {
        if (member == m && in_sys) {
#pragma unroll
            for (int c = 0; c < 6; c++) {
                a += ta[c];
                b += tb[c];
            }
        }
        a = __shfl_sync(mask, a, base + m);
        b = __shfl_sync(mask, b, base + m);
    }
    sa = a;
    sb = b;
}

#define GRHS(mask_, yin_, kout_) group_rhs<SCF>(pot, fr, (mask_), base, member, nmem, A.nbody, bod, (yin_), (kout_))

template <bool STREAM, bool DENSE, bool SCF>
__global__ void __launch_bounds__(NB_THREADS)
nbody_dop853_kernel(const __grid_constant__ DevPot pot, const __grid_constant__ DevFrame fr,
                    const __grid_constant__ NbArgs A) {
    using namespace dop;
    const int lane = threadIdx.x & 31;
    const int gs = A.gs;
    const int g = lane / gs;
    const int member = lane - g * gs;
    const int base = g * gs;
    const bool lane_ok = g < 32 / gs;
    const unsigned gmask = lane_ok ? (((gs == 32) ? 0xffffffffu : ((1u << gs) - 1u)) << base) : 0u;

    const double safe = 0.9, fac1 = 0.333, fac2 = 6.0;  // and beta = 0
    const double facc1 = 1.0 / fac1, facc2 = 1.0 / fac2;
    const double atoli = A.atol, rtoli = A.rtol;

    double y[6], k1[6], k2[6], k3[6], k4[6], k5[6], k6[6], k7[6], k8[6], k9[6], k10[6], yy1[6];
    int64_t sys = 0, si = 0, ss = 0;
    int nmem = 0;
    const gx_body *bod = A.bodies;
    double x = 0., xend = 0., h = 0., hmax = 0., posneg = 1., uround = 0., facold = 0., hlamb = 0.;
    int64_t nmax = 0, nstiff = 0, nfcn = 0, nstep = 0, naccpt = 0, nrejct = 0, out_idx = 0, out_slot = 0;
    int last = 0, reject = 0, iasti = 0, nonsti = 0, idid = 0;
    bool have = false, done = !lane_ok, need_init = false;

    for (;;) {
        // -- a group without a system takes the next one (group-local) --------
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
                sys = (int64_t)id;
                if constexpr (STREAM) {
                    si = sys / A.n_streams;
                    ss = sys - si * A.n_streams;
                    const int64_t o0 = A.offset[si], o1 = A.offset[si + 1];
                    // nothing released at this time (gala skips it), or an offset
                    // table inconsistent with the particle array (rejected, no access)
                    const bool bad = o1 < o0 || o0 < 0 || o1 > A.n_particles || o1 - o0 > gs - A.nbody;
                    if (o1 == o0 || bad) {
                        if (member == 0) {
                            (void)GX_DBG_CHECK(!bad, DBG_OFFSET, si, A.n_release);
                            A.status[ss * A.n_release + si] = bad ? -1 : 0;
                            if (A.stats)
                                for (int k = 0; k < 4; k++) A.stats[(ss * A.n_release + si) * 4 + k] = 0;
                        }
                        continue;
                    }
                    nmem = A.nbody + (int)(o1 - o0);
                    bod = A.bodies + ss * A.nbody;
                    if (member < A.nbody) {
                        const double *src = A.nbody_w + ((ss * A.n_release + si) * A.nbody + member) * 6;
#pragma unroll
                        for (int c = 0; c < 6; c++) y[c] = src[c];
                    } else if (member < nmem) {
                        const double *src = A.stream_w0 + (ss * A.n_particles + o0 + (member - A.nbody)) * 6;
#pragma unroll
                        for (int c = 0; c < 6; c++) y[c] = src[c];
                    } else {
#pragma unroll
                        for (int c = 0; c < 6; c++) y[c] = 0.;
                    }
                    // dop853_step's dop853() arguments (dop853.pyx:46-72) and front-end defaults
                    x = A.release_t[si];
                    xend = A.t_final;
                    h = A.dt0;
                    uround = 2.3E-16;
                    nstiff = 1;
                    hmax = xend - x;
                } else {
                    nmem = A.nparticles;
                    bod = A.bodies + sys * A.nbody;
                    if (member < nmem) {
                        const double *src = A.w0 + (sys * A.nparticles + member) * 6;
#pragma unroll
                        for (int c = 0; c < 6; c++) y[c] = src[c];
                    } else {
#pragma unroll
                        for (int c = 0; c < 6; c++) y[c] = 0.;
                    }
                    // dop853_helper's dop853() arguments (dop853.pyx:157-182)
                    x = A.t[0];
                    xend = A.t[A.ntimes - 1];
                    h = A.t[1] - A.t[0];
                    uround = 2.220446049250313e-16;
                    nstiff = A.nstiff;
                    hmax = A.dt_max;
                    if (hmax == 0.0) hmax = xend - x;
                }
                nmax = A.nmax;
                if (!nmax) nmax = 1000000;
                if (!nstiff) nstiff = 1000;
                else if (nstiff < 0) nstiff = nmax + 10;
                posneg = nb_sign(1.0, xend - x);
                facold = 1.0E-4;
                hlamb = 0.0;
                last = reject = iasti = nonsti = idid = 0;
                nfcn = nstep = naccpt = nrejct = 0;
                out_idx = out_slot = 0;
                have = true;
                need_init = true;
                break;
            }
        }
        const unsigned act = __ballot_sync(0xffffffffu, have);
        if (act == 0u) break;
        if (!have) continue;
        const bool in_sys = member < nmem;

        // -- first derivative and, when h0 == 0, hinit (dop853.cpp:18-86) ------
        {
            const unsigned im = __ballot_sync(act, need_init);
            if (need_init) {
                GRHS(im, y, k1);
                hmax = fabs(hmax);
                if (h == 0.0) {
                    double ta[6], tb[6];
#pragma unroll
                    for (int c = 0; c < 6; c++) {
                        const double sk = atoli + rtoli * fabs(y[c]);
                        double sqr = k1[c] / sk;
                        ta[c] = sqr * sqr;
                        sqr = y[c] / sk;
                        tb[c] = sqr * sqr;
                    }
                    double dnf, dny;
                    chain_sum2(im, gs, base, member, in_sys, ta, tb, dnf, dny);
                    double hh = ((dnf <= 1.0E-10) || (dny <= 1.0E-10)) ? 1.0E-6 : sqrt(dny / dnf) * 0.01;
                    hh = nb_min(hh, hmax);
                    hh = nb_sign(hh, posneg);
#pragma unroll
                    for (int c = 0; c < 6; c++) yy1[c] = y[c] + hh * k1[c];
                    GRHS(im, yy1, k2);
#pragma unroll
                    for (int c = 0; c < 6; c++) {
                        const double sk = atoli + rtoli * fabs(y[c]);
                        const double sqr = (k2[c] - k1[c]) / sk;
                        ta[c] = sqr * sqr;
                        tb[c] = 0.;
                    }
                    double der2, unused;
                    chain_sum2(im, gs, base, member, in_sys, ta, tb, der2, unused);
                    der2 = sqrt(der2) / hh;
                    const double der12 = nb_max(fabs(der2), sqrt(dnf));
                    const double h1 =
                        (der12 <= 1.0E-15) ? nb_max(1.0E-6, fabs(hh) * 1.0E-3) : pow(0.01 / der12, 1.0 / 8.0);
                    hh = nb_min(100.0 * fabs(hh), nb_min(h1, hmax));
                    h = nb_sign(hh, posneg);
                }
                nfcn += 2;
                need_init = false;
            }
        }

        // -- step guards (dop853.cpp:321-334) ----------------------------------
        bool fin = false;
        if (nstep > nmax || h != h) {
            // a NaN step size never recovers: gala would reject until nstep > nmax
            // and return -2; that outcome is returned at once
            idid = -2;
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
            const double xold = x, hout = h;
            nstep++;

            // the twelve stages (dop853.cpp:368-414)
#pragma unroll
            for (int c = 0; c < 6; c++) yy1[c] = fma(h * a21, k1[c], y[c]);
            GRHS(am, yy1, k2);
#pragma unroll
            for (int c = 0; c < 6; c++) yy1[c] = fma(h, fma(a32, k2[c], a31 * k1[c]), y[c]);
            GRHS(am, yy1, k3);
#pragma unroll
            for (int c = 0; c < 6; c++) yy1[c] = fma(h, fma(a43, k3[c], a41 * k1[c]), y[c]);
            GRHS(am, yy1, k4);
#pragma unroll
            for (int c = 0; c < 6; c++) yy1[c] = fma(h, fma(a54, k4[c], fma(a53, k3[c], a51 * k1[c])), y[c]);
            GRHS(am, yy1, k5);
#pragma unroll
            for (int c = 0; c < 6; c++) yy1[c] = fma(h, fma(a65, k5[c], fma(a64, k4[c], a61 * k1[c])), y[c]);
            GRHS(am, yy1, k6);
#pragma unroll
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a76, k6[c], fma(a75, k5[c], fma(a74, k4[c], a71 * k1[c]))), y[c]);
            GRHS(am, yy1, k7);
#pragma unroll
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a87, k7[c], fma(a86, k6[c], fma(a85, k5[c], fma(a84, k4[c], a81 * k1[c])))), y[c]);
            GRHS(am, yy1, k8);
#pragma unroll
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a98, k8[c], fma(a97, k7[c], fma(a96, k6[c], fma(a95, k5[c],
                    fma(a94, k4[c], a91 * k1[c]))))), y[c]);
            GRHS(am, yy1, k9);
#pragma unroll
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a109, k9[c], fma(a108, k8[c], fma(a107, k7[c], fma(a106, k6[c], fma(a105, k5[c],
                    fma(a104, k4[c], a101 * k1[c])))))), y[c]);
            GRHS(am, yy1, k10);
#pragma unroll
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a1110, k10[c], fma(a119, k9[c], fma(a118, k8[c], fma(a117, k7[c], fma(a116, k6[c],
                    fma(a115, k5[c], fma(a114, k4[c], a111 * k1[c]))))))), y[c]);
            GRHS(am, yy1, k2);
            const double xph = x + h;
#pragma unroll
            for (int c = 0; c < 6; c++)
                yy1[c] = fma(h, fma(a1211, k2[c], fma(a1210, k10[c], fma(a129, k9[c], fma(a128, k8[c], fma(a127, k7[c],
                    fma(a126, k6[c], fma(a125, k5[c], fma(a124, k4[c], a121 * k1[c])))))))), y[c]);
            GRHS(am, yy1, k3);
            nfcn += 11;
#pragma unroll
            for (int c = 0; c < 6; c++) {
                k4[c] = fma(b12, k3[c], fma(b11, k2[c], fma(b10, k10[c], fma(b9, k9[c], fma(b8, k8[c], fma(b7, k7[c],
                            fma(b6, k6[c], b1 * k1[c])))))));
                k5[c] = fma(h, k4[c], y[c]);
            }

            // error estimation (:416-444), sequential over the system
            double err, err2;
            {
                double t1[6], t2[6];
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    const double isk = fast::rcp_f(fma(rtoli, fmax(fabs(y[c]), fabs(k5[c])), atoli));
                    double erri = fma(-bhh3, k3[c], fma(-bhh2, k9[c], fma(-bhh1, k1[c], k4[c])));
                    double sqr = erri * isk;
                    t2[c] = sqr * sqr;
                    erri = fma(er12, k3[c], fma(er11, k2[c], fma(er10, k10[c], fma(er9, k9[c], fma(er8, k8[c],
                               fma(er7, k7[c], fma(er6, k6[c], er1 * k1[c])))))));
                    sqr = erri * isk;
                    t1[c] = sqr * sqr;
                }
                chain_sum2(am, gs, base, member, in_sys, t1, t2, err, err2);
            }
            double deno = err + 0.01 * err2;
            if (deno <= 0.0) deno = 1.0;
            err = fabs(h) * err * sqrt(1.0 / (deno * (double)(6 * nmem)));

            // computation of hnew (:446-452)
            // pow(err, expo1) with expo1 = 1/8 (beta = 0): three square roots
            const double fac11 = sqrt(sqrt(sqrt(err)));
            double fac = fac11;  // gala divides by pow(facold, beta) == 1 for its beta = 0
            (void)facold;
            fac = nb_max(facc2, nb_min(facc1, fac / safe));
            double hnew = h / fac;
            const bool acc = err <= 1.0;

            // FSAL derivative for every group; a rejected group never reads it
            GRHS(am, k5, k4);
            if (acc) {
                facold = nb_max(err, 1.0E-4);
                naccpt++;
                nfcn++;
            }

            // stiffness detection (:463-486); the first detection returns -4 as in gala
            bool stiff = false;
            const bool test_st = acc && (!(naccpt % nstiff) || (iasti > 0));
            if (__ballot_sync(am, test_st)) {
                double ta[6], tb[6];
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    double sqr = k4[c] - k3[c];
                    ta[c] = sqr * sqr;
                    sqr = k5[c] - yy1[c];
                    tb[c] = sqr * sqr;
                }
                double stnum, stden;
                chain_sum2(am, gs, base, member, in_sys, ta, tb, stnum, stden);
                if (test_st) {
                    if (stden > 0.0) hlamb = h * sqrt(stnum / stden);
                    if (hlamb > 6.1) {
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

            if constexpr (DENSE) {
                // dense output (:492-612), evaluated by every group, written by accepted ones
                double r5[6], r6[6], r7[6], r8[6];
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    r5[c] = d41 * k1[c] + d46 * k6[c] + d47 * k7[c] + d48 * k8[c] + d49 * k9[c] + d410 * k10[c] +
                            d411 * k2[c] + d412 * k3[c];
                    r6[c] = d51 * k1[c] + d56 * k6[c] + d57 * k7[c] + d58 * k8[c] + d59 * k9[c] + d510 * k10[c] +
                            d511 * k2[c] + d512 * k3[c];
                    r7[c] = d61 * k1[c] + d66 * k6[c] + d67 * k7[c] + d68 * k8[c] + d69 * k9[c] + d610 * k10[c] +
                            d611 * k2[c] + d612 * k3[c];
                    r8[c] = d71 * k1[c] + d76 * k6[c] + d77 * k7[c] + d78 * k8[c] + d79 * k9[c] + d710 * k10[c] +
                            d711 * k2[c] + d712 * k3[c];
                }
#pragma unroll
                for (int c = 0; c < 6; c++)
                    yy1[c] = fma(h, fma(a1413, k4[c], fma(a1412, k3[c], fma(a1411, k2[c], fma(a1410, k10[c],
                        fma(a149, k9[c], fma(a148, k8[c], fma(a147, k7[c], a141 * k1[c]))))))), y[c]);
                GRHS(am, yy1, k10);
#pragma unroll
                for (int c = 0; c < 6; c++)
                    yy1[c] = fma(h, fma(a1514, k10[c], fma(a1513, k4[c], fma(a1512, k3[c], fma(a1511, k2[c],
                        fma(a158, k8[c], fma(a157, k7[c], fma(a156, k6[c], a151 * k1[c]))))))), y[c]);
                GRHS(am, yy1, k2);
#pragma unroll
                for (int c = 0; c < 6; c++)
                    yy1[c] = fma(h, fma(a1615, k2[c], fma(a1614, k10[c], fma(a1613, k4[c], fma(a169, k9[c],
                        fma(a168, k8[c], fma(a167, k7[c], fma(a166, k6[c], a161 * k1[c]))))))), y[c]);
                GRHS(am, yy1, k3);
                if (acc && !stiff) {
                    nfcn += 3;
                    double r1[6], r2[6], r3[6], r4[6];
#pragma unroll
                    for (int c = 0; c < 6; c++) {
                        r5[c] = h * (r5[c] + d413 * k4[c] + d414 * k10[c] + d415 * k2[c] + d416 * k3[c]);
                        r6[c] = h * (r6[c] + d513 * k4[c] + d514 * k10[c] + d515 * k2[c] + d516 * k3[c]);
                        r7[c] = h * (r7[c] + d613 * k4[c] + d614 * k10[c] + d615 * k2[c] + d616 * k3[c]);
                        r8[c] = h * (r8[c] + d713 * k4[c] + d714 * k10[c] + d715 * k2[c] + d716 * k3[c]);
                        r1[c] = y[c];
                        const double ydiff = k5[c] - y[c];
                        r2[c] = ydiff;
                        const double bspl = h * k1[c] - ydiff;
                        r3[c] = bspl;
                        r4[c] = ydiff - h * k4[c] - bspl;
                    }
                    const double x0 = xold, x1 = x0 + hout;
                    while (out_idx < A.ntimes) {
                        const double t_out = A.t[out_idx];
                        if (!((x0 <= t_out && t_out <= x1) || (x1 <= t_out && t_out <= x0))) break;
                        if (out_idx % A.out_stride == 0) {
                            const double s = (t_out - xold) / hout;
                            const double s1 = 1.0 - s;
                            if (in_sys) {
                                double *o = A.w_out + ((sys * A.n_out + out_slot) * A.nparticles + member) * 6;
#pragma unroll
                                for (int c = 0; c < 6; c++)
                                    o[c] = r1[c] + s * (r2[c] + s1 * (r3[c] + s * (r4[c] +
                                                    s1 * (r5[c] + s * (r6[c] + s1 * (r7[c] + s * r8[c]))))));
                            }
                            out_slot++;
                        }
                        out_idx++;
                    }
                }
            }

            if (acc && !stiff) {
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    k1[c] = k4[c];
                    y[c] = k5[c];
                }
                x = xph;
                if (last) {
                    idid = 1;
                } else {
                    if (fabs(hnew) > hmax) hnew = posneg * hmax;
                    if (reject) hnew = posneg * nb_min(fabs(hnew), fabs(h));
                    reject = 0;
                }
            } else if (!acc) {
                hnew = h / nb_min(facc1, fac11 / safe);
                reject = 1;
                if (naccpt >= 1) nrejct = nrejct + 1;
                last = 0;
            }
            h = hnew;
        }

        // -- a finished system writes its results --------------------------------
        if (idid != 0) {
            if constexpr (STREAM) {
                const int64_t o0 = A.offset[si];
                if (member >= A.nbody && member < nmem) {
                    double *o = A.stream_w_out + (ss * A.n_particles + o0 + (member - A.nbody)) * 6;
#pragma unroll
                    for (int c = 0; c < 6; c++) o[c] = y[c];
                }
                // the bodies after the last release system (mockstream.pyx:287-289)
                if (member < A.nbody && A.nbody_w_out && A.offset[si + 1] == A.offset[A.n_release]) {
                    double *o = A.nbody_w_out + (ss * A.nbody + member) * 6;
#pragma unroll
                    for (int c = 0; c < 6; c++) o[c] = y[c];
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
            } else {
                if (!A.save_all && in_sys) {
                    double *o = A.w_out + (sys * A.nparticles + member) * 6;
#pragma unroll
                    for (int c = 0; c < 6; c++) o[c] = y[c];
                }
                if (member == 0) {
                    A.status[sys] = idid;
                    if (A.stats) {
                        A.stats[4 * sys + 0] = nfcn;
                        A.stats[4 * sys + 1] = nstep;
                        A.stats[4 * sys + 2] = naccpt;
                        A.stats[4 * sys + 3] = nrejct;
                    }
                }
            }
            have = false;
        }
    }
    (void)nonsti;
}
#undef GRHS

// ---------------------------------------------------------------------------
// Fardal release sampler: FardalStreamDF._sample (df.pyx:363-457) with
// BaseStreamDF.get_rj_vj_R (:61-92), transform_from_sat (:94-106), the helpers
// of _coord.pyx (cross, norm, apply_3matrix) and c_d2_dr2 (cpotential.cpp:346-371).
// One thread per (stream, time).  The normal draws are made on the host by the
// caller's random state in gala's order and passed in.
// ---------------------------------------------------------------------------
struct FardalArgs {
    int64_t n_streams, ntimes, n_particles;
    const double *prog_w;   // (n_streams, ntimes, row_stride): x, v of the progenitor first
    int64_t row_stride;
    const double *prog_m;   // (n_streams, ntimes)
    const double *t;        // (ntimes)
    const int64_t *offset;  // (ntimes + 1) first row of the particles released at each time
    const double *draws;    // (n_streams, n_particles, ndraw), see release_offsets
    double G;
    int32_t lead, trail, gala_modified;
    int32_t kind, ndraw;    // 0 Fardal (4 draws), 1 Lagrange cloud (3), 2 Chen (6)
    double *w_out;          // (n_streams, n_particles, 6)
};

// Release placement in the satellite frame (x along the progenitor's radius
// vector, z along its angular momentum) of one particle of tail `tail` (0
// trailing, 1 leading):
//   kind 0, FardalStreamDF (df.pyx:410-450): draws kx, kz, kvt, kvz;
//   kind 1, LagrangeCloudStreamDF (df.pyx:515-552): (+-rj, 0, 0), velocity the
//     three draws (each normal(0, v_disp), drawn by the caller);
//   kind 2, ChenStreamDF (df.pyx:614-700): the six multivariate-normal draws
//     r, phi, theta, v, alpha, beta (degrees); Dr = r rj, Dv = v sqrt(2 G m / Dr);
//     the leading tail adds pi to phi and alpha.
// Components gala leaves unset are zero.
__device__ __forceinline__ void release_offsets(int kind, int gala_modified, const double *d, int tail, double rj,
                                                double vj, double G, double m, double *tx, double *tv) {
    const double sr = (tail == 0) ? rj : -rj, sv = (tail == 0) ? vj : -vj;
    tx[0] = tx[1] = tx[2] = 0.;
    tv[0] = tv[1] = tv[2] = 0.;
    if (kind == 0) {
        const double kx = d[0];
        tx[0] = kx * sr;
        tx[2] = d[1] * sr;
        tv[1] = d[2] * sv;
        if (gala_modified) tv[1] *= kx;
        tv[2] = d[3] * sv;
    } else if (kind == 1) {
        tx[0] = sr;
        tv[0] = d[0];
        tv[1] = d[1];
        tv[2] = d[2];
    } else {
        const double pi = 3.14159265358979323846;
        const double Dr = d[0] * rj;
        const double Dv = d[3] * sqrt(2 * G * m / Dr);
        double p1 = d[1] * (pi / 180), p2 = d[2] * (pi / 180), p4 = d[4] * (pi / 180), p5 = d[5] * (pi / 180);
        if (tail == 1) {
            p1 = p1 + pi;
            p4 = p4 + pi;
        }
        tx[0] = Dr * cos(p2) * cos(p1);
        tx[1] = Dr * cos(p2) * sin(p1);
        tx[2] = Dr * sin(p2);
        tv[0] = Dv * cos(p5) * cos(p4);
        tv[1] = Dv * cos(p5) * sin(p4);
        tv[2] = Dv * sin(p5);
    }
}

// c_potential at one point (cpotential.cpp:170-189).
template <bool SCF>
__device__ __noinline__ double fardal_phi(const DevPot &pot, V3 q) {
    return potential_value<SCF>(pot, q.v);
}

template <bool SCF>
__global__ void __launch_bounds__(128) fardal_sample_kernel(const __grid_constant__ DevPot pot, const FardalArgs A) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= A.n_streams * A.ntimes) return;
    const int64_t s = idx / A.ntimes, i = idx - s * A.ntimes;
    const int64_t o0 = A.offset[i], o1 = A.offset[i + 1];
    const int ntail = A.lead + A.trail;
    if (o1 <= o0 || o0 < 0 || o1 > A.n_particles || ntail == 0) return;
    const int64_t np = (o1 - o0) / ntail;
    const double *pw = A.prog_w + (s * A.ntimes + i) * A.row_stride;
    const double px[3] = {pw[0], pw[1], pw[2]}, pv[3] = {pw[3], pw[4], pw[5]};
    const double m = A.prog_m[s * A.ntimes + i];

    // get_rj_vj_R
    double dist = 0.;
    for (int k = 0; k < 3; k++) dist += px[k] * px[k];
    dist = sqrt(dist);
    double L[3];
    L[0] = px[1] * pv[2] - px[2] * pv[1];
    L[1] = -px[0] * pv[2] + px[2] * pv[0];
    L[2] = px[0] * pv[1] - px[1] * pv[0];
    double Lnorm = 0.;
    for (int k = 0; k < 3; k++) Lnorm += L[k] * L[k];
    Lnorm = sqrt(Lnorm);
    double R[3][3];
    for (int k = 0; k < 3; k++) {
        R[0][k] = px[k] / dist;
        R[2][k] = L[k] / Lnorm;
    }
    const double Om = Lnorm / (dist * dist);
    // c_d2_dr2 with h = 1e-2
    double d2r;
    {
        double r2 = 0;
        for (int j = 0; j < 3; j++) r2 = r2 + px[j] * px[j];
        const double hh = 1E-2;
        const double r = sqrt(r2);
        V3 e;
        for (int j = 0; j < 3; j++) e.v[j] = px[j] + hh * px[j] / r;
        d2r = fardal_phi<SCF>(pot, e);
        V3 q0;
        for (int j = 0; j < 3; j++) q0.v[j] = px[j];
        d2r = d2r - 2. * fardal_phi<SCF>(pot, q0);
        for (int j = 0; j < 3; j++) e.v[j] = px[j] - hh * px[j] / r;
        d2r = d2r + fardal_phi<SCF>(pot, e);
        d2r = d2r / (hh * hh);
    }
    const double rj = pow(A.G * m / (Om * Om - d2r), 1 / 3.);
    const double vj = Om * rj;
    R[1][0] = -(R[0][1] * R[2][2] - R[0][2] * R[2][1]);
    R[1][1] = -(-R[0][0] * R[2][2] + R[0][2] * R[2][0]);
    R[1][2] = -(R[0][0] * R[2][1] - R[0][1] * R[2][0]);

    int64_t row = o0;
    for (int tail = 0; tail < 2; tail++) {
        if (tail == 0 && !A.trail) continue;
        if (tail == 1 && !A.lead) continue;
        for (int64_t k = 0; k < np; k++, row++) {
            double tx[3], tv[3];
            release_offsets(A.kind, A.gala_modified, A.draws + (s * A.n_particles + row) * A.ndraw, tail, rj, vj,
                            A.G, m, tx, tv);
            double *o = A.w_out + (s * A.n_particles + row) * 6;
            for (int n = 0; n < 3; n++) {
                double ox = R[0][n] * tx[0] + R[1][n] * tx[1] + R[2][n] * tx[2];
                double ov = R[0][n] * tv[0] + R[1][n] * tv[1] + R[2][n] * tv[2];
                ox += px[n];
                ov += pv[n];
                o[n] = ox;
                o[3 + n] = ov;
            }
        }
    }
}

template <bool STREAM, bool DENSE>
int launch_nbody(const DevPot &dp, const DevFrame &df, const NbArgs &A, cudaStream_t st) {
    int dev = 0, sms = 0, per_sm = 0;
    GX_CUDA_TRY(cudaGetDevice(&dev));
    GX_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (dp.has_scf)
        GX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nbody_dop853_kernel<STREAM, DENSE, true>,
                                                                  NB_THREADS, 0));
    else
        GX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nbody_dop853_kernel<STREAM, DENSE, false>,
                                                                  NB_THREADS, 0));
    if (per_sm < 1) per_sm = 1;
    const int64_t groups_per_block = (int64_t)(NB_THREADS / 32) * (32 / A.gs);
    int64_t need = (A.n_sys + groups_per_block - 1) / groups_per_block;
    int64_t grid = (int64_t)sms * per_sm;
    if (need < grid) grid = need;
    if (grid < 1) grid = 1;
    GX_CUDA_TRY(cudaMemsetAsync(A.counter, 0, sizeof(unsigned long long), st));
    if (dp.has_scf)
        nbody_dop853_kernel<STREAM, DENSE, true><<<(unsigned)grid, NB_THREADS, 0, st>>>(dp, df, A);
    else
        nbody_dop853_kernel<STREAM, DENSE, false><<<(unsigned)grid, NB_THREADS, 0, st>>>(dp, df, A);
    return check_launch(STREAM ? "mockstream_dop853" : "nbody_dop853");
}


}  // namespace gx

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" int gx_nbody_dop853(const gx_potential *pot, const gx_frame *frame, int64_t n_systems,
                               int32_t nparticles, int32_t nbody, const gx_body *bodies, const double *w0,
                               const double *t, int64_t ntimes, double atol, double rtol, int64_t nmax,
                               double dt_max, int64_t nstiff, int32_t save_all, int64_t out_stride, double *w_out,
                               int32_t *status, int64_t *stats, int64_t *queue_counter, void *stream) {
    gx::DevPot dp;
    gx::DevFrame df;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    rc = gx::pack_frame(frame, &df);
    if (rc) return rc;
    GX_CHECK_ARG(n_systems >= 0, "n_systems < 0");
    GX_CHECK_ARG(nparticles >= 1 && nparticles <= 32, "nparticles must be in [1, 32] (got %d)", nparticles);
    GX_CHECK_ARG(nbody >= 0 && nbody <= nparticles, "nbody must be in [0, nparticles] (got %d)", nbody);
    GX_CHECK_ARG(ntimes >= 2, "ntimes must be >= 2 (got %lld)", (long long)ntimes);
    GX_CHECK_ARG(out_stride >= 1, "out_stride must be >= 1");
    GX_CHECK_ARG(nmax >= 0, "nmax must be >= 0 (0 = gala's default 1e6)");
    GX_CHECK_ARG(atol >= 0 && rtol >= 0, "tolerances must be non-negative");
    if (n_systems == 0) return GX_OK;
    GX_CHECK_ARG(w0 && t && w_out && status && queue_counter, "NULL array");
    GX_CHECK_ARG(nbody == 0 || bodies, "bodies is NULL");
    gx::NbArgs A;
    memset(&A, 0, sizeof(A));
    A.gs = nparticles;
    A.nbody = nbody;
    A.n_sys = n_systems;
    A.bodies = bodies;
    A.atol = atol;
    A.rtol = rtol;
    A.nmax = nmax;
    A.nparticles = nparticles;
    A.save_all = save_all ? 1 : 0;
    A.w0 = w0;
    A.t = t;
    A.ntimes = ntimes;
    A.out_stride = out_stride;
    A.n_out = (ntimes - 1) / out_stride + 1;
    A.nstiff = nstiff;
    A.dt_max = dt_max;
    A.w_out = w_out;
    A.status = status;
    A.stats = stats;
    A.counter = reinterpret_cast<unsigned long long *>(queue_counter);
    A.cancel = gx::cancel_flag();
    cudaStream_t st = gx::as_stream(stream);
    return save_all ? gx::launch_nbody<false, true>(dp, df, A, st) : gx::launch_nbody<false, false>(dp, df, A, st);
}

extern "C" int gx_mockstream_dop853(const gx_potential *pot, const gx_frame *frame, int64_t n_streams,
                                    int32_t nbody, const gx_body *bodies, const double *nbody_w, int64_t n_release,
                                    const double *release_t, const int64_t *release_offset,
                                    int32_t max_per_release, const double *stream_w0, int64_t n_particles,
                                    double t_final, double dt0, double atol, double rtol, int64_t nmax,
                                    double *stream_w_out, double *nbody_w_out, int32_t *status, int64_t *stats,
                                    int64_t *queue_counter, void *stream) {
    gx::DevPot dp;
    gx::DevFrame df;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    rc = gx::pack_frame(frame, &df);
    if (rc) return rc;
    GX_CHECK_ARG(n_streams >= 0 && n_release >= 0 && n_particles >= 0, "negative size");
    GX_CHECK_ARG(nbody >= 1, "nbody must be >= 1 (the progenitor)");
    GX_CHECK_ARG(max_per_release >= 0 && nbody + max_per_release <= 32,
                 "nbody + max_per_release must be <= 32 (got %d + %d)", nbody, max_per_release);
    GX_CHECK_ARG(nmax >= 0, "nmax must be >= 0 (0 = gala's default 1e6)");
    GX_CHECK_ARG(atol >= 0 && rtol >= 0, "tolerances must be non-negative");
    if (n_streams == 0 || n_release == 0) return GX_OK;
    GX_CHECK_ARG(bodies && nbody_w && release_t && release_offset && status && queue_counter, "NULL array");
    GX_CHECK_ARG(n_particles == 0 || (stream_w0 && stream_w_out), "NULL particle array");
    gx::NbArgs A;
    memset(&A, 0, sizeof(A));
    A.gs = nbody + (max_per_release > 0 ? max_per_release : 0);
    A.nbody = nbody;
    A.n_sys = n_streams * n_release;
    A.bodies = bodies;
    A.atol = atol;
    A.rtol = rtol;
    A.nmax = nmax;
    A.n_streams = n_streams;
    A.n_release = n_release;
    A.n_particles = n_particles;
    A.nbody_w = nbody_w;
    A.release_t = release_t;
    A.offset = release_offset;
    A.stream_w0 = stream_w0;
    A.t_final = t_final;
    A.dt0 = dt0;
    A.stream_w_out = stream_w_out;
    A.nbody_w_out = nbody_w_out;
    A.status = status;
    A.stats = stats;
    A.counter = reinterpret_cast<unsigned long long *>(queue_counter);
    A.cancel = gx::cancel_flag();
    return gx::launch_nbody<true, false>(dp, df, A, gx::as_stream(stream));
}

extern "C" int gx_stream_sample(const gx_potential *pot, int64_t n_streams, int64_t ntimes, const double *prog_w,
                                int64_t row_stride, const double *prog_m, const double *t,
                                const int64_t *release_offset, int64_t n_particles, int32_t kind,
                                const double *draws, double G, int32_t lead, int32_t trail, int32_t gala_modified,
                                double *w_out, void *stream) {
    GX_CHECK_ARG(kind >= 0 && kind <= 2, "kind must be 0 (Fardal), 1 (Lagrange cloud) or 2 (Chen)");
    gx::DevPot dp;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(n_streams >= 0 && ntimes >= 0 && n_particles >= 0, "negative size");
    GX_CHECK_ARG(row_stride >= 6, "row_stride must be >= 6");
    GX_CHECK_ARG(lead || trail, "at least one of lead / trail must be set");
    if (n_streams == 0 || ntimes == 0 || n_particles == 0) return GX_OK;
    GX_CHECK_ARG(prog_w && prog_m && t && release_offset && draws && w_out, "NULL array");
    gx::FardalArgs A;
    A.n_streams = n_streams;
    A.ntimes = ntimes;
    A.n_particles = n_particles;
    A.prog_w = prog_w;
    A.row_stride = row_stride;
    A.prog_m = prog_m;
    A.t = t;
    A.offset = release_offset;
    A.draws = draws;
    A.G = G;
    A.lead = lead ? 1 : 0;
    A.trail = trail ? 1 : 0;
    A.gala_modified = gala_modified ? 1 : 0;
    A.kind = kind;
    A.ndraw = kind == 0 ? 4 : kind == 1 ? 3 : 6;
    A.w_out = w_out;
    const int64_t n = n_streams * ntimes;
    const unsigned grid = (unsigned)((n + 127) / 128);
    cudaStream_t st = gx::as_stream(stream);
    if (dp.has_scf)
        gx::fardal_sample_kernel<true><<<grid, 128, 0, st>>>(dp, A);
    else
        gx::fardal_sample_kernel<false><<<grid, 128, 0, st>>>(dp, A);
    return gx::check_launch("stream_sample");
}

extern "C" int gx_fardal_sample(const gx_potential *pot, int64_t n_streams, int64_t ntimes, const double *prog_w,
                                int64_t row_stride, const double *prog_m, const double *t,
                                const int64_t *release_offset, int64_t n_particles, const double *draws, double G,
                                int32_t lead, int32_t trail, int32_t gala_modified, double *w_out, void *stream) {
    return gx_stream_sample(pot, n_streams, ntimes, prog_w, row_stride, prog_m, t, release_offset, n_particles, 0,
                            draws, G, lead, trail, gala_modified, w_out, stream);
}
