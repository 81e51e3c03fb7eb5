// gx_nbody_wide.cu -- FP64 DOP853 for mock-stream release systems wider than a
// warp: one CTA per system, the system's state in device scratch.
//
// gala integrates every release of mockstream_dop853 (src/gala/dynamics/
// mockstream/mockstream.pyx:176-303) as ONE dop853_step problem (dop853.pyx:
// 27-75 -> dopcor, dopri/dop853.cpp:89-650) over [massive bodies, the particles
// released at that time]: one step size, one error norm, one accept/reject and
// stiffness decision for the whole system.  A release of thousands of particles
// (gala's one-burst setting) does not fit the 32-lane groups of gx_nbody.cu, so
// such systems run here:
//   * one CTA per system; thread t owns members t, t + blockDim, ...;
//   * the state (y, the stage derivatives, the stage argument) lives in device
//     scratch as SoA rows [array][component][member] (L2-resident);
//   * every stage is two passes separated by a barrier: all stage arguments,
//     then all right-hand sides -- a member's right-hand side reads the massive
//     bodies' stage positions (c_nbody_acceleration, cpotential.cpp:389-415);
//   * the error and stiffness sums are CTA sums in a fixed order (each thread
//     over its members in order, a warp butterfly, then the warps in order), so
//     the run is deterministic; the order differs from gala's sequential loop,
//     so results agree with gala to rounding, not bit for bit;
//   * every scalar of the controller is computed identically by all threads from
//     the same sums (uniform control flow), and the loop is bounded by nmax.
#include "gx_host.h"
#include "gx_scf.cuh"
#include "gx_dop853_tableau.cuh"
#include "gx_body.cuh"
#include "gx_fast64.cuh"

namespace gx {

constexpr int WD_THREADS = 256;
constexpr int WD_ARRAYS = 12;     // Y, K1..K10, YY1
constexpr int WD_ARRAYS_D = 16;   // and the dense-output coefficients R5..R8 (DirectNBody)

enum { A_Y = 0, A_K1, A_K2, A_K3, A_K4, A_K5, A_K6, A_K7, A_K8, A_K9, A_K10, A_YY1, A_R5, A_R6, A_R7, A_R8 };

struct WideArgs {
    int32_t nbody;
    int32_t max_members;
    int64_t n_streams, n_release, n_particles;
    const gx_body *bodies;    // (n_streams, nbody)
    const double *nbody_w;    // (n_streams, n_release, nbody, 6)
    const double *release_t;  // (n_release)
    const int64_t *offset;    // (n_release + 1)
    const double *stream_w0;  // (n_streams, n_particles, 6)
    double t_final, dt0, atol, rtol;
    int64_t nmax;
    const int64_t *systems;   // system ids si * n_streams + ss handled here
    int64_t n_systems;
    double *scratch;          // n_systems x WD_ARRAYS x 6 x max_members doubles
    double *stream_w_out, *nbody_w_out;
    int32_t *status;
    int64_t *stats;
    const int32_t *cancel;    // host cancel flag (mapped memory) or nullptr
};

// Deterministic CTA sums of two values (each thread passes its partials).
__device__ __forceinline__ void cta_sum2(double &a, double &b, double *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
        red[wid] = a;
        red[32 + wid] = b;
    }
    __syncthreads();
    double sa = 0., sb = 0.;
    for (int w = 0; w < nw; w++) {
        sa += red[w];
        sb += red[32 + w];
    }
    __syncthreads();
    a = sa;
    b = sb;
}

// Fwrapper_direct_nbody (dop853.cpp:990-1006) for member m of the system:
// Hamilton's equations in the external potential, then the pull of every
// non-null massive body j != m at its stage position.
template <bool SCF>
__device__ __forceinline__ void wide_rhs(const DevPot &pot, const DevFrame &fr, const gx_body *__restrict__ bod,
                                         int nbody, const double *__restrict__ arg, int64_t M, int m,
                                         double *__restrict__ kout) {
    V6 w;
#pragma unroll
    for (int c = 0; c < 6; c++) w.v[c] = arg[c * M + m];
    V6 k = fast::rhs_call_f<SCF>(pot, fr, w);
    for (int j = 0; j < nbody; j++) {
        const int type = __ldg(&bod[j].type);
        if (j == m || type == GX_POT_NULL) continue;
        double f2[3];
        body_gradient(type, bod[j].params, w.v[0] - arg[j], w.v[1] - arg[M + j], w.v[2] - arg[2 * M + j], f2);
        k.v[3] += -f2[0];
        k.v[4] += -f2[1];
        k.v[5] += -f2[2];
    }
#pragma unroll
    for (int c = 0; c < 6; c++) kout[c * M + m] = k.v[c];
}

// The dop853() arguments that differ between gala's two callers of these
// systems: dop853_step (dop853.pyx:27-75; mock-stream releases and the animate
// mode: uround 2.3e-16, nstiff 1, hmax = the interval) and dop853_helper
// (dop853.pyx:90-193; DirectNBody: uround = eps, nstiff and dt_max as given).
struct WideOpts {
    double uround;
    int64_t nstiff;  // after the front-end defaults (0 -> 1000, < 0 -> nmax + 10)
    double hmax;     // > 0
};

// Dense output of a DirectNBody system onto the output grid: w_out (n_systems,
// n_out, nparticles, 6) for every out_stride-th time of t (dop853.cpp:584-612).
struct WideDense {
    const double *t;
    int64_t ntimes, out_stride, n_out, sys;
    double *w_out;
    int64_t out_idx, out_slot;  // the same on every thread
};

// One dop853() call on the system of the first nmem members, from x to xend
// with the initial step h, run by the whole CTA.  The state is Ar[A_Y] (SoA rows
// of stride M); the other arrays are the stage derivatives, the stage argument
// and, with DENSE, the dense-output coefficients.  Adds {nfcn, nstep, naccpt,
// nrejct} to ctr and returns gala's idid; every thread returns the same value,
// after a barrier.
template <bool SCF, bool DENSE = false>
__device__ __forceinline__ int wide_dop853(const DevPot &pot, const DevFrame &fr, const gx_body *__restrict__ bod,
                                           int nbody, int nmem, int64_t M, double *const *Ar, double *red, double x,
                                           const double xend, double h, const double atoli, const double rtoli,
                                           const int64_t nmax_in, int64_t *ctr, const WideOpts &opt,
                                           WideDense *dn = nullptr) {
    using namespace dop;
    const int tid = threadIdx.x, nt = blockDim.x;
    __syncthreads();
    for (int m = tid; m < nmem; m += nt) wide_rhs<SCF>(pot, fr, bod, nbody, Ar[A_Y], M, m, Ar[A_K1]);
    __syncthreads();

    const double uround = opt.uround;
    const int64_t nmax = nmax_in ? nmax_in : 1000000;
    const int64_t nstiff = opt.nstiff;
    const double hmax = opt.hmax;
    const double posneg = (xend - x < 0.0) ? -1.0 : 1.0;
    const double safe = 0.9, facc1 = 1.0 / 0.333, facc2 = 1.0 / 6.0;
    int last = 0, reject = 0, iasti = 0, nonsti = 0, idid = 0;
    double hlamb = 0.0;
    int64_t nfcn = 2, nstep = 0, naccpt = 0, nrejct = 0;

#define WSTAGE(dst, expr)                                                                              \
    for (int m = tid; m < nmem; m += nt)                                                               \
        for (int c = 0; c < 6; c++) {                                                                  \
            const int64_t o = c * M + m;                                                               \
            Ar[A_YY1][o] = (expr);                                                                     \
        }                                                                                              \
    __syncthreads();                                                                                   \
    for (int m = tid; m < nmem; m += nt) wide_rhs<SCF>(pot, fr, bod, nbody, Ar[A_YY1], M, m, Ar[dst]); \
    __syncthreads()
#define K(a) Ar[a][o]

    for (;;) {
        if (nstep > nmax || h != h) {
            idid = -2;  // a NaN step never recovers: gala's -2 after nmax rejections, at once
            break;
        }
        if (0.1 * fabs(h) <= fabs(x) * uround) {
            idid = -3;
            break;
        }
        if ((x + 1.01 * h - xend) * posneg > 0.0) {
            h = xend - x;
            last = 1;
        }
        nstep++;
        // the twelve stages (dop853.cpp:368-414), gala's term order as FMA chains
        WSTAGE(A_K2, fma(h * a21, K(A_K1), K(A_Y)));
        WSTAGE(A_K3, fma(h, fma(a32, K(A_K2), a31 * K(A_K1)), K(A_Y)));
        WSTAGE(A_K4, fma(h, fma(a43, K(A_K3), a41 * K(A_K1)), K(A_Y)));
        WSTAGE(A_K5, fma(h, fma(a54, K(A_K4), fma(a53, K(A_K3), a51 * K(A_K1))), K(A_Y)));
        WSTAGE(A_K6, fma(h, fma(a65, K(A_K5), fma(a64, K(A_K4), a61 * K(A_K1))), K(A_Y)));
        WSTAGE(A_K7, fma(h, fma(a76, K(A_K6), fma(a75, K(A_K5), fma(a74, K(A_K4), a71 * K(A_K1)))), K(A_Y)));
        WSTAGE(A_K8, fma(h, fma(a87, K(A_K7), fma(a86, K(A_K6), fma(a85, K(A_K5), fma(a84, K(A_K4),
                     a81 * K(A_K1))))), K(A_Y)));
        WSTAGE(A_K9, fma(h, fma(a98, K(A_K8), fma(a97, K(A_K7), fma(a96, K(A_K6), fma(a95, K(A_K5),
                     fma(a94, K(A_K4), a91 * K(A_K1)))))), K(A_Y)));
        WSTAGE(A_K10, fma(h, fma(a109, K(A_K9), fma(a108, K(A_K8), fma(a107, K(A_K7), fma(a106, K(A_K6),
                      fma(a105, K(A_K5), fma(a104, K(A_K4), a101 * K(A_K1))))))), K(A_Y)));
        WSTAGE(A_K2, fma(h, fma(a1110, K(A_K10), fma(a119, K(A_K9), fma(a118, K(A_K8), fma(a117, K(A_K7),
                     fma(a116, K(A_K6), fma(a115, K(A_K5), fma(a114, K(A_K4), a111 * K(A_K1)))))))), K(A_Y)));
        const double xph = x + h;
        WSTAGE(A_K3, fma(h, fma(a1211, K(A_K2), fma(a1210, K(A_K10), fma(a129, K(A_K9), fma(a128, K(A_K8),
                     fma(a127, K(A_K7), fma(a126, K(A_K6), fma(a125, K(A_K5), fma(a124, K(A_K4),
                     a121 * K(A_K1))))))))), K(A_Y)));
        nfcn += 11;
        // 8th-order solution (k4), new state (k5) and error terms (:416-444)
        double err = 0.0, err2 = 0.0;
        for (int m = tid; m < nmem; m += nt)
            for (int c = 0; c < 6; c++) {
                const int64_t o = c * M + m;
                const double k4 = fma(b12, K(A_K3), fma(b11, K(A_K2), fma(b10, K(A_K10), fma(b9, K(A_K9),
                                  fma(b8, K(A_K8), fma(b7, K(A_K7), fma(b6, K(A_K6), b1 * K(A_K1))))))));
                const double k5 = fma(h, k4, K(A_Y));
                const double isk = fast::rcp_f(fma(rtoli, fmax(fabs(K(A_Y)), fabs(k5)), atoli));
                double erri = fma(-bhh3, K(A_K3), fma(-bhh2, K(A_K9), fma(-bhh1, K(A_K1), k4)));
                double sqr = erri * isk;
                err2 = fma(sqr, sqr, err2);
                erri = fma(er12, K(A_K3), fma(er11, K(A_K2), fma(er10, K(A_K10), fma(er9, K(A_K9), fma(er8, K(A_K8),
                       fma(er7, K(A_K7), fma(er6, K(A_K6), er1 * K(A_K1))))))));
                sqr = erri * isk;
                err = fma(sqr, sqr, err);
                K(A_K4) = k4;
                K(A_K5) = k5;
            }
        cta_sum2(err, err2, red);
        double deno = err + 0.01 * err2;
        if (deno <= 0.0) deno = 1.0;
        err = fabs(h) * err * sqrt(1.0 / (deno * (double)(6 * nmem)));
        const double fac11 = sqrt(sqrt(sqrt(err)));  // gala's pow(err, 1/8) (beta = 0)
        const double fac = fmax(facc2, fmin(facc1, fac11 / safe));
        double hnew = h / fac;
        if (err <= 1.0) {
            naccpt++;
            // FSAL: k4 = f(k5), the new state; k5 holds the positions the pulls need
            for (int m = tid; m < nmem; m += nt) wide_rhs<SCF>(pot, fr, bod, nbody, Ar[A_K5], M, m, Ar[A_K4]);
            __syncthreads();
            nfcn++;
            // stiffness detection (:463-486) after every accepted step (nstiff =
            // 1); the first detection returns -4 as in gala
            double stnum = 0.0, stden = 0.0;
            for (int m = tid; m < nmem; m += nt)
                for (int c = 0; c < 6; c++) {
                    const int64_t o = c * M + m;
                    double d = K(A_K4) - K(A_K3);
                    stnum += d * d;
                    d = K(A_K5) - K(A_YY1);
                    stden += d * d;
                }
            cta_sum2(stnum, stden, red);
            if (!(naccpt % nstiff) || iasti > 0) {
                if (stden > 0.0) hlamb = h * sqrt(stnum / stden);
                if (hlamb > 6.1) {
                    nonsti = 0;
                    iasti++;
                    idid = -4;
                    break;
                }
                nonsti++;
                if (nonsti == 6) iasti = 0;
            }
            if constexpr (DENSE) {
                // dense output (dop853.cpp:492-612) for a step that holds an output
                // time (the trajectory does not depend on it): the coefficients
                // from the stages, three more stages, then contd8 at each time
                const double x0 = x, x1 = x + h;
                auto inside = [&](double to) { return (x0 <= to && to <= x1) || (x1 <= to && to <= x0); };
                if (dn->out_idx < dn->ntimes && inside(dn->t[dn->out_idx])) {
                    for (int m = tid; m < nmem; m += nt)
                        for (int c = 0; c < 6; c++) {
                            const int64_t o = c * M + m;
                            K(A_R5) = d41 * K(A_K1) + d46 * K(A_K6) + d47 * K(A_K7) + d48 * K(A_K8) + d49 * K(A_K9) +
                                      d410 * K(A_K10) + d411 * K(A_K2) + d412 * K(A_K3);
                            K(A_R6) = d51 * K(A_K1) + d56 * K(A_K6) + d57 * K(A_K7) + d58 * K(A_K8) + d59 * K(A_K9) +
                                      d510 * K(A_K10) + d511 * K(A_K2) + d512 * K(A_K3);
                            K(A_R7) = d61 * K(A_K1) + d66 * K(A_K6) + d67 * K(A_K7) + d68 * K(A_K8) + d69 * K(A_K9) +
                                      d610 * K(A_K10) + d611 * K(A_K2) + d612 * K(A_K3);
                            K(A_R8) = d71 * K(A_K1) + d76 * K(A_K6) + d77 * K(A_K7) + d78 * K(A_K8) + d79 * K(A_K9) +
                                      d710 * K(A_K10) + d711 * K(A_K2) + d712 * K(A_K3);
                        }
                    __syncthreads();
                    WSTAGE(A_K10, fma(h, fma(a1413, K(A_K4), fma(a1412, K(A_K3), fma(a1411, K(A_K2),
                                  fma(a1410, K(A_K10), fma(a149, K(A_K9), fma(a148, K(A_K8), fma(a147, K(A_K7),
                                  a141 * K(A_K1)))))))), K(A_Y)));
                    WSTAGE(A_K2, fma(h, fma(a1514, K(A_K10), fma(a1513, K(A_K4), fma(a1512, K(A_K3),
                                 fma(a1511, K(A_K2), fma(a158, K(A_K8), fma(a157, K(A_K7), fma(a156, K(A_K6),
                                 a151 * K(A_K1)))))))), K(A_Y)));
                    WSTAGE(A_K3, fma(h, fma(a1615, K(A_K2), fma(a1614, K(A_K10), fma(a1613, K(A_K4),
                                 fma(a169, K(A_K9), fma(a168, K(A_K8), fma(a167, K(A_K7), fma(a166, K(A_K6),
                                 a161 * K(A_K1)))))))), K(A_Y)));
                    nfcn += 3;
                    int64_t oi = dn->out_idx, os = dn->out_slot;
                    while (oi < dn->ntimes && inside(dn->t[oi])) {
                        if (oi % dn->out_stride == 0) {
                            const double s_ = (dn->t[oi] - x0) / h, s1 = 1.0 - s_;
                            for (int m = tid; m < nmem; m += nt) {
                                double *w = dn->w_out + ((dn->sys * dn->n_out + os) * (int64_t)M + m) * 6;
                                for (int c = 0; c < 6; c++) {
                                    const int64_t o = c * M + m;
                                    const double r1 = K(A_Y), ydiff = K(A_K5) - K(A_Y);
                                    const double bspl = h * K(A_K1) - ydiff;
                                    const double r4 = ydiff - h * K(A_K4) - bspl;
                                    const double r5 = h * (K(A_R5) + d413 * K(A_K4) + d414 * K(A_K10) +
                                                           d415 * K(A_K2) + d416 * K(A_K3));
                                    const double r6 = h * (K(A_R6) + d513 * K(A_K4) + d514 * K(A_K10) +
                                                           d515 * K(A_K2) + d516 * K(A_K3));
                                    const double r7 = h * (K(A_R7) + d613 * K(A_K4) + d614 * K(A_K10) +
                                                           d615 * K(A_K2) + d616 * K(A_K3));
                                    const double r8 = h * (K(A_R8) + d713 * K(A_K4) + d714 * K(A_K10) +
                                                           d715 * K(A_K2) + d716 * K(A_K3));
                                    w[c] = r1 + s_ * (ydiff + s1 * (bspl + s_ * (r4 + s1 * (r5 + s_ * (r6 +
                                                 s1 * (r7 + s_ * r8))))));
                                }
                            }
                            os++;
                        }
                        oi++;
                    }
                    dn->out_idx = oi;
                    dn->out_slot = os;
                }
            }
            for (int m = tid; m < nmem; m += nt)
                for (int c = 0; c < 6; c++) {
                    const int64_t o = c * M + m;
                    K(A_K1) = K(A_K4);
                    K(A_Y) = K(A_K5);
                }
            __syncthreads();
            x = xph;
            if (last) {
                idid = 1;
                break;
            }
            if (fabs(hnew) > hmax) hnew = posneg * hmax;
            if (reject) hnew = posneg * fmin(fabs(hnew), fabs(h));
            reject = 0;
        } else {
            hnew = h / fmin(facc1, fac11 / safe);
            reject = 1;
            if (naccpt >= 1) nrejct++;
            last = 0;
        }
        h = hnew;
    }
#undef K
#undef WSTAGE
    (void)nonsti;
    __syncthreads();
    ctr[0] += nfcn;
    ctr[1] += nstep;
    ctr[2] += naccpt;
    ctr[3] += nrejct;
    return idid;
}

template <bool SCF>
__global__ void __launch_bounds__(WD_THREADS)
nbody_wide_kernel(const __grid_constant__ DevPot pot, const __grid_constant__ DevFrame fr,
                  const __grid_constant__ WideArgs A) {
    __shared__ double red[64];
    const int64_t b = blockIdx.x;
    if (b >= A.n_systems) return;
    // a CTA that starts after cancellation integrates nothing (one reader, CTA-uniform)
    if (__syncthreads_or(threadIdx.x == 0 && cancel_requested(A.cancel))) return;
    const int64_t sys = A.systems[b];
    const int64_t si = sys / A.n_streams, ss = sys - si * A.n_streams;
    // an id outside the release grid: nothing to address (recorded in the debug build)
    if (!GX_DBG_CHECK(si >= 0 && si < A.n_release, DBG_SYSTEM, sys, A.n_release * A.n_streams)) return;
    const int64_t o0 = A.offset[si], o1 = A.offset[si + 1];
    const int64_t M = A.max_members;
    const int nbody = A.nbody;
    if (o1 < o0 || o0 < 0 || o1 > A.n_particles || nbody + (o1 - o0) > M) {
        // inconsistent offsets: no access
        if (threadIdx.x == 0) {
            (void)GX_DBG_CHECK(false, DBG_OFFSET, si, A.n_release);
            A.status[ss * A.n_release + si] = -1;
        }
        return;
    }
    const int nmem = nbody + (int)(o1 - o0);
    const gx_body *bod = A.bodies + ss * nbody;
    double *base = A.scratch + b * (int64_t)WD_ARRAYS * 6 * M;
    double *Ar[WD_ARRAYS];
#pragma unroll
    for (int a = 0; a < WD_ARRAYS; a++) Ar[a] = base + (int64_t)a * 6 * M;
    const int tid = threadIdx.x, nt = blockDim.x;

    // the system at the release time: bodies, then the released particles
    for (int m = tid; m < nmem; m += nt) {
        const double *src = (m < nbody) ? A.nbody_w + ((ss * A.n_release + si) * nbody + m) * 6
                                        : A.stream_w0 + (ss * A.n_particles + o0 + (m - nbody)) * 6;
#pragma unroll
        for (int c = 0; c < 6; c++) Ar[A_Y][c * M + m] = src[c];
    }
    int64_t ctr[4] = {0, 0, 0, 0};
    const WideOpts opt = {2.3E-16, 1, fabs(A.t_final - A.release_t[si])};  // dop853_step (dop853.pyx:46-72)
    const int idid = wide_dop853<SCF>(pot, fr, bod, nbody, nmem, M, Ar, red, A.release_t[si], A.t_final, A.dt0,
                                      A.atol, A.rtol, A.nmax, ctr, opt);
    for (int m = tid; m < nmem; m += nt) {
        double *dst = nullptr;
        if (m >= nbody) dst = A.stream_w_out + (ss * A.n_particles + o0 + (m - nbody)) * 6;
        else if (A.nbody_w_out && o1 == A.offset[A.n_release]) dst = A.nbody_w_out + (ss * nbody + m) * 6;
        if (dst)
            for (int c = 0; c < 6; c++) dst[c] = Ar[A_Y][c * M + m];
    }
    if (tid == 0) {
        const int64_t k = ss * A.n_release + si;
        A.status[k] = idid;
        if (A.stats)
            for (int q = 0; q < 4; q++) A.stats[4 * k + q] = ctr[q];
    }
}

// mockstream_dop853_animate (mockstream.pyx:306-440) for many streams: one CTA
// per stream steps the growing system [bodies, particles released so far]
// interval by interval over the whole orbit grid and writes snapshots.
struct AnimArgs {
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
    double *scratch;           // n_streams x WD_ARRAYS x 6 x M doubles
    double *snap;              // (n_streams, 6, n_output, M) or NULL
    double *w_out;             // (n_streams, M, 6)
    int32_t *status;           // (n_streams, ntimes): [0] = 1, [i] = idid of interval i
    int64_t *stats;            // (n_streams, 4) summed over the intervals, or NULL
    const int32_t *cancel;     // host cancel flag (mapped memory) or nullptr
};

template <bool SCF>
__global__ void __launch_bounds__(WD_THREADS)
animate_wide_kernel(const __grid_constant__ DevPot pot, const __grid_constant__ DevFrame fr,
                    const __grid_constant__ AnimArgs A) {
    __shared__ double red[64];
    const int64_t s = blockIdx.x;
    if (s >= A.n_streams) return;
    const int64_t M = A.M;
    const int nbody = A.nbody;
    const gx_body *bod = A.bodies + s * nbody;
    double *base = A.scratch + s * (int64_t)WD_ARRAYS * 6 * M;
    double *Ar[WD_ARRAYS];
#pragma unroll
    for (int a = 0; a < WD_ARRAYS; a++) Ar[a] = base + (int64_t)a * 6 * M;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int m = tid; m < M; m += nt) {
        const double *src = (m < nbody) ? A.nbody_w0 + (s * nbody + m) * 6
                                        : A.stream_w0 + (s * A.n_particles + (m - nbody)) * 6;
#pragma unroll
        for (int c = 0; c < 6; c++) Ar[A_Y][c * M + m] = src[c];
    }
    __syncthreads();
    // members beyond the released ones are NaN in a snapshot (the HDF5 fill value)
    const double qnan = __longlong_as_double(0x7ff8000000000000LL);
    auto snapshot = [&](int64_t j, int64_t live) {
        if (!A.snap) return;
        for (int m = tid; m < M; m += nt)
#pragma unroll
            for (int c = 0; c < 6; c++)
                A.snap[((s * 6 + c) * A.n_output + j) * M + m] = (m < live) ? Ar[A_Y][c * M + m] : qnan;
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
        // after cancellation the stream stops between intervals (one reader, CTA-uniform);
        // the intervals not run keep status 0
        if (__syncthreads_or(tid == 0 && cancel_requested(A.cancel))) {
            for (int64_t k = i + tid; k < A.ntimes; k += nt) A.status[s * A.ntimes + k] = 0;
            while (j < A.n_output) snapshot(j++, 0);  // snapshots not reached: all NaN
            break;
        }
        const WideOpts opt = {2.3E-16, 1, fabs(A.t[i] - A.t[i - 1])};  // dop853_step (dop853.pyx:46-72)
        const int idid = wide_dop853<SCF>(pot, fr, bod, nbody, (int)(nbody + n), M, Ar, red, A.t[i - 1], A.t[i],
                                          A.dt0, A.atol, A.rtol, A.nmax, ctr, opt);
        n = grow(n, i, bad);
        if (tid == 0) A.status[s * A.ntimes + i] = bad ? -1 : idid;
        if (i % A.output_every == 0 || i == A.ntimes - 1) snapshot(j++, nbody + n);
    }
    __syncthreads();
    for (int m = tid; m < M; m += nt)
#pragma unroll
        for (int c = 0; c < 6; c++) A.w_out[(s * M + m) * 6 + c] = Ar[A_Y][c * M + m];
    if (tid == 0 && A.stats)
        for (int q = 0; q < 4; q++) A.stats[4 * s + q] = ctr[q];
}

// DirectNBody systems of any size (direct_nbody_dop853, nbody.pyx:30-115 ->
// dop853_helper, dop853.pyx:90-193): one CTA per system, gala's dop853_helper
// arguments, dense output onto the time grid when save_all.
struct NbWideArgs {
    int32_t nparticles, nbody, save_all;
    int64_t n_systems, ntimes, out_stride, n_out;
    const gx_body *bodies;   // (n_systems, max(nbody, 1))
    const double *w0;        // (n_systems, nparticles, 6)
    const double *t;         // (ntimes)
    double atol, rtol, dt_max;
    int64_t nmax, nstiff;
    double *scratch;         // n_systems x WD_ARRAYS_D x 6 x nparticles doubles
    double *w_out;           // (n_systems, n_out, nparticles, 6) or (n_systems, nparticles, 6)
    int32_t *status;
    int64_t *stats;
    const int32_t *cancel;
};

template <bool SCF, bool DENSE>
__global__ void __launch_bounds__(WD_THREADS)
nbody_system_wide_kernel(const __grid_constant__ DevPot pot, const __grid_constant__ DevFrame fr,
                         const __grid_constant__ NbWideArgs A) {
    __shared__ double red[64];
    const int64_t sys = blockIdx.x;
    if (sys >= A.n_systems) return;
    // a CTA that starts after cancellation integrates nothing (one reader, CTA-uniform)
    if (__syncthreads_or(threadIdx.x == 0 && cancel_requested(A.cancel))) return;
    const int64_t M = A.nparticles;
    const int tid = threadIdx.x, nt = blockDim.x;
    double *base = A.scratch + sys * (int64_t)WD_ARRAYS_D * 6 * M;
    double *Ar[WD_ARRAYS_D];
#pragma unroll
    for (int a = 0; a < WD_ARRAYS_D; a++) Ar[a] = base + (int64_t)a * 6 * M;
    for (int m = tid; m < M; m += nt)
#pragma unroll
        for (int c = 0; c < 6; c++) Ar[A_Y][c * M + m] = A.w0[(sys * M + m) * 6 + c];
    // dop853_helper's dop853() arguments (dop853.pyx:157-182) and front-end defaults
    const double x0 = A.t[0], xend = A.t[A.ntimes - 1];
    const int64_t nmax = A.nmax ? A.nmax : 1000000;
    WideOpts opt;
    opt.uround = 2.220446049250313e-16;  // np.finfo(float).eps
    opt.nstiff = A.nstiff == 0 ? 1000 : (A.nstiff < 0 ? nmax + 10 : A.nstiff);
    opt.hmax = fabs(A.dt_max == 0.0 ? xend - x0 : A.dt_max);
    WideDense dn = {A.t, A.ntimes, A.out_stride, A.n_out, sys, A.w_out, 0, 0};
    int64_t ctr[4] = {0, 0, 0, 0};
    const gx_body *bod = A.bodies + sys * (A.nbody > 0 ? A.nbody : 1);
    const int idid = wide_dop853<SCF, DENSE>(pot, fr, bod, A.nbody, (int)M, M, Ar, red, x0, xend, A.t[1] - A.t[0],
                                             A.atol, A.rtol, A.nmax, ctr, opt, &dn);
    if constexpr (!DENSE) {
        for (int m = tid; m < M; m += nt)
#pragma unroll
            for (int c = 0; c < 6; c++) A.w_out[(sys * M + m) * 6 + c] = Ar[A_Y][c * M + m];
    }
    if (tid == 0) {
        A.status[sys] = idid;
        if (A.stats)
            for (int q = 0; q < 4; q++) A.stats[4 * sys + q] = ctr[q];
    }
}

}  // namespace gx

extern "C" int64_t gx_mockstream_wide_scratch_bytes(int64_t n_systems, int32_t max_members) {
    if (n_systems <= 0 || max_members <= 0) return 0;
    return n_systems * (int64_t)gx::WD_ARRAYS * 6 * (int64_t)max_members * (int64_t)sizeof(double);
}

extern "C" int gx_mockstream_dop853_wide(const gx_potential *pot, const gx_frame *frame, int64_t n_streams,
                                         int32_t nbody, const gx_body *bodies, const double *nbody_w,
                                         int64_t n_release, const double *release_t, const int64_t *release_offset,
                                         const double *stream_w0, int64_t n_particles, double t_final, double dt0,
                                         double atol, double rtol, int64_t nmax, const int64_t *systems,
                                         int64_t n_systems, int32_t max_members, double *scratch,
                                         int64_t scratch_bytes, double *stream_w_out, double *nbody_w_out,
                                         int32_t *status, int64_t *stats, void *stream) {
    gx::DevPot dp;
    gx::DevFrame df;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    rc = gx::pack_frame(frame, &df);
    if (rc) return rc;
    GX_CHECK_ARG(n_streams >= 1 && n_release >= 0 && n_particles >= 0 && n_systems >= 0, "bad size");
    GX_CHECK_ARG(nbody >= 1, "nbody must be >= 1 (the progenitor)");
    GX_CHECK_ARG(max_members > nbody, "max_members must exceed nbody");
    GX_CHECK_ARG(nmax >= 0, "nmax must be >= 0 (0 = gala's default 1e6)");
    GX_CHECK_ARG(atol >= 0 && rtol >= 0, "tolerances must be non-negative");
    GX_CHECK_ARG(dt0 != 0.0, "dt0 (the release grid's step, gala's h0) must be non-zero");
    if (n_systems == 0) return GX_OK;
    GX_CHECK_ARG(bodies && nbody_w && release_t && release_offset && stream_w0 && systems && scratch && status &&
                     stream_w_out,
                 "NULL array");
    GX_CHECK_ARG(n_systems <= (int64_t)INT32_MAX, "too many systems");
    const int64_t need = gx_mockstream_wide_scratch_bytes(n_systems, max_members);
    GX_CHECK_ARG(scratch_bytes >= need, "scratch of %lld bytes, %lld needed", (long long)scratch_bytes,
                 (long long)need);
    gx::WideArgs A;
    memset(&A, 0, sizeof(A));
    A.nbody = nbody;
    A.max_members = max_members;
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
    A.systems = systems;
    A.n_systems = n_systems;
    A.scratch = scratch;
    A.stream_w_out = stream_w_out;
    A.nbody_w_out = nbody_w_out;
    A.status = status;
    A.stats = stats;
    A.cancel = gx::cancel_flag();
    cudaStream_t st = gx::as_stream(stream);
    if (dp.has_scf)
        gx::nbody_wide_kernel<true><<<(unsigned)n_systems, gx::WD_THREADS, 0, st>>>(dp, df, A);
    else
        gx::nbody_wide_kernel<false><<<(unsigned)n_systems, gx::WD_THREADS, 0, st>>>(dp, df, A);
    return gx::check_launch("mockstream_dop853_wide");
}

extern "C" int64_t gx_mockstream_animate_snapshots(int64_t ntimes, int64_t output_every) {
    if (ntimes < 2 || output_every < 1) return 0;
    return (ntimes - 1) / output_every + 1 + ((ntimes - 1) % output_every != 0);
}

extern "C" int gx_mockstream_dop853_animate(const gx_potential *pot, const gx_frame *frame, int64_t n_streams,
                                            int32_t nbody, const gx_body *bodies, const double *nbody_w0,
                                            int64_t ntimes, const double *t, double dt0,
                                            const int32_t *nstream, const double *stream_w0,
                                            int64_t n_particles, int64_t output_every, double atol, double rtol,
                                            int64_t nmax, double *scratch, int64_t scratch_bytes, double *snap,
                                            double *w_out, int32_t *status, int64_t *stats, void *stream) {
    gx::DevPot dp;
    gx::DevFrame df;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    rc = gx::pack_frame(frame, &df);
    if (rc) return rc;
    GX_CHECK_ARG(n_streams >= 1 && n_particles >= 0, "bad size");
    GX_CHECK_ARG(ntimes >= 2, "the time grid needs at least two points");
    GX_CHECK_ARG(nbody >= 1, "nbody must be >= 1 (the progenitor)");
    GX_CHECK_ARG(output_every >= 1, "output_every must be >= 1");
    GX_CHECK_ARG(nmax >= 0, "nmax must be >= 0 (0 = gala's default 1e6)");
    GX_CHECK_ARG(atol >= 0 && rtol >= 0, "tolerances must be non-negative");
    GX_CHECK_ARG(bodies && nbody_w0 && t && nstream && (stream_w0 || n_particles == 0) && scratch && w_out &&
                     status,
                 "NULL array");
    GX_CHECK_ARG(n_streams <= (int64_t)INT32_MAX && nbody + n_particles <= (int64_t)INT32_MAX, "too large");
    GX_CHECK_ARG(dt0 != 0.0, "dt0 (t[1] - t[0], gala's h0) must be non-zero");
    const int64_t M = nbody + n_particles;
    const int64_t need = gx_mockstream_wide_scratch_bytes(n_streams, (int32_t)M);
    GX_CHECK_ARG(scratch_bytes >= need, "scratch of %lld bytes, %lld needed", (long long)scratch_bytes,
                 (long long)need);
    gx::AnimArgs A;
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
    A.scratch = scratch;
    A.snap = snap;
    A.w_out = w_out;
    A.status = status;
    A.stats = stats;
    A.cancel = gx::cancel_flag();
    cudaStream_t st = gx::as_stream(stream);
    if (dp.has_scf)
        gx::animate_wide_kernel<true><<<(unsigned)n_streams, gx::WD_THREADS, 0, st>>>(dp, df, A);
    else
        gx::animate_wide_kernel<false><<<(unsigned)n_streams, gx::WD_THREADS, 0, st>>>(dp, df, A);
    return gx::check_launch("mockstream_dop853_animate");
}

extern "C" int64_t gx_nbody_wide_scratch_bytes(int64_t n_systems, int32_t nparticles) {
    if (n_systems <= 0 || nparticles <= 0) return 0;
    return n_systems * (int64_t)gx::WD_ARRAYS_D * 6 * (int64_t)nparticles * (int64_t)sizeof(double);
}

extern "C" int gx_nbody_dop853_wide(const gx_potential *pot, const gx_frame *frame, int64_t n_systems,
                                    int32_t nparticles, int32_t nbody, const gx_body *bodies, const double *w0,
                                    const double *t, int64_t ntimes, double atol, double rtol, int64_t nmax,
                                    double dt_max, int64_t nstiff, int32_t save_all, int64_t out_stride,
                                    double *scratch, int64_t scratch_bytes, double *w_out, int32_t *status,
                                    int64_t *stats, void *stream) {
    gx::DevPot dp;
    gx::DevFrame df;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    rc = gx::pack_frame(frame, &df);
    if (rc) return rc;
    GX_CHECK_ARG(n_systems >= 0 && nparticles >= 1 && nbody >= 0 && nbody <= nparticles, "bad size");
    GX_CHECK_ARG(ntimes >= 2, "ntimes must be >= 2 (got %lld)", (long long)ntimes);
    GX_CHECK_ARG(out_stride >= 1, "out_stride must be >= 1");
    GX_CHECK_ARG(nmax >= 0, "nmax must be >= 0 (0 = gala's default 1e6)");
    GX_CHECK_ARG(atol >= 0 && rtol >= 0, "tolerances must be non-negative");
    if (n_systems == 0) return GX_OK;
    GX_CHECK_ARG(bodies && w0 && t && scratch && w_out && status, "NULL array");
    GX_CHECK_ARG(n_systems <= (int64_t)INT32_MAX, "too many systems");
    const int64_t need = gx_nbody_wide_scratch_bytes(n_systems, nparticles);
    GX_CHECK_ARG(scratch_bytes >= need, "scratch of %lld bytes, %lld needed", (long long)scratch_bytes,
                 (long long)need);
    gx::NbWideArgs A;
    memset(&A, 0, sizeof(A));
    A.nparticles = nparticles;
    A.nbody = nbody;
    A.save_all = save_all ? 1 : 0;
    A.n_systems = n_systems;
    A.ntimes = ntimes;
    A.out_stride = out_stride;
    A.n_out = (ntimes - 1) / out_stride + 1;
    A.bodies = bodies;
    A.w0 = w0;
    A.t = t;
    A.atol = atol;
    A.rtol = rtol;
    A.dt_max = dt_max;
    A.nmax = nmax;
    A.nstiff = nstiff;
    A.scratch = scratch;
    A.w_out = w_out;
    A.status = status;
    A.stats = stats;
    A.cancel = gx::cancel_flag();
    cudaStream_t st = gx::as_stream(stream);
    const unsigned grid = (unsigned)n_systems;
    if (dp.has_scf) {
        if (save_all) gx::nbody_system_wide_kernel<true, true><<<grid, gx::WD_THREADS, 0, st>>>(dp, df, A);
        else gx::nbody_system_wide_kernel<true, false><<<grid, gx::WD_THREADS, 0, st>>>(dp, df, A);
    } else {
        if (save_all) gx::nbody_system_wide_kernel<false, true><<<grid, gx::WD_THREADS, 0, st>>>(dp, df, A);
        else gx::nbody_system_wide_kernel<false, false><<<grid, gx::WD_THREADS, 0, st>>>(dp, df, A);
    }
    return gx::check_launch("nbody_dop853_wide");
}
