// gx_batch.cu -- batched integration of many orbits with uneven step counts,
// step sizes and integrators, in FP32 with compensated state accumulation.
//
// Work queue: the caller supplies a processing order (a permutation of the
// orbits, padded with -1 to whole chunks) in which each chunk holds orbits of
// one integrator and similar cost, chunks sorted longest first.  A persistent
// grid (a few CTAs per SM) pulls work from the counters of gx_queue.cuh: the
// longest 32-orbit blocks one per SM sub-partition (one orbit per lane), then
// the other chunks in order (two orbits per lane where a chunk holds 64 or
// more).  Longest-first order plus dynamic pulling keeps the SMs busy until
// the very end.
//
// Per orbit: positions and velocities are carried as FP32 (hi, lo) pairs with
// Kahan-compensated updates; forces are evaluated in FP32 at hi (gx_fp32.cuh).
// Initial and final states are FP64 (hi + lo), so FP32 rounding of the state
// does not accumulate over tens of thousands of steps.
//   leapfrog  kick-drift-kick as c_leapfrog_step (leapfrog.pyx:35-51)
//   ruth4     c_ruth4_step (ruth4.pyx:24-35); the d = 0 sub-step's gradient is
//             skipped here (FP32 form, no bit-parity claim); each later sub-step's
//             kick and drift are fused (kick_drift), the step ending on a drift
//             so that a resumed run repeats the bits of an uninterrupted one
#include <mutex>

#include <cuda.h>

#include "gx_host.h"
#include "gx_fp32.cuh"
#include "gx_queue.cuh"
#include "gx_scf.cuh"

namespace gx {

struct BatchArgs {
    int64_t n;        // number of orbits
    int64_t slots;    // length of the order array (multiple of chunk)
    int64_t n_lead;   // chunks in the lead region (gx_queue.cuh)
    int32_t chunk;    // orbits per queue item (multiple of 32)
    int32_t pad;
    float c[4], d[4];  // Ruth4 coefficients
    const int32_t *cancel;  // host cancel flag (mapped memory) or nullptr
    // integrator state (12, n) float32: position hi, lo; velocity hi, lo (the
    // half-step velocity for Leapfrog), read to resume and / or written at the end
    const float *state_in;
    float *state_out;
};

__device__ __forceinline__ void split(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

// One orbit's integrator state in registers: position and velocity as FP32
// (hi, lo) pairs (for Leapfrog the velocity is the half-step v_{n+1/2}), the
// last gradient, the step and the Ruth4 coefficients times the step.
struct OrbitF {
    float xh[3], xl[3], vh[3], vl[3], g[3];
    float h, ch[4], dh[4];
};

// Load an orbit: from A.state_in in a resumed run, else split from the FP64
// initial conditions; then the Leapfrog start (c_init_velocity,
// v_{1/2} = v - g h / 2, which a resumed run already holds; the gradient at the
// start also serves the output velocity when no step follows) or the Ruth4
// coefficients times the step (shorter dependent chains per sub-step).
template <typename S, bool STATE>
__device__ __forceinline__ void orbit_begin(const DevPotF &pot, const BatchArgs &A, const double *w0, int64_t n,
                                            int64_t i, int64_t nsteps, float h, int meth, OrbitF &o) {
    const bool resume = STATE && A.state_in != nullptr;
    if (resume) {
        for (int k = 0; k < 3; k++) {
            o.xh[k] = A.state_in[k * n + i];
            o.xl[k] = A.state_in[(3 + k) * n + i];
            o.vh[k] = A.state_in[(6 + k) * n + i];
            o.vl[k] = A.state_in[(9 + k) * n + i];
        }
    } else {
        for (int k = 0; k < 3; k++) {
            split(w0[k * n + i], o.xh[k], o.xl[k]);
            split(w0[(3 + k) * n + i], o.vh[k], o.vl[k]);
        }
    }
    o.h = h;
    if (meth == 0) {
        if (!resume || nsteps == 0) potential_gradient_f<S>(pot, o.xh, o.g);
        if (!resume)
            for (int k = 0; k < 3; k++) kahan_add(o.vh[k], o.vl[k], -o.g[k] * h * 0.5f);
    } else {
#pragma unroll
        for (int s = 0; s < 4; s++) {
            o.ch[s] = A.c[s] * h;
            o.dh[s] = -A.d[s] * h;
        }
    }
}

// One Leapfrog step (c_leapfrog_step: drift, gradient, kick).
template <typename S>
__device__ __forceinline__ void lf_step(const DevPotF &pot, OrbitF &o) {
    for (int k = 0; k < 3; k++) kahan_add(o.xh[k], o.xl[k], fmaf(o.vh[k], o.h, o.vl[k] * o.h));
    potential_gradient_f<S>(pot, o.xh, o.g);
    for (int k = 0; k < 3; k++) kick(o.vh[k], o.vl[k], -o.h, o.g[k]);
}

// One Ruth4 step: sub-step 0 has d = 0 (drift only); each later sub-step's kick
// and drift are fused (kick_drift).  The step ends on a drift, so a resumed run
// repeats the bits of an uninterrupted one.
template <typename S>
__device__ __forceinline__ void r4_step(const DevPotF &pot, OrbitF &o) {
    for (int k = 0; k < 3; k++) kahan_add(o.xh[k], o.xl[k], fmaf(o.vh[k], o.ch[0], o.vl[k] * o.ch[0]));
#pragma unroll
    for (int s = 1; s < 4; s++) {
        potential_gradient_f<S>(pot, o.xh, o.g);
        for (int k = 0; k < 3; k++) kick_drift(o.xh[k], o.xl[k], o.vh[k], o.vl[k], o.dh[s], o.g[k], o.ch[s]);
    }
}

// Finish an orbit: the state for a checkpoint (A.state_out, before the output
// velocity is formed), the Leapfrog output velocity v_{n+1/2} + g h / 2 and the
// FP64 final state hi + lo.
template <bool STATE>
__device__ __forceinline__ void orbit_end(const BatchArgs &A, const double *w0, int64_t n, int64_t i,
                                          int64_t nsteps, int meth, OrbitF &o, double *w_out) {
    if constexpr (STATE) {
        if (A.state_out)
            for (int k = 0; k < 3; k++) {
                A.state_out[k * n + i] = o.xh[k];
                A.state_out[(3 + k) * n + i] = o.xl[k];
                A.state_out[(6 + k) * n + i] = o.vh[k];
                A.state_out[(9 + k) * n + i] = o.vl[k];
            }
    }
    if (nsteps == 0 && !(STATE && A.state_in != nullptr)) {  // no step taken: the initial conditions as given
        for (int k = 0; k < 6; k++) w_out[k * n + i] = w0[k * n + i];
        return;
    }
    if (meth == 0)
        for (int k = 0; k < 3; k++) kahan_add(o.vh[k], o.vl[k], o.g[k] * o.h * 0.5f);
    for (int k = 0; k < 3; k++) {
        w_out[k * n + i] = (double)o.xh[k] + (double)o.xl[k];
        w_out[(3 + k) * n + i] = (double)o.vh[k] + (double)o.vl[k];
    }
}

__device__ __forceinline__ void swap_orbits(OrbitF &a, OrbitF &b, bool doit) {
    float *pa = reinterpret_cast<float *>(&a), *pb = reinterpret_cast<float *>(&b);
#pragma unroll
    for (int k = 0; k < (int)(sizeof(OrbitF) / sizeof(float)); k++) {
        const float x = pa[k], y = pb[k];
        pa[k] = doit ? y : x;
        pb[k] = doit ? x : y;
    }
}

// Orbit ia, and orbit ib (>= 0, same integrator) in the same lane: both step
// together, two independent dependent chains the scheduler interleaves, while
// both have steps left; the longer one then finishes alone.  ib = -1 runs ia
// alone.  Each orbit's arithmetic is the same either way (its result does not
// depend on its partner).  With STATE, the integrator state is read from
// A.state_in when given and written to A.state_out when given, so that a run
// of k steps followed by a resumed run of n - k steps gives the bits of one run
// of n steps.
template <typename S, bool STATE>
__device__ __forceinline__ void integrate_fp32(const DevPotF &pot, const BatchArgs &A, const double *w0,
                                               const int64_t *nsteps, const double *dt, const int32_t *method,
                                               int32_t ia, int32_t ib, double *w_out) {
    const int64_t n = A.n;
    const bool keep = STATE && (A.state_in != nullptr || A.state_out != nullptr);
    int64_t na = nsteps[ia];
    const int meth = method[ia];
    if (ib < 0 && na == 0 && !keep) {
        for (int k = 0; k < 6; k++) w_out[k * n + ia] = w0[k * n + ia];
        return;
    }
    const int64_t nb = ib >= 0 ? nsteps[ib] : 0;
    OrbitF a, b;
    orbit_begin<S, STATE>(pot, A, w0, n, ia, na, (float)dt[ia], meth, a);
    if (ib >= 0) orbit_begin<S, STATE>(pot, A, w0, n, ib, nb, (float)dt[ib], meth, b);
    const int64_t common = ib >= 0 ? (na < nb ? na : nb) : 0;
    if (meth == 0) {
        for (int64_t j = 0; j < common; j++) {
            lf_step<S>(pot, a);
            lf_step<S>(pot, b);
        }
    } else {
        for (int64_t j = 0; j < common; j++) {
            r4_step<S>(pot, a);
            r4_step<S>(pot, b);
        }
    }
    // the remaining steps of the longer orbit, in a
    int32_t ja = ia, jb = ib;
    int64_t ma = na, mb = nb;
    if (ib >= 0) {
        const bool sw = nb > na;
        swap_orbits(a, b, sw);
        ja = sw ? ib : ia;
        jb = sw ? ia : ib;
        ma = sw ? nb : na;
        mb = sw ? na : nb;
    }
    if (meth == 0)
        for (int64_t j = common; j < ma; j++) lf_step<S>(pot, a);
    else
        for (int64_t j = common; j < ma; j++) r4_step<S>(pot, a);
    orbit_end<STATE>(A, w0, n, ja, ma, meth, a, w_out);
    if (ib >= 0) orbit_end<STATE>(A, w0, n, jb, mb, meth, b, w_out);
}

// Persistent grid over the queue of gx_queue.cuh: a lead block (32 of the
// longest orbits, at most one per SM sub-partition) runs one orbit per lane, so
// its dependent chains keep their latency; a main-region chunk runs its 32-orbit
// blocks two at a time, lane l pairing orbit l of one block with orbit l of the
// next (one integrator, similar cost), which doubles the independent work per
// warp where throughput, not latency, decides.
template <typename S, bool STATE>
__global__ void __launch_bounds__(256) batch_fp32_kernel(const __grid_constant__ DevPotF pot, BatchArgs A,
                                                         const double *__restrict__ w0,
                                                         const int64_t *__restrict__ nsteps,
                                                         const double *__restrict__ dt,
                                                         const int32_t *__restrict__ method,
                                                         const int32_t *__restrict__ order,
                                                         int32_t *__restrict__ counter, double *__restrict__ w_out) {
    const int lane = threadIdx.x & 31;
    const int64_t nchunks = A.slots / A.chunk;
    const int subs = A.chunk / 32;
    int phase = 0;
    for (;;) {
        // a cancelled launch takes no further work (lane 0 decides for the warp)
        int64_t c = -1;
        int sub = -1;
        if (lane == 0 && !cancel_requested(A.cancel)) c = queue_next(counter, nchunks, A.n_lead, subs, phase, sub);
        c = __shfl_sync(0xffffffffu, c, 0);
        sub = __shfl_sync(0xffffffffu, sub, 0);
        if (c < 0) break;
        // blocks [b0, b1) of chunk c, paired (b, b + 1) in the main region
        const int b0 = sub >= 0 ? sub : 0, b1 = sub >= 0 ? sub + 1 : subs;
        for (int b = b0; b < b1; b += 2) {
            // -1 pads the order; any other id outside [0, n) is skipped (and recorded in the debug build)
            int32_t ia = order[c * A.chunk + 32 * b + lane];
            int32_t ib = b + 1 < b1 ? order[c * A.chunk + 32 * (b + 1) + lane] : -1;
            if (ia != -1 && !GX_DBG_CHECK(ia >= 0 && ia < A.n, DBG_ORDER, ia, A.n)) ia = -1;
            if (ib != -1 && !GX_DBG_CHECK(ib >= 0 && ib < A.n, DBG_ORDER, ib, A.n)) ib = -1;
            if (ia < 0) {
                ia = ib;
                ib = -1;
            }
            const bool pair = ib >= 0 && method[ia] == method[ib];
            // at most two calls: (ia, ib) as a pair, or ia and then ib alone
#pragma unroll 1
            for (int pass = 0; pass < 2; pass++) {
                const int32_t x = pass == 0 ? ia : (pair ? -1 : ib);
                const int32_t y = pass == 0 && pair ? ib : -1;
                if (x < 0) continue;
                integrate_fp32<S, STATE>(pot, A, w0, nsteps, dt, method, x, y, w_out);
                GX_DBG_DONE(x, nsteps[x]);
                if (y >= 0) GX_DBG_DONE(y, nsteps[y]);
            }
        }
    }
}

// FP32 descriptor from the FP64 one (gala packing [G, ...]) with the per-type
// constants the FP32 force code wants.
int pack_potential_f32(const gx_potential *pot, DevPotF *out) {
    DevPot dp;
    int rc = pack_potential(pot, &dp);
    if (rc) return rc;
    if (dp.cdev) {
        set_error("the FP32 forms take at most GX_MAX_COMPONENTS = %d components (got %d)", GX_MAX_COMPONENTS,
                  dp.ncomp);
        return GX_ERR_CAPACITY;
    }
    if (dp.has_scf) {
        set_error("the FP32 batched integrator supports closed-form components only (no SCF)");
        return GX_ERR_UNSUPPORTED;
    }
    memset(out, 0, sizeof(*out));
    out->ncomp = dp.ncomp;
    for (int i = 0; i < dp.ncomp; i++) {
        const DevComp &c = dp.c[i];
        DevCompF &f = out->c[i];
        const double *p = dp.p + c.poff;
        f.type = c.type;
        f.do_sr = c.do_sr;
        for (int k = 0; k < 3; k++) f.q0[k] = (float)c.q0[k];
        for (int k = 0; k < 9; k++) f.R[k] = (float)c.R[k];
        switch (c.type) {
        case GX_POT_NULL: break;
        case GX_POT_KEPLER: f.p[0] = (float)(p[0] * p[1]); break;
        case GX_POT_HERNQUIST: f.p[0] = (float)(p[0] * p[1]); f.p[1] = (float)p[2]; break;
        case GX_POT_PLUMMER: f.p[0] = (float)(p[0] * p[1]); f.p[1] = (float)(p[2] * p[2]); break;
        case GX_POT_MIYAMOTONAGAI:
            f.p[0] = (float)(p[0] * p[1]); f.p[1] = (float)p[2]; f.p[2] = (float)(p[3] * p[3]);
            break;
        case GX_POT_SPHERICALNFW:
        case GX_POT_FLATTENEDNFW:
        case GX_POT_TRIAXIALNFW:
            f.p[0] = (float)(p[0] * p[1] / (p[2] * p[2] * p[2]));
            f.p[1] = (float)(1.0 / p[2]);
            f.p[2] = (float)p[2];
            if (c.type == GX_POT_FLATTENEDNFW) f.p[3] = (float)(1.0 / (p[5] * p[5]));
            if (c.type == GX_POT_TRIAXIALNFW) {
                f.p[3] = (float)(1.0 / (p[3] * p[3]));
                f.p[4] = (float)(1.0 / (p[4] * p[4]));
                f.p[5] = (float)(1.0 / (p[5] * p[5]));
            }
            break;
        default:
            set_error("component %d: type %d has no FP32 implementation", i, c.type);
            return GX_ERR_UNSUPPORTED;
        }
    }
    return GX_OK;
}

// Launch the persistent kernel, specialised when the component list is one of
// the compiled signatures (no shift/rotate), generic otherwise.
static void launch_batch_fp32(const DevPotF &dp, const BatchArgs &A, const double *w0, const int64_t *nsteps,
                              const double *dt, const int32_t *method, const int32_t *order, int32_t *counter,
                              double *w_out, int grid, int block, cudaStream_t st) {
    auto is = [&](int a, int b, int c, int d) {
        const int want[4] = {a, b, c, d};
        int nc = 0;
        for (int k = 0; k < 4; k++) nc += want[k] >= 0;
        if (dp.ncomp != nc) return false;
        for (int k = 0; k < nc; k++)
            if (dp.c[k].type != want[k] || dp.c[k].do_sr) return false;
        return true;
    };
    constexpr int H = GX_POT_HERNQUIST, MN = GX_POT_MIYAMOTONAGAI, NFW = GX_POT_SPHERICALNFW, P = GX_POT_PLUMMER;
#define GX_LAUNCH(SIG)                                                                                    \
    do {                                                                                                  \
        if (A.state_in || A.state_out)                                                                    \
            batch_fp32_kernel<SIG, true><<<grid, block, 0, st>>>(dp, A, w0, nsteps, dt, method, order,     \
                                                                 counter, w_out);                         \
        else                                                                                              \
            batch_fp32_kernel<SIG, false><<<grid, block, 0, st>>>(dp, A, w0, nsteps, dt, method, order,    \
                                                                  counter, w_out);                        \
    } while (0)
    using SigHHMN = PotSig<H, H, MN, NFW>;
    using SigMNHH = PotSig<MN, H, H, NFW>;
    using SigH = PotSig<H, -1, -1, -1>;
    using SigP = PotSig<P, -1, -1, -1>;
    if (is(H, H, MN, NFW)) GX_LAUNCH(SigHHMN);
    else if (is(MN, H, H, NFW)) GX_LAUNCH(SigMNHH);
    else if (is(H, -1, -1, -1)) GX_LAUNCH(SigH);
    else if (is(P, -1, -1, -1)) GX_LAUNCH(SigP);
    else GX_LAUNCH(SigGeneric);
#undef GX_LAUNCH
}

}  // namespace gx

static int batch_fp32_entry(const gx_potential *pot, const double *w0, int64_t n, const int64_t *n_steps,
                            const double *dt, const int32_t *method, const int32_t *order, int64_t n_slots,
                            int32_t chunk, int32_t block, int32_t grid, int32_t *queue_counter,
                            const float *state_in, float *state_out, double *w_out, void *stream) {
    gx::DevPotF dp;
    int rc = gx::pack_potential_f32(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0 && n < (int64_t)INT32_MAX, "n out of range");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(w0 && n_steps && dt && method && order && queue_counter && w_out, "NULL array");
    GX_CHECK_ARG(chunk >= 32 && chunk % 32 == 0 && chunk <= 4096, "chunk must be a multiple of 32 in [32, 4096]");
    GX_CHECK_ARG(n_slots >= n && n_slots % chunk == 0, "order length must be >= n and a multiple of chunk");
    GX_CHECK_ARG(block >= 32 && block <= 256 && block % 32 == 0, "block must be a multiple of 32 in [32, 256]");
    GX_CHECK_ARG(grid >= 1, "grid must be >= 1");
    gx::BatchArgs A;
    memset(&A, 0, sizeof(A));
    A.n = n;
    A.slots = n_slots;
    A.chunk = chunk;
    A.pad = 0;
    A.cancel = gx::cancel_flag();
    A.state_in = state_in;
    A.state_out = state_out;
    const double two_13 = std::pow(2., 1. / 3.);
    const double c[4] = {1. / (2. * (2. - two_13)), (1. - two_13) / (2. * (2. - two_13)),
                         (1. - two_13) / (2. * (2. - two_13)), 1. / (2. * (2. - two_13))};
    const double d[4] = {0., 1. / (2. - two_13), -two_13 / (2. - two_13), 1. / (2. - two_13)};
    for (int k = 0; k < 4; k++) {
        A.c[k] = (float)c[k];
        A.d[k] = (float)d[k];
    }
    A.n_lead = gx::queue_lead_chunks(n_slots / chunk, chunk);
    cudaStream_t st = gx::as_stream(stream);
    GX_CUDA_TRY(cudaMemsetAsync(queue_counter, 0, GX_BATCH_QUEUE_WORDS * sizeof(int32_t), st));
    gx::launch_batch_fp32(dp, A, w0, n_steps, dt, method, order, queue_counter, w_out, grid, block, st);
    return gx::check_launch("batch_fp32");
}

extern "C" int gx_batch_integrate_fp32(const gx_potential *pot, const double *w0, int64_t n,
                                       const int64_t *n_steps, const double *dt, const int32_t *method,
                                       const int32_t *order, int64_t n_slots, int32_t chunk, int32_t block,
                                       int32_t grid, int32_t *queue_counter, double *w_out, void *stream) {
    return batch_fp32_entry(pot, w0, n, n_steps, dt, method, order, n_slots, chunk, block, grid, queue_counter,
                            nullptr, nullptr, w_out, stream);
}

extern "C" int gx_batch_integrate_fp32_state(const gx_potential *pot, const double *w0, int64_t n,
                                             const int64_t *n_steps, const double *dt, const int32_t *method,
                                             const int32_t *order, int64_t n_slots, int32_t chunk, int32_t block,
                                             int32_t grid, int32_t *queue_counter, const float *state_in,
                                             float *state_out, double *w_out, void *stream) {
    GX_CHECK_ARG(state_in || state_out, "state_in and state_out are both NULL (use gx_batch_integrate_fp32)");
    GX_CHECK_ARG(state_in != state_out, "state_in and state_out must not alias");
    return batch_fp32_entry(pot, w0, n, n_steps, dt, method, order, n_slots, chunk, block, grid, queue_counter,
                            state_in, state_out, w_out, stream);
}

// ===========================================================================
// Fixed-step FP32-compensated integration on one time grid with snapshots:
// the FP32 form of leapfrog_integrate_hamiltonian / ruth4_integrate_hamiltonian
// (leapfrog.pyx:54-121, ruth4.pyx:37-113).  One thread per orbit; the step is
// t[1] - t[0]; every out_stride-th of the ntimes grid points is stored as FP64
// (hi + lo), in gala's (6, n_out, N) layout, or only the final state.
// ===========================================================================
namespace gx {

struct FixedArgs {
    int64_t n, nsteps, out_stride, n_out;
    int32_t save_all, method;
    float c[4], d[4];
};

__device__ __forceinline__ void store_state(double *out, int64_t n_out, int64_t n, int64_t slot, int64_t i,
                                            const float *xh, const float *xl, const double *v) {
    for (int k = 0; k < 3; k++) {
        __stcs(&out[((int64_t)k * n_out + slot) * n + i], (double)xh[k] + (double)xl[k]);
        __stcs(&out[((int64_t)(3 + k) * n_out + slot) * n + i], v[k]);
    }
}

template <typename S>
__global__ void __launch_bounds__(128) fixed_fp32_kernel(const __grid_constant__ DevPotF pot, FixedArgs A,
                                                         const double *__restrict__ w0,
                                                         const double *__restrict__ t, double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const int64_t n = A.n;
    const float h = (float)(t[1] - t[0]);
    float xh[3], xl[3], vh[3], vl[3], g[3];
    double v[3];
    for (int k = 0; k < 3; k++) {
        split(w0[k * n + i], xh[k], xl[k]);
        split(w0[(3 + k) * n + i], vh[k], vl[k]);
        v[k] = w0[(3 + k) * n + i];
    }
    int64_t slot = 0;
    if (A.save_all) {
        // snapshot 0 is the initial state, exactly
        for (int k = 0; k < 6; k++) __stcs(&out[((int64_t)k * A.n_out + slot) * n + i], w0[k * n + i]);
        slot++;
    }
    if (A.method == 0) {
        potential_gradient_f<S>(pot, xh, g);
        for (int k = 0; k < 3; k++) kahan_add(vh[k], vl[k], -g[k] * h * 0.5f);
        for (int64_t j = 1; j <= A.nsteps; j++) {
            for (int k = 0; k < 3; k++) kahan_add(xh[k], xl[k], fmaf(vh[k], h, vl[k] * h));
            potential_gradient_f<S>(pot, xh, g);
            for (int k = 0; k < 3; k++) kick(vh[k], vl[k], -h, g[k]);
            if (A.save_all && j % A.out_stride == 0) {
                // output velocity of c_leapfrog_step: v_{j+1/2} + g h / 2
                for (int k = 0; k < 3; k++) v[k] = (double)vh[k] + ((double)vl[k] + (double)(g[k] * h * 0.5f));
                store_state(out, A.n_out, n, slot++, i, xh, xl, v);
            }
        }
        for (int k = 0; k < 3; k++) v[k] = (double)vh[k] + ((double)vl[k] + (double)(g[k] * h * 0.5f));
    } else {
        for (int64_t j = 1; j <= A.nsteps; j++) {
            for (int k = 0; k < 3; k++) kahan_add(xh[k], xl[k], A.c[0] * fmaf(vh[k], h, vl[k] * h));
#pragma unroll
            for (int s = 1; s < 4; s++) {
                potential_gradient_f<S>(pot, xh, g);
                for (int k = 0; k < 3; k++) kick_drift(xh[k], xl[k], vh[k], vl[k], -A.d[s] * h, g[k], A.c[s] * h);
            }
            if (A.save_all && j % A.out_stride == 0) {
                for (int k = 0; k < 3; k++) v[k] = (double)vh[k] + (double)vl[k];
                store_state(out, A.n_out, n, slot++, i, xh, xl, v);
            }
        }
        for (int k = 0; k < 3; k++) v[k] = (double)vh[k] + (double)vl[k];
    }
    if (!A.save_all)
        for (int k = 0; k < 3; k++) {
            out[k * n + i] = (double)xh[k] + (double)xl[k];
            out[(3 + k) * n + i] = v[k];
        }
}

}  // namespace gx

extern "C" int gx_fixed_fp32(const gx_potential *pot, int32_t method, const double *w0, int64_t n,
                             const double *t, int64_t ntimes, int32_t save_all, int64_t out_stride, double *w_out,
                             void *stream) {
    gx::DevPotF dp;
    int rc = gx::pack_potential_f32(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(method == 0 || method == 1, "method must be 0 (leapfrog) or 1 (ruth4)");
    GX_CHECK_ARG(n >= 0, "n < 0");
    GX_CHECK_ARG(ntimes >= 2, "ntimes must be >= 2 (got %lld)", (long long)ntimes);
    GX_CHECK_ARG(out_stride >= 1, "out_stride must be >= 1");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(w0 && t && w_out, "NULL array");
    gx::FixedArgs A;
    memset(&A, 0, sizeof(A));
    A.n = n;
    A.nsteps = ntimes - 1;
    A.out_stride = out_stride;
    A.n_out = (ntimes - 1) / out_stride + 1;
    A.save_all = save_all ? 1 : 0;
    A.method = method;
    const double two_13 = std::pow(2., 1. / 3.);
    const double c[4] = {1. / (2. * (2. - two_13)), (1. - two_13) / (2. * (2. - two_13)),
                         (1. - two_13) / (2. * (2. - two_13)), 1. / (2. * (2. - two_13))};
    const double d[4] = {0., 1. / (2. - two_13), -two_13 / (2. - two_13), 1. / (2. - two_13)};
    for (int k = 0; k < 4; k++) {
        A.c[k] = (float)c[k];
        A.d[k] = (float)d[k];
    }
    cudaStream_t st = gx::as_stream(stream);
    const unsigned grid = (unsigned)((n + 127) / 128);
    auto is = [&](int a) { return dp.ncomp == 1 && dp.c[0].type == a && !dp.c[0].do_sr; };
    const bool mw = dp.ncomp == 4 && dp.c[0].type == GX_POT_HERNQUIST && dp.c[1].type == GX_POT_HERNQUIST &&
                    dp.c[2].type == GX_POT_MIYAMOTONAGAI && dp.c[3].type == GX_POT_SPHERICALNFW &&
                    !(dp.c[0].do_sr | dp.c[1].do_sr | dp.c[2].do_sr | dp.c[3].do_sr);
    using namespace gx;
    if (mw)
        fixed_fp32_kernel<PotSig<GX_POT_HERNQUIST, GX_POT_HERNQUIST, GX_POT_MIYAMOTONAGAI, GX_POT_SPHERICALNFW>>
            <<<grid, 128, 0, st>>>(dp, A, w0, t, w_out);
    else if (is(GX_POT_HERNQUIST))
        fixed_fp32_kernel<PotSig<GX_POT_HERNQUIST, -1, -1, -1>><<<grid, 128, 0, st>>>(dp, A, w0, t, w_out);
    else
        fixed_fp32_kernel<SigGeneric><<<grid, 128, 0, st>>>(dp, A, w0, t, w_out);
    return gx::check_launch("fixed_fp32");
}

// ===========================================================================
// The processing order of a batch, built on the device without a host sync:
// per integrator the orbits sorted by cost (n_steps x gradient evaluations per
// step, 1 for Leapfrog and 3 for Ruth4) into 128 bins per octave -- a 0.54 %
// resolution, the most expensive first -- and cut into chunks padded with -1;
// the chunks of the two integrators merged by the bin of their first orbit
// (Ruth4 first on ties).  Orbits of one bin keep no particular order; each
// orbit's result does not depend on the order.
// ===========================================================================
namespace gx {

constexpr int SB_PER_OCT = 128;
constexpr int SB_BINS = 64 * SB_PER_OCT;    // bins per integrator (cost below 2^64)
constexpr int SB_HIST = 2 * SB_BINS;        // Ruth4 bins, then Leapfrog bins
constexpr int SB_INFO = 4;                  // chunks of each integrator
constexpr int SB_SCAN_T = 1024;             // threads of the scan
constexpr int SB_PER_T = SB_BINS / SB_SCAN_T;  // bins of each half per scan thread

__device__ __forceinline__ int sched_bin(int64_t nsteps, int32_t method) {
    const double cost = (double)(nsteps > 0 ? nsteps : 0) * (method == 0 ? 1.0 : 3.0);
    const int b = SB_BINS - 1 - (int)(log2(cost + 1.0) * SB_PER_OCT);
    return b < 0 ? 0 : (b > SB_BINS - 1 ? SB_BINS - 1 : b);
}
__device__ __forceinline__ int sched_key(int64_t nsteps, int32_t method) {
    return (method == 0 ? SB_BINS : 0) + sched_bin(nsteps, method);
}

__global__ void sched_histogram(int32_t *hist, const int64_t *__restrict__ nsteps,
                                const int32_t *__restrict__ method, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&hist[sched_key(nsteps[i], method[i])], 1);
}

// Exclusive prefix sums of both halves of the histogram (one CTA of SB_SCAN_T
// threads, thread t owning SB_PER_T consecutive bins of each half); the Leapfrog
// list starts after the Ruth4 list padded to whole chunks.
// info = {Ruth4 chunks, Leapfrog chunks}.
__global__ void __launch_bounds__(SB_SCAN_T) sched_scan(int32_t *hist, int32_t *info, int chunk) {
    __shared__ int32_t sr[SB_SCAN_T], sl[SB_SCAN_T];
    const int t = threadIdx.x;
    int32_t cr[SB_PER_T], cl[SB_PER_T], tr = 0, tl = 0;
#pragma unroll
    for (int k = 0; k < SB_PER_T; k++) {
        cr[k] = hist[t * SB_PER_T + k];
        cl[k] = hist[SB_BINS + t * SB_PER_T + k];
        tr += cr[k];
        tl += cl[k];
    }
    sr[t] = tr;
    sl[t] = tl;
    __syncthreads();
    for (int o = 1; o < SB_SCAN_T; o <<= 1) {  // inclusive Hillis-Steele scans of the threads' totals
        const int32_t ar = t >= o ? sr[t - o] : 0, al = t >= o ? sl[t - o] : 0;
        __syncthreads();
        sr[t] += ar;
        sl[t] += al;
        __syncthreads();
    }
    const int32_t nr = sr[SB_SCAN_T - 1], nl = sl[SB_SCAN_T - 1];
    const int32_t ncr = (nr + chunk - 1) / chunk, ncl = (nl + chunk - 1) / chunk;
    int32_t orr = sr[t] - tr, ol = ncr * chunk + sl[t] - tl;
#pragma unroll
    for (int k = 0; k < SB_PER_T; k++) {
        hist[t * SB_PER_T + k] = orr;
        hist[SB_BINS + t * SB_PER_T + k] = ol;
        orr += cr[k];
        ol += cl[k];
    }
    if (t == 0) {
        info[0] = ncr;
        info[1] = ncl;
    }
}

__global__ void sched_scatter(int32_t *hist, int32_t *tmp, const int64_t *__restrict__ nsteps,
                              const int32_t *__restrict__ method, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) tmp[atomicAdd(&hist[sched_key(nsteps[i], method[i])], 1)] = (int32_t)i;
}

// Bin of each chunk's first orbit (never padding: a list pads only its end).
__global__ void sched_heads(const int32_t *info, const int32_t *__restrict__ tmp, int32_t *heads,
                            const int64_t *__restrict__ nsteps, const int32_t *__restrict__ method, int chunk) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= info[0] + info[1]) return;
    const int32_t i = tmp[(int64_t)c * chunk];
    heads[c] = sched_bin(nsteps[i], method[i]);
}

// Merge the two chunk lists (each sorted by head bin) into the order: one warp
// per chunk; lane 0 finds the chunk's place by binary search in the other list.
__global__ void sched_merge(const int32_t *info, const int32_t *__restrict__ tmp, const int32_t *__restrict__ heads,
                            int32_t *order, int chunk) {
    const int c = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    const int ncr = info[0], ncl = info[1];
    if (c >= ncr + ncl) return;
    int f = 0;
    if (lane == 0) {
        const bool ruth4 = c < ncr;
        const int32_t key = heads[c];
        const int32_t *other = ruth4 ? heads + ncr : heads;
        int lo = 0, hi = ruth4 ? ncl : ncr;
        while (lo < hi) {  // Ruth4: Leapfrog heads < key; Leapfrog: Ruth4 heads <= key
            const int mid = (lo + hi) >> 1;
            if (ruth4 ? other[mid] < key : other[mid] <= key) lo = mid + 1;
            else hi = mid;
        }
        f = (ruth4 ? c : c - ncr) + lo;
    }
    f = __shfl_sync(0xffffffffu, f, 0);
    for (int k = lane; k < chunk; k += 32) order[(int64_t)f * chunk + k] = tmp[(int64_t)c * chunk + k];
}

}  // namespace gx

namespace gx {

// Build the order of n orbits (see above) into order[0 .. n_slots) with the
// work words `work`; sizes checked by the caller.
static int launch_schedule(const int64_t *n_steps, const int32_t *method, int64_t n, int32_t chunk, int32_t *order,
                           int64_t n_slots, int64_t slots, int32_t *work, cudaStream_t st) {
    int32_t *hist = work, *info = work + SB_HIST, *heads = info + SB_INFO;
    int32_t *tmp = heads + slots / chunk;
    GX_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(int32_t) * (SB_HIST + SB_INFO), st));
    GX_CUDA_TRY(cudaMemsetAsync(tmp, 0xff, sizeof(int32_t) * slots, st));    // -1: padding
    GX_CUDA_TRY(cudaMemsetAsync(order, 0xff, sizeof(int32_t) * n_slots, st));
    if (n == 0) return GX_OK;
    const int tb = 256;
    const unsigned gn = (unsigned)((n + tb - 1) / tb);
    const int64_t max_chunks = slots / chunk;
    sched_histogram<<<gn, tb, 0, st>>>(hist, n_steps, method, n);
    sched_scan<<<1, SB_SCAN_T, 0, st>>>(hist, info, chunk);
    sched_scatter<<<gn, tb, 0, st>>>(hist, tmp, n_steps, method, n);
    sched_heads<<<(unsigned)((max_chunks + tb - 1) / tb), tb, 0, st>>>(info, tmp, heads, n_steps, method, chunk);
    sched_merge<<<(unsigned)((max_chunks * 32 + tb - 1) / tb), tb, 0, st>>>(info, tmp, heads, order, chunk);
    return check_launch("batch_schedule");
}

}  // namespace gx

extern "C" int64_t gx_batch_schedule_slots(int64_t n, int32_t chunk) {
    if (n < 0 || chunk < 1) return 0;
    return ((n + chunk - 1) / chunk + 1) * (int64_t)chunk;
}

extern "C" int64_t gx_batch_schedule_work_words(int64_t n, int32_t chunk) {
    const int64_t slots = gx_batch_schedule_slots(n, chunk);
    if (slots == 0) return 0;
    return gx::SB_HIST + gx::SB_INFO + slots / chunk + slots;
}

extern "C" int gx_batch_schedule(const int64_t *n_steps, const int32_t *method, int64_t n, int32_t chunk,
                                 int32_t *order, int64_t n_slots, int32_t *work, int64_t work_words, void *stream) {
    GX_CHECK_ARG(n >= 0 && n < (int64_t)INT32_MAX, "n out of range");
    GX_CHECK_ARG(chunk >= 32 && chunk % 32 == 0 && chunk <= 4096, "chunk must be a multiple of 32 in [32, 4096]");
    const int64_t slots = gx_batch_schedule_slots(n, chunk);
    GX_CHECK_ARG(n_slots >= slots, "order holds %lld slots, %lld needed", (long long)n_slots, (long long)slots);
    GX_CHECK_ARG(work_words >= gx_batch_schedule_work_words(n, chunk), "work of %lld words, %lld needed",
                 (long long)work_words, (long long)gx_batch_schedule_work_words(n, chunk));
    GX_CHECK_ARG(order && work && (n == 0 || (n_steps && method)), "NULL array");
    return gx::launch_schedule(n_steps, method, n, chunk, order, n_slots, slots, work, gx::as_stream(stream));
}

// ===========================================================================
// Allocation-free variant of the batched FP32 integrator.
//
// Some callers cannot allocate device memory: an application whose memory
// manager owns the whole GPU (a framework's caching allocator, or a service
// that reserves HBM up front) must not have a library call cudaMalloc behind
// its back; a host in another language that only receives device pointers from
// a different runtime has no allocator to call; and cudaMalloc / cudaFree can
// synchronize the device, which a latency-critical asynchronous pipeline cannot
// afford.  gx_batch_integrate_fp32_noalloc serves them: the caller passes only
// inputs and outputs, and the work queue (its counter and the processing order,
// which gx_batch_integrate_fp32 takes from the caller) lives in the file-scope
// array below, sized for at most GX_NOALLOC_MAX_ORBITS orbits.  The array exists
// on every GPU that loads this library until the process exits.
//
// The processing order is built in the array as gx_batch_schedule builds it
// (cost bins, chunk lists merged by head cost); the order within a bin comes
// from atomics, which changes only which warp runs an orbit, never its
// arithmetic -- results are bit-identical to the caller-order entry point.
// ===========================================================================
namespace gx {

constexpr int NA_CHUNK = 32;
constexpr int64_t NA_SLOTS = GX_NOALLOC_MAX_ORBITS + 2 * NA_CHUNK;   // >= gx_batch_schedule_slots(max, 32)
constexpr int64_t NA_WORK = SB_HIST + SB_INFO + NA_SLOTS / NA_CHUNK + NA_SLOTS;
// int32 layout: [0, GX_BATCH_QUEUE_WORDS) queue | [NA_WORK_OFF, + NA_WORK) schedule work | order
constexpr int64_t NA_WORK_OFF = ((GX_BATCH_QUEUE_WORDS + 63) / 64) * 64;
constexpr int64_t NA_ORDER_OFF = ((NA_WORK_OFF + NA_WORK + 63) / 64) * 64;
constexpr int64_t NA_WORDS = NA_ORDER_OFF + NA_SLOTS;

static __device__ __align__(256) int32_t g_noalloc_scratch[NA_WORDS];

// Identity of the CUDA context current on this thread (cuCtxGetId through the
// runtime's driver entry points, so the library links no driver library).
typedef CUresult (*ctx_get_current_fn)(CUcontext *);
typedef CUresult (*ctx_get_id_fn)(CUcontext, unsigned long long *);

static int current_context_id(unsigned long long *id) {
    static ctx_get_current_fn get_cur = nullptr;
    static ctx_get_id_fn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<ctx_get_current_fn>(fn);
        fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<ctx_get_id_fn>(fn);
    });
    CUcontext ctx = nullptr;
    if (!get_cur || !get_id || get_cur(&ctx) != CUDA_SUCCESS || ctx == nullptr || get_id(ctx, id) != CUDA_SUCCESS)
        *id = 0;  // unknown: look the address up again
    return GX_OK;
}

// Device address of g_noalloc_scratch in the current context.  It is looked up
// with cudaGetSymbolAddress (that device current) on a device's first call and
// again whenever the context has changed since (after cudaDeviceReset the
// module is loaded again and the array may sit elsewhere).
static int noalloc_scratch_address(int32_t **out) {
    static std::mutex mu;
    static int32_t *addr[64] = {nullptr};
    static unsigned long long ctx_of[64] = {0};
    int dev = 0;
    GX_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return GX_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(mu);
    unsigned long long ctx = 0;
    current_context_id(&ctx);
    if (addr[dev] == nullptr || ctx == 0 || ctx != ctx_of[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            set_error("cudaGetSymbolAddress(g_noalloc_scratch) failed on device %d: %s", dev, cudaGetErrorString(e));
            return GX_ERR_CUDA;
        }
        addr[dev] = static_cast<int32_t *>(p);
        // the lookup makes the context current if it was not yet: record its id now
        current_context_id(&ctx_of[dev]);
    }
    *out = addr[dev];
    return GX_OK;
}

}  // namespace gx

extern "C" int gx_batch_integrate_fp32_noalloc(const gx_potential *pot, const double *w0, int64_t n,
                                               const int64_t *n_steps, const double *dt, const int32_t *method,
                                               int32_t block, int32_t grid, double *w_out, void *stream) {
    gx::DevPotF dp;
    int rc = gx::pack_potential_f32(pot, &dp);
    if (rc) return rc;
    if (n < 0 || n > GX_NOALLOC_MAX_ORBITS) {
        gx::set_error("gx_batch_integrate_fp32_noalloc: n = %lld is outside [0, %d]; its fixed work-queue "
                      "scratch holds at most GX_NOALLOC_MAX_ORBITS orbits (use gx_batch_integrate_fp32 for more)",
                      (long long)n, GX_NOALLOC_MAX_ORBITS);
        return GX_ERR_CAPACITY;
    }
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(w0 && n_steps && dt && method && w_out, "NULL array");
    GX_CHECK_ARG(block >= 32 && block <= 256 && block % 32 == 0, "block must be a multiple of 32 in [32, 256]");
    GX_CHECK_ARG(grid >= 1, "grid must be >= 1");
    int32_t *s = nullptr;
    rc = gx::noalloc_scratch_address(&s);
    if (rc) return rc;
    const int64_t slots = gx_batch_schedule_slots(n, gx::NA_CHUNK);
    static_assert(gx::NA_SLOTS >= GX_NOALLOC_MAX_ORBITS + gx::NA_CHUNK, "order capacity");
    cudaStream_t st = gx::as_stream(stream);
    GX_CUDA_TRY(cudaMemsetAsync(s, 0, GX_BATCH_QUEUE_WORDS * sizeof(int32_t), st));  // queue
    rc = gx::launch_schedule(n_steps, method, n, gx::NA_CHUNK, s + gx::NA_ORDER_OFF, slots, slots,
                             s + gx::NA_WORK_OFF, st);
    if (rc) return rc;
    gx::BatchArgs A;
    memset(&A, 0, sizeof(A));
    A.n = n;
    A.slots = slots;
    A.n_lead = gx::queue_lead_chunks(slots / gx::NA_CHUNK, gx::NA_CHUNK);
    A.chunk = gx::NA_CHUNK;
    A.pad = 0;
    A.cancel = gx::cancel_flag();
    A.state_in = nullptr;
    A.state_out = nullptr;
    const double two_13 = std::pow(2., 1. / 3.);
    const double c[4] = {1. / (2. * (2. - two_13)), (1. - two_13) / (2. * (2. - two_13)),
                         (1. - two_13) / (2. * (2. - two_13)), 1. / (2. * (2. - two_13))};
    const double d[4] = {0., 1. / (2. - two_13), -two_13 / (2. - two_13), 1. / (2. - two_13)};
    for (int k = 0; k < 4; k++) {
        A.c[k] = (float)c[k];
        A.d[k] = (float)d[k];
    }
    gx::launch_batch_fp32(dp, A, w0, n_steps, dt, method, s + gx::NA_ORDER_OFF, s, w_out, grid, block, st);
    return gx::check_launch("batch_fp32 (noalloc)");
}
