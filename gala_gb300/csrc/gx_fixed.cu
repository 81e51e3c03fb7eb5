// gx_fixed.cu -- FP64 Leapfrog and Ruth4, one thread per orbit.
//
// Each thread carries its orbit's state in registers for the whole run and
// evaluates the composite gradient in registers (no per-step kernel launch, no
// state round trip through memory).  Snapshots go straight to gala's
// (6, ntimes, N) layout: at every step a warp writes 6 fully coalesced 256-byte
// rows.  The per-orbit arithmetic is gala's, expression by expression:
//   leapfrog  c_init_velocity / c_leapfrog_step (leapfrog.pyx:24-51,99-116)
//   ruth4     c_ruth4_step with gala's coefficients (ruth4.pyx:24-35,65-78,98-108)
#include "gx_host.h"
#include "gx_queue.cuh"
#include "gx_scf.cuh"

namespace gx {

struct Ruth4Coef {
    double c[4], d[4];
};

template <bool SCF>
__device__ __forceinline__ void grad_impl(const DevPot &pot, const double *x, double *g) {
    V3 q;
    q.v[0] = x[0]; q.v[1] = x[1]; q.v[2] = x[2];
    const V3 r = gradient_call<SCF>(pot, q);
    g[0] = r.v[0]; g[1] = r.v[1]; g[2] = r.v[2];
}
#define grad(pot, x, g) grad_impl<SCF>(pot, x, g)

template <bool SAVE_ALL, bool SCF>
__global__ void __launch_bounds__(128, 1) leapfrog_kernel(const __grid_constant__ DevPot pot, const double *__restrict__ w0, int64_t n,
                                                       const double *__restrict__ t, int64_t ntimes,
                                                       double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x[3], v[3], vh[3], g[3];
    for (int k = 0; k < 3; k++) {
        x[k] = w0[k * n + i];
        v[k] = w0[(3 + k) * n + i];
    }
    const double dt = t[1] - t[0];
    if (SAVE_ALL) {
        for (int k = 0; k < 3; k++) {
            out[(k * ntimes) * n + i] = x[k];
            out[((3 + k) * ntimes) * n + i] = v[k];
        }
    }
    // c_init_velocity: v_{1/2} = v - grad * dt / 2
    grad(pot, x, g);
    for (int k = 0; k < 3; k++) vh[k] = v[k] - g[k] * dt / 2.;
    for (int64_t j = 1; j < ntimes; j++) {
        // c_leapfrog_step: drift, gradient, half kick (output v), full kick
        for (int k = 0; k < 3; k++) x[k] = x[k] + vh[k] * dt;
        grad(pot, x, g);
        for (int k = 0; k < 3; k++) {
            v[k] = vh[k] - g[k] * dt / 2.;
            vh[k] = vh[k] - g[k] * dt;
        }
        if (SAVE_ALL) {
            for (int k = 0; k < 3; k++) {
                __stcs(&out[(k * ntimes + j) * n + i], x[k]);
                __stcs(&out[((3 + k) * ntimes + j) * n + i], v[k]);
            }
        }
    }
    if (!SAVE_ALL) {
        for (int k = 0; k < 3; k++) {
            out[k * n + i] = x[k];
            out[(3 + k) * n + i] = v[k];
        }
    }
}

template <bool SAVE_ALL, bool SCF>
__global__ void __launch_bounds__(128, 1) ruth4_kernel(const __grid_constant__ DevPot pot, Ruth4Coef co, const double *__restrict__ w0,
                                                    int64_t n, const double *__restrict__ t, int64_t ntimes,
                                                    double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double w[6], g[3];
    for (int k = 0; k < 6; k++) w[k] = w0[k * n + i];
    const double dt = t[1] - t[0];
    if (SAVE_ALL)
        for (int k = 0; k < 6; k++) out[(k * ntimes) * n + i] = w[k];
    for (int64_t j = 1; j < ntimes; j++) {
#pragma unroll
        for (int s = 0; s < 4; s++) {
            // The first sub-step has d = 0, yet gala still evaluates the gradient
            // there: a non-finite gradient (an orbit sitting on a singular point)
            // turns v into NaN through 0 * inf.  This FP64 form keeps that
            // evaluation so that it reproduces gala in every case.
            grad(pot, w, g);
            for (int k = 0; k < 3; k++) {
                w[3 + k] = w[3 + k] - co.d[s] * g[k] * dt;
                w[k] = w[k] + co.c[s] * w[3 + k] * dt;
            }
        }
        if (SAVE_ALL)
            for (int k = 0; k < 6; k++) __stcs(&out[(k * ntimes + j) * n + i], w[k]);
    }
    if (!SAVE_ALL)
        for (int k = 0; k < 6; k++) out[k * n + i] = w[k];
}

// ---------------------------------------------------------------------------
// Batched FP64 form of the same two integrators (the plain form of the batched
// workload): per orbit its own n_steps, dt and integrator, final state only,
// gala's arithmetic exactly as in the kernels above.  Same work queue as the
// FP32 batch kernel (gx_batch.cu, gx_queue.cuh): chunks of the caller's order
// pulled by a persistent grid.
// ---------------------------------------------------------------------------
template <bool SCF>
__global__ void __launch_bounds__(128, 1) batch_fp64_kernel(const __grid_constant__ DevPot pot, Ruth4Coef co,
                                                            int64_t n, int64_t slots, int32_t chunk, int64_t n_lead,
                                                            const double *__restrict__ w0,
                                                            const int64_t *__restrict__ nsteps,
                                                            const double *__restrict__ dtv,
                                                            const int32_t *__restrict__ method,
                                                            const int32_t *__restrict__ order,
                                                            int32_t *__restrict__ counter,
                                                            double *__restrict__ out,
                                                            const int32_t *__restrict__ cancel) {
    const int lane = threadIdx.x & 31;
    const int64_t nchunks = slots / chunk;
    const int subs = chunk / 32;
    int phase = 0;
    for (;;) {
        // a cancelled launch takes no further work (lane 0 decides for the warp)
        int64_t c = -1;
        int sub = -1;
        if (lane == 0 && !cancel_requested(cancel)) c = queue_next(counter, nchunks, n_lead, subs, phase, sub);
        c = __shfl_sync(0xffffffffu, c, 0);
        sub = __shfl_sync(0xffffffffu, sub, 0);
        if (c < 0) break;
        // one lead block, or every block of a main-region chunk
        const int b0 = sub >= 0 ? sub : 0, b1 = sub >= 0 ? sub + 1 : subs;
        for (int b = b0; b < b1; b++) {
            const int32_t i = order[c * chunk + 32 * b + lane];
            // -1 pads the order; any other id outside [0, n) is skipped (and recorded in the debug build)
            if (i == -1 || !GX_DBG_CHECK(i >= 0 && i < n, DBG_ORDER, i, n)) continue;
            GX_DBG_DONE(i, nsteps[i]);
            double w[6], g[3];
            for (int k = 0; k < 6; k++) w[k] = w0[k * n + i];
            const int64_t ns = nsteps[i];
            const double dt = dtv[i];
            if (ns > 0 && method[i] == 0) {
                double vh[3];
                grad(pot, w, g);
                for (int k = 0; k < 3; k++) vh[k] = w[3 + k] - g[k] * dt / 2.;
                for (int64_t j = 0; j < ns; j++) {
                    for (int k = 0; k < 3; k++) w[k] = w[k] + vh[k] * dt;
                    grad(pot, w, g);
                    for (int k = 0; k < 3; k++) {
                        w[3 + k] = vh[k] - g[k] * dt / 2.;
                        vh[k] = vh[k] - g[k] * dt;
                    }
                }
            } else if (ns > 0) {
                for (int64_t j = 0; j < ns; j++) {
                    for (int s = 0; s < 4; s++) {
                        grad(pot, w, g);
                        for (int k = 0; k < 3; k++) {
                            w[3 + k] = w[3 + k] - co.d[s] * g[k] * dt;
                            w[k] = w[k] + co.c[s] * w[3 + k] * dt;
                        }
                    }
                }
            }
            for (int k = 0; k < 6; k++) out[k * n + i] = w[k];
        }
    }
}

static int fixed_common(const gx_potential *pot, const gx_frame *frame, const double *w0, int64_t n,
                        const double *t, int64_t ntimes, double *w_out, DevPot *dp, const char *name) {
    int rc = pack_potential(pot, dp);
    if (rc) return rc;
    if (frame != nullptr && frame->type != GX_FRAME_STATIC) {
        set_error("%s integration is currently only supported for StaticFrame", name);
        return GX_ERR_UNSUPPORTED;
    }
    GX_CHECK_ARG(n >= 0, "n < 0");
    GX_CHECK_ARG(ntimes >= 2, "ntimes must be >= 2 (got %lld)", (long long)ntimes);
    GX_CHECK_ARG(n == 0 || (w0 && t && w_out), "NULL array");
    return GX_OK;
}

}  // namespace gx

extern "C" {

int gx_leapfrog_integrate_hamiltonian(const gx_potential *pot, const gx_frame *frame, const double *w0, int64_t n,
                                      const double *t, int64_t ntimes, int32_t save_all, double *w_out,
                                      void *stream) {
    gx::DevPot dp;
    int rc = gx::fixed_common(pot, frame, w0, n, t, ntimes, w_out, &dp, "Leapfrog");
    if (rc || n == 0) return rc;
    const int bs = 128;
    const unsigned grid = (unsigned)((n + bs - 1) / bs);
    cudaStream_t st = gx::as_stream(stream);
    if (save_all && dp.has_scf)
        gx::leapfrog_kernel<true, true><<<grid, bs, 0, st>>>(dp, w0, n, t, ntimes, w_out);
    else if (save_all)
        gx::leapfrog_kernel<true, false><<<grid, bs, 0, st>>>(dp, w0, n, t, ntimes, w_out);
    else if (dp.has_scf)
        gx::leapfrog_kernel<false, true><<<grid, bs, 0, st>>>(dp, w0, n, t, ntimes, w_out);
    else
        gx::leapfrog_kernel<false, false><<<grid, bs, 0, st>>>(dp, w0, n, t, ntimes, w_out);
    return gx::check_launch("leapfrog");
}

int gx_batch_integrate_fp64(const gx_potential *pot, const double *w0, int64_t n, const int64_t *n_steps,
                            const double *dt, const int32_t *method, const int32_t *order, int64_t n_slots,
                            int32_t chunk, int32_t block, int32_t grid, int32_t *queue_counter, double *w_out,
                            void *stream) {
    gx::DevPot dp;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0 && n < (int64_t)INT32_MAX, "n out of range");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(w0 && n_steps && dt && method && order && queue_counter && w_out, "NULL array");
    GX_CHECK_ARG(chunk >= 32 && chunk % 32 == 0 && chunk <= 4096, "chunk must be a multiple of 32 in [32, 4096]");
    GX_CHECK_ARG(n_slots >= n && n_slots % chunk == 0, "order length must be >= n and a multiple of chunk");
    GX_CHECK_ARG(block >= 32 && block <= 128 && block % 32 == 0, "block must be a multiple of 32 in [32, 128]");
    GX_CHECK_ARG(grid >= 1, "grid must be >= 1");
    const double two_13 = std::pow(2., 1. / 3.);
    gx::Ruth4Coef co;
    co.c[0] = 1. / (2. * (2. - two_13));
    co.c[1] = (1. - two_13) / (2. * (2. - two_13));
    co.c[2] = (1. - two_13) / (2. * (2. - two_13));
    co.c[3] = 1. / (2. * (2. - two_13));
    co.d[0] = 0.;
    co.d[1] = 1. / (2. - two_13);
    co.d[2] = -two_13 / (2. - two_13);
    co.d[3] = 1. / (2. - two_13);
    cudaStream_t st = gx::as_stream(stream);
    GX_CUDA_TRY(cudaMemsetAsync(queue_counter, 0, GX_BATCH_QUEUE_WORDS * sizeof(int32_t), st));
    const int64_t n_lead = gx::queue_lead_chunks(n_slots / chunk, chunk);
    if (dp.has_scf)
        gx::batch_fp64_kernel<true><<<grid, block, 0, st>>>(dp, co, n, n_slots, chunk, n_lead, w0, n_steps, dt,
                                                            method, order, queue_counter, w_out, gx::cancel_flag());
    else
        gx::batch_fp64_kernel<false><<<grid, block, 0, st>>>(dp, co, n, n_slots, chunk, n_lead, w0, n_steps, dt,
                                                             method, order, queue_counter, w_out, gx::cancel_flag());
    return gx::check_launch("batch_fp64");
}

int gx_ruth4_integrate_hamiltonian(const gx_potential *pot, const gx_frame *frame, const double *w0, int64_t n,
                                   const double *t, int64_t ntimes, int32_t save_all, double *w_out,
                                   void *stream) {
    gx::DevPot dp;
    int rc = gx::fixed_common(pot, frame, w0, n, t, ntimes, w_out, &dp, "Ruth4");
    if (rc || n == 0) return rc;
    // ruth4.pyx:65-78, evaluated on the host in double like Cython does.
    const double two_13 = std::pow(2., 1. / 3.);
    gx::Ruth4Coef co;
    co.c[0] = 1. / (2. * (2. - two_13));
    co.c[1] = (1. - two_13) / (2. * (2. - two_13));
    co.c[2] = (1. - two_13) / (2. * (2. - two_13));
    co.c[3] = 1. / (2. * (2. - two_13));
    co.d[0] = 0.;
    co.d[1] = 1. / (2. - two_13);
    co.d[2] = -two_13 / (2. - two_13);
    co.d[3] = 1. / (2. - two_13);
    const int bs = 128;
    const unsigned grid = (unsigned)((n + bs - 1) / bs);
    cudaStream_t st = gx::as_stream(stream);
    if (save_all && dp.has_scf)
        gx::ruth4_kernel<true, true><<<grid, bs, 0, st>>>(dp, co, w0, n, t, ntimes, w_out);
    else if (save_all)
        gx::ruth4_kernel<true, false><<<grid, bs, 0, st>>>(dp, co, w0, n, t, ntimes, w_out);
    else if (dp.has_scf)
        gx::ruth4_kernel<false, true><<<grid, bs, 0, st>>>(dp, co, w0, n, t, ntimes, w_out);
    else
        gx::ruth4_kernel<false, false><<<grid, bs, 0, st>>>(dp, co, w0, n, t, ntimes, w_out);
    return gx::check_launch("ruth4");
}

}  // extern "C"
