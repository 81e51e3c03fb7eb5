// gx_lfnbody.cu -- FP64 Leapfrog for small direct n-body systems and for the
// release systems of Leapfrog mock streams (gala's arithmetic, -fmad=false).
#include "gx_host.h"
#include "gx_scf.cuh"
#include "gx_body.cuh"

namespace gx {

// ---------------------------------------------------------------------------
// Leapfrog n-body systems: leapfrog_integrate_nbody (leapfrog.pyx:161-255) and
// the release systems of mockstream_leapfrog (mockstream.pyx:548-593).  One
// THREAD per system (a few bodies: the whole state fits in registers), bodies
// updated in gala's order within a step: body k drifts, feels the external
// potential and every other non-null massive body at its CURRENT position
// (already moved this step when j < k: c_nbody_gradient_symplectic,
// cpotential.cpp:418-442), and kicks.  Consecutive threads are consecutive
// systems of one release time, so a warp runs systems of equal length.
// ---------------------------------------------------------------------------
struct LfArgs {
    int64_t n_sys;
    int32_t nbody;          // massive bodies (first in every system)
    int32_t nparticles;     // direct n-body: bodies per system
    const gx_body *bodies;  // (n_streams or n_sys, nbody)
    double dt;
    // direct n-body systems
    const double *w0;       // (n_sys, nparticles, 6)
    const double *t;
    int64_t ntimes;
    int32_t save_all;
    double *w_out;
    // release systems
    int64_t n_streams, n_release, n_particles;
    const double *nbody_w;  // (n_streams, n_release, nbody, 6)
    const double *release_t;
    const int64_t *offset;
    const double *stream_w0;
    double t_final;
    double *stream_w_out, *nbody_w_out;
    int32_t *status;
};

template <int MAXB, bool SCF>
__device__ __forceinline__ void lf_grad(const DevPot &pot, const gx_body *__restrict__ bod, int nbody, int b,
                                        const double (&x)[MAXB][3], double *g) {
    V3 q;
    q.v[0] = x[b][0];
    q.v[1] = x[b][1];
    q.v[2] = x[b][2];
    const V3 ge = gradient_call<SCF>(pot, q);
    g[0] = ge.v[0];
    g[1] = ge.v[1];
    g[2] = ge.v[2];
#pragma unroll
    for (int j = 0; j < MAXB; j++) {
        if (j >= nbody || j == b) continue;
        const int type = __ldg(&bod[j].type);
        if (type == GX_POT_NULL) continue;
        const V3 f2 = body_gradient_call(type, bod[j].params, x[b][0] - x[j][0], x[b][1] - x[j][1],
                                         x[b][2] - x[j][2]);
        g[0] += f2.v[0];
        g[1] += f2.v[1];
        g[2] += f2.v[2];
    }
}

template <int MAXB, bool STREAM, bool SAVE_ALL, bool SCF>
__global__ void __launch_bounds__(128) lf_nbody_kernel(const __grid_constant__ DevPot pot, const LfArgs A) {
    const int64_t sys = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= A.n_sys) return;
    double x[MAXB][3], v[MAXB][3], vh[MAXB][3];
    int nsys;
    const gx_body *bod;
    int64_t si = 0, ss = 0, o0 = 0;
    double t0;
    int64_t n_steps;
    const double dt = A.dt;
    if constexpr (STREAM) {
        si = sys / A.n_streams;
        ss = sys - si * A.n_streams;
        o0 = A.offset[si];
        const int64_t o1 = A.offset[si + 1];
        if (o1 == o0) {
            A.status[ss * A.n_release + si] = 0;
            return;
        }
        if (!GX_DBG_CHECK(!(o1 < o0 || o0 < 0 || o1 > A.n_particles || A.nbody + (o1 - o0) > MAXB), DBG_OFFSET,
                          si, A.n_release)) {
            A.status[ss * A.n_release + si] = -1;
            return;
        }
        nsys = A.nbody + (int)(o1 - o0);
        bod = A.bodies + ss * A.nbody;
        t0 = A.release_t[si];
        n_steps = (int64_t)((A.t_final - t0) / dt + 0.5);  // mockstream.pyx:582
    } else {
        nsys = A.nparticles;
        bod = A.bodies + sys * A.nbody;
        t0 = A.t[0];
        n_steps = A.ntimes - 1;
    }
#pragma unroll
    for (int b = 0; b < MAXB; b++) {
        const double *src = nullptr;
        if (b < nsys) {
            if constexpr (STREAM)
                src = (b < A.nbody) ? A.nbody_w + ((ss * A.n_release + si) * A.nbody + b) * 6
                                    : A.stream_w0 + (ss * A.n_particles + o0 + (b - A.nbody)) * 6;
            else
                src = A.w0 + (sys * A.nparticles + b) * 6;
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            x[b][k] = src ? src[k] : 0.;
            v[b][k] = src ? src[3 + k] : 0.;
        }
    }
    if constexpr (!STREAM && SAVE_ALL) {
#pragma unroll
        for (int b = 0; b < MAXB; b++)
            if (b < nsys) {
                double *o = A.w_out + ((sys * A.ntimes) * A.nparticles + b) * 6;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    o[k] = x[b][k];
                    o[3 + k] = v[b][k];
                }
            }
    }
    // c_init_velocity_nbody (leapfrog.pyx:126-138), every body at the start positions
#pragma unroll
    for (int b = 0; b < MAXB; b++) {
        if (b >= nsys) continue;
        double g[3];
        lf_grad<MAXB, SCF>(pot, bod, A.nbody, b, x, g);
#pragma unroll
        for (int k = 0; k < 3; k++) vh[b][k] = v[b][k] - g[k] * dt / 2.;
    }
    (void)t0;
    for (int64_t j = 0; j < n_steps; j++) {
        // c_leapfrog_step_nbody (leapfrog.pyx:140-158), bodies in order
#pragma unroll
        for (int b = 0; b < MAXB; b++) {
            if (b >= nsys) continue;
#pragma unroll
            for (int k = 0; k < 3; k++) x[b][k] = x[b][k] + vh[b][k] * dt;
            double g[3];
            lf_grad<MAXB, SCF>(pot, bod, A.nbody, b, x, g);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                v[b][k] = vh[b][k] - g[k] * dt / 2.;
                vh[b][k] = vh[b][k] - g[k] * dt;
            }
        }
        if constexpr (!STREAM && SAVE_ALL) {
#pragma unroll
            for (int b = 0; b < MAXB; b++)
                if (b < nsys) {
                    double *o = A.w_out + (((sys * A.ntimes) + j + 1) * A.nparticles + b) * 6;
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        o[k] = x[b][k];
                        o[3 + k] = v[b][k];
                    }
                }
        }
    }
    if constexpr (STREAM) {
#pragma unroll
        for (int b = 0; b < MAXB; b++) {
            if (b >= nsys) continue;
            double *o;
            if (b >= A.nbody)
                o = A.stream_w_out + (ss * A.n_particles + o0 + (b - A.nbody)) * 6;
            else if (A.nbody_w_out && A.offset[si + 1] == A.offset[A.n_release])
                o = A.nbody_w_out + (ss * A.nbody + b) * 6;
            else
                continue;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                o[k] = x[b][k];
                o[3 + k] = v[b][k];
            }
        }
        A.status[ss * A.n_release + si] = 1;
    } else if constexpr (!SAVE_ALL) {
#pragma unroll
        for (int b = 0; b < MAXB; b++)
            if (b < nsys) {
                double *o = A.w_out + (sys * A.nparticles + b) * 6;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    o[k] = x[b][k];
                    o[3 + k] = v[b][k];
                }
            }
    }
}

template <bool STREAM, bool SAVE_ALL>
int launch_lf(const DevPot &dp, const LfArgs &A, int maxb, cudaStream_t st) {
    const unsigned grid = (unsigned)((A.n_sys + 127) / 128);
    if (maxb > 8) {
        set_error("leapfrog n-body systems of %d bodies: at most 8", maxb);
        return GX_ERR_UNSUPPORTED;
    }
    // three bodies (a progenitor and one particle per tail) is the common mock
    // stream; everything else up to eight bodies shares one instantiation
    if (dp.has_scf)
        lf_nbody_kernel<8, STREAM, SAVE_ALL, true><<<grid, 128, 0, st>>>(dp, A);
    else if (maxb <= 3)
        lf_nbody_kernel<3, STREAM, SAVE_ALL, false><<<grid, 128, 0, st>>>(dp, A);
    else
        lf_nbody_kernel<8, STREAM, SAVE_ALL, false><<<grid, 128, 0, st>>>(dp, A);
    return check_launch(STREAM ? "mockstream_leapfrog" : "nbody_leapfrog");
}

}  // namespace gx

extern "C" int gx_nbody_leapfrog(const gx_potential *pot, int64_t n_systems, int32_t nparticles, int32_t nbody,
                                 const gx_body *bodies, const double *w0, const double *t, int64_t ntimes,
                                 int32_t save_all, double *w_out, void *stream) {
    gx::DevPot dp;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(n_systems >= 0, "n_systems < 0");
    GX_CHECK_ARG(nparticles >= 1 && nparticles <= 8, "nparticles must be in [1, 8] (got %d)", nparticles);
    GX_CHECK_ARG(nbody >= 0 && nbody <= nparticles, "nbody must be in [0, nparticles] (got %d)", nbody);
    GX_CHECK_ARG(ntimes >= 2, "ntimes must be >= 2 (got %lld)", (long long)ntimes);
    if (n_systems == 0) return GX_OK;
    GX_CHECK_ARG(w0 && t && w_out, "NULL array");
    GX_CHECK_ARG(nbody == 0 || bodies, "bodies is NULL");
    double t01[2];
    GX_CUDA_TRY(cudaMemcpyAsync(t01, t, sizeof(t01), cudaMemcpyDeviceToHost, gx::as_stream(stream)));
    GX_CUDA_TRY(cudaStreamSynchronize(gx::as_stream(stream)));
    gx::LfArgs A;
    memset(&A, 0, sizeof(A));
    A.n_sys = n_systems;
    A.nbody = nbody;
    A.nparticles = nparticles;
    A.bodies = bodies;
    A.dt = t01[1] - t01[0];
    A.w0 = w0;
    A.t = t;
    A.ntimes = ntimes;
    A.save_all = save_all ? 1 : 0;
    A.w_out = w_out;
    cudaStream_t st = gx::as_stream(stream);
    return save_all ? gx::launch_lf<false, true>(dp, A, nparticles, st)
                    : gx::launch_lf<false, false>(dp, A, nparticles, st);
}

extern "C" int gx_mockstream_leapfrog(const gx_potential *pot, int64_t n_streams, int32_t nbody,
                                      const gx_body *bodies, const double *nbody_w, int64_t n_release,
                                      const double *release_t, const int64_t *release_offset,
                                      int32_t max_per_release, const double *stream_w0, int64_t n_particles,
                                      double t_final, double dt, double *stream_w_out, double *nbody_w_out,
                                      int32_t *status, void *stream) {
    gx::DevPot dp;
    int rc = gx::pack_potential(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(n_streams >= 0 && n_release >= 0 && n_particles >= 0, "negative size");
    GX_CHECK_ARG(nbody >= 1, "nbody must be >= 1 (the progenitor)");
    GX_CHECK_ARG(max_per_release >= 0 && nbody + max_per_release <= 8,
                 "nbody + max_per_release must be <= 8 (got %d + %d)", nbody, max_per_release);
    GX_CHECK_ARG(dt != 0.0, "dt must be non-zero");
    if (n_streams == 0 || n_release == 0) return GX_OK;
    GX_CHECK_ARG(bodies && nbody_w && release_t && release_offset && status, "NULL array");
    GX_CHECK_ARG(n_particles == 0 || (stream_w0 && stream_w_out), "NULL particle array");
    gx::LfArgs A;
    memset(&A, 0, sizeof(A));
    A.n_sys = n_streams * n_release;
    A.nbody = nbody;
    A.bodies = bodies;
    A.dt = dt;
    A.n_streams = n_streams;
    A.n_release = n_release;
    A.n_particles = n_particles;
    A.nbody_w = nbody_w;
    A.release_t = release_t;
    A.offset = release_offset;
    A.stream_w0 = stream_w0;
    A.t_final = t_final;
    A.stream_w_out = stream_w_out;
    A.nbody_w_out = nbody_w_out;
    A.status = status;
    return gx::launch_lf<true, false>(dp, A, nbody + max_per_release, gx::as_stream(stream));
}
