// gx_stream32.cu -- Leapfrog mock-stream release systems in FP32 with
// compensated state (the fast form of gx_mockstream_leapfrog).
//
// Same system layout and step order as the FP64 kernel (mockstream.pyx:548-593,
// leapfrog.pyx:126-158): one thread per release system, bodies updated in order
// within a step, a particle feeling the external potential and every massive
// body at its current position.  Positions and half-step velocities are FP32
// (hi, lo) pairs with Kahan-compensated updates; forces are FP32 on the MUFU
// unit (gx_fp32.cuh), the body pull evaluated at the separation
// (x_hi - x0_hi) + (x_lo - x0_lo), which keeps the particle-progenitor distance
// accurate although both positions are ~1e2 times larger.  Initial and final
// states are FP64.  No bit-parity claim: accuracy is measured against the FP64
// kernel.
#include "gx_host.h"
#include "gx_fp32.cuh"
#include "gx_scf.cuh"

namespace gx {

int pack_potential_f32(const gx_potential *pot, DevPotF *out);

struct Lf32Args {
    int64_t n_sys, n_streams, n_release, n_particles;
    int32_t nbody;
    int32_t pad;
    const gx_body *bodies;   // (n_streams, nbody)
    const double *nbody_w;   // (n_streams, n_release, nbody, 6)
    const double *release_t;
    const int64_t *offset;
    const double *stream_w0;
    double t_final, dt;
    double *stream_w_out, *nbody_w_out;
    int32_t *status;
};

__device__ __forceinline__ void split2(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

// The FP32 constants of one body's component (the packing of pack_potential_f32).
__device__ __forceinline__ void body_to_f32(const gx_body *b, DevCompF &c) {
    const int type = __ldg(&b->type);
    const double G = __ldg(b->params + 0), m = __ldg(b->params + 1);
    const double p2 = __ldg(b->params + 2), p3 = __ldg(b->params + 3);
    c.type = type;
    c.do_sr = 0;
#pragma unroll
    for (int k = 0; k < 6; k++) c.p[k] = 0.f;
    switch (type) {
    case GX_POT_KEPLER: c.p[0] = (float)(G * m); break;
    case GX_POT_HERNQUIST: c.p[0] = (float)(G * m); c.p[1] = (float)p2; break;
    case GX_POT_PLUMMER: c.p[0] = (float)(G * m); c.p[1] = (float)(p2 * p2); break;
    case GX_POT_MIYAMOTONAGAI: c.p[0] = (float)(G * m); c.p[1] = (float)p2; c.p[2] = (float)(p3 * p3); break;
    case GX_POT_SPHERICALNFW: c.p[0] = (float)(G * m / (p2 * p2 * p2)); c.p[1] = (float)(1.0 / p2); c.p[2] = (float)p2; break;
    default: c.type = GX_POT_NULL; break;
    }
}

template <int MAXB, typename S>
__global__ void __launch_bounds__(128) lf_stream_fp32_kernel(const __grid_constant__ DevPotF pot, const Lf32Args A) {
    const int64_t sys = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= A.n_sys) return;
    const int64_t si = sys / A.n_streams, ss = sys - si * A.n_streams;
    const int64_t o0 = A.offset[si], o1 = A.offset[si + 1];
    if (o1 == o0) {
        A.status[ss * A.n_release + si] = 0;
        return;
    }
    if (!GX_DBG_CHECK(!(o1 < o0 || o0 < 0 || o1 > A.n_particles || A.nbody + (o1 - o0) > MAXB), DBG_OFFSET, si,
                      A.n_release)) {
        A.status[ss * A.n_release + si] = -1;
        return;
    }
    const int nsys = A.nbody + (int)(o1 - o0);
    const int nbody = A.nbody;
    DevCompF bc[MAXB];
#pragma unroll
    for (int j = 0; j < MAXB; j++) {
        if (j < nbody) body_to_f32(A.bodies + ss * nbody + j, bc[j]);
        else bc[j].type = GX_POT_NULL;
    }
    float xh[MAXB][3], xl[MAXB][3], vh[MAXB][3], vl[MAXB][3], g[MAXB][3];
#pragma unroll
    for (int b = 0; b < MAXB; b++) {
        const double *src = nullptr;
        if (b < nsys)
            src = (b < nbody) ? A.nbody_w + ((ss * A.n_release + si) * nbody + b) * 6
                              : A.stream_w0 + (ss * A.n_particles + o0 + (b - nbody)) * 6;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            split2(src ? src[k] : 0., xh[b][k], xl[b][k]);
            split2(src ? src[3 + k] : 0., vh[b][k], vl[b][k]);
            g[b][k] = 0.f;
        }
    }
    const float h = (float)A.dt;

    auto force = [&](int b) {
        float q[3] = {xh[b][0], xh[b][1], xh[b][2]};
        potential_gradient_f<S>(pot, q, g[b]);
#pragma unroll
        for (int j = 0; j < MAXB; j++) {
            if (j >= nbody || j == b || bc[j].type == GX_POT_NULL) continue;
            const float d[3] = {(xh[b][0] - xh[j][0]) + (xl[b][0] - xl[j][0]),
                                (xh[b][1] - xh[j][1]) + (xl[b][1] - xl[j][1]),
                                (xh[b][2] - xh[j][2]) + (xl[b][2] - xl[j][2])};
            comp_gradient_f(bc[j], d, g[b]);
        }
    };

    // c_init_velocity_nbody: v_{1/2} = v - g h / 2
#pragma unroll
    for (int b = 0; b < MAXB; b++) {
        if (b >= nsys) continue;
        force(b);
#pragma unroll
        for (int k = 0; k < 3; k++) kahan_add(vh[b][k], vl[b][k], -g[b][k] * h * 0.5f);
    }
    const int64_t n_steps = (int64_t)((A.t_final - A.release_t[si]) / A.dt + 0.5);
    for (int64_t j = 0; j < n_steps; j++) {
#pragma unroll
        for (int b = 0; b < MAXB; b++) {
            if (b >= nsys) continue;
#pragma unroll
            for (int k = 0; k < 3; k++) kahan_add(xh[b][k], xl[b][k], fmaf(vh[b][k], h, vl[b][k] * h));
            force(b);
#pragma unroll
            for (int k = 0; k < 3; k++) kahan_add(vh[b][k], vl[b][k], -g[b][k] * h);
        }
    }
    // output velocity at the last step: v_{n+1/2} + g h / 2 (the init value when n_steps == 0)
#pragma unroll
    for (int b = 0; b < MAXB; b++) {
        if (b >= nsys) continue;
        double *o;
        if (b >= nbody)
            o = A.stream_w_out + (ss * A.n_particles + o0 + (b - nbody)) * 6;
        else if (A.nbody_w_out && o1 == A.offset[A.n_release])
            o = A.nbody_w_out + (ss * nbody + b) * 6;
        else
            continue;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float vhk = vh[b][k], vlk = vl[b][k];
            kahan_add(vhk, vlk, g[b][k] * h * 0.5f);
            o[k] = (double)xh[b][k] + (double)xl[b][k];
            o[3 + k] = (double)vhk + (double)vlk;
        }
    }
    A.status[ss * A.n_release + si] = 1;
}

}  // namespace gx

extern "C" int gx_mockstream_leapfrog_fp32(const gx_potential *pot, int64_t n_streams, int32_t nbody,
                                           const gx_body *bodies, const double *nbody_w, int64_t n_release,
                                           const double *release_t, const int64_t *release_offset,
                                           int32_t max_per_release, const double *stream_w0, int64_t n_particles,
                                           double t_final, double dt, double *stream_w_out, double *nbody_w_out,
                                           int32_t *status, void *stream) {
    gx::DevPotF dp;
    int rc = gx::pack_potential_f32(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(n_streams >= 0 && n_release >= 0 && n_particles >= 0, "negative size");
    GX_CHECK_ARG(nbody >= 1, "nbody must be >= 1 (the progenitor)");
    GX_CHECK_ARG(max_per_release >= 0 && nbody + max_per_release <= 8,
                 "nbody + max_per_release must be <= 8 (got %d + %d)", nbody, max_per_release);
    GX_CHECK_ARG(dt != 0.0, "dt must be non-zero");
    if (n_streams == 0 || n_release == 0) return GX_OK;
    GX_CHECK_ARG(bodies && nbody_w && release_t && release_offset && status, "NULL array");
    GX_CHECK_ARG(n_particles == 0 || (stream_w0 && stream_w_out), "NULL particle array");
    gx::Lf32Args A;
    memset(&A, 0, sizeof(A));
    A.n_sys = n_streams * n_release;
    A.n_streams = n_streams;
    A.n_release = n_release;
    A.n_particles = n_particles;
    A.nbody = nbody;
    A.bodies = bodies;
    A.nbody_w = nbody_w;
    A.release_t = release_t;
    A.offset = release_offset;
    A.stream_w0 = stream_w0;
    A.t_final = t_final;
    A.dt = dt;
    A.stream_w_out = stream_w_out;
    A.nbody_w_out = nbody_w_out;
    A.status = status;
    const unsigned grid = (unsigned)((A.n_sys + 127) / 128);
    cudaStream_t st = gx::as_stream(stream);
    constexpr int H = GX_POT_HERNQUIST, MN = GX_POT_MIYAMOTONAGAI, NFW = GX_POT_SPHERICALNFW;
    bool mw = dp.ncomp == 4;
    const int want[4] = {H, H, MN, NFW};
    for (int k = 0; k < 4 && mw; k++) mw = dp.c[k].type == want[k] && !dp.c[k].do_sr;
    const int maxb = nbody + max_per_release;
    if (mw && maxb <= 3)
        gx::lf_stream_fp32_kernel<3, gx::PotSig<H, H, MN, NFW>><<<grid, 128, 0, st>>>(dp, A);
    else if (maxb <= 3)
        gx::lf_stream_fp32_kernel<3, gx::SigGeneric><<<grid, 128, 0, st>>>(dp, A);
    else
        gx::lf_stream_fp32_kernel<8, gx::SigGeneric><<<grid, 128, 0, st>>>(dp, A);
    return gx::check_launch("mockstream_leapfrog_fp32");
}
