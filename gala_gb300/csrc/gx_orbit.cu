// gx_orbit.cu -- per-orbit extremum statistics over stored snapshots: gala's
// Orbit.pericenter / apocenter / zmax (src/gala/dynamics/orbit.py:391-656) in
// one pass over HBM.
//
// gala finds the interior strict local maxima of q(t) (argrelmax with the two
// ends removed; q = -r for pericentres, r for apocentres, |z| for z maxima) and
// refines each with the parabola through the three samples around it, taking
// its vertex.  Here one thread per orbit streams its x, y, z rows of the
// (6, ntimes, N) snapshot array once (consecutive threads read consecutive
// orbits: every load is coalesced) and updates the three statistics together,
// keeping a three-sample window.  The vertex is computed in coordinates centred
// on the middle sample (q = a + b s + c s^2, s = t - t_j), the same parabola as
// gala's polyfit through the raw times but without their cancellation.
// Per orbit and kind it returns the number of extrema, their sum (in time order),
// minimum and maximum, and the first `keep` values and times.
#include "gx_host.h"

namespace gx {

struct ExtArgs {
    const double *w;   // (6, ntimes, n)
    const double *t;   // (ntimes)
    int64_t ntimes, n;
    int32_t reverse;   // time grid runs backwards: scan from the end (gala reverses the orbit)
    int32_t approximate;
    int32_t keep;
    int32_t pad;
    int32_t *count;    // (3, n)
    double *sum, *vmin, *vmax;  // (3, n)
    double *vals, *times;       // (3, n, keep) or NULL
};

struct ExtAcc {
    int32_t count;
    double sum, mn, mx;
};

__device__ __forceinline__ void ext_push(const ExtArgs &A, ExtAcc &acc, int kind, int64_t i, double v, double tv) {
    if (A.vals && acc.count < A.keep) {
        const int64_t o = ((int64_t)kind * A.n + i) * A.keep + acc.count;
        A.vals[o] = v;
        A.times[o] = tv;
    }
    acc.count++;
    acc.sum += v;
    acc.mn = fmin(acc.mn, v);
    acc.mx = fmax(acc.mx, v);
}

// Interior strict maximum of q at the middle of (q0, q1, q2) sampled at
// (t0, t1, t2); the vertex of the interpolating parabola (orbit.py:411-424).
__device__ __forceinline__ bool refine(double q0, double q1, double q2, double t0, double t1, double t2,
                                       bool approximate, double &v, double &tv) {
    if (!(q1 > q0 && q1 > q2)) return false;
    if (approximate) {
        v = q1;
        tv = t1;
        return true;
    }
    const double s0 = t0 - t1, s2 = t2 - t1;
    const double d0 = (q0 - q1) / s0, d2 = (q2 - q1) / s2;
    const double c = (d2 - d0) / (s2 - s0);
    const double b = d2 - c * s2;
    const double sv = -b / (2.0 * c);
    v = q1 + sv * (b + c * sv);
    tv = t1 + sv;
    return true;
}

// FP64 is 1/64 of the FP32 rate on this part (and double -> float conversion
// runs on the FP64 pipe), so the scan over all samples uses neither: each
// coordinate's FP32 approximation is built from the high word of the double
// with integer operations (sign cleared, exponent rebiased, top 20 mantissa
// bits: relative error below 2^-20), and r^2 and |z| are compared in FP32 with
// a relative margin of 1e-5.  Samples that pass -- a superset of gala's
// extrema, in practice the extrema themselves -- are only recorded (index and
// kinds) in a per-thread list during the scan.  The FP64 work (r and |z|,
// gala's strict comparisons, the parabola) runs afterwards over the lists, all
// lanes of a warp processing their k-th candidate together, instead of one lane
// at a time inside the scan: an extremum is rare per orbit but, across 32
// orbits, present in almost every stretch of samples.  r is sqrt(x^2 + y^2 +
// z^2) with fused multiply-adds, within an ulp of astropy's
// hypot(hypot(x, y), z) for a fifth of the FP64 work.  Loads are issued EXT_U
// samples ahead and the window is indexed at compile time.
constexpr int EXT_U = 8;
constexpr int EXT_LIST = 48;

// |x| as an FP32 value from the high word of x (0 below 2^-126, for the scan only).
__device__ __forceinline__ float abs_f32_from_hi(double x) {
    const unsigned hi = (unsigned)__double2hiint(x) & 0x7fffffffu;
    const unsigned bits = (hi - (896u << 20)) << 3;
    return (hi >= (897u << 20)) ? __uint_as_float(bits) : 0.0f;
}

__device__ __forceinline__ int ext_flags(float r0, float r1, float r2, float a0, float a1, float a2) {
    const float lo = 1.0f - 1e-5f, hi = 1.0f + 1e-5f;
    int f = 0;
    if (r1 <= r0 * hi && r1 <= r2 * hi) f |= 1;  // pericentre candidate
    if (r1 >= r0 * lo && r1 >= r2 * lo) f |= 2;  // apocentre candidate
    if (a1 >= a0 * lo && a1 >= a2 * lo) f |= 4;  // |z| maximum candidate
    return f;
}

struct ExtOrbit {
    const double *x, *y, *z;
};

// FP64 test and refinement of candidate sample jc (orbit.py:391-426), kinds f.
__device__ __forceinline__ void ext_check(const ExtArgs &A, const ExtOrbit &O, int64_t i, int64_t jc, int f,
                                          ExtAcc *acc) {
    const int64_t nt = A.ntimes;
    double px[3], py[3], pz[3], pt[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int64_t j = jc - 1 + k;
        const int64_t rr = A.reverse ? nt - 1 - j : j;
        px[k] = O.x[rr * A.n];
        py[k] = O.y[rr * A.n];
        pz[k] = O.z[rr * A.n];
        pt[k] = __ldg(A.t + rr);
    }
    double v, tv;
    if (f & 3) {
        double r[3];
#pragma unroll
        for (int k = 0; k < 3; k++) r[k] = sqrt(fma(px[k], px[k], fma(py[k], py[k], pz[k] * pz[k])));
        if ((f & 1) && refine(-r[0], -r[1], -r[2], pt[0], pt[1], pt[2], A.approximate, v, tv))
            ext_push(A, acc[0], 0, i, -v, tv);
        if ((f & 2) && refine(r[0], r[1], r[2], pt[0], pt[1], pt[2], A.approximate, v, tv))
            ext_push(A, acc[1], 1, i, v, tv);
    }
    if ((f & 4) && refine(fabs(pz[0]), fabs(pz[1]), fabs(pz[2]), pt[0], pt[1], pt[2], A.approximate, v, tv))
        ext_push(A, acc[2], 2, i, v, tv);
}

__global__ void __launch_bounds__(128) orbit_extrema_kernel(const ExtArgs A) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < A.n;
    const int64_t nt = A.ntimes;
    const int64_t ii = live ? i : 0;
    const ExtOrbit O = {A.w + ii, A.w + nt * A.n + ii, A.w + 2 * nt * A.n + ii};
    ExtAcc acc[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        acc[k].count = 0;
        acc[k].sum = 0.;
        acc[k].mn = __longlong_as_double(0x7ff0000000000000LL);
        acc[k].mx = -__longlong_as_double(0x7ff0000000000000LL);
    }
    int list[EXT_LIST];  // candidate sample index << 3 | kinds, in increasing time
    int ncand = 0;
    // process the list: all lanes of the warp take their k-th candidate together
    auto flush = [&]() {
        int most = ncand;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) most = max(most, __shfl_xor_sync(0xffffffffu, most, o));
        for (int k = 0; k < most; k++)
            if (k < ncand) ext_check(A, O, ii, list[k] >> 3, list[k] & 7, acc);
        ncand = 0;
    };
    auto note = [&](int64_t jc, int f) {
        if (f != 0 && jc >= 1 && jc <= nt - 2 && live) list[ncand++] = (int)(jc << 3) | f;
    };
    float wr[EXT_U + 2], wa[EXT_U + 2];
    wr[0] = wr[1] = wa[0] = wa[1] = 0.f;
    int64_t j0 = 0;
    for (; j0 + EXT_U <= nt; j0 += EXT_U) {
        double bx[EXT_U], by[EXT_U], bz[EXT_U];
#pragma unroll
        for (int u = 0; u < EXT_U; u++) {
            const int64_t rr = A.reverse ? nt - 1 - (j0 + u) : j0 + u;
            bx[u] = __ldcs(O.x + rr * A.n);
            by[u] = __ldcs(O.y + rr * A.n);
            bz[u] = __ldcs(O.z + rr * A.n);
        }
#pragma unroll
        for (int u = 0; u < EXT_U; u++) {
            const float fx = abs_f32_from_hi(bx[u]), fy = abs_f32_from_hi(by[u]), fz = abs_f32_from_hi(bz[u]);
            wr[u + 2] = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
            wa[u + 2] = fz;
        }
#pragma unroll
        for (int c = 1; c <= EXT_U; c++)
            note(j0 + c - 2, ext_flags(wr[c - 1], wr[c], wr[c + 1], wa[c - 1], wa[c], wa[c + 1]));
        if (__any_sync(0xffffffffu, ncand > EXT_LIST - EXT_U)) flush();
        wr[0] = wr[EXT_U]; wr[1] = wr[EXT_U + 1];
        wa[0] = wa[EXT_U]; wa[1] = wa[EXT_U + 1];
    }
    // remaining samples one at a time (window positions 0, 1 hold the two before)
    for (; j0 < nt; j0++) {
        const int64_t rr = A.reverse ? nt - 1 - j0 : j0;
        const float fx = abs_f32_from_hi(__ldcs(O.x + rr * A.n)), fy = abs_f32_from_hi(__ldcs(O.y + rr * A.n));
        const float fz = abs_f32_from_hi(__ldcs(O.z + rr * A.n));
        wr[2] = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
        wa[2] = fz;
        note(j0 - 1, ext_flags(wr[0], wr[1], wr[2], wa[0], wa[1], wa[2]));
        if (__any_sync(0xffffffffu, ncand >= EXT_LIST)) flush();
        wr[0] = wr[1]; wa[0] = wa[1];
        wr[1] = wr[2]; wa[1] = wa[2];
    }
    flush();
    if (!live) return;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        A.count[k * A.n + i] = acc[k].count;
        A.sum[k * A.n + i] = acc[k].sum;
        A.vmin[k * A.n + i] = acc[k].mn;
        A.vmax[k * A.n + i] = acc[k].mx;
    }
}

}  // namespace gx

extern "C" int gx_orbit_extrema(const double *w, const double *t, int64_t ntimes, int64_t n, int32_t approximate,
                                int32_t keep, int32_t *count, double *sum, double *vmin, double *vmax, double *vals,
                                double *times, void *stream) {
    GX_CHECK_ARG(ntimes >= 0 && n >= 0, "negative size");
    GX_CHECK_ARG(keep >= 0, "keep must be >= 0");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(w && t && count && sum && vmin && vmax, "NULL array");
    GX_CHECK_ARG(keep == 0 || (vals && times), "keep > 0 needs vals and times");
    gx::ExtArgs A;
    A.w = w;
    A.t = t;
    A.ntimes = ntimes;
    A.n = n;
    A.approximate = approximate ? 1 : 0;
    A.keep = keep;
    A.pad = 0;
    A.count = count;
    A.sum = sum;
    A.vmin = vmin;
    A.vmax = vmax;
    A.vals = keep ? vals : nullptr;
    A.times = keep ? times : nullptr;
    A.reverse = 0;
    if (ntimes >= 2) {
        double tt[2];
        cudaStream_t st = gx::as_stream(stream);
        GX_CUDA_TRY(cudaMemcpyAsync(&tt[0], t, sizeof(double), cudaMemcpyDeviceToHost, st));
        GX_CUDA_TRY(cudaMemcpyAsync(&tt[1], t + ntimes - 1, sizeof(double), cudaMemcpyDeviceToHost, st));
        GX_CUDA_TRY(cudaStreamSynchronize(st));
        A.reverse = tt[1] < tt[0] ? 1 : 0;
    }
    const unsigned grid = (unsigned)((n + 127) / 128);
    gx::orbit_extrema_kernel<<<grid, 128, 0, gx::as_stream(stream)>>>(A);
    return gx::check_launch("orbit_extrema");
}
