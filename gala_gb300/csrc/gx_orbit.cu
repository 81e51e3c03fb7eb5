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
// keeping a sliding window of samples.  The vertex is computed in coordinates
// centred on the middle sample (s = t - t_j), the same parabola as gala's
// polyfit through the raw times but without their cancellation.
// Per orbit and kind it returns the number of extrema, their sum (in time order),
// minimum and maximum, and the first `keep` values and times.
#include <algorithm>

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
    double sum;
    long long kmin, kmax;  // order keys of the minimum and maximum (see order_key)
};

// Signed 64-bit key with the order of the doubles (for non-NaN values): min and
// max on the integer pipes instead of the FP64 pipe.
__device__ __forceinline__ long long order_key(double v) {
    const long long b = __double_as_longlong(v);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double from_key(long long k) {
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL));
}

__device__ __forceinline__ void ext_push(const ExtArgs &A, ExtAcc &acc, int kind, int64_t i, double v, double tv) {
    if (A.vals && acc.count < A.keep) {
        const int64_t o = ((int64_t)kind * A.n + i) * A.keep + acc.count;
        A.vals[o] = v;
        A.times[o] = tv;
    }
    acc.count++;
    acc.sum += v;
    const long long k = order_key(v);
    acc.kmin = min(acc.kmin, k);
    acc.kmax = max(acc.kmax, k);
}

// Vertex of the parabola through (t0, q0), (t1, q1), (t2, q2) (orbit.py:411-424),
// in coordinates centred on the middle sample, s = t - t1: with e = q - q1 and
// D = s0 s2 (s2 - s0), q = q1 + (B s + C s^2) / D where C = e2 s0 - e0 s2 and
// B = e2 s0 (s2 - s0) - C s2; the vertex is at s = -B / (2C), value
// q1 - B^2 / (4 C D).  One reciprocal instead of gala's polyfit.
__device__ __forceinline__ void vertex(double q0, double q1, double q2, double t0, double t1, double t2, double &v,
                                       double &tv) {
    const double s0 = t0 - t1, s2 = t2 - t1, w = s2 - s0;
    const double e0 = q0 - q1, e2 = q2 - q1;
    const double C = fma(e2, s0, -e0 * s2);
    const double B = fma(e2 * s0, w, -C * s2);
    const double D = s0 * s2 * w;
    const double inv = 1.0 / (2.0 * C * D);
    tv = t1 - B * D * inv;
    v = q1 - 0.5 * B * B * inv;
}

// FP64 is 1/64 of the FP32 rate on this part (and double -> float conversion
// runs on the FP64 pipe), so the scan over all samples uses neither: each
// coordinate's FP32 approximation is built from the high word of the double
// with integer operations (sign cleared, exponent rebiased, top 20 mantissa
// bits: relative error below 2^-20), and r^2 and |z| are compared in FP32 with
// a relative margin of 1e-5.  Samples that pass -- a superset of gala's
// extrema -- are staged with their two neighbours (the doubles are still in
// registers) in per-warp rings in shared memory: one for r candidates (x, y, z)
// and one for |z| candidates (z).  When a ring fills, the warp checks its
// candidates one per lane, whatever orbit they belong to (no divergence, no
// re-read from HBM): r = sqrt(x^2 + y^2 + z^2) with fused multiply-adds
// (within an ulp of astropy's hypot(hypot(x, y), z)), gala's strict
// comparisons, the vertex.  Each lane then folds in the results of its own
// orbit in time order, following a chain of slot indices built when the
// candidates were staged.  Pericentre and apocentre share the parabola of r:
// the vertex of -r is minus the vertex of r, bit for bit.
constexpr int EXT_U = 2;        // samples per chunk
constexpr int EXT_STAGES = 2;   // chunks in shared memory: one being scanned, one in flight
static_assert(EXT_U >= 2, "the window carries two samples out of each chunk");
constexpr int EXT_CAP = 64;     // ring slots per warp and kind
constexpr int EXT_WARPS = 8;    // warps per CTA (time segments per orbit group)
constexpr int EXT_THREADS = 32 * EXT_WARPS;

// |x| as an FP32 value from the high word of x (top 20 mantissa bits), clamped
// to the FP32 normal range; for the scan only.  The sign is shifted out, and the
// exponent is rebiased modulo 2^9 after the shift drops its top two bits
// (e - 896 = (e mod 512) - 384 mod 512 for e in [897, 1150]).
__device__ __forceinline__ float abs_f32_from_hi(double x) {
    unsigned h = (unsigned)__double2hiint(x) << 1;
    h = min(max(h, 897u << 21), (1150u << 21) | 0x1fffffu);
    return __uint_as_float((h << 2) - (384u << 23));
}

// Candidate kinds of the middle sample; z1nz says its exact z is not 0 (z = 0
// is never a strict maximum of |z|, which keeps orbits in the plane z = 0 cheap).
__device__ __forceinline__ int ext_flags(float r0, float r1, float r2, float a0, float a1, float a2, bool z1nz) {
    const float lo = 1.0f - 1e-5f, hi = 1.0f + 1e-5f;
    return (r1 <= fminf(r0, r2) * hi ? 1 : 0)             // pericentre candidate
           | (r1 >= fmaxf(r0, r2) * lo ? 2 : 0)           // apocentre candidate
           | (z1nz && a1 >= fmaxf(a0, a2) * lo ? 4 : 0);  // |z| maximum candidate
}

struct ExtRings {
    double r[9][EXT_CAP];  // x, y, z at (j-1, j, j+1); after the check: [0] value, [1] time
    int rj[EXT_CAP];       // centre sample; after the check: 0 none, 1 pericentre, 2 apocentre
    int rnext[EXT_CAP];    // next slot of the same orbit, -1 at the end
    double z[3][EXT_CAP];  // z at (j-1, j, j+1); after the check: [0] value, [1] time
    int zj[EXT_CAP];       // centre sample; after the check: 0 none, 1 maximum
    int znext[EXT_CAP];
};

// sqrt(u) for u >= 0 from an FP32 reciprocal-square-root seed and STEPS Newton
// (Heron) steps in FP64: relative error below 1e-13 after one step (the seed's
// ~3e-7, squared), a few ulp after two; three FP64 instructions a step instead
// of a correctly rounded square root.
template <int STEPS>
__device__ __forceinline__ double sqrt_newton(double u) {
    const unsigned hi = (unsigned)__double2hiint(u);
    if (hi < (897u << 20) || hi >= (1151u << 20)) return sqrt(u);  // outside the FP32 normal range
    const unsigned lo = (unsigned)__double2loint(u);
    const float uf = __uint_as_float(((hi - (896u << 20)) << 3) | (lo >> 29));
    const unsigned yb = __float_as_uint(rsqrtf(uf));
    // the FP32 seed as a double, and half of it, built from its bits
    const int yhi = (int)(((yb >> 23) + 896u) << 20 | ((yb >> 3) & 0xfffffu));
    const int ylo = (int)(yb << 29);
    const double y = __hiloint2double(yhi, ylo), h = __hiloint2double(yhi - (1 << 20), ylo);
    double r = u * y;
#pragma unroll
    for (int k = 0; k < STEPS; k++) r = fma(fma(-r, r, u), h, r);
    return r;
}

// The vertex of the parabola through (t_k, r_k), r_k = sqrt(u_k), as vertex()
// computes it, with the differences r_k - r_1 taken as (u_k - u_1) / (r_k + r_1):
// exact up to the rounding of u, so the square roots (from sqrt_newton) only
// need the accuracy of a ratio.  With a_k = r_k + r_1 and P = a_0 a_2 the
// centred coefficients are C' / P and B' / P (C' and B' as in vertex() with
// e_0 a_0 a_2 = (u_0 - u_1) a_2 and e_2 a_0 a_2 = (u_2 - u_1) a_0); P cancels in
// the vertex position and one reciprocal serves both outputs.
__device__ __forceinline__ void vertex_r(double u0, double u1, double u2, double t0, double t1, double t2,
                                         double &v, double &tv) {
    // r_0, r_2 enter only through the ratios; r_1 is the value's leading term
    const double r0 = sqrt_newton<1>(u0), r1 = sqrt_newton<2>(u1), r2 = sqrt_newton<1>(u2);
    const double s0 = t0 - t1, s2 = t2 - t1, w = s2 - s0;
    const double a0 = r0 + r1, a2 = r2 + r1;
    const double p0 = (u0 - u1) * a2, p2 = (u2 - u1) * a0;  // e_k a_0 a_2
    const double C = fma(p2, s0, -p0 * s2);
    const double B = fma(p2 * s0, w, -C * s2);
    const double DP = (s0 * s2 * w) * (a0 * a2);
    const double inv = 1.0 / (2.0 * C * DP);
    tv = t1 - B * DP * inv;
    v = r1 - 0.5 * B * B * inv;
}

// Non-negative doubles (and +inf) order like their bit patterns; NaN patterns
// are above that of +inf.
constexpr long long EXT_INF_BITS = 0x7ff0000000000000LL;

// Check a warp's staged candidates (one per lane, any orbit) and fold each
// lane's results into its accumulators in time order.  Out of line: it runs
// once per EXT_CAP candidates, and inlining it at every staging site would
// overflow the instruction cache of the scan loop.  gala's strict comparisons
// (orbit.py:405, argrelmax) are made on r^2 and |z| as integers (FP64
// comparisons cost a slot of the FP64 pipe); a NaN sample is never an extremum
// and has none next to it, as in argrelmax.
__device__ __noinline__ void ext_flush(const ExtArgs &A, ExtRings &R, ExtAcc *acc, int64_t i, int lane, int nr,
                                       int nz, int rhead, int zhead) {
    const int nt = (int)A.ntimes;
    auto tval = [&](int j) { return __ldg(A.t + (A.reverse ? nt - 1 - j : j)); };
    __syncwarp();
    for (int s = lane; s < nr; s += 32) {
        double u[3];
        long long ku[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            u[k] = fma(R.r[k][s], R.r[k][s], fma(R.r[3 + k][s], R.r[3 + k][s], R.r[6 + k][s] * R.r[6 + k][s]));
            ku[k] = __double_as_longlong(u[k]);
        }
        const int j = R.rj[s];
        const bool num = ku[0] <= EXT_INF_BITS && ku[1] <= EXT_INF_BITS && ku[2] <= EXT_INF_BITS;
        const bool peri = num && ku[1] < ku[0] && ku[1] < ku[2];
        const bool apo = num && ku[1] > ku[0] && ku[1] > ku[2];
        int kind = 0;
        if (peri || apo) {
            kind = peri ? 1 : 2;
            const double t1 = tval(j);
            double v, tv = t1;
            if (A.approximate)
                v = sqrt(u[1]);
            else
                vertex_r(u[0], u[1], u[2], tval(j - 1), t1, tval(j + 1), v, tv);
            R.r[0][s] = v;
            R.r[1][s] = tv;
        }
        R.rj[s] = kind;
    }
    for (int s = lane; s < nz; s += 32) {
        const long long k0 = __double_as_longlong(R.z[0][s]) & 0x7fffffffffffffffLL;
        const long long k1 = __double_as_longlong(R.z[1][s]) & 0x7fffffffffffffffLL;
        const long long k2 = __double_as_longlong(R.z[2][s]) & 0x7fffffffffffffffLL;
        const int j = R.zj[s];
        int kind = 0;
        if (k0 <= EXT_INF_BITS && k1 <= EXT_INF_BITS && k2 <= EXT_INF_BITS && k1 > k0 && k1 > k2) {
            kind = 1;
            const double a1 = __longlong_as_double(k1);
            const double t1 = tval(j);
            double v = a1, tv = t1;
            if (!A.approximate)
                vertex(__longlong_as_double(k0), a1, __longlong_as_double(k2), tval(j - 1), t1, tval(j + 1), v,
                       tv);
            R.z[0][s] = v;
            R.z[1][s] = tv;
        }
        R.zj[s] = kind;
    }
    __syncwarp();
    int cr = rhead, cz = zhead;
    while (__any_sync(0xffffffffu, cr >= 0)) {
        if (cr >= 0) {
            const int kind = R.rj[cr];
            if (kind == 1) ext_push(A, acc[0], 0, i, R.r[0][cr], R.r[1][cr]);
            else if (kind == 2) ext_push(A, acc[1], 1, i, R.r[0][cr], R.r[1][cr]);
            cr = R.rnext[cr];
        }
    }
    while (__any_sync(0xffffffffu, cz >= 0)) {
        if (cz >= 0) {
            if (R.zj[cz]) ext_push(A, acc[2], 2, i, R.z[0][cz], R.z[1][cz]);
            cz = R.znext[cz];
        }
    }
    __syncwarp();
}

// Per warp: the chunk buffers (x, y, z of EXT_U samples of the warp's 32
// orbits, filled with cp.async while the previous chunk is scanned) and the
// candidate rings.
struct ExtWarp {
    double buf[EXT_STAGES][3][EXT_U][32];
    ExtRings rings;
};

// A warp's statistics of one time segment, laid over its ring storage once the
// segment's last candidates are folded in.
struct ExtPart {
    int32_t count[3][32];
    double sum[3][32];
    long long kmin[3][32], kmax[3][32];
};
static_assert(sizeof(ExtPart) <= sizeof(double) * 9 * EXT_CAP, "partials must fit in the r ring");

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Scan samples [js, je) of orbit ii (scan order) and fold the extrema centred
// in [clo, chi) into acc.  All lanes of the warp call it together.
__device__ __forceinline__ void ext_scan(const ExtArgs &A, ExtWarp &Wp, ExtAcc *acc, int64_t ii, bool live, int js,
                                         int je, int clo, int chi) {
    ExtRings &R = Wp.rings;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int64_t nt = A.ntimes;
    // sample j of the scan is row (reverse ? nt-1-j : j); rows are n doubles apart
    const int64_t step = A.reverse ? -A.n : A.n;
    const double *p0 = A.w + ii + (A.reverse ? (nt - 1) * A.n : 0) + js * step;
    const int64_t plane = nt * A.n;  // x -> y -> z
    int nr = 0, nz = 0;                                  // ring fill (warp-uniform)
    int rhead = -1, rlast = -1, zhead = -1, zlast = -1;  // this lane's chains

    // stage the candidates centred on sample jc (samples jc-1, jc, jc+1)
    auto stage = [&](int jc, int f, double x0, double x1, double x2, double y0, double y1, double y2, double z0,
                     double z1, double z2) {
        const bool ok = live && jc >= clo && jc < chi;
        const bool vr = ok && (f & 3), vz = ok && (f & 4);
        const unsigned br = __ballot_sync(0xffffffffu, vr), bz = __ballot_sync(0xffffffffu, vz);
        if ((br | bz) == 0u) return;
        if (nr + __popc(br) > EXT_CAP || nz + __popc(bz) > EXT_CAP) {
            ext_flush(A, R, acc, ii, lane, nr, nz, rhead, zhead);
            nr = nz = 0;
            rhead = rlast = zhead = zlast = -1;
        }
        if (vr) {
            const int s = nr + __popc(br & below);
            R.r[0][s] = x0; R.r[1][s] = x1; R.r[2][s] = x2;
            R.r[3][s] = y0; R.r[4][s] = y1; R.r[5][s] = y2;
            R.r[6][s] = z0; R.r[7][s] = z1; R.r[8][s] = z2;
            R.rj[s] = jc;
            R.rnext[s] = -1;
            if (rlast >= 0) R.rnext[rlast] = s; else rhead = s;
            rlast = s;
        }
        if (vz) {
            const int s = nz + __popc(bz & below);
            R.z[0][s] = z0; R.z[1][s] = z1; R.z[2][s] = z2;
            R.zj[s] = jc;
            R.znext[s] = -1;
            if (zlast >= 0) R.znext[zlast] = s; else zhead = s;
            zlast = s;
        }
        nr += __popc(br);
        nz += __popc(bz);
    };
    // chunk k (samples js + k EXT_U ...) -> buffer k % EXT_STAGES, each lane
    // copying its own orbit's doubles
    const int nchunk = (je - js) / EXT_U;
    auto issue = [&](int k) {
        // chunk k starts (k EXT_U) rows after sample js
        const double *q = p0 + (int64_t)(k * EXT_U) * step;
        double(*b)[EXT_U][32] = Wp.buf[k % EXT_STAGES];
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int u = 0; u < EXT_U; u++) cp_async8(&b[c][u][lane], q + c * plane + u * step);
    };

    // window positions 0, 1: the two samples before the chunk (registers);
    // positions 2 .. EXT_U+1: the chunk (shared memory).  At the start they
    // are placeholders: the centres next to them lie before clo.
    double cx0 = 0., cx1 = 0., cy0 = 0., cy1 = 0., cz0 = 0., cz1 = 0.;
    float wr[EXT_U + 2], wa[EXT_U + 2];
    bool znz[EXT_U + 2];
    wr[0] = wr[1] = wa[0] = wa[1] = 0.f;
    znz[0] = znz[1] = false;
    if (nchunk > 0) issue(0);
    cp_async_commit();
    for (int k = 0; k < nchunk; k++) {
        if (k + 1 < nchunk) issue(k + 1);
        cp_async_commit();
        cp_async_wait_prev();  // this lane's copies of chunk k have landed
        const double(*b)[EXT_U][32] = Wp.buf[k % EXT_STAGES];
#pragma unroll
        for (int u = 0; u < EXT_U; u++) {
            const double z = b[2][u][lane];
            const float fx = abs_f32_from_hi(b[0][u][lane]), fy = abs_f32_from_hi(b[1][u][lane]);
            const float fz = abs_f32_from_hi(z);
            wr[u + 2] = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
            wa[u + 2] = fz;
            znz[u + 2] = ((__double2hiint(z) << 1) | __double2loint(z)) != 0;
        }
        const int j0 = js + k * EXT_U;
#pragma unroll
        for (int c = 1; c <= EXT_U; c++) {
            const int f = ext_flags(wr[c - 1], wr[c], wr[c + 1], wa[c - 1], wa[c], wa[c + 1], znz[c]);
            // doubles at window positions c-1, c, c+1 (p < 2: registers, else the chunk)
#define GX_WIN(coord, p, r0, r1) ((p) == 0 ? (r0) : (p) == 1 ? (r1) : b[coord][(p)-2][lane])
            stage(j0 + c - 2, f, GX_WIN(0, c - 1, cx0, cx1), GX_WIN(0, c, cx0, cx1), b[0][c - 1][lane],
                  GX_WIN(1, c - 1, cy0, cy1), GX_WIN(1, c, cy0, cy1), b[1][c - 1][lane],
                  GX_WIN(2, c - 1, cz0, cz1), GX_WIN(2, c, cz0, cz1), b[2][c - 1][lane]);
#undef GX_WIN
        }
        cx0 = b[0][EXT_U - 2][lane]; cx1 = b[0][EXT_U - 1][lane];
        cy0 = b[1][EXT_U - 2][lane]; cy1 = b[1][EXT_U - 1][lane];
        cz0 = b[2][EXT_U - 2][lane]; cz1 = b[2][EXT_U - 1][lane];
        wr[0] = wr[EXT_U]; wr[1] = wr[EXT_U + 1];
        wa[0] = wa[EXT_U]; wa[1] = wa[EXT_U + 1];
        znz[0] = znz[EXT_U]; znz[1] = znz[EXT_U + 1];
    }
    // remaining samples one at a time
    for (int j0 = js + nchunk * EXT_U; j0 < je; j0++) {
        const double *q = p0 + (int64_t)(j0 - js) * step;
        const double x = __ldcs(q), y = __ldcs(q + plane), z = __ldcs(q + 2 * plane);
        const float fx = abs_f32_from_hi(x), fy = abs_f32_from_hi(y), fz = abs_f32_from_hi(z);
        wr[2] = fmaf(fx, fx, fmaf(fy, fy, fz * fz));
        wa[2] = fz;
        stage(j0 - 1, ext_flags(wr[0], wr[1], wr[2], wa[0], wa[1], wa[2], znz[1]), cx0, cx1, x, cy0, cy1, y, cz0,
              cz1, z);
        znz[1] = ((__double2hiint(z) << 1) | __double2loint(z)) != 0;
        cx0 = cx1; cy0 = cy1; cz0 = cz1; wr[0] = wr[1]; wa[0] = wa[1];
        cx1 = x; cy1 = y; cz1 = z; wr[1] = wr[2]; wa[1] = wa[2];
    }
    ext_flush(A, R, acc, ii, lane, nr, nz, rhead, zhead);
}

__device__ __forceinline__ void ext_reset(ExtAcc *acc) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        acc[k].count = 0;
        acc[k].sum = 0.;
        acc[k].kmin = 0x7fffffffffffffffLL;
        acc[k].kmax = -0x7fffffffffffffffLL - 1;
    }
}

__device__ __forceinline__ void ext_store(const ExtArgs &A, int k, int64_t i, int32_t count, double sum,
                                          long long kmin, long long kmax) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    A.count[k * A.n + i] = count;
    A.sum[k * A.n + i] = sum;
    A.vmin[k * A.n + i] = count ? from_key(kmin) : nan;
    A.vmax[k * A.n + i] = count ? from_key(kmax) : nan;
}

// Persistent CTAs of EXT_WARPS warps over groups of 32 orbits (one orbit per
// lane).  Statistics only (keep = 0): the CTA's warps split one group's time
// range into EXT_WARPS segments and the partial statistics are merged in
// shared memory in segment (time) order, so every SM stays busy to the end
// whatever N is.  With keep > 0 (the first extrema themselves, in time order)
// each warp scans a whole group.
__global__ void __launch_bounds__(EXT_THREADS, 2) orbit_extrema_kernel(const ExtArgs A) {
    extern __shared__ __align__(16) unsigned char ext_smem[];
    ExtWarp *warps = reinterpret_cast<ExtWarp *>(ext_smem);  // [EXT_WARPS]
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    ExtWarp &Wp = warps[wid];
    const int nt = (int)A.ntimes;
    const int64_t ngroups = (A.n + 31) / 32;
    const bool split = A.vals == nullptr;
    const int64_t units = split ? ngroups : (ngroups + EXT_WARPS - 1) / EXT_WARPS;
    ExtAcc acc[3];
    for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
        const int64_t g = split ? u : u * EXT_WARPS + wid;
        const int64_t i = g * 32 + lane;
        const bool live = g < ngroups && i < A.n;
        const int64_t ii = live ? i : 0;
        ext_reset(acc);
        if (split) {
            const int seg = (nt + EXT_WARPS - 1) / EXT_WARPS;
            const int lo = wid * seg, hi = min(nt, lo + seg);
            if (lo < hi) ext_scan(A, Wp, acc, ii, live, max(lo - 1, 0), min(hi + 1, nt), max(lo, 1), min(hi, nt - 1));
            ExtPart &P = *reinterpret_cast<ExtPart *>(&Wp.rings.r[0][0]);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                P.count[k][lane] = acc[k].count;
                P.sum[k][lane] = acc[k].sum;
                P.kmin[k][lane] = acc[k].kmin;
                P.kmax[k][lane] = acc[k].kmax;
            }
            __syncthreads();
            if (threadIdx.x < 96) {
                const int k = threadIdx.x >> 5;
                const int64_t io = g * 32 + lane;
                int32_t count = 0;
                double sum = 0.;
                long long kmin = 0x7fffffffffffffffLL, kmax = -0x7fffffffffffffffLL - 1;
                for (int w = 0; w < EXT_WARPS; w++) {
                    const ExtPart &Q = *reinterpret_cast<const ExtPart *>(&warps[w].rings.r[0][0]);
                    if (Q.count[k][lane] == 0) continue;
                    count += Q.count[k][lane];
                    sum += Q.sum[k][lane];
                    kmin = min(kmin, Q.kmin[k][lane]);
                    kmax = max(kmax, Q.kmax[k][lane]);
                }
                if (io < A.n) ext_store(A, k, io, count, sum, kmin, kmax);
            }
            __syncthreads();
        } else if (g < ngroups) {
            ext_scan(A, Wp, acc, ii, live, 0, nt, 1, nt - 1);
            if (live)
#pragma unroll
                for (int k = 0; k < 3; k++) ext_store(A, k, i, acc[k].count, acc[k].sum, acc[k].kmin, acc[k].kmax);
        }
    }
}

}  // namespace gx

extern "C" int gx_orbit_extrema(const double *w, const double *t, int64_t ntimes, int64_t n, int32_t approximate,
                                int32_t keep, int32_t *count, double *sum, double *vmin, double *vmax, double *vals,
                                double *times, void *stream) {
    GX_CHECK_ARG(ntimes >= 0 && n >= 0, "negative size");
    GX_CHECK_ARG(keep >= 0, "keep must be >= 0");
    GX_CHECK_ARG(ntimes < ((int64_t)1 << 31), "ntimes must be below 2^31");
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
    int dev = 0, sms = 0, per_sm = 0;
    const size_t smem = sizeof(gx::ExtWarp) * gx::EXT_WARPS;
    GX_CUDA_TRY(cudaGetDevice(&dev));
    GX_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GX_CUDA_TRY(
        cudaFuncSetAttribute(gx::orbit_extrema_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    GX_CUDA_TRY(
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gx::orbit_extrema_kernel, gx::EXT_THREADS, smem));
    const int64_t groups = (n + 31) / 32;
    const int64_t units = keep ? (groups + gx::EXT_WARPS - 1) / gx::EXT_WARPS : groups;
    const unsigned grid = (unsigned)std::min<int64_t>(units, (int64_t)sms * std::max(per_sm, 1));
    gx::orbit_extrema_kernel<<<grid, gx::EXT_THREADS, smem, gx::as_stream(stream)>>>(A);
    return gx::check_launch("orbit_extrema");
}
