// gx_mlp_map.cuh -- the surrogate's input map, output chain rule and FP32
// analytic fallback, shared by the surrogate inference kernels.
#pragma once

#include <cstdint>

namespace gx {
namespace mlpi {

struct InferArgs {
    // input map / output scaling
    float r_min, r_max, rho0, inv_log_ratio;   // inv_log_ratio = 1 / ln(r_max / r_min)
    float GM, r_s;                              // Hernquist base (the S000 term)
    // analytic fallback (FP32 SCF, gala packing [G, nmax, lmax, M, r_s, S, T])
    const float *scf;                           // float copy of the packed SCF parameters
};

// Spherical (l = 0) part of the SCF expansion and its radial derivative, FP32:
//   Phi_0 = -(G M / r_s) sum_n S_n00 C_n^{3/2}(xi) / (1 + s),
//   dPhi_0/dr = (G M / r_s^2) sum_n S_n00 [(1+s)^-2 (n = 0); (1+s)^-3 ((1+s) C_n^{3/2} - 6 C_{n-1}^{5/2}) (n > 0)],
// s = r / r_s, xi = (s - 1)/(s + 1) (phi_nl and dPhi_nl/dr of bfe_helper.cpp:24-64 at l = 0).
__device__ __forceinline__ void scf_l0(const float *p, float r, float &phi0, float &dphi0) {
    const float GM = p[0] * p[3], rs = p[4];
    const int nmax = (int)p[1], lmax = (int)p[2];
    const int stride = (lmax + 1) * (lmax + 1);
    const float s = r / rs, xi = (s - 1.f) / (s + 1.f);
    const float i1 = 1.f / (1.f + s);
    float C = 1.f, Cm1 = 0.f, Cm2 = 0.f, D = 1.f, Dm1 = 0.f, Dm2 = 0.f;
    float sp = 0.f, sd = 0.f;
    for (int n = 0; n <= nmax; n++) {
        if (n == 1) { Cm1 = 1.f; C = 3.f * xi; }
        else if (n > 1) { Cm2 = Cm1; Cm1 = C; C = (2.f * xi * (n + 0.5f) * Cm1 - (n + 1.f) * Cm2) / n; }
        const int nd = n - 1;
        if (nd == 1) { Dm1 = 1.f; D = 5.f * xi; }
        else if (nd > 1) { Dm2 = Dm1; Dm1 = D; D = (2.f * xi * (nd + 1.5f) * Dm1 - (nd + 3.f) * Dm2) / nd; }
        const float Sn = p[5 + n * stride];
        sp += Sn * C;
        sd += Sn * ((n == 0) ? i1 : i1 * ((1.f + s) * C - 6.f * D) * i1);
    }
    phi0 = -GM / rs * sp * i1;
    dphi0 = GM / (rs * rs) * sd * i1;
}

// input map and chain rule (gx_mlp.cuh): Phi = Phi_0 + Phi_H y
struct MapPt {
    float r, nx, ny, nz, rho, drho, phiH, dphiH, phi0, dphi0;
};

__device__ __forceinline__ MapPt map_point(const InferArgs &A, float x, float y, float z) {
    MapPt m;
    const float r2 = x * x + y * y + z * z;
    const float ri = rsqrtf(r2);
    m.r = r2 * ri;
    m.nx = x * ri;
    m.ny = y * ri;
    m.nz = z * ri;
    m.rho = A.rho0 + (1.f - A.rho0) * __logf(m.r / A.r_min) * A.inv_log_ratio;
    m.drho = (1.f - A.rho0) * A.inv_log_ratio * ri;
    const float irs = 1.f / (m.r + A.r_s);
    m.phiH = -A.GM * irs;
    m.dphiH = A.GM * irs * irs;  // d Phi_H / dr
    scf_l0(A.scf, m.r, m.phi0, m.dphi0);
    return m;
}

// grad Phi from the network value y and input gradient g
__device__ __forceinline__ void surrogate_grad(const MapPt &m, float yv, const float *g, float *out) {
    const float ng = m.nx * g[0] + m.ny * g[1] + m.nz * g[2];
    const float a = m.rho / m.r;
    const float jx = a * (g[0] - m.nx * ng) + m.drho * m.nx * ng;
    const float jy = a * (g[1] - m.ny * ng) + m.drho * m.ny * ng;
    const float jz = a * (g[2] - m.nz * ng) + m.drho * m.nz * ng;
    const float radial = m.dphi0 + m.dphiH * yv;
    out[0] = radial * m.nx + m.phiH * jx;
    out[1] = radial * m.ny + m.phiH * jy;
    out[2] = radial * m.nz + m.phiH * jz;
}

// Analytic SCF gradient in FP32 (same series as gx_scf.cuh, gala's packing),
// computed by a whole warp for one point: lane q handles the (l, m) pairs
// q, q + 32, ... (P_l^m by its recurrence in l at fixed m, Gegenbauer terms by
// their recurrence in n); the three spherical components are warp-reduced.
// Every lane returns the gradient.
static __device__ __noinline__ void scf_grad_f32_warp(const float *p, const float *q, float *g) {
    const float SQRT_FOURPI = 3.544907701811031f, PI = 3.14159265358979f;
    const int lane = threadIdx.x & 31;
    const float G = p[0], M = p[3], r_s = p[4];
    const int nmax = (int)p[1], lmax = (int)p[2];
    const int ncoef = (nmax + 1) * (lmax + 1) * (lmax + 1);
    const float *S = p + 5, *T = p + 5 + ncoef;
    const float r = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    const float s = r / r_s, X = q[2] / r, phi = atan2f(q[1], q[0]);
    // on the z axis 1 - X^2 rounds to 0 in FP32; the series' 1/sin(theta) terms
    // have finite limits there, approached here by a floor on sin(theta)
    const float sint = fmaxf(sqrtf(fmaxf(1.f - X * X, 0.f)), 1e-6f), xi = (s - 1.f) / (s + 1.f);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    const int npairs = (lmax + 1) * (lmax + 2) / 2;
    for (int qi = lane; qi < npairs; qi += 32) {
        int l = (int)((sqrtf(8.f * qi + 1.f) - 1.f) * 0.5f);
        while ((l + 1) * (l + 2) / 2 <= qi) l++;
        while (l * (l + 1) / 2 > qi) l--;
        const int m = qi - l * (l + 1) / 2;
        // P_l^m and P_{l-1}^m (Condon-Shortley phase)
        float pmm = 1.f;
        for (int i = 1; i <= m; i++) pmm *= -(2.f * i - 1.f) * sint;
        float Plm = pmm, Pl1m = 0.f;
        if (l > m) {
            float pm2 = pmm, pm1 = X * (2.f * m + 1.f) * pmm;
            for (int ll = m + 2; ll <= l; ll++) {
                const float pl = (X * (2.f * ll - 1.f) * pm1 - (ll + m - 1.f) * pm2) / (float)(ll - m);
                pm2 = pm1;
                pm1 = pl;
            }
            Plm = pm1;
            Pl1m = pm2;
        }
        float fl = 1.f;  // (l-m)!/(l+m)!
        for (int i = l - m + 1; i <= l + m; i++) fl /= (float)i;
        const float norm = sqrtf((2 * l + 1) / (4.f * PI) * fl);
        const float Y = norm * Plm;
        const float dY = (l > 0) ? norm / sint * (l * X * Plm - (l + m) * Pl1m) : 0.f;
        float sm, cm;
        __sincosf(m * phi, &sm, &cm);
        const float a1c = 2 * l + 1.5f, a2c = 2 * l + 2.5f;
        const float psl = __powf(s, (float)l), pslm1 = __powf(s, (float)(l - 1));
        const float p1 = __powf(1.f + s, -2.f * l - 1.f), p3 = __powf(1.f + s, -3.f - 2.f * l);
        float Cm1 = 0.f, C = 1.f, Dm1 = 0.f, D = 1.f;
        for (int n = 0; n <= nmax; n++) {
            if (n == 1) { Cm1 = 1.f; C = 2.f * a1c * xi; }
            else if (n > 1) {
                const float Cn = (2.f * xi * (n + a1c - 1.f) * C - (n + 2.f * a1c - 2.f) * Cm1) / n;
                Cm1 = C;
                C = Cn;
            }
            const int nd = n - 1;
            if (nd == 1) { Dm1 = 1.f; D = 2.f * a2c * xi; }
            else if (nd > 1) {
                const float Dn = (2.f * xi * (nd + a2c - 1.f) * D - (nd + 2.f * a2c - 2.f) * Dm1) / nd;
                Dm1 = D;
                D = Dn;
            }
            const int i = m + (lmax + 1) * (l + (lmax + 1) * n);
            const float Sv = S[i], Tv = T[i];
            if (Sv == 0.f && Tv == 0.f) continue;
            const float rad = -SQRT_FOURPI * psl * p1 * C;
            const float drad = (n == 0) ? SQRT_FOURPI * pslm1 * p3 * (1 + s) * (l * (s - 1) + s)
                                        : SQRT_FOURPI * pslm1 * p3 * (-2 * (3 + 4 * l) * s * D + (1 + s) * (l * (s - 1) + s) * C);
            const float tmp = Sv * cm + Tv * sm;
            a0 += drad * Y * tmp;
            a1 += dY * rad / s * tmp;
            a2 += (float)m * Y * rad * (Tv * cm - Sv * sm) / (s * sint);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    float cphi, sphi;
    __sincosf(phi, &sphi, &cphi);
    const float f = G * M / (r_s * r_s);
    g[0] = (sint * cphi * a0 + X * cphi * a1 - sphi * a2) * f;
    g[1] = (sint * sphi * a0 + X * sphi * a1 + cphi * a2) * f;
    g[2] = (X * a0 - sint * a1) * f;
}

}  // namespace mlpi
}  // namespace gx
