// gx_mlp_infer.cu -- surrogate force on BF16 tensor cores, and the FP32
// leapfrog that integrates orbits in it.
//
// One CTA (8 warps) owns a tile of 64 positions.  For the tile it runs the
// network forward (layer 1 in FP32 on the CUDA cores, layers 2-4 as 64x256x256
// BF16 MMAs with FP32 accumulation) and the input-gradient backward pass
// (three more 64x256x256 MMAs against the transposed weights), then the
// chain rule through the input map (gx_mlp.cuh) gives grad Phi.  Layout:
//   * activations / deltas: BF16 [64][256] in shared memory, double-buffered
//     (rows padded by 16 bytes so ldmatrix is conflict-free);
//   * weights: BF16 [256][256] in global memory (L2-resident, 768 KB for the
//     six matrices W2, W3, W4, W4^T, W3^T, W2^T), staged per GEMM in four
//     64-wide K slabs, double-buffered with cp.async;
//   * silu'(z_l) for the backward pass stays in registers (FP16 pairs), in the
//     MMA accumulator layout, so it never leaves the SM;
//   * y (the value) and G = dy/dxh are reduced from the accumulators.
// Warp tiling: 2 (rows) x 4 (columns) warps, 32 x 64 outputs per warp,
// mma.sync.m16n8k16 (2 x 8 tiles per k16 step).
//
// Orbits (the integrating form): threads 0..63 own one orbit each, carried as
// FP32 (hi, lo) Kahan pairs like gx_batch.cu; every step: drift, surrogate
// force for the tile, kick.  Positions outside the trained radius range use the
// analytic SCF force in FP32 instead (per-orbit fallback).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <atomic>

#include "gx_host.h"
#include "gx_mlp.cuh"
#include "gx_mlp_map.cuh"

namespace gx {
namespace mlpi {

using namespace gx::mlp;

constexpr int TM = 64;                 // positions per CTA
constexpr int NT = 256;                // threads per CTA
constexpr int AST = H + 8;             // activation row stride (bf16 elements): 528 bytes
constexpr int KS = 64;                 // K slab
constexpr int WST = KS + 8;            // weight slab row stride (bf16): 144 bytes
constexpr int SMEM_A = 2 * 2 * TM * AST * 2;  // two activation buffers, each a hi and a lo part
constexpr int SMEM_W = 2 * H * WST * 2;      // two weight slabs
constexpr int SMEM_MISC = TM * 8 * 4 + 4 * TM * 4 * 4 + TM * 16 + TM * 3 * 4 + 16;
constexpr int SMEM_BYTES = SMEM_A + SMEM_W + SMEM_MISC;


__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float *c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;"); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;"); }

// Stage K slab `s` (columns s*64 .. s*64+63) of a [256][256] bf16 matrix into ws.
__device__ __forceinline__ void load_slab(__nv_bfloat16 *ws, const __nv_bfloat16 *Wg, int s) {
    // 256 rows x 64 bf16 = 256 x 128 bytes = 2048 chunks of 16 bytes, 8 per thread
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int chunk = threadIdx.x + i * NT;
        const int row = chunk >> 3, c16 = chunk & 7;
        cp_async16(ws + row * WST + c16 * 8, Wg + (size_t)row * H + s * KS + c16 * 8);
    }
    cp_commit();
}

// acc[2][8][4] = A(64x256, smem) x W^T where W (global [256 n][256 k]) is the
// B operand (k contiguous per output n).  A is held as a BF16 pair hi + lo
// (lo = the rounding remainder of hi); SPLIT = 2 multiplies both parts
// (activation precision ~2^-17), SPLIT = 1 only hi.  The first slab of W must
// already be in flight in slab buffer 0.
template <int SPLIT>
__device__ __forceinline__ void gemm_tile(float (&acc)[2][8][4], const __nv_bfloat16 *As,
                                          __nv_bfloat16 *Ws, const __nv_bfloat16 *Wg) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = warp >> 2, wn = warp & 3;
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 8; j++)
#pragma unroll
            for (int k = 0; k < 4; k++) acc[i][j][k] = 0.f;
    for (int s = 0; s < H / KS; s++) {
        if (s + 1 < H / KS) {
            load_slab(Ws + ((s + 1) & 1) * H * WST, Wg, s + 1);
            cp_wait1();
        } else {
            cp_wait0();
        }
        __syncthreads();
        const __nv_bfloat16 *wsb = Ws + (s & 1) * H * WST;
#pragma unroll
        for (int kk = 0; kk < KS; kk += 16) {
            uint32_t a[SPLIT][2][4];
#pragma unroll
            for (int p = 0; p < SPLIT; p++)
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    const int row = wm * 32 + i * 16 + (lane & 15);
                    const int col = s * KS + kk + (lane >> 4) * 8;
                    ldsm_x4(smem_u32(As + p * TM * AST + row * AST + col), a[p][i][0], a[p][i][1], a[p][i][2],
                            a[p][i][3]);
                }
#pragma unroll
            for (int j = 0; j < 8; j += 2) {
                // two n-tiles (16 outputs) x k16 from the slab: matrices (n0..7,k0..7), (n0..7,k8..15),
                // (n8..15,k0..7), (n8..15,k8..15)
                const int n = wn * 64 + j * 8 + (lane & 7) + ((lane >> 4) << 3);
                const int k = kk + ((lane >> 3) & 1) * 8;
                uint32_t b0, b1, b2, b3;
                ldsm_x4(smem_u32(wsb + n * WST + k), b0, b1, b2, b3);
#pragma unroll
                for (int p = 0; p < SPLIT; p++)
#pragma unroll
                    for (int i = 0; i < 2; i++) {
                        mma_bf16(acc[i][j], a[p][i][0], a[p][i][1], a[p][i][2], a[p][i][3], b0, b1);
                        mma_bf16(acc[i][j + 1], a[p][i][0], a[p][i][1], a[p][i][2], a[p][i][3], b2, b3);
                    }
            }
        }
        __syncthreads();
    }
}

// store v (two consecutive columns) as hi + lo BF16 parts
__device__ __forceinline__ void store_split(__nv_bfloat16 *buf, int r, int c, float v0, float v1) {
    const __nv_bfloat162 hi = __floats2bfloat162_rn(v0, v1);
    const float2 hf = __bfloat1622float2(hi);
    *reinterpret_cast<__nv_bfloat162 *>(buf + r * AST + c) = hi;
    *reinterpret_cast<__nv_bfloat162 *>(buf + TM * AST + r * AST + c) = __floats2bfloat162_rn(v0 - hf.x, v1 - hf.y);
}

// Accumulator element (i, j, k) of this thread -> (row, col) of the 64x256 tile.
__device__ __forceinline__ int acc_row(int i, int k) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    return (warp >> 2) * 32 + i * 16 + (lane >> 2) + ((k >> 1) << 3);
}
__device__ __forceinline__ int acc_col(int j, int k) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    return (warp & 3) * 64 + j * 8 + ((lane & 3) << 1) + (k & 1);
}

// Sum over the columns of a per-thread partial (row-indexed by (i, k>>1)) into
// red[4 col-warps][64 rows]; the caller sums the 4 column-warps.
__device__ __forceinline__ void row_reduce(float (&part)[2][2], float *red) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float v = part[i][h];
            v += __shfl_xor_sync(0xffffffffu, v, 1);
            v += __shfl_xor_sync(0xffffffffu, v, 2);
            if ((lane & 3) == 0) red[(warp & 3) * TM + (warp >> 2) * 32 + i * 16 + (lane >> 2) + h * 8] = v;
        }
}

// One surrogate evaluation for the tile whose inputs xh[64][3] are in smem.
// Outputs: yv[64] (network value) and G[64][3] (dy/dxh) in smem.
template <int SPLIT>
__device__ __forceinline__ void tile_eval(const float *__restrict__ P, const __nv_bfloat16 *__restrict__ Wb, char *smem,
                          const float *xh, float *yv, float *G) {
    __nv_bfloat16 *Abuf = reinterpret_cast<__nv_bfloat16 *>(smem);
    __nv_bfloat16 *Ws = reinterpret_cast<__nv_bfloat16 *>(smem + SMEM_A);
    float *red = reinterpret_cast<float *>(smem + SMEM_A + SMEM_W + TM * 8 * 4);  // [4][4][64]
    float acc[2][8][4];
    __half2 sp[4][2][8][2];  // silu'(z_l) for l = 1..4 (index l-1), accumulator layout
    const __nv_bfloat16 *Wfwd[3] = {Wb, Wb + H * H, Wb + 2 * H * H};           // W2, W3, W4
    const __nv_bfloat16 *Wbwd[3] = {Wb + 3 * H * H, Wb + 4 * H * H, Wb + 5 * H * H};  // W4^T, W3^T, W2^T

    // prefetch the first slab of W2 while layer 1 runs on the CUDA cores
    load_slab(Ws, Wfwd[0], 0);

    // layer 1 (K = 3, FP32) directly in the accumulator layout
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 8; j++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                float s1v[2];
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int k = h * 2 + e;
                    const int r = acc_row(i, k), c = acc_col(j, k);
                    const float z = P[OFF_W1 + c * 3 + 0] * xh[r * 3 + 0] + P[OFF_W1 + c * 3 + 1] * xh[r * 3 + 1] +
                                    P[OFF_W1 + c * 3 + 2] * xh[r * 3 + 2] + P[OFF_B1 + c];
                    float a, s1, s2;
                    silu3(z, a, s1, s2);
                    (void)s2;
                    acc[i][j][k] = a;
                    s1v[e] = s1;
                }
                sp[0][i][j][h] = __floats2half2_rn(s1v[0], s1v[1]);
            }
    // write a1 (bf16 hi + lo) into activation buffer 0
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 8; j++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int r = acc_row(i, h * 2), c = acc_col(j, h * 2);
                store_split(Abuf, r, c, acc[i][j][h * 2], acc[i][j][h * 2 + 1]);
            }
    __syncthreads();

    // layers 2..4
    int cur = 0;
#pragma unroll
    for (int l = 2; l <= 4; l++) {
        gemm_tile<SPLIT>(acc, Abuf + cur * 2 * TM * AST, Ws, Wfwd[l - 2]);
        if (l < 4) load_slab(Ws, Wfwd[l - 1], 0);
        const float *b = P + off_b(l);
        __nv_bfloat16 *nxt = Abuf + (cur ^ 1) * 2 * TM * AST;
        float ypart[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 8; j++)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    float av[2], s1v[2];
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const int k = h * 2 + e;
                        const int c = acc_col(j, k);
                        float a, s1, s2;
                        silu3(acc[i][j][k] + b[c], a, s1, s2);
                        (void)s2;
                        av[e] = a;
                        s1v[e] = s1;
                        if (l == 4) ypart[i][h] += a * P[OFF_W5 + c];
                    }
                    sp[l - 1][i][j][h] = __floats2half2_rn(s1v[0], s1v[1]);
                    if (l == 4) {
                        // backward seed: delta_4 = w5 * silu'(z4)
                        const int c = acc_col(j, h * 2);
                        av[0] = P[OFF_W5 + c] * s1v[0];
                        av[1] = P[OFF_W5 + c + 1] * s1v[1];
                    }
                    const int r = acc_row(i, h * 2), c = acc_col(j, h * 2);
                    store_split(nxt, r, c, av[0], av[1]);
                }
        if (l == 4) row_reduce(ypart, red);
        cur ^= 1;
        __syncthreads();
    }
    if (threadIdx.x < TM) {
        const int r = threadIdx.x;
        yv[r] = red[r] + red[TM + r] + red[2 * TM + r] + red[3 * TM + r] + P[OFF_B5];
    }

    // backward: u_l = delta_{l+1} W_{l+1}, delta_l = u_l * silu'(z_l), l = 3, 2, 1
    load_slab(Ws, Wbwd[0], 0);
#pragma unroll
    for (int t = 0; t < 3; t++) {
        const int l = 3 - t;  // layer whose silu' multiplies
        gemm_tile<SPLIT>(acc, Abuf + cur * 2 * TM * AST, Ws, Wbwd[t]);
        if (t < 2) load_slab(Ws, Wbwd[t + 1], 0);
        __nv_bfloat16 *nxt = Abuf + (cur ^ 1) * 2 * TM * AST;
        float gpart[3][2][2] = {};
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 8; j++)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const float2 s = __half22float2(sp[l - 1][i][j][h]);
                    const float d0 = acc[i][j][h * 2] * s.x, d1 = acc[i][j][h * 2 + 1] * s.y;
                    if (l > 1) {
                        const int r = acc_row(i, h * 2), c = acc_col(j, h * 2);
                        store_split(nxt, r, c, d0, d1);
                    } else {
                        const int c = acc_col(j, h * 2);
#pragma unroll
                        for (int q = 0; q < 3; q++)
                            gpart[q][i][h] += d0 * P[OFF_W1 + c * 3 + q] + d1 * P[OFF_W1 + (c + 1) * 3 + q];
                    }
                }
        if (l == 1) {
#pragma unroll
            for (int q = 0; q < 3; q++) row_reduce(gpart[q], red + (q + 1) * 4 * TM);
        }
        cur ^= 1;
        __syncthreads();
    }
    if (threadIdx.x < TM) {
        const int r = threadIdx.x;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const float *rq = red + (q + 1) * 4 * TM;
            G[r * 3 + q] = rq[r] + rq[TM + r] + rq[2 * TM + r] + rq[3 * TM + r];
        }
    }
    __syncthreads();
}

// Points of the tile outside [r_min, r_max]: each warp computes the analytic
// force of every 8th listed point; results land in fb[64][3].  Uses the
// caller's smem list of (row, x, y, z) and count; ends with __syncthreads.
__device__ __forceinline__ void tile_fallback(const InferArgs &A, const int *cnt, const float4 *list, float *fb) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nfb = *cnt;
    for (int e = warp; e < nfb; e += NT / 32) {
        const float4 pt = list[e];
        const float q[3] = {pt.y, pt.z, pt.w};
        float g[3];
        scf_grad_f32_warp(A.scf, q, g);
        if (lane == 0) {
            const int row = (int)pt.x;
            fb[row * 3 + 0] = g[0];
            fb[row * 3 + 1] = g[1];
            fb[row * 3 + 2] = g[2];
        }
    }
    __syncthreads();
}

// Evaluate the surrogate force at n points (q: 3 x n SoA, float64), into
// out (3 x n, float64) and the potential (n) -- for tests and diagnostics.
template <int SPLIT>
__global__ void __launch_bounds__(NT, 1) surrogate_eval_kernel(InferArgs A, const float *__restrict__ P,
                                                                const __nv_bfloat16 *__restrict__ Wb,
                                                                const double *__restrict__ q, int64_t n,
                                                                double *__restrict__ grad, double *__restrict__ phi) {
    extern __shared__ __align__(16) char smem[];
    float *xh = reinterpret_cast<float *>(smem + SMEM_A + SMEM_W);   // [64][3]
    float *yv = xh + TM * 3;                                          // [64]
    float *G = yv + TM;                                               // [64][3]
    char *fbbase = smem + SMEM_A + SMEM_W + TM * 8 * 4 + 4 * TM * 4 * 4;
    float4 *fblist = reinterpret_cast<float4 *>(fbbase);              // [64] (row, x, y, z)
    float *fbg = reinterpret_cast<float *>(fbbase + TM * 16);         // [64][3]
    int *fbcnt = reinterpret_cast<int *>(fbbase + TM * 16 + TM * 3 * 4);
    const int64_t ntiles = (n + TM - 1) / TM;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t i = tile * TM + threadIdx.x;
        MapPt m;
        if (threadIdx.x < TM) {
            float x = 1.f, y = 0.f, z = 0.f;
            if (i < n) { x = (float)q[i]; y = (float)q[n + i]; z = (float)q[2 * n + i]; }
            m = map_point(A, x, y, z);
            xh[threadIdx.x * 3 + 0] = m.rho * m.nx;
            xh[threadIdx.x * 3 + 1] = m.rho * m.ny;
            xh[threadIdx.x * 3 + 2] = m.rho * m.nz;
        }
        if (threadIdx.x == 0) *fbcnt = 0;
        __syncthreads();
        tile_eval<SPLIT>(P, Wb, smem, xh, yv, G);
        const bool outside = threadIdx.x < TM && i < n && !(m.r >= A.r_min && m.r <= A.r_max);
        if (outside) {
            const int e = atomicAdd(fbcnt, 1);
            fblist[e] = make_float4((float)threadIdx.x, (float)q[i], (float)q[n + i], (float)q[2 * n + i]);
        }
        __syncthreads();
        tile_fallback(A, fbcnt, fblist, fbg);
        if (threadIdx.x < TM && i < n) {
            float gr[3];
            if (!outside) {
                surrogate_grad(m, yv[threadIdx.x], G + threadIdx.x * 3, gr);
            } else {
                gr[0] = fbg[threadIdx.x * 3 + 0];
                gr[1] = fbg[threadIdx.x * 3 + 1];
                gr[2] = fbg[threadIdx.x * 3 + 2];
            }
            grad[i] = gr[0];
            grad[n + i] = gr[1];
            grad[2 * n + i] = gr[2];
            if (phi) phi[i] = (double)m.phi0 + (double)m.phiH * (double)yv[threadIdx.x];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void split(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}
// compensated accumulation into (s, c), value s + c (the split's convention)
__device__ __forceinline__ void kahan(float &s, float &c, float d) {
    const float y = __fadd_rn(d, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(y, __fsub_rn(t, s));
    s = t;
}

// Leapfrog (kick-drift-kick as c_leapfrog_step, leapfrog.pyx:35-51) in the
// surrogate potential; n_steps and dt shared by all orbits; FP32 state with
// Kahan compensation; final state (6 x n, float64) and the count of force
// evaluations that used the analytic fallback.
template <int SPLIT>
__global__ void __launch_bounds__(NT, 1) surrogate_leapfrog_kernel(InferArgs A, const float *__restrict__ P,
                                                                    const __nv_bfloat16 *__restrict__ Wb,
                                                                    const double *__restrict__ w0, int64_t n,
                                                                    int64_t nsteps, float dt, int analytic,
                                                                    double *__restrict__ w_out,
                                                                    unsigned long long *__restrict__ fallbacks) {
    extern __shared__ __align__(16) char smem[];
    float *xh = reinterpret_cast<float *>(smem + SMEM_A + SMEM_W);
    float *yv = xh + TM * 3;
    float *G = yv + TM;
    char *fbbase = smem + SMEM_A + SMEM_W + TM * 8 * 4 + 4 * TM * 4 * 4;
    float4 *fblist = reinterpret_cast<float4 *>(fbbase);
    float *fbg = reinterpret_cast<float *>(fbbase + TM * 16);
    int *fbcnt = reinterpret_cast<int *>(fbbase + TM * 16 + TM * 3 * 4);
    const int64_t ntiles = (n + TM - 1) / TM;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t i = tile * TM + threadIdx.x;
        const bool own = threadIdx.x < TM && i < n;
        float xh_[3] = {1.f, 0.f, 0.f}, xl[3] = {0.f, 0.f, 0.f}, vh[3] = {0.f, 0.f, 0.f}, vl[3] = {0.f, 0.f, 0.f};
        float g[3] = {0.f, 0.f, 0.f};
        unsigned long long nfb = 0;
        if (own)
            for (int k = 0; k < 3; k++) {
                split(w0[k * n + i], xh_[k], xl[k]);
                split(w0[(3 + k) * n + i], vh[k], vl[k]);
            }
        // force at the start, then nsteps x (drift, force, kick); the first kick is a half kick
        for (int64_t step = 0; step <= nsteps; step++) {
            if (step > 0 && own)
                for (int k = 0; k < 3; k++) kahan(xh_[k], xl[k], fmaf(vh[k], dt, vl[k] * dt));
            MapPt m;
            if (threadIdx.x < TM) {
                m = map_point(A, xh_[0], xh_[1], xh_[2]);
                xh[threadIdx.x * 3 + 0] = m.rho * m.nx;
                xh[threadIdx.x * 3 + 1] = m.rho * m.ny;
                xh[threadIdx.x * 3 + 2] = m.rho * m.nz;
            }
            if (threadIdx.x == 0) *fbcnt = 0;
            __syncthreads();
            if (!analytic) tile_eval<SPLIT>(P, Wb, smem, xh, yv, G);
            const bool outside = own && (analytic || !(m.r >= A.r_min && m.r <= A.r_max));
            if (outside) {
                const int e = atomicAdd(fbcnt, 1);
                fblist[e] = make_float4((float)threadIdx.x, xh_[0], xh_[1], xh_[2]);
            }
            __syncthreads();
            tile_fallback(A, fbcnt, fblist, fbg);
            if (own) {
                if (!outside) {
                    surrogate_grad(m, yv[threadIdx.x], G + threadIdx.x * 3, g);
                } else {
                    g[0] = fbg[threadIdx.x * 3 + 0];
                    g[1] = fbg[threadIdx.x * 3 + 1];
                    g[2] = fbg[threadIdx.x * 3 + 2];
                    nfb++;
                }
                const float f = (step == 0) ? 0.5f : 1.0f;
                for (int k = 0; k < 3; k++) kahan(vh[k], vl[k], -g[k] * dt * f);
            }
        }
        if (own) {
            // undo the last half of the final kick to report v at the last step
            for (int k = 0; k < 3; k++) kahan(vh[k], vl[k], g[k] * dt * 0.5f);
            for (int k = 0; k < 3; k++) {
                w_out[k * n + i] = (double)xh_[k] + (double)xl[k];
                w_out[(3 + k) * n + i] = (double)vh[k] + (double)vl[k];
            }
            if (nfb) atomicAdd(fallbacks, nfb);
        }
        __syncthreads();
    }
}

}  // namespace mlpi
}  // namespace gx

using namespace gx::mlpi;

static int infer_args(const float *scf_params, double r_min, double r_max, double GM, double r_s, int32_t split,
                      InferArgs *A) {
    GX_CHECK_ARG(scf_params != nullptr, "NULL SCF parameters (analytic base and fallback)");
    GX_CHECK_ARG(r_min > 0 && r_max > r_min && GM > 0 && r_s > 0, "bad surrogate input map");
    GX_CHECK_ARG(split == 1 || split == 2, "split must be 1 (BF16 activations) or 2 (BF16 hi + lo)");
    A->r_min = (float)r_min;
    A->r_max = (float)r_max;
    A->rho0 = 0.1f;
    A->inv_log_ratio = (float)(1.0 / std::log(r_max / r_min));
    A->GM = (float)GM;
    A->r_s = (float)r_s;
    A->scf = scf_params;
    // the shared-memory opt-in belongs to a device's context: once per device
    static std::atomic<unsigned long long> configured{0};
    int dev = 0;
    GX_CUDA_TRY(cudaGetDevice(&dev));
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(configured.load() & bit)) {
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_eval_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM_BYTES));
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_eval_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM_BYTES));
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_leapfrog_kernel<1>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_leapfrog_kernel<2>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        configured.fetch_or(bit);
    }
    return GX_OK;
}

extern "C" int gx_surrogate_gradient(const float *params, const void *wbf16, const float *scf_params, double r_min,
                                     double r_max, double GM, double r_s, int32_t split, const double *q, int64_t n,
                                     double *grad, double *phi, int32_t grid, void *stream) {
    InferArgs A;
    int rc = infer_args(scf_params, r_min, r_max, GM, r_s, split, &A);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(params && wbf16 && q && grad && grid >= 1, "NULL array or bad grid");
    const __nv_bfloat16 *w = static_cast<const __nv_bfloat16 *>(wbf16);
    cudaStream_t st = gx::as_stream(stream);
    if (split == 2)
        surrogate_eval_kernel<2><<<grid, NT, SMEM_BYTES, st>>>(A, params, w, q, n, grad, phi);
    else
        surrogate_eval_kernel<1><<<grid, NT, SMEM_BYTES, st>>>(A, params, w, q, n, grad, phi);
    return gx::check_launch("surrogate_gradient");
}

extern "C" int gx_surrogate_leapfrog(const float *params, const void *wbf16, const float *scf_params, double r_min,
                                     double r_max, double GM, double r_s, int32_t split, int32_t analytic,
                                     const double *w0, int64_t n, int64_t n_steps, double dt, double *w_out,
                                     unsigned long long *fallbacks, int32_t grid, void *stream) {
    InferArgs A;
    int rc = infer_args(scf_params, r_min, r_max, GM, r_s, split, &A);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0 && n_steps >= 0, "n and n_steps must be >= 0");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(w0 && w_out && fallbacks && grid >= 1, "NULL array or bad grid");
    GX_CHECK_ARG(analytic || (params && wbf16), "NULL network parameters");
    const __nv_bfloat16 *w = static_cast<const __nv_bfloat16 *>(wbf16);
    cudaStream_t st = gx::as_stream(stream);
    if (split == 2)
        surrogate_leapfrog_kernel<2><<<grid, NT, SMEM_BYTES, st>>>(A, params, w, w0, n, n_steps, (float)dt,
                                                                   analytic, w_out, fallbacks);
    else
        surrogate_leapfrog_kernel<1><<<grid, NT, SMEM_BYTES, st>>>(A, params, w, w0, n, n_steps, (float)dt,
                                                                   analytic, w_out, fallbacks);
    return gx::check_launch("surrogate_leapfrog");
}

extern "C" int gx_surrogate_smem_bytes(void) { return SMEM_BYTES; }
