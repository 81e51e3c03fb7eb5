// gx_mlp_tc.cu -- surrogate force on the 5th-generation tensor cores
// (tcgen05.mma with the accumulator in tensor memory), and the FP32 leapfrog
// that integrates orbits in it.
//
// One CTA (16 warps) per SM, persistent over tiles of 128 positions.  Row r of
// the tile is TMEM lane r; warp w reads lane quadrant w % 4 (the lanes a warp may
// access) and column slice w / 4 (64 columns), so each row's epilogue is shared
// by four threads and every scheduler has four warps to hide latency.  Per tile:
//   * layer 1 (3 -> 256) in FP32 on the CUDA cores;
//   * layers 2-4 and the three input-gradient GEMMs are 128 x 256 x 256
//     tcgen05.mma (kind::f16, FP32 accumulation into TMEM columns 0..255) with
//     BF16 operands (the A operand -- activations / deltas -- optionally as
//     BF16 hi + lo parts) or FP16 operands, both K-major in shared memory with
//     the 128-byte swizzle;
//   * the weights (W2, W3, W4, W4^T, W3^T, W2^T) are kept in global memory as
//     pre-swizzled 32 KB images of 64-wide K chunks (768 KB, L2-resident) and
//     streamed into two shared buffers with cp.async.bulk, one chunk ahead of
//     the MMAs (mbarrier complete_tx); tcgen05.commit frees a buffer when the
//     MMAs that read it have finished;
//   * epilogues read the accumulator with tcgen05.ld (thread t reads its row),
//     apply bias and SiLU and write the next A operand; silu'(z2), silu'(z3) are
//     kept in TMEM as FP16 pairs (columns 256..511) for the backward pass,
//     silu'(z1) is recomputed from the three inputs.
// One thread (thread 0) issues the MMAs and the weight copies.  Every wait on
// an mbarrier is bounded; on timeout the kernel records an error, stops issuing
// work, waits (bounded) for its copies in flight, frees TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <atomic>

#include "gx_host.h"
#include "gx_mlp.cuh"
#include "gx_mlp_map.cuh"
#include "gx_scf.cuh"

namespace gx {
namespace mltc {

using namespace gx::mlp;
using gx::mlpi::InferArgs;
using gx::mlpi::MapPt;
using gx::mlpi::map_point;
using gx::mlpi::surrogate_grad;

constexpr int TM = 128;                 // rows per tile (= TMEM lanes)
constexpr int NT = 512;                 // threads per CTA: 4 column slices x 4 lane quadrants
constexpr int SLICE = 64;               // columns handled by one thread of a row
constexpr int KCH = H / 64;             // 64-wide K chunks of a 256-wide operand
constexpr int A_CHUNK = TM * 128;       // bytes of one K chunk of A (128 rows x 128 B)
constexpr int A_PART = KCH * A_CHUNK;   // 64 KB: one part (hi or lo) of A
constexpr int W_CHUNK = H * 128;        // 32 KB: one K chunk of a 256 x 256 weight matrix
constexpr int NGEMM = 6;
constexpr int NCHUNK = NGEMM * KCH;     // weight chunks per tile
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t COL_SP2 = 256, COL_SP3 = 384;
constexpr long WAIT_LIMIT = 1L << 26;   // polls of an mbarrier before giving up

struct Shared {
    uint64_t wfull[2];
    uint64_t wempty[2];
    uint64_t mma_done;
    uint32_t tmem_base;
    int abort;
    int fbcnt;
    int pad;
    float4 fblist[TM];
    float fbg[TM * 3];
    float xh[TM * 3];        // network inputs of the tile
    float part[4][TM * 4];   // per-slice partial sums: y and G (4 per row)
    float4 w1b1[H];          // layer 1: {W1[j][0], W1[j][1], W1[j][2], b1[j]}
    float bias[3][H];        // b2, b3, b4
    float w5[H];
};
constexpr int SMEM_BYTES = 1024 + 2 * A_PART + 2 * W_CHUNK + (int)sizeof(Shared);

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: K-major operand with the 128-byte swizzle,
// 8-row groups 1024 bytes apart (tcgen05 descriptor version 1).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Operand modes (the `split` argument): 1 = BF16 operands, 2 = BF16 weights
// with the activations as BF16 hi + lo parts (two MMAs per K step), 3 = FP16
// operands (11-bit mantissa for weights and activations, one MMA per K step).
template <int SPLIT>
constexpr int NPART = SPLIT == 2 ? 2 : 1;

// Instruction descriptor (kind::f16): FP32 accumulator, A and B of the same
// type -- BF16 (type code 1) or FP16 (code 0) -- both K-major, M = 128, N = 256.
template <int SPLIT>
constexpr uint32_t IDESC = (1u << 4) | ((SPLIT == 3 ? 0u : 1u) << 7) | ((SPLIT == 3 ? 0u : 1u) << 10) |
                           ((uint32_t)(H >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count));
}

__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity) {
    const uint32_t a = su32(b);
    for (long it = 0; it < WAIT_LIMIT; it++) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(su32(dst)),
        "l"(src), "r"(bytes), "r"(su32(bar))
        : "memory");
}

template <int SPLIT>
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(IDESC<SPLIT>), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

__device__ __forceinline__ void tm_ld32(uint32_t addr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; k++) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void tm_ld16(uint32_t addr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tm_st16(uint32_t addr, const uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
            addr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
        "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
        : "memory");
}

// SiLU and its derivative with the logistic function as 0.5 + 0.5 tanh(z / 2):
// one MUFU instruction (tanh.approx, max relative error ~2^-11, below the BF16
// rounding the activations get anyway).
__device__ __forceinline__ float tanh_approx(float x) {
    float r;
    asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void silu2(float z, float &a, float &s1) {
    const float sg = fmaf(0.5f, tanh_approx(0.5f * z), 0.5f);
    a = z * sg;
    s1 = sg * fmaf(z, 1.0f - sg, 1.0f);
}

// Write 32 consecutive values (columns j0..j0+31, j0 a multiple of 32) of row
// `row` of the A operand: BF16 hi part and the BF16 rounding remainder (lo), or
// FP16 values (SPLIT 3).
template <int SPLIT>
__device__ __forceinline__ void put_a(uint8_t *sA, int row, int j0, const float (&v)[32]) {
    const int c = j0 >> 6, g0 = (j0 & 63) >> 3;
#pragma unroll
    for (int u = 0; u < 4; u++) {
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float a = v[u * 8 + 2 * e], b = v[u * 8 + 2 * e + 1];
            if constexpr (SPLIT == 3) {
                const __half2 hh = __floats2half2_rn(a, b);
                hw[e] = *reinterpret_cast<const uint32_t *>(&hh);
                lw[e] = 0u;
                continue;
            }
            const __nv_bfloat162 hi = __floats2bfloat162_rn(a, b);
            hw[e] = *reinterpret_cast<const uint32_t *>(&hi);
            if constexpr (SPLIT == 2) {
                const float2 hf = __bfloat1622float2(hi);
                const __nv_bfloat162 lo = __floats2bfloat162_rn(a - hf.x, b - hf.y);
                lw[e] = *reinterpret_cast<const uint32_t *>(&lo);
            } else {
                lw[e] = 0u;
            }
        }
        const int off = c * A_CHUNK + row * 128 + (((g0 + u) ^ (row & 7)) << 4);
        *reinterpret_cast<uint4 *>(sA + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        if constexpr (SPLIT == 2)
            *reinterpret_cast<uint4 *>(sA + A_PART + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
    }
}

// Per-CTA state of the MMA / copy issuer (thread 0).
struct Issuer {
    const uint8_t *wimg;  // NCHUNK chunk images of W_CHUNK bytes
    uint8_t *sW;          // two W_CHUNK buffers
    uint32_t q;           // next weight chunk to consume (global count)
    uint32_t issued;      // weight chunks whose copy has been issued
    uint32_t gemms;       // GEMMs committed so far
};

__device__ __forceinline__ void issue_copy(Issuer &I, Shared &S) {
    const uint32_t b = I.issued & 1;
    bulk_copy(I.sW + b * W_CHUNK, I.wimg + (size_t)(I.issued % NCHUNK) * W_CHUNK, W_CHUNK, &S.wfull[b]);
    I.issued++;
}

// One 128 x 256 x 256 GEMM into TMEM columns [0, 256): A from sA (hi and lo
// parts), B = the next four weight chunks.  Thread 0 only.  Returns false on a
// wait timeout.
template <int SPLIT>
__device__ bool issue_gemm(Issuer &I, Shared &S, uint8_t *sA, uint32_t tmem) {
    for (int c = 0; c < KCH; c++) {
        const uint32_t q = I.q, b = q & 1;
        if (!mbar_wait(&S.wfull[b], (q >> 1) & 1)) return false;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t wbase = su32(I.sW + b * W_CHUNK);
#pragma unroll
        for (int s = 0; s < 4; s++) {
            const uint64_t bd = desc_sw128(wbase + s * 32);
#pragma unroll
            for (int part = 0; part < NPART<SPLIT>; part++) {
                const uint64_t ad = desc_sw128(su32(sA + part * A_PART + c * A_CHUNK + s * 32));
                mma<SPLIT>(tmem, ad, bd, (c | s | part) ? 1u : 0u);
            }
        }
        commit(&S.wempty[b]);
        I.q++;
        // refill the other buffer once the MMAs of the previous chunk are done
        if (I.q >= 2) {
            const uint32_t pq = I.q - 2, pb = pq & 1;
            if (I.issued == I.q && !mbar_wait(&S.wempty[pb], (pq >> 1) & 1)) return false;
            if (I.issued == I.q) issue_copy(I, S);
        }
    }
    commit(&S.mma_done);
    I.gemms++;
    return true;
}

// Hand-off between the issuer and the epilogue threads.
__device__ __forceinline__ void to_mma() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
}

// Run one GEMM and wait for its result (all threads).  False on timeout.
template <int SPLIT>
__device__ __forceinline__ bool gemm(Issuer &I, Shared &S, uint8_t *sA, uint32_t tmem, uint32_t &phase) {
    to_mma();
    if (threadIdx.x == 0 && !S.abort && !issue_gemm<SPLIT>(I, S, sA, tmem)) S.abort = 1;
    __syncthreads();
    if (S.abort) return false;
    if (!mbar_wait(&S.mma_done, phase)) S.abort = 1;
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    return !S.abort;
}

// One surrogate evaluation of the tile whose inputs are in S.xh.  Every thread
// works on row `row`, columns [col0, col0 + 64); threads 0..127 (slice 0) get
// the row's value yv and input gradient G.  Returns false on a wait timeout.
template <int SPLIT>
__device__ bool tile_eval(const float *__restrict__ P, Issuer &I, Shared &S, uint8_t *sA, uint32_t tmem,
                          uint32_t &phase, float &yv, float (&G)[3]) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quad = warp & 3, slice = warp >> 2;
    const int row = quad * 32 + lane, col0 = slice * SLICE;
    const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
    const float x0 = S.xh[row * 3], x1 = S.xh[row * 3 + 1], x2 = S.xh[row * 3 + 2];
    // layer 1 (K = 3) in FP32
#pragma unroll 1
    for (int j0 = col0; j0 < col0 + SLICE; j0 += 32) {
        float v[32];
#pragma unroll
        for (int k = 0; k < 32; k++) {
            const float4 w = S.w1b1[j0 + k];
            const float z = fmaf(w.x, x0, fmaf(w.y, x1, fmaf(w.z, x2, w.w)));
            float s1;
            silu2(z, v[k], s1);
        }
        put_a<SPLIT>(sA, row, j0, v);
    }
    // layers 2..4
    float y = 0.f;
#pragma unroll 1
    for (int l = 2; l <= 4; l++) {
        if (!gemm<SPLIT>(I, S, sA, tmem, phase)) return false;
        const float *b = S.bias[l - 2];
#pragma unroll 1
        for (int j0 = col0; j0 < col0 + SLICE; j0 += 32) {
            float v[32];
            tm_ld32(tmem + lane_base + j0, v);
            uint32_t sp[16];
#pragma unroll
            for (int k = 0; k < 32; k += 2) {
                float a0, s0, a1, s1;
                const float2 bb = *reinterpret_cast<const float2 *>(b + j0 + k);
                silu2(v[k] + bb.x, a0, s0);
                silu2(v[k + 1] + bb.y, a1, s1);
                if (l == 4) {
                    const float2 ww = *reinterpret_cast<const float2 *>(S.w5 + j0 + k);
                    const float w0 = ww.x, w1 = ww.y;
                    y += a0 * w0 + a1 * w1;
                    v[k] = w0 * s0;  // backward seed delta_4 = w5 * silu'(z4)
                    v[k + 1] = w1 * s1;
                } else {
                    v[k] = a0;
                    v[k + 1] = a1;
                    const __half2 h = __floats2half2_rn(s0, s1);
                    sp[k >> 1] = *reinterpret_cast<const uint32_t *>(&h);
                }
            }
            if (l < 4) tm_st16(tmem + lane_base + (l == 2 ? COL_SP2 : COL_SP3) + (j0 >> 1), sp);
            put_a<SPLIT>(sA, row, j0, v);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    S.part[slice][row * 4] = y;
    // backward: u_l = delta_{l+1} W_{l+1}, delta_l = u_l silu'(z_l), l = 3, 2, 1
    float g0 = 0.f, g1 = 0.f, g2 = 0.f;
#pragma unroll 1
    for (int l = 3; l >= 1; l--) {
        if (!gemm<SPLIT>(I, S, sA, tmem, phase)) return false;
#pragma unroll 1
        for (int j0 = col0; j0 < col0 + SLICE; j0 += 32) {
            float v[32];
            tm_ld32(tmem + lane_base + j0, v);
            if (l > 1) {
                uint32_t sp[16];
                tm_ld16(tmem + lane_base + (l == 2 ? COL_SP2 : COL_SP3) + (j0 >> 1), sp);
#pragma unroll
                for (int k = 0; k < 32; k += 2) {
                    const float2 sv = __half22float2(*reinterpret_cast<const __half2 *>(&sp[k >> 1]));
                    v[k] *= sv.x;
                    v[k + 1] *= sv.y;
                }
                put_a<SPLIT>(sA, row, j0, v);
            } else {
#pragma unroll
                for (int k = 0; k < 32; k++) {
                    const float4 w = S.w1b1[j0 + k];
                    const float z = fmaf(w.x, x0, fmaf(w.y, x1, fmaf(w.z, x2, w.w)));
                    float a, s1;
                    silu2(z, a, s1);
                    const float d = v[k] * s1;
                    g0 = fmaf(d, w.x, g0);
                    g1 = fmaf(d, w.y, g1);
                    g2 = fmaf(d, w.z, g2);
                }
            }
        }
    }
    S.part[slice][row * 4 + 1] = g0;
    S.part[slice][row * 4 + 2] = g1;
    S.part[slice][row * 4 + 3] = g2;
    __syncthreads();
    if (threadIdx.x < TM) {
        const int r = threadIdx.x;
        float acc[4];
#pragma unroll
        for (int k = 0; k < 4; k++) acc[k] = S.part[0][r * 4 + k] + S.part[1][r * 4 + k] + S.part[2][r * 4 + k] +
                                             S.part[3][r * 4 + k];
        yv = acc[0] + __ldg(P + OFF_B5);
        G[0] = acc[1];
        G[1] = acc[2];
        G[2] = acc[3];
    }
    return true;
}

// Analytic SCF force (FP32) for the tile's points outside [r_min, r_max]:
// each warp takes every 4th listed point.  Ends with __syncthreads.
__device__ __forceinline__ void tile_fallback(const InferArgs &A, Shared &S) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nfb = S.fbcnt;
    for (int e = warp; e < nfb; e += NT / 32) {
        const float4 pt = S.fblist[e];
        const float q[3] = {pt.y, pt.z, pt.w};
        float g[3];
        gx::mlpi::scf_grad_f32_warp(A.scf, q, g);
        if (lane == 0) {
            const int r = (int)pt.x;
            S.fbg[r * 3 + 0] = g[0];
            S.fbg[r * 3 + 1] = g[1];
            S.fbg[r * 3 + 2] = g[2];
        }
    }
    __syncthreads();
}

struct Ctx {
    Shared *S;
    uint8_t *sA;
    Issuer I;
    uint32_t tmem;
    uint32_t phase;
};

// Set up shared state, barriers and TMEM; start the first two weight copies.
__device__ __forceinline__ void ctx_init(Ctx &C, const float *__restrict__ P, const uint8_t *wimg, char *smem_raw) {
    uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    C.sA = base;
    C.I.sW = base + 2 * A_PART;
    C.S = reinterpret_cast<Shared *>(base + 2 * A_PART + 2 * W_CHUNK);
    C.I.wimg = wimg;
    C.I.q = C.I.issued = C.I.gemms = 0;
    C.phase = 0;
    Shared &S = *C.S;
    if (threadIdx.x == 0) {
        mbar_init(&S.wfull[0], 1);
        mbar_init(&S.wfull[1], 1);
        mbar_init(&S.wempty[0], 1);
        mbar_init(&S.wempty[1], 1);
        mbar_init(&S.mma_done, 1);
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int j = threadIdx.x; j < H; j += blockDim.x) {
        S.w1b1[j] = make_float4(P[OFF_W1 + j * 3], P[OFF_W1 + j * 3 + 1], P[OFF_W1 + j * 3 + 2], P[OFF_B1 + j]);
        S.bias[0][j] = P[OFF_B2 + j];
        S.bias[1][j] = P[OFF_B3 + j];
        S.bias[2][j] = P[OFF_B4 + j];
        S.w5[j] = P[OFF_W5 + j];
    }
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&S.tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    C.tmem = S.tmem_base;
    if (threadIdx.x == 0) {
        issue_copy(C.I, S);
        issue_copy(C.I, S);
    }
}

// Drain the weight copies still in flight, free TMEM, report a timeout.
__device__ __forceinline__ void ctx_finish(Ctx &C, int *status) {
    Shared &S = *C.S;
    __syncthreads();
    if (threadIdx.x == 0) {
        // every issued copy completes its wfull barrier; wait for those not consumed
        for (uint32_t k = C.I.q; k < C.I.issued; k++) mbar_wait(&S.wfull[k & 1], (k >> 1) & 1);
        // and for the last MMAs (their commit on wempty) before TMEM is released
        if (C.I.q > 0) mbar_wait(&S.wempty[(C.I.q - 1) & 1], ((C.I.q - 1) >> 1) & 1);
        if (S.abort && status) atomicExch(status, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(C.tmem), "r"(TMEM_COLS));
}

template <int SPLIT>
__global__ void __launch_bounds__(NT, 1) surrogate_eval_tc_kernel(InferArgs A, const float *__restrict__ P,
                                                                   const uint8_t *__restrict__ wimg,
                                                                   const double *__restrict__ q, int64_t n,
                                                                   double *__restrict__ grad, double *__restrict__ phi,
                                                                   int *status) {
    extern __shared__ char smem_raw[];
    Ctx C;
    ctx_init(C, P, wimg, smem_raw);
    Shared &S = *C.S;
    const bool owner = threadIdx.x < TM;
    const int64_t ntiles = (n + TM - 1) / TM;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t i = tile * TM + threadIdx.x;
        float x = 1.f, y = 0.f, z = 0.f;
        MapPt m;
        if (owner) {
            if (i < n) {
                x = (float)q[i];
                y = (float)q[n + i];
                z = (float)q[2 * n + i];
            }
            m = map_point(A, x, y, z);
            S.xh[threadIdx.x * 3 + 0] = m.rho * m.nx;
            S.xh[threadIdx.x * 3 + 1] = m.rho * m.ny;
            S.xh[threadIdx.x * 3 + 2] = m.rho * m.nz;
        }
        if (threadIdx.x == 0) S.fbcnt = 0;
        __syncthreads();
        float yv = 0.f, G[3] = {0.f, 0.f, 0.f};
        if (!tile_eval<SPLIT>(P, C.I, S, C.sA, C.tmem, C.phase, yv, G)) break;
        const bool outside = owner && i < n && !(m.r >= A.r_min && m.r <= A.r_max);
        if (outside) {
            const int e = atomicAdd(&S.fbcnt, 1);
            S.fblist[e] = make_float4((float)threadIdx.x, x, y, z);
        }
        __syncthreads();
        tile_fallback(A, S);
        if (owner && i < n) {
            float gr[3];
            if (!outside) {
                surrogate_grad(m, yv, G, gr);
            } else {
                gr[0] = S.fbg[threadIdx.x * 3 + 0];
                gr[1] = S.fbg[threadIdx.x * 3 + 1];
                gr[2] = S.fbg[threadIdx.x * 3 + 2];
            }
            grad[i] = gr[0];
            grad[n + i] = gr[1];
            grad[2 * n + i] = gr[2];
            if (phi) phi[i] = (double)m.phi0 + (double)m.phiH * (double)yv;
        }
        __syncthreads();
    }
    ctx_finish(C, status);
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
// surrogate potential, FP32 state with Kahan compensation (as
// surrogate_leapfrog_kernel of gx_mlp_infer.cu, with 128-orbit tiles).
template <int SPLIT>
__global__ void __launch_bounds__(NT, 1) surrogate_leapfrog_tc_kernel(InferArgs A, const float *__restrict__ P,
                                                                       const uint8_t *__restrict__ wimg,
                                                                       const double *__restrict__ w0, int64_t n,
                                                                       int64_t nsteps, float dt,
                                                                       double *__restrict__ w_out,
                                                                       unsigned long long *__restrict__ fallbacks,
                                                                       int *status) {
    extern __shared__ char smem_raw[];
    Ctx C;
    ctx_init(C, P, wimg, smem_raw);
    Shared &S = *C.S;
    const int64_t ntiles = (n + TM - 1) / TM;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t i = tile * TM + threadIdx.x;
        const bool owner = threadIdx.x < TM;
        const bool own = owner && i < n;
        float xh_[3] = {1.f, 0.f, 0.f}, xl[3] = {0.f, 0.f, 0.f}, vh[3] = {0.f, 0.f, 0.f}, vl[3] = {0.f, 0.f, 0.f};
        float g[3] = {0.f, 0.f, 0.f};
        unsigned long long nfb = 0;
        if (own)
            for (int k = 0; k < 3; k++) {
                split(w0[k * n + i], xh_[k], xl[k]);
                split(w0[(3 + k) * n + i], vh[k], vl[k]);
            }
        for (int64_t step = 0; step <= nsteps; step++) {
            MapPt m;
            if (owner) {
                if (step > 0 && own)
                    for (int k = 0; k < 3; k++) kahan(xh_[k], xl[k], fmaf(vh[k], dt, vl[k] * dt));
                m = map_point(A, xh_[0], xh_[1], xh_[2]);
                S.xh[threadIdx.x * 3 + 0] = m.rho * m.nx;
                S.xh[threadIdx.x * 3 + 1] = m.rho * m.ny;
                S.xh[threadIdx.x * 3 + 2] = m.rho * m.nz;
            }
            if (threadIdx.x == 0) S.fbcnt = 0;
            __syncthreads();
            float yv = 0.f, G[3] = {0.f, 0.f, 0.f};
            if (!tile_eval<SPLIT>(P, C.I, S, C.sA, C.tmem, C.phase, yv, G)) {
                ok = false;
                break;
            }
            const bool outside = own && !(m.r >= A.r_min && m.r <= A.r_max);
            if (outside) {
                const int e = atomicAdd(&S.fbcnt, 1);
                S.fblist[e] = make_float4((float)threadIdx.x, xh_[0], xh_[1], xh_[2]);
            }
            __syncthreads();
            tile_fallback(A, S);
            if (own) {
                if (!outside) {
                    surrogate_grad(m, yv, G, g);
                } else {
                    g[0] = S.fbg[threadIdx.x * 3 + 0];
                    g[1] = S.fbg[threadIdx.x * 3 + 1];
                    g[2] = S.fbg[threadIdx.x * 3 + 2];
                    nfb++;
                }
                const float f = (step == 0) ? 0.5f : 1.0f;
                for (int k = 0; k < 3; k++) kahan(vh[k], vl[k], -g[k] * dt * f);
            }
        }
        if (own && ok) {
            for (int k = 0; k < 3; k++) kahan(vh[k], vl[k], g[k] * dt * 0.5f);
            for (int k = 0; k < 3; k++) {
                w_out[k * n + i] = (double)xh_[k] + (double)xl[k];
                w_out[(3 + k) * n + i] = (double)vh[k] + (double)vl[k];
            }
            if (nfb) atomicAdd(fallbacks, nfb);
        }
        __syncthreads();
    }
    ctx_finish(C, status);
}

}  // namespace mltc
}  // namespace gx

using namespace gx::mltc;

static int tc_args(const float *scf_params, double r_min, double r_max, double GM, double r_s, InferArgs *A) {
    GX_CHECK_ARG(scf_params != nullptr, "NULL SCF parameters (analytic base and fallback)");
    GX_CHECK_ARG(r_min > 0 && r_max > r_min && GM > 0 && r_s > 0, "bad surrogate input map");
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
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_eval_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM_BYTES));
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_eval_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM_BYTES));
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_leapfrog_tc_kernel<1>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_leapfrog_tc_kernel<2>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_eval_tc_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM_BYTES));
        GX_CUDA_TRY(cudaFuncSetAttribute(surrogate_leapfrog_tc_kernel<3>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        configured.fetch_or(bit);
    }
    return GX_OK;
}

extern "C" int gx_surrogate_gradient_tc(const float *params, const void *wimg, const float *scf_params, double r_min,
                                        double r_max, double GM, double r_s, int32_t split, const double *q, int64_t n,
                                        double *grad, double *phi, int32_t grid, int32_t *status, void *stream) {
    InferArgs A;
    int rc = tc_args(scf_params, r_min, r_max, GM, r_s, &A);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(params && wimg && q && grad && status && grid >= 1, "NULL array or bad grid");
    GX_CHECK_ARG(((uintptr_t)wimg & 15) == 0, "weight image must be 16-byte aligned");
    GX_CHECK_ARG(split >= 1 && split <= 3,
                 "split must be 1 (BF16 activations), 2 (BF16 hi + lo) or 3 (FP16 operands)");
    if (split == 3)
        surrogate_eval_tc_kernel<3><<<grid, NT, SMEM_BYTES, gx::as_stream(stream)>>>(
            A, params, static_cast<const uint8_t *>(wimg), q, n, grad, phi, status);
    else if (split == 2)
        surrogate_eval_tc_kernel<2><<<grid, NT, SMEM_BYTES, gx::as_stream(stream)>>>(
            A, params, static_cast<const uint8_t *>(wimg), q, n, grad, phi, status);
    else
        surrogate_eval_tc_kernel<1><<<grid, NT, SMEM_BYTES, gx::as_stream(stream)>>>(
            A, params, static_cast<const uint8_t *>(wimg), q, n, grad, phi, status);
    return gx::check_launch("surrogate_gradient_tc");
}

extern "C" int gx_surrogate_leapfrog_tc(const float *params, const void *wimg, const float *scf_params, double r_min,
                                        double r_max, double GM, double r_s, int32_t split, const double *w0,
                                        int64_t n, int64_t n_steps, double dt, double *w_out,
                                        unsigned long long *fallbacks, int32_t grid, int32_t *status, void *stream) {
    InferArgs A;
    int rc = tc_args(scf_params, r_min, r_max, GM, r_s, &A);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0 && n_steps >= 0, "n and n_steps must be >= 0");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(params && wimg && w0 && w_out && fallbacks && status && grid >= 1, "NULL array or bad grid");
    GX_CHECK_ARG(((uintptr_t)wimg & 15) == 0, "weight image must be 16-byte aligned");
    GX_CHECK_ARG(split >= 1 && split <= 3,
                 "split must be 1 (BF16 activations), 2 (BF16 hi + lo) or 3 (FP16 operands)");
    if (split == 3)
        surrogate_leapfrog_tc_kernel<3><<<grid, NT, SMEM_BYTES, gx::as_stream(stream)>>>(
            A, params, static_cast<const uint8_t *>(wimg), w0, n, n_steps, (float)dt, w_out, fallbacks, status);
    else if (split == 2)
        surrogate_leapfrog_tc_kernel<2><<<grid, NT, SMEM_BYTES, gx::as_stream(stream)>>>(
            A, params, static_cast<const uint8_t *>(wimg), w0, n, n_steps, (float)dt, w_out, fallbacks, status);
    else
        surrogate_leapfrog_tc_kernel<1><<<grid, NT, SMEM_BYTES, gx::as_stream(stream)>>>(
            A, params, static_cast<const uint8_t *>(wimg), w0, n, n_steps, (float)dt, w_out, fallbacks, status);
    return gx::check_launch("surrogate_leapfrog_tc");
}

extern "C" int gx_surrogate_tc_smem_bytes(void) { return SMEM_BYTES; }
