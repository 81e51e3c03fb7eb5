// gx_mlp_train.cu -- training of the potential surrogate (gx_mlp.cuh) on the GPU.
//
// The loss fits both the value and the input gradient of the target:
//   L = alpha * mean_b (y_b - y*_b)^2 + beta * mean_b |G_b - G*_b|^2,  G = d y / d xh,
// so the parameter gradient needs the derivative of the input gradient with
// respect to the parameters ("double backward").  One training step runs, in
// FP32 on the CUDA cores:
//   forward      Z_l = A_{l-1} W_l^T + b_l, A_l = silu(Z_l), keeping S_l = silu'(Z_l), T_l = silu''(Z_l)
//   input grad   D_4 = w5 * S_4, U_l = D_{l+1} W_{l+1}, D_l = U_l * S_l, G = D_1 W_1
//   adjoint      E = dL/dG, e = dL/dy;  back through the input-gradient pass
//                (W1g += D_1^T E, Dbar_1 = E W_1^T, Ubar_l = Dbar_l * S_l,
//                 Zbar_l = Dbar_l * U_l * T_l, W_{l+1}g += D_{l+1}^T Ubar_l,
//                 Dbar_{l+1} = Ubar_l W_{l+1}^T, w5g += sum Dbar_4 * S_4,
//                 Zbar_4 = Dbar_4 * w5 * T_4), then ordinary backprop of the
//                forward pass (Zbar_4 += e w5 * S_4, W_l g += Zbar_l^T A_{l-1},
//                Abar = Zbar_l W_l, Zbar_{l-1} += Abar * S_{l-1}).
// Parameter gradients are written to `grads`; gx_mlp_adam applies Adam.
// Every GEMM is one tiled SIMT kernel (64x64 tiles, 4x4 outputs per thread).
#include "gx_host.h"
#include "gx_mlp.cuh"

namespace gx {
namespace mlp {

// C[M,N] = alpha * op(A)[M,K] op(B)[K,N] + beta * C.  TA: A is stored [K][M]
// (element (m,k) at A[k*lda+m]) instead of [M][K]; TB: B stored [N][K].
// 128 x 128 block tile, K slabs of 8 staged through shared memory (double
// buffered), 256 threads each computing an 8 x 8 register tile.
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm_f32(int M, int N, int K, float alpha, const float *__restrict__ A,
                                                int lda, const float *__restrict__ B, int ldb, float beta,
                                                float *__restrict__ C, int ldc) {
    constexpr int BM = 128, BN = 128, BK = 8;
    __shared__ __align__(16) float As[2][BK][BM];
    __shared__ __align__(16) float Bs[2][BK][BN];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    // split-K: this CTA covers K range [kbeg, kend)
    const int kchunk = ((K + gridDim.z - 1) / gridDim.z + BK - 1) / BK * BK;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(K, kbeg + kchunk);
    float acc[8][8] = {};
    float ra[4], rb[4];
    auto gload = [&](int k0) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = tid + q * 256;
            int kk, mm;
            if (TA) { mm = e % BM; kk = e / BM; } else { kk = e % BK; mm = e / BK; }
            const int gm = m0 + mm, gk = k0 + kk;
            ra[q] = (gm < M && gk < kend) ? (TA ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk]) : 0.f;
            int kb, nn;
            if (TB) { kb = e % BK; nn = e / BK; } else { nn = e % BN; kb = e / BN; }
            const int gn = n0 + nn, gkb = k0 + kb;
            rb[q] = (gn < N && gkb < kend) ? (TB ? B[(int64_t)gn * ldb + gkb] : B[(int64_t)gkb * ldb + gn]) : 0.f;
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = tid + q * 256;
            int kk, mm;
            if (TA) { mm = e % BM; kk = e / BM; } else { kk = e % BK; mm = e / BK; }
            As[buf][kk][mm] = ra[q];
            int kb, nn;
            if (TB) { kb = e % BK; nn = e / BK; } else { nn = e % BN; kb = e / BN; }
            Bs[buf][kb][nn] = rb[q];
        }
    };
    gload(kbeg);
    sstore(0);
    __syncthreads();
    int buf = 0;
    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        const bool more = k0 + BK < kend;
        if (more) gload(k0 + BK);
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            float a[8], b[8];
            const float4 a0 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4 *>(&As[buf][kk][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][64 + tx * 4]);
            a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w; a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
            b[0] = b0.x; b[1] = b0.y; b[2] = b0.z; b[3] = b0.w; b[4] = b1.x; b[5] = b1.y; b[6] = b1.z; b[7] = b1.w;
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (more) {
            sstore(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int gm = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int gn = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
            if (gn >= N) continue;
            float *c = &C[(int64_t)gm * ldc + gn];
            if (gridDim.z > 1)
                atomicAdd(c, alpha * acc[i][j]);  // split-K: C already holds beta * C
            else
                *c = alpha * acc[i][j] + (beta == 0.f ? 0.f : beta * *c);
        }
    }
}

// Split K over extra CTAs when the output tile grid is small (weight gradients:
// 256 x 256 outputs, K = batch).  Split-K accumulates into C, so it is used
// only with beta = 1.
template <bool TA, bool TB>
static void gemm(cudaStream_t st, int M, int N, int K, float alpha, const float *A, int lda, const float *B,
                 int ldb, float beta, float *C, int ldc) {
    const int tiles = ((N + 127) / 128) * ((M + 127) / 128);
    int split = 1;
    if (beta == 1.f && tiles < 152) {
        split = (2 * 152 + tiles - 1) / tiles;
        const int maxsplit = (K + 255) / 256;
        if (split > maxsplit) split = maxsplit;
        if (split < 1) split = 1;
    }
    dim3 grid((N + 127) / 128, (M + 127) / 128, split);
    gemm_f32<TA, TB><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}

// Z (already A W^T, in place in `a`) + bias -> a = silu, s = silu', t = silu''.
__global__ void act_kernel(int64_t n, const float *__restrict__ bias, float *__restrict__ a, float *__restrict__ s,
                           float *__restrict__ t) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float z = a[i] + bias[i % H];
    float av, s1, s2;
    silu3(z, av, s1, s2);
    a[i] = av;
    s[i] = s1;
    t[i] = s2;
}

// out[b] = dot(A[b,:], w) + c  (one warp per row)
__global__ void rowdot_kernel(int64_t B, const float *__restrict__ A, const float *__restrict__ w,
                              const float *__restrict__ c, float *__restrict__ out) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (row >= B) return;
    float acc = 0.f;
    for (int k = lane; k < H; k += 32) acc = fmaf(A[row * H + k], w[k], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[row] = acc + (c ? *c : 0.f);
}

// D4 = w5 * S4 (row-broadcast)
__global__ void d4_kernel(int64_t n, const float *__restrict__ w5, const float *__restrict__ S4,
                          float *__restrict__ D4) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) D4[i] = w5[i % H] * S4[i];
}

// out = x * y (elementwise)
__global__ void mul_kernel(int64_t n, const float *__restrict__ x, const float *__restrict__ y,
                           float *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = x[i] * y[i];
}

// loss terms and their seeds: e = 2 alpha (y - y*) / B, E = 2 beta w (G - G*) / B
// (w = per-sample weight of the gradient term, 1 if wg is NULL)
__global__ void loss_kernel(int64_t B, float alpha, float beta, const float *__restrict__ y,
                            const float *__restrict__ ys, const float *__restrict__ G, const float *__restrict__ Gs,
                            const float *__restrict__ wg, float *__restrict__ e, float *__restrict__ E,
                            float *__restrict__ loss) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float lv = 0.f, lg = 0.f;
    if (b < B) {
        const float dv = y[b] - ys[b];
        e[b] = 2.f * alpha * dv / (float)B;
        lv = dv * dv;
        const float wb = wg ? wg[b] : 1.f;
        for (int j = 0; j < 3; j++) {
            const float dg = G[b * 3 + j] - Gs[b * 3 + j];
            E[b * 3 + j] = 2.f * beta * wb * dg / (float)B;
            lg += wb * dg * dg;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lv += __shfl_xor_sync(0xffffffffu, lv, o);
        lg += __shfl_xor_sync(0xffffffffu, lg, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&loss[0], lv / (float)B);
        atomicAdd(&loss[1], lg / (float)B);
    }
}

// Ubar = Dbar * S ; Zbar = Dbar * U * T
__global__ void adj_kernel(int64_t n, const float *__restrict__ Dbar, const float *__restrict__ S,
                           const float *__restrict__ U, const float *__restrict__ T, float *__restrict__ Ubar,
                           float *__restrict__ Zbar) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float d = Dbar[i];
    Ubar[i] = d * S[i];
    Zbar[i] = d * U[i] * T[i];
}

// Zbar4 = Dbar4 * w5 * T4 + e * w5 * S4
__global__ void zbar4_kernel(int64_t n, const float *__restrict__ Dbar4, const float *__restrict__ w5,
                             const float *__restrict__ T4, const float *__restrict__ S4, const float *__restrict__ e,
                             float *__restrict__ Zbar4) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = (int)(i % H);
    Zbar4[i] = w5[k] * (Dbar4[i] * T4[i] + e[i / H] * S4[i]);
}

// Zbar += Abar * S
__global__ void addmul_kernel(int64_t n, const float *__restrict__ Abar, const float *__restrict__ S,
                              float *__restrict__ Zbar) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) Zbar[i] += Abar[i] * S[i];
}

// column sums over the batch: out[k] = sum_b X[b, k] (+ sum_b e[b] Y[b, k] if e)
__global__ void colsum_kernel(int64_t B, const float *__restrict__ X, const float *__restrict__ e,
                              const float *__restrict__ Y, float *__restrict__ out) {
    const int k = threadIdx.x;  // blockDim = H
    const int64_t r0 = (int64_t)blockIdx.x * 256;
    float acc = 0.f;
    for (int64_t r = r0; r < r0 + 256 && r < B; r++) {
        acc += X[r * H + k];
        if (e) acc += e[r] * Y[r * H + k];
    }
    atomicAdd(&out[k], acc);
}

// out += sum_b x[b]
__global__ void sum_kernel(int64_t B, const float *__restrict__ x, float *__restrict__ out) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float v = b < B ? x[b] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, v);
}

// layer-1 forward with K = 3 inputs
__global__ void layer1_kernel(int64_t B, const float *__restrict__ X, const float *__restrict__ P,
                              float *__restrict__ A, float *__restrict__ S, float *__restrict__ T) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * H) return;
    const int64_t b = i / H;
    const int o = (int)(i % H);
    const float *W1 = P + OFF_W1;
    const float z = W1[o * 3 + 0] * X[b * 3 + 0] + W1[o * 3 + 1] * X[b * 3 + 1] + W1[o * 3 + 2] * X[b * 3 + 2] +
                    P[OFF_B1 + o];
    float a, s1, s2;
    silu3(z, a, s1, s2);
    A[i] = a;
    S[i] = s1;
    T[i] = s2;
}

// Adam (bias-corrected), FP32 master weights
__global__ void adam_kernel(int64_t n, float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

static inline unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace mlp
}  // namespace gx

using namespace gx::mlp;

extern "C" int64_t gx_mlp_param_count(void) { return NPARAM; }

extern "C" int64_t gx_mlp_train_workspace_floats(int64_t batch) { return batch * (26 * (int64_t)H + 16); }

extern "C" int gx_mlp_forward(const float *params, const float *xh, int64_t B, float *y, float *G, float *workspace,
                              void *stream) {
    GX_CHECK_ARG(params && xh && y && workspace && B > 0 && B < (1 << 26), "bad arguments");
    cudaStream_t st = gx::as_stream(stream);
    const int64_t n = B * H;
    float *w = workspace;
    float *A[5], *S[5], *T[5], *D[5], *U[4];
    for (int l = 1; l <= 4; l++) {
        A[l] = w; w += n;
        S[l] = w; w += n;
        T[l] = w; w += n;
        D[l] = w; w += n;
    }
    for (int l = 1; l <= 3; l++) { U[l] = w; w += n; }
    layer1_kernel<<<nblk(n, 256), 256, 0, st>>>(B, xh, params, A[1], S[1], T[1]);
    for (int l = 2; l <= 4; l++) {
        gemm<false, true>(st, (int)B, H, H, 1.f, A[l - 1], H, params + off_W(l), H, 0.f, A[l], H);
        act_kernel<<<nblk(n, 256), 256, 0, st>>>(n, params + off_b(l), A[l], S[l], T[l]);
    }
    rowdot_kernel<<<nblk(B * 32, 256), 256, 0, st>>>(B, A[4], params + OFF_W5, params + OFF_B5, y);
    if (G) {
        d4_kernel<<<nblk(n, 256), 256, 0, st>>>(n, params + OFF_W5, S[4], D[4]);
        for (int l = 3; l >= 1; l--) {
            gemm<false, false>(st, (int)B, H, H, 1.f, D[l + 1], H, params + off_W(l + 1), H, 0.f, U[l], H);
            mul_kernel<<<nblk(n, 256), 256, 0, st>>>(n, U[l], S[l], D[l]);
        }
        gemm<false, false>(st, (int)B, 3, H, 1.f, D[1], H, params + OFF_W1, 3, 0.f, G, 3);
    }
    return gx::check_launch("mlp_forward");
}

extern "C" int gx_mlp_train_step(const float *params, float *grads, const float *xh, const float *ystar,
                                 const float *Gstar, const float *gweight, int64_t B, float alpha, float beta,
                                 float *workspace, float *loss, void *stream) {
    GX_CHECK_ARG(params && grads && xh && ystar && Gstar && workspace && loss, "NULL pointer");
    GX_CHECK_ARG(B > 0 && B < (1 << 26), "batch out of range");
    cudaStream_t st = gx::as_stream(stream);
    const int64_t n = B * H;
    float *w = workspace;
    float *A[5], *S[5], *T[5], *D[5], *U[4];
    for (int l = 1; l <= 4; l++) {
        A[l] = w; w += n;
        S[l] = w; w += n;
        T[l] = w; w += n;
        D[l] = w; w += n;
    }
    for (int l = 1; l <= 3; l++) { U[l] = w; w += n; }
    float *Zb[5];
    for (int l = 1; l <= 4; l++) { Zb[l] = w; w += n; }
    float *Dbar = w; w += n;
    float *Ubar = w; w += n;
    float *Abar = w; w += n;
    float *y = w; w += B;
    float *e = w; w += B;
    float *G = w; w += 3 * B;
    float *E = w; w += 3 * B;
    const float *W5 = params + OFF_W5;
    float *g = grads;

    GX_CUDA_TRY(cudaMemsetAsync(grads, 0, sizeof(float) * NPARAM, st));
    GX_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float) * 2, st));
    // forward and input gradient
    int rc = gx_mlp_forward(params, xh, B, y, G, workspace, stream);
    if (rc) return rc;
    loss_kernel<<<nblk(B, 256), 256, 0, st>>>(B, alpha, beta, y, ystar, G, Gstar, gweight, e, E, loss);

    // adjoint of the input-gradient pass
    gemm<true, false>(st, H, 3, (int)B, 1.f, D[1], H, E, 3, 1.f, g + OFF_W1, 3);      // W1g += D1^T E
    // Dbar_1 = E W1^T : [B,3] x [3,256] where W1 is [256][3] -> B operand stored [N][K]
    gemm<false, true>(st, (int)B, H, 3, 1.f, E, 3, params + OFF_W1, 3, 0.f, Dbar, H);
    for (int l = 1; l <= 3; l++) {
        adj_kernel<<<nblk(n, 256), 256, 0, st>>>(n, Dbar, S[l], U[l], T[l], Ubar, Zb[l]);
        // W_{l+1} g += D_{l+1}^T Ubar_l  : [256 x B] x [B x 256]
        gemm<true, false>(st, H, H, (int)B, 1.f, D[l + 1], H, Ubar, H, 1.f, g + off_W(l + 1), H);
        // Dbar_{l+1} = Ubar_l W_{l+1}^T
        gemm<false, true>(st, (int)B, H, H, 1.f, Ubar, H, params + off_W(l + 1), H, 0.f, Dbar, H);
    }
    // w5g += colsum(Dbar4 * S4) + A4^T e ; Zbar4 = w5 * (Dbar4 * T4 + e * S4)
    mul_kernel<<<nblk(n, 256), 256, 0, st>>>(n, Dbar, S[4], Abar);
    colsum_kernel<<<nblk(B, 256), H, 0, st>>>(B, Abar, e, A[4], g + OFF_W5);
    zbar4_kernel<<<nblk(n, 256), 256, 0, st>>>(n, Dbar, W5, T[4], S[4], e, Zb[4]);
    // b5g = sum e
    sum_kernel<<<nblk(B, 256), 256, 0, st>>>(B, e, g + OFF_B5);
    // backprop through the forward pass
    for (int l = 4; l >= 2; l--) {
        gemm<true, false>(st, H, H, (int)B, 1.f, Zb[l], H, A[l - 1], H, 1.f, g + off_W(l), H);  // W_l g += Zbar^T A
        colsum_kernel<<<nblk(B, 256), H, 0, st>>>(B, Zb[l], nullptr, nullptr, g + off_b(l));
        gemm<false, false>(st, (int)B, H, H, 1.f, Zb[l], H, params + off_W(l), H, 0.f, Abar, H);  // Abar = Zbar W_l
        addmul_kernel<<<nblk(n, 256), 256, 0, st>>>(n, Abar, S[l - 1], Zb[l - 1]);
    }
    gemm<true, false>(st, H, 3, (int)B, 1.f, Zb[1], H, xh, 3, 1.f, g + OFF_W1, 3);  // W1g += Zbar1^T X
    colsum_kernel<<<nblk(B, 256), H, 0, st>>>(B, Zb[1], nullptr, nullptr, g + OFF_B1);
    return gx::check_launch("mlp_train_step");
}

extern "C" int gx_mlp_adam(float *params, const float *grads, float *m, float *v, int64_t n, float lr, float beta1,
                           float beta2, float eps, int64_t step, void *stream) {
    GX_CHECK_ARG(params && grads && m && v && n > 0 && step >= 1, "bad arguments");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    adam_kernel<<<nblk(n, 256), 256, 0, gx::as_stream(stream)>>>(n, params, grads, m, v, lr, beta1, beta2, eps, c1,
                                                                  c2);
    return gx::check_launch("mlp_adam");
}
