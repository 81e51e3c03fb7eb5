// gx_mlp.cuh -- the potential surrogate network: layout and maths shared by the
// training kernels (gx_mlp_train.cu) and the inference kernels (gx_mlp_infer.cu).
//
// Network: y(xh) = w5 . a4 + b5,  a_l = silu(W_l a_{l-1} + b_l), l = 1..4,
// a_0 = xh (3 inputs), hidden width 256.  Parameters in one FP32 buffer:
//   W1 [256][3] | b1 [256] | W2 [256][256] | b2 | W3 | b3 | W4 | b4 | w5 [256] | b5
//
// Input map and output (so the network only learns a bounded correction):
//   r in [r_min, r_max], n = x / r, rho(r) = rho0 + (1 - rho0) ln(r / r_min) / ln(r_max / r_min)
//   xh = rho(r) n                                 (a ball of radius <= 1)
//   Phi(x) = Phi_H(r) (1 + y(xh)),  Phi_H = -G M / (r + r_s)  (the S000 term of SCF)
//   grad Phi = grad Phi_H (1 + y) + Phi_H J^T grad_xh y,
//   J^T g = (rho / r) (g - n (n.g)) + rho' n (n.g),  rho' = (1 - rho0) / (r ln(r_max / r_min))
#pragma once

#include <cstdint>

namespace gx {
namespace mlp {

constexpr int H = 256;
constexpr int DIN = 3;
constexpr int64_t OFF_W1 = 0;
constexpr int64_t OFF_B1 = OFF_W1 + H * DIN;
constexpr int64_t OFF_W2 = OFF_B1 + H;
constexpr int64_t OFF_B2 = OFF_W2 + H * H;
constexpr int64_t OFF_W3 = OFF_B2 + H;
constexpr int64_t OFF_B3 = OFF_W3 + H * H;
constexpr int64_t OFF_W4 = OFF_B3 + H;
constexpr int64_t OFF_B4 = OFF_W4 + H * H;
constexpr int64_t OFF_W5 = OFF_B4 + H;
constexpr int64_t OFF_B5 = OFF_W5 + H;
constexpr int64_t NPARAM = OFF_B5 + 1;

__host__ __device__ constexpr int64_t off_W(int l) {
    return l == 1 ? OFF_W1 : l == 2 ? OFF_W2 : l == 3 ? OFF_W3 : OFF_W4;
}
__host__ __device__ constexpr int64_t off_b(int l) {
    return l == 1 ? OFF_B1 : l == 2 ? OFF_B2 : l == 3 ? OFF_B3 : OFF_B4;
}

// SiLU and its first two derivatives.
__device__ __forceinline__ void silu3(float z, float &a, float &s1, float &s2) {
    const float sg = 1.0f / (1.0f + __expf(-z));
    a = z * sg;
    s1 = sg * (1.0f + z * (1.0f - sg));
    s2 = sg * (1.0f - sg) * (2.0f + z * (1.0f - 2.0f * sg));
}

}  // namespace mlp
}  // namespace gx
