// gx_nfw_poly.cuh -- generated by gen_nfw_poly.py; do not edit.
// Degree-10 Chebyshev approximations on [-1, 1] (monomial coefficients c0..c10) of
//   H(x) = 2 f(u) / u^2,           u = (x + 1) / 2   (NFW factor inside r_s)
//   K(y) = ln(1 + w) - 1 / (1 + w), w = (y + 1) / 2   (NFW factor outside r_s)
// with f(u) = ln(1 + u) - u / (1 + u), evaluated in Estrin's scheme (depth 4 after x).
#pragma once

namespace gx {

__device__ __forceinline__ float estrin10(float x, float c0, float c1, float c2, float c3, float c4, float c5,
                                          float c6, float c7, float c8, float c9, float c10) {
    const float x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
    const float b0 = fmaf(fmaf(c3, x, c2), x2, fmaf(c1, x, c0));
    const float b1 = fmaf(fmaf(c7, x, c6), x2, fmaf(c5, x, c4));
    const float b2 = fmaf(c10, x2, fmaf(c9, x, c8));
    return fmaf(b2, x8, fmaf(b1, x4, b0));
}

__device__ __forceinline__ float nfw_poly_h(float x) {
    return estrin10(x, 0.5770542025566101f, -0.2652195990085602f, 0.10153299570083618f, -0.036609869450330734f, 0.01284234132617712f, -0.004448618274182081f, 0.0015229814453050494f, -0.0004927248228341341f, 0.00016704715380910784f, -8.19876222521998e-05f, 2.7610502002062276e-05f);
}

__device__ __forceinline__ float nfw_poly_k(float x) {
    return estrin10(x, -0.26120156049728394f, 0.5555556416511536f, -0.12962965667247772f, 0.03703578561544418f, -0.011316459625959396f, 0.0035734311677515507f, -0.0011453976621851325f, 0.00035481899976730347f, -0.00011559890845092013f, 5.39281900273636e-05f, -1.7742417185218073e-05f);
}

}  // namespace gx

