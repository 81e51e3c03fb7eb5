// gx_peaks.cu -- arithmetic-pipe calibration kernels.
//
// MEASURED_PEAKS-style denominators exist for HBM and bf16 tensor throughput;
// the FP64 and FP32 integrators are bound by the FP64 / FP32 pipes instead, so
// the library carries its own throughput probes: each thread runs 8
// independent multiply-add chains (enough ILP to keep the pipe busy) for
// `iters` iterations; the grid is a multiple of the SM count.  The result
// buffer keeps the chains live.  Flop count = 2 * 8 * iters per thread.
#include "gx_host.h"

namespace gx {

template <typename T>
__global__ void __launch_bounds__(256) fma_chain_kernel(int64_t iters, T a, T b, T *__restrict__ sink) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int64_t i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)12345.678) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;  // practically never taken
}

}  // namespace gx

extern "C" int gx_calibrate_fma(int32_t fp64, int32_t blocks, int32_t threads, int64_t iters, void *sink,
                                void *stream) {
    GX_CHECK_ARG(blocks > 0 && threads > 0 && threads <= 256 && iters > 0, "bad calibration launch shape");
    GX_CHECK_ARG(sink != nullptr, "NULL sink");
    cudaStream_t st = gx::as_stream(stream);
    if (fp64)
        gx::fma_chain_kernel<double><<<blocks, threads, 0, st>>>(iters, 0.999999, 1e-7, (double *)sink);
    else
        gx::fma_chain_kernel<float><<<blocks, threads, 0, st>>>(iters, 0.999999f, 1e-7f, (float *)sink);
    return gx::check_launch("calibrate_fma");
}
