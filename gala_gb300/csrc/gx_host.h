// gx_host.h -- host-side helpers shared by the C-ABI entry points: descriptor
// validation and packing into the by-value kernel descriptor, and the
// thread-local error message behind gx_last_error_message().
#pragma once

#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>

#include "gx_debug.cuh"
#include "gx_device.cuh"

namespace gx {

void set_error(const char *fmt, ...);

#define GX_CHECK_ARG(cond, ...)          \
    do {                                 \
        if (!(cond)) {                   \
            ::gx::set_error(__VA_ARGS__); \
            return GX_ERR_INVALID_ARGUMENT; \
        }                                \
    } while (0)

#define GX_CUDA_TRY(expr)                                                              \
    do {                                                                               \
        cudaError_t e_ = (expr);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            ::gx::set_error("%s failed: %s", #expr, cudaGetErrorString(e_));            \
            return GX_ERR_CUDA;                                                        \
        }                                                                              \
    } while (0)

// Number of doubles a component of this type must carry ([G, ...]).
int expected_params(int type, const double *p, int64_t avail);

// Validate a gx_potential and copy it into the kernel descriptor.
int pack_potential(const gx_potential *pot, DevPot *out);
int pack_frame(const gx_frame *fr, DevFrame *out);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// The cancel flag that gx_set_cancel_flag installed on the calling host thread
// (a device-readable int32; nullptr = none).  The persistent kernels launched
// from that thread receive it and stop taking new work once it reads non-zero.
const int32_t *cancel_flag();

// Device side: the host has asked the launch to stop.  The flag lives in
// mapped host memory and is written while the kernel runs, so every reader
// loads it through a volatile pointer; callers that need one answer for a
// whole warp or CTA read it on one thread and broadcast it.
__device__ __forceinline__ bool cancel_requested(const int32_t *flag) {
    return flag != nullptr && *reinterpret_cast<const volatile int32_t *>(flag) != 0;
}

// Launch-error check after a <<<>>> launch.
inline int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: kernel launch failed: %s", what, cudaGetErrorString(e));
        return GX_ERR_CUDA;
    }
    return GX_OK;
}

}  // namespace gx
