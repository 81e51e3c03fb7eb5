// gx_host.cu -- descriptor packing, error reporting and the potential /
// Hamiltonian evaluation entry points (gx_potential_value, gx_potential_gradient,
// gx_potential_density, gx_hamiltonian_value, gx_hamiltonian_gradient).
#include <cmath>
#include <vector>

#include "gx_host.h"
#include "gx_queue.cuh"
#include "gx_scf.cuh"

namespace gx {

static thread_local char g_errmsg[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_errmsg, sizeof(g_errmsg), fmt, ap);
    va_end(ap);
}

int expected_params(int type, const double *p, int64_t avail) {
    switch (type) {
    case GX_POT_NULL: return 1;
    case GX_POT_KEPLER: return 2;
    case GX_POT_HERNQUIST: return 3;
    case GX_POT_PLUMMER: return 3;
    case GX_POT_MIYAMOTONAGAI: return 4;
    case GX_POT_SPHERICALNFW:
    case GX_POT_FLATTENEDNFW:
    case GX_POT_TRIAXIALNFW: return 6;
    case GX_POT_SCF: {
        if (avail < 5) return -1;
        const double nmax = p[1], lmax = p[2];
        if (!(nmax >= 0 && lmax >= 0 && nmax + 1 <= SCF_MAX_N && lmax + 1 <= SCF_MAX_L)) return -1;
        const int n = (int)nmax, l = (int)lmax;
        return 5 + 2 * (n + 1) * (l + 1) * (l + 1);
    }
    default: return -1;
    }
}

// Host-derived constants of a component for the FP64-pipe-lean forms
// (gx_fast64.cuh); P is the component's [G, ...] block.
static void derived_constants(int type, const double *P, DevComp &d) {
    d.dc[0] = P[0] * P[1];
    switch (type) {
    case GX_POT_PLUMMER: d.dc[1] = P[2] * P[2]; break;
    case GX_POT_MIYAMOTONAGAI: d.dc[1] = P[3] * P[3]; break;
    case GX_POT_SPHERICALNFW:
    case GX_POT_FLATTENEDNFW:
    case GX_POT_TRIAXIALNFW:
        d.dc[1] = 1.0 / P[2];
        d.dc[2] = type == GX_POT_TRIAXIALNFW ? 1.0 / (P[3] * P[3]) : 1.0;
        d.dc[3] = type == GX_POT_TRIAXIALNFW ? 1.0 / (P[4] * P[4]) : 1.0;
        d.dc[4] = type != GX_POT_SPHERICALNFW ? 1.0 / (P[5] * P[5]) : 1.0;
        break;
    default: break;
    }
}

// Validate the descriptor's header and component i; *need = the doubles its type uses.
static int check_header(const gx_potential *pot) {
    GX_CHECK_ARG(pot != nullptr, "potential descriptor is NULL");
    GX_CHECK_ARG(pot->n_dim == 3, "n_dim must be 3 (got %d)", pot->n_dim);
    GX_CHECK_ARG(pot->n_components >= 0, "n_components < 0");
    GX_CHECK_ARG(pot->n_components == 0 || (pot->components && pot->params), "NULL component or param array");
    return GX_OK;
}

static int check_component(const gx_potential *pot, int i, int *need) {
    const gx_component &c = pot->components[i];
    GX_CHECK_ARG(c.param_offset >= 0 && c.param_offset + c.n_params <= pot->n_params_total,
                 "component %d parameter range outside params[]", i);
    GX_CHECK_ARG(c.param_offset < (int64_t)INT32_MAX, "component %d: parameter offset too large", i);
    *need = expected_params(c.type, pot->params + c.param_offset, c.n_params);
    GX_CHECK_ARG(*need > 0, "component %d: unknown type %d or bad SCF header", i, c.type);
    GX_CHECK_ARG(c.n_params >= *need, "component %d: %d parameters, type %d needs %d", i, c.n_params, c.type,
                 *need);
    return GX_OK;
}

int pack_potential(const gx_potential *pot, DevPot *out) {
    int rc = check_header(pot);
    if (rc) return rc;
    memset(out, 0, sizeof(*out));
    out->ncomp = pot->n_components;
    out->pdev = pot->params_device;
    if (pot->n_components > GX_MAX_COMPONENTS) {
        // a large composite: components from the device table, parameters
        // from the device copy
        if (pot->table_device == nullptr || pot->params_device == nullptr) {
            set_error("%d components exceed GX_MAX_COMPONENTS = %d: pass the component table in device memory "
                      "(table_device, packed by gx_pack_component_table) and params_device",
                      pot->n_components, GX_MAX_COMPONENTS);
            return GX_ERR_CAPACITY;
        }
        for (int i = 0; i < pot->n_components; i++) {
            int need = 0;
            rc = check_component(pot, i, &need);
            if (rc) return rc;
            if (pot->components[i].type == GX_POT_SCF) out->has_scf = 1;
        }
        out->cdev = static_cast<const DevComp *>(pot->table_device);
        return GX_OK;
    }
    int ninl = 0;
    for (int i = 0; i < pot->n_components; i++) {
        const gx_component &c = pot->components[i];
        int need = 0;
        rc = check_component(pot, i, &need);
        if (rc) return rc;
        DevComp &d = out->c[i];
        d.type = c.type;
        d.do_sr = c.do_shift_rotate ? 1 : 0;
        for (int k = 0; k < 3; k++) d.q0[k] = c.q0[k];
        for (int k = 0; k < 9; k++) d.R[k] = c.R[k];
        if (c.type == GX_POT_SCF) {
            if (pot->params_device == nullptr) {
                set_error("component %d is SCF: params_device (device copy of params) is required", i);
                return GX_ERR_INVALID_ARGUMENT;
            }
            d.inl = 0;
            d.poff = (int32_t)c.param_offset;
            out->has_scf = 1;
        } else {
            if (ninl + need > GX_MAX_INLINE_PARAMS) {
                set_error("inline parameters exceed GX_MAX_INLINE_PARAMS = %d", GX_MAX_INLINE_PARAMS);
                return GX_ERR_CAPACITY;
            }
            d.inl = 1;
            d.poff = ninl;
            for (int k = 0; k < need; k++) out->p[ninl + k] = pot->params[c.param_offset + k];
            ninl += need;
            derived_constants(c.type, pot->params + c.param_offset, d);
        }
    }
    out->n_inline = ninl;
    return GX_OK;
}

int pack_frame(const gx_frame *fr, DevFrame *out) {
    memset(out, 0, sizeof(*out));
    if (fr == nullptr) {
        out->type = GX_FRAME_STATIC;
        return GX_OK;
    }
    GX_CHECK_ARG(fr->type == GX_FRAME_STATIC || fr->type == GX_FRAME_CONSTANT_ROTATING, "unknown frame type %d",
                 fr->type);
    out->type = fr->type;
    for (int k = 0; k < 3; k++) out->O[k] = fr->params[k];
    return GX_OK;
}

// ---------------------------------------------------------------------------
// Evaluation kernels: one thread per point, SoA in and out.
// ---------------------------------------------------------------------------
template <int KIND, bool SCF>  // KIND 0 value, 1 gradient, 2 density
__global__ void eval_kernel(const __grid_constant__ DevPot pot, const double *__restrict__ q, int64_t n, double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double qi[3] = {q[i], q[n + i], q[2 * n + i]};
    if (KIND == 0) {
        out[i] = potential_value<SCF>(pot, qi);
    } else if (KIND == 2) {
        out[i] = potential_density<SCF>(pot, qi);
    } else {
        double g[3];
        potential_gradient<SCF>(pot, qi, g);
        out[i] = g[0];
        out[n + i] = g[1];
        out[2 * n + i] = g[2];
    }
}

template <int KIND, bool SCF>  // KIND 0 energy, 1 Hamilton's equations
__global__ void ham_kernel(const __grid_constant__ DevPot pot, const __grid_constant__ DevFrame fr, const double *__restrict__ w, int64_t n, double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double wi[6];
    for (int k = 0; k < 6; k++) wi[k] = w[k * n + i];
    if (KIND == 0) {
        out[i] = potential_value<SCF>(pot, wi) + frame_energy(fr, wi);
    } else {
        double f[6];
        hamiltonian_rhs<SCF>(pot, fr, wi, f);
        for (int k = 0; k < 6; k++) out[k * n + i] = f[k];
    }
}

template <int KIND>
static int launch_eval(const gx_potential *pot, const double *q, int64_t n, double *out, void *stream) {
    DevPot dp;
    int rc = pack_potential(pot, &dp);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(q && out, "NULL array");
    const int bs = 128;
    const int64_t grid = (n + bs - 1) / bs;
    if (dp.has_scf)
        eval_kernel<KIND, true><<<(unsigned)grid, bs, 0, as_stream(stream)>>>(dp, q, n, out);
    else
        eval_kernel<KIND, false><<<(unsigned)grid, bs, 0, as_stream(stream)>>>(dp, q, n, out);
    return check_launch("gx_potential eval");
}

template <int KIND>
static int launch_ham(const gx_potential *pot, const gx_frame *fr, const double *w, int64_t n, double *out,
                      void *stream) {
    DevPot dp;
    DevFrame df;
    int rc = pack_potential(pot, &dp);
    if (rc) return rc;
    rc = pack_frame(fr, &df);
    if (rc) return rc;
    GX_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return GX_OK;
    GX_CHECK_ARG(w && out, "NULL array");
    const int bs = 128;
    const int64_t grid = (n + bs - 1) / bs;
    if (dp.has_scf)
        ham_kernel<KIND, true><<<(unsigned)grid, bs, 0, as_stream(stream)>>>(dp, df, w, n, out);
    else
        ham_kernel<KIND, false><<<(unsigned)grid, bs, 0, as_stream(stream)>>>(dp, df, w, n, out);
    return check_launch("gx_hamiltonian eval");
}

static thread_local const int32_t *g_cancel = nullptr;
const int32_t *cancel_flag() { return g_cancel; }

// Readers of the debug records, one per translation unit (debug build only).
static std::vector<DbgReader> &dbg_readers() {
    static std::vector<DbgReader> r;
    return r;
}
void dbg_register(DbgReader r) { dbg_readers().push_back(r); }

// The lead region of the batched integrators' queue: at most one 32-orbit
// block per SM sub-partition of the current device (four per multiprocessor),
// in whole chunks.
int64_t queue_lead_chunks(int64_t n_chunks, int32_t chunk) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms = 0;
    const int64_t lead = 4 * (int64_t)sms / (chunk / 32);
    return n_chunks < lead ? n_chunks : lead;
}

}  // namespace gx

extern "C" {

int gx_abi_version(void) { return GX_ABI_VERSION; }

int64_t gx_component_table_bytes(int32_t n_components) {
    return n_components > 0 ? (int64_t)n_components * (int64_t)sizeof(gx::DevComp) : 0;
}

int gx_pack_component_table(const gx_potential *pot, void *host_out, int64_t bytes) {
    int rc = gx::check_header(pot);
    if (rc) return rc;
    const int64_t want = gx_component_table_bytes(pot->n_components);
    GX_CHECK_ARG(bytes >= want, "table buffer of %lld bytes, %lld needed", (long long)bytes, (long long)want);
    GX_CHECK_ARG(want == 0 || host_out != nullptr, "NULL table buffer");
    gx::DevComp *t = static_cast<gx::DevComp *>(host_out);
    for (int i = 0; i < pot->n_components; i++) {
        int need = 0;
        rc = gx::check_component(pot, i, &need);
        if (rc) return rc;
        const gx_component &c = pot->components[i];
        gx::DevComp d;
        memset(&d, 0, sizeof(d));
        d.type = c.type;
        d.do_sr = c.do_shift_rotate ? 1 : 0;
        d.inl = 0;  // parameters from the device copy of params[]
        d.poff = (int32_t)c.param_offset;
        for (int k = 0; k < 3; k++) d.q0[k] = c.q0[k];
        for (int k = 0; k < 9; k++) d.R[k] = c.R[k];
        if (c.type != GX_POT_SCF) gx::derived_constants(c.type, pot->params + c.param_offset, d);
        memcpy(&t[i], &d, sizeof(d));
    }
    return GX_OK;
}

const char *gx_last_error_message(void) { return gx::g_errmsg; }

void gx_set_cancel_flag(const int32_t *flag) { gx::g_cancel = flag; }

int gx_cancel_flag_create(int32_t **host_ptr, int32_t **device_ptr) {
    GX_CHECK_ARG(host_ptr && device_ptr, "NULL pointer");
    void *h = nullptr;
    GX_CUDA_TRY(cudaHostAlloc(&h, 64, cudaHostAllocMapped | cudaHostAllocPortable));
    *reinterpret_cast<volatile int32_t *>(h) = 0;
    void *d = nullptr;
    const cudaError_t e = cudaHostGetDevicePointer(&d, h, 0);
    if (e != cudaSuccess) {
        cudaFreeHost(h);
        gx::set_error("cudaHostGetDevicePointer failed: %s", cudaGetErrorString(e));
        return GX_ERR_CUDA;
    }
    *host_ptr = static_cast<int32_t *>(h);
    *device_ptr = static_cast<int32_t *>(d);
    return GX_OK;
}

int gx_debug_enabled(void) {
#ifdef GX_DEBUG_CHECKS
    return 1;
#else
    return 0;
#endif
}

int gx_debug_read(int64_t *out, int32_t reset) {
    GX_CHECK_ARG(out, "NULL pointer");
    for (int k = 0; k < 9; k++) out[k] = 0;
    if (!gx_debug_enabled()) {
        gx::set_error("the release library keeps no debug records (load libgala_gb300_debug.so)");
        return GX_ERR_UNSUPPORTED;
    }
    GX_CUDA_TRY(cudaDeviceSynchronize());
    for (gx::DbgReader rd : gx::dbg_readers()) {
        gx::DbgRecord r;
        if (rd(&r, reset != 0) != 0) {
            gx::set_error("reading a debug record failed");
            return GX_ERR_CUDA;
        }
        if (r.first && !out[0]) {
            out[0] = (int64_t)(r.first >> 32);
            out[1] = (int64_t)(r.first & 0xffffffffu);
            out[2] = r.index;
            out[3] = r.bound;
        }
        out[4] += (int64_t)r.fails;
        out[5] += (int64_t)r.done;
        out[6] += (int64_t)r.id_sum;
        out[7] += (int64_t)r.id_sq;
        out[8] += (int64_t)r.steps;
    }
    return GX_OK;
}

int gx_cancel_flag_destroy(int32_t *host_ptr) {
    GX_CHECK_ARG(host_ptr, "NULL pointer");
    GX_CUDA_TRY(cudaFreeHost(host_ptr));
    return GX_OK;
}

int gx_potential_value(const gx_potential *pot, double t, const double *q, int64_t n, double *out, void *stream) {
    (void)t;
    return gx::launch_eval<0>(pot, q, n, out, stream);
}

int gx_potential_gradient(const gx_potential *pot, double t, const double *q, int64_t n, double *out,
                          void *stream) {
    (void)t;
    return gx::launch_eval<1>(pot, q, n, out, stream);
}

int gx_potential_density(const gx_potential *pot, double t, const double *q, int64_t n, double *out,
                         void *stream) {
    (void)t;
    return gx::launch_eval<2>(pot, q, n, out, stream);
}

int gx_hamiltonian_value(const gx_potential *pot, const gx_frame *frame, double t, const double *w, int64_t n,
                         double *out, void *stream) {
    (void)t;
    return gx::launch_ham<0>(pot, frame, w, n, out, stream);
}

int gx_hamiltonian_gradient(const gx_potential *pot, const gx_frame *frame, double t, const double *w, int64_t n,
                            double *out, void *stream) {
    (void)t;
    return gx::launch_ham<1>(pot, frame, w, n, out, stream);
}

}  // extern "C"
