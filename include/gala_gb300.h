/*
 * gala_gb300.h -- C ABI of the GB300 orbit-integration library (libgala_gb300.so).
 *
 * This is the drop-in boundary for gala's orbit-integration hot path.  Every entry
 * point below replaces one function of gala's Cython/C layer; the citation next to
 * each declaration names the gala function (path inside the gala project) whose
 * argument meaning, output layout and error behaviour it reproduces.
 *
 * Conventions
 *   - All array arguments are DEVICE pointers (e.g. torch.Tensor.data_ptr() of a
 *     CUDA tensor).  Descriptors (gx_potential, gx_frame, option structs) are HOST
 *     structs; the library copies them into kernel parameters at launch.
 *   - Phase-space arrays use gala's structure-of-arrays layout: w0 is (6, N)
 *     row-major (x, y, z, vx, vy, vz rows), snapshots are (6, ntimes, N).
 *   - Units are whatever the caller packed (gala_gb300 uses kpc, Myr, Msun with
 *     G = 4.498502151469553e-12 kpc^3 / (Msun Myr^2)).
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     asynchronous with respect to the host unless stated otherwise.
 *   - Return value: GX_OK (0) or a negative gx_error code.  The call never aborts
 *     the process; gx_last_error_message() describes the most recent failure of
 *     the calling thread.
 */
#ifndef GALA_GB300_H
#define GALA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GX_ABI_VERSION 3

/* Capacity of the by-value potential descriptor handed to every kernel.  A
 * potential with more components (gala's composites have no limit) is read by
 * the FP64 kernels from a component table in device memory instead
 * (gx_potential.table_device); the FP32 forms take at most GX_MAX_COMPONENTS. */
#define GX_MAX_COMPONENTS 16
/* Scratch of the batched integrators' work queue (gx_batch_integrate_fp32,
 * _fp32_state, _fp64), in int32: two counters and one flag per SM
 * sub-partition for up to 256 multiprocessors.  The order's first n_lead =
 * min(n_chunks, 4 x multiprocessors / (chunk / 32)) chunks (the longest) go
 * out in blocks of 32 orbits, at most one per sub-partition, before the rest in
 * whole chunks.  After a run (also a cancelled one) the integrated orbits are
 * the first min(q[1], n_lead x chunk / 32) blocks of 32 slots and the first
 * min(q[0], n_chunks - n_lead) chunks after the lead region. */
#define GX_BATCH_QUEUE_WORDS 1026
#define GX_MAX_INLINE_PARAMS 128

/* ------------------------------------------------------------------------- */
/* Error codes                                                               */
/* ------------------------------------------------------------------------- */
typedef enum gx_error {
    GX_OK = 0,
    GX_ERR_INVALID_ARGUMENT = -1,   /* bad size, NULL pointer, unknown type      */
    GX_ERR_UNSUPPORTED = -2,        /* combination not implemented on the GPU    */
    GX_ERR_CUDA = -3,               /* a CUDA runtime call failed                */
    GX_ERR_CAPACITY = -4,           /* descriptor exceeds GX_MAX_* capacities    */
    GX_ERR_KERNEL_STATUS = -5       /* a kernel reported a bounded-wait timeout  */
} gx_error;

/* DOP853 per-batch status, same values as gala's dop853() return code
 * (src/gala/integrate/cyintegrators/dopri/dop853.cpp:340-354, 474-480). */
#define GX_DOP853_OK            1
#define GX_DOP853_BAD_INPUT    -1
#define GX_DOP853_NMAX         -2
#define GX_DOP853_SMALL_STEP   -3
#define GX_DOP853_STIFF        -4

/* ------------------------------------------------------------------------- */
/* Potential descriptor: the device analogue of gala's struct _CPotential     */
/* (src/gala/potential/potential/src/cpotential.h:10-36).  Function pointers  */
/* are replaced by a type tag; parameters keep gala's packing [G, p0, p1, ...] */
/* (CPotentialWrapper.init, src/gala/potential/potential/cpotential.pyx:57-102)*/
/* ------------------------------------------------------------------------- */
typedef enum gx_potential_type {
    GX_POT_NULL = 0,           /* null_* (builtin_potentials.cpp:18-21)            */
    GX_POT_KEPLER = 1,         /* [G, m]          kepler_*  (:58-88)               */
    GX_POT_HERNQUIST = 2,      /* [G, m, c]       hernquist_* (:211-244)           */
    GX_POT_PLUMMER = 3,        /* [G, m, b]       plummer_* (:292-324)             */
    GX_POT_MIYAMOTONAGAI = 4,  /* [G, m, a, b]    miyamotonagai_* (:1287-1332)     */
    GX_POT_SPHERICALNFW = 5,   /* [G, m, r_s, a, b, c] sphericalnfw_* (:819-864)   */
    GX_POT_FLATTENEDNFW = 6,   /* [G, m, r_s, a, b, c] flattenednfw_* (:925-962)   */
    GX_POT_TRIAXIALNFW = 7,    /* [G, m, r_s, a, b, c] triaxialnfw_* (:1028-1072)  */
    GX_POT_SCF = 8             /* [G, nmax, lmax, m, r_s, Snlm..., Tnlm...]
                                  scf_* (src/gala/potential/scf/src/bfe.cpp:191-259) */
} gx_potential_type;

typedef struct gx_component {
    int32_t type;              /* gx_potential_type                                 */
    int32_t n_params;          /* number of doubles of this component in params[]   */
    int64_t param_offset;      /* offset of this component's [G, ...] in params[]   */
    int32_t do_shift_rotate;   /* 0 iff q0 == 0 and R == I (cpotential.pyx:99-102)  */
    int32_t reserved;
    double q0[3];              /* origin                                            */
    double R[9];               /* rotation, row-major                               */
} gx_component;

typedef struct gx_potential {
    int32_t n_components;      /* components are summed in this order (composite   */
    int32_t n_dim;             /* insertion order); n_dim must be 3                 */
    const gx_component* components;   /* HOST array[n_components]                   */
    const double* params;             /* HOST packed parameters                     */
    const double* params_device;      /* DEVICE copy of params; required when a      */
                                      /* component is GX_POT_SCF or when there are  */
                                      /* more than GX_MAX_COMPONENTS, else may be NULL */
    int64_t n_params_total;
    const void* table_device;         /* DEVICE component table for more than        */
                                      /* GX_MAX_COMPONENTS components: the bytes     */
                                      /* gx_pack_component_table wrote for this same */
                                      /* descriptor, copied to the device; else NULL */
} gx_potential;

/* Reference frame: gala's CFrameType (src/gala/potential/frame/src/cframe.h:7-17). */
typedef enum gx_frame_type {
    GX_FRAME_STATIC = 0,              /* static_frame_* (builtin_frames.cpp:8-24)   */
    GX_FRAME_CONSTANT_ROTATING = 1    /* constant_rotating_frame_3d_* (:73-112),     */
                                      /* params = Omega (3)                          */
} gx_frame_type;

typedef struct gx_frame {
    int32_t type;
    int32_t reserved;
    double params[3];
} gx_frame;

/* Potential of one massive body of an n-body system: gala's particle potentials
 * of DirectNBody / MockStreamGenerator (src/gala/dynamics/nbody/core.py,
 * mockstream.pyx:49-78).  One unrotated component, shifted by the integrator to
 * the body's position (c_nbody_acceleration, cpotential.cpp:389-415); a body of
 * type GX_POT_NULL exerts no force (gala's NullPotential, `null == 1`). */
typedef struct gx_body {
    int32_t type;        /* gx_potential_type of the single component             */
    int32_t n_params;    /* entries of params in use: [G, p1, p2, ...]            */
    double params[7];
} gx_body;               /* 64 bytes */

/* ------------------------------------------------------------------------- */
/* Library                                                                   */
/* ------------------------------------------------------------------------- */
/* Component table for a potential of more than GX_MAX_COMPONENTS components.
 * gala keeps the component pointers of a composite in host arrays (struct
 * _CPotential, cpotential.h:10-36); on the GPU a large composite lives in a
 * device table that every thread reads through the L1 cache.
 *   gx_component_table_bytes(n)      bytes of the table for n components
 *   gx_pack_component_table(pot, host_out, bytes)
 *       validates pot (its components and params, HOST) and writes the table
 *       into host_out; copy those bytes to device memory and set
 *       pot->table_device (and pot->params_device) before calling any FP64
 *       entry point with this descriptor.  The table is valid for the
 *       descriptor it was packed from.  Returns GX_OK or an error code. */
int64_t gx_component_table_bytes(int32_t n_components);
int gx_pack_component_table(const gx_potential* pot, void* host_out, int64_t bytes);

/* ABI version of the loaded library (compare with GX_ABI_VERSION). */
int gx_abi_version(void);

/* Message of the last failed call on this host thread ("" if none). */
const char* gx_last_error_message(void);

/* Cancelling long launches.  gala's mock-stream loop polls for a keyboard
 * interrupt between releases (PyErr_CheckSignals, mockstream.pyx:277); the
 * GPU work of one call is a single launch, so its kernels poll a flag in
 * mapped host memory instead.
 *   gx_cancel_flag_create   allocates the flag (pinned, mapped, zero) and
 *                           returns its host address and the device address
 *                           kernels read it through
 *   gx_set_cancel_flag      installs a device address (NULL: none) for the
 *                           launches made afterwards from the calling host
 *                           thread
 *   gx_cancel_flag_destroy  frees it; only after every launch that reads it
 *                           has completed (a CUDA graph captured while it was
 *                           installed reads it at every replay)
 * The host requests cancellation by storing a non-zero int32 through the host
 * address, at any time.  What a launch then skips, per entry point:
 *   gx_batch_integrate_fp32, gx_batch_integrate_fp64: no further queue chunk
 *     is taken; chunks already taken complete.  The queue counter then holds
 *     the number of chunks taken (at most n_slots / chunk); the orbits of the
 *     first that many chunks of `order` are integrated, the others untouched;
 *   gx_dop853_fp32, gx_nbody_dop853, gx_mockstream_dop853,
 *     gx_mockstream_dop853_fp32: no further orbit or system is taken; ones in
 *     flight complete; the status of the ones not taken is left as the caller
 *     initialised it;
 *   gx_dop853_integrate_hamiltonian: batches whose CTA starts after the request are not
 *     integrated (their status is left as initialised);
 *   gx_mockstream_dop853_wide: systems whose CTA starts after the request are
 *     not integrated;
 *   gx_mockstream_dop853_animate: each stream stops after its current
 *     interval; the status of the intervals not run is 0, the snapshots not
 *     reached are all NaN, and the final state is the one reached.
 * Every other entry point ignores the flag. */
int gx_cancel_flag_create(int32_t** host_ptr, int32_t** device_ptr);
void gx_set_cancel_flag(const int32_t* device_ptr);
int gx_cancel_flag_destroy(int32_t* host_ptr);

/* The debug build.  The kernels test every index that comes from a caller's
 * device array (queue orders, system ids, release offsets and counts) and skip
 * what is out of range.  libgala_gb300_debug.so (the same sources compiled with
 * GX_DEBUG_CHECKS) also records each failed test in device memory, and the
 * persistent queues of gx_batch_integrate_fp32 / _fp64 and gx_dop853_fp32 add
 * every orbit they complete to a count, sum(id + 1), sum((id + 1)^2) and a
 * step total.  No check traps.  gala has no counterpart (its loops are compiled
 * without bounds checks, boundscheck=False).
 *   gx_debug_enabled()      1 in the debug build, 0 in the release library
 *   gx_debug_read(out, r)   synchronises the device and writes int64[9] =
 *       {code of the first failure (1 order id, 2 system id, 3 release offsets,
 *        4 release count; 0 none), its source line, index, bound, failures,
 *        orbits completed, sum(id + 1), sum((id + 1)^2), steps}
 *     summed over the library's translation units; r != 0 clears the records.
 *     GX_ERR_UNSUPPORTED in the release library. */
int gx_debug_enabled(void);
int gx_debug_read(int64_t* out, int32_t reset);

/* ------------------------------------------------------------------------- */
/* Potential evaluation over N points.                                       */
/* q is (3, N) SoA; out is (N,) for value/density and (3, N) for gradient.   */
/* ------------------------------------------------------------------------- */

/* c_potential (src/gala/potential/potential/src/cpotential.cpp:170-189),
 * applied to every column of q (CPotentialWrapper.energy, cpotential.pyx:104-122). */
int gx_potential_value(const gx_potential* pot, double t, const double* q,
                       int64_t n, double* out, void* stream);

/* c_gradient (cpotential.cpp:214-287): out = sum over components of grad Phi,
 * with the shift/rotate path q' = R (q - q0), g += R^T g'.  out is overwritten. */
int gx_potential_gradient(const gx_potential* pot, double t, const double* q,
                          int64_t n, double* out, void* stream);

/* c_density (cpotential.cpp:192-211). */
int gx_potential_density(const gx_potential* pot, double t, const double* q,
                         int64_t n, double* out, void* stream);

/* Hamiltonian.energy (src/gala/potential/hamiltonian/chamiltonian.pyx:83-86,
 * 107-128): c_potential (shift/rotate aware) + the frame's energy
 * (static_frame_hamiltonian / constant_rotating_frame_3d_hamiltonian,
 * builtin_frames.cpp:8-16, 78-94) for every column of w (6, N). */
int gx_hamiltonian_value(const gx_potential* pot, const gx_frame* frame, double t,
                         const double* w, int64_t n, double* out, void* stream);

/* hamiltonian_gradient_T (chamiltonian.cpp:38-57): dH/dt of every column of
 * w (6, N) into out (6, N) = (qdot, pdot). */
int gx_hamiltonian_gradient(const gx_potential* pot, const gx_frame* frame, double t,
                            const double* w, int64_t n, double* out, void* stream);

/* ------------------------------------------------------------------------- */
/* Fixed-step symplectic integrators (FP64, one thread per orbit).           */
/* t (ntimes) are the output times (t[1]-t[0] is the step, as in gala).      */
/* save_all != 0: w_out is (6, ntimes, N), snapshot 0 = w0.                  */
/* save_all == 0: w_out is (6, N), the state at t[ntimes-1].                 */
/* ------------------------------------------------------------------------- */

/* leapfrog_integrate_hamiltonian
 * (src/gala/integrate/cyintegrators/leapfrog.pyx:54-121): kick-drift-kick with
 * c_init_velocity (:24-32) and c_leapfrog_step (:35-51).  Frame must be static. */
int gx_leapfrog_integrate_hamiltonian(const gx_potential* pot, const gx_frame* frame,
                                      const double* w0, int64_t n, const double* t,
                                      int64_t ntimes, int32_t save_all, double* w_out,
                                      void* stream);

/* ruth4_integrate_hamiltonian (src/gala/integrate/cyintegrators/ruth4.pyx:37-113),
 * c_ruth4_step (:24-35) with gala's coefficients (:65-78).  Frame must be static. */
int gx_ruth4_integrate_hamiltonian(const gx_potential* pot, const gx_frame* frame,
                                   const double* w0, int64_t n, const double* t,
                                   int64_t ntimes, int32_t save_all, double* w_out,
                                   void* stream);

/* dop853_integrate_hamiltonian
 * (src/gala/integrate/cyintegrators/dop853.pyx:196-250) -> dop853_helper (:90-193)
 * -> dop853()/dopcor() (dopri/dop853.cpp:89-866).  Orbits are integrated in
 * batches of `nbatch` consecutive orbits that share one step size and one RMS
 * error norm over all 6*nb components, exactly as gala's batching does.
 *   atol, rtol, nmax, dt_max, nstiff : gala's meaning and defaults (0 -> default)
 *   save_all != 0 : w_out is (6, n_out, N) holding the dense output at
 *                   t[0], t[out_stride], t[2*out_stride], ... (n_out =
 *                   (ntimes - 1) / out_stride + 1); out_stride = 1 is gala's layout.
 *   save_all == 0 : w_out is (6, N), the state at t[ntimes-1].
 *   status        : DEVICE int32[ceil(N / nbatch)], gala's dop853() return code
 *                   per batch (1 = success, -2 nmax, -3 step too small, -4 stiff).
 *   stats         : DEVICE int64[4 * ceil(N / nbatch)] or NULL; per batch the
 *                   counters gala's dopcor keeps: nfcn, nstep, naccpt, nrejct.
 *   nbatch        : 1..1024 (gala default 100). */
int gx_dop853_integrate_hamiltonian(const gx_potential* pot, const gx_frame* frame,
                                    const double* w0, int64_t n, const double* t,
                                    int64_t ntimes, double atol, double rtol,
                                    int64_t nmax, double dt_max, int64_t nstiff,
                                    int32_t save_all, int32_t nbatch,
                                    int64_t out_stride, double* w_out,
                                    int32_t* status, int64_t* stats, void* stream);

/* FP32-compensated form of leapfrog_integrate_hamiltonian / ruth4_integrate_
 * hamiltonian (src/gala/integrate/cyintegrators/leapfrog.pyx:54-121,
 * ruth4.pyx:37-113) on gala's time grid (step t[1] - t[0]): FP32 forces,
 * Kahan-compensated FP32 state, FP64 input and output.  method 0 = leapfrog,
 * 1 = ruth4.  save_all != 0: w_out (6, n_out, N) with every out_stride-th of
 * the ntimes grid points (n_out = (ntimes - 1) / out_stride + 1); save_all == 0:
 * w_out (6, N) at t[ntimes-1].  Static frames, closed-form components only. */
int gx_fixed_fp32(const gx_potential* pot, int32_t method, const double* w0, int64_t n,
                  const double* t, int64_t ntimes, int32_t save_all, int64_t out_stride,
                  double* w_out, void* stream);

/* DOP853 with FP32 stages and forces and FP64 step control.  gala's
 * dop853_integrate_hamiltonian (src/gala/integrate/cyintegrators/dop853.pyx:
 * 196-250) with nbatch = 1 -- every orbit is its own system with its own step
 * size -- over gala's dopcor (dopri/dop853.cpp:89-650): the stages, forces and
 * dense-output polynomial are FP32, the state is a double-float pair, and the
 * time, step size, error-norm combination (:441-444) and accept/reject are FP64.
 * Results are not bit-compatible with gala; accuracy is that of an FP32 force
 * (relative ~1e-7 per evaluation).  Tolerances below ~1e-8 relative ask for
 * more than FP32 stages resolve and only shrink the steps.
 *   arguments as gx_dop853_integrate_hamiltonian (no nbatch), plus
 *   order         : DEVICE int32[N] processing order (a permutation of the
 *                   orbits), or NULL for 0..N-1; orbits of similar cost next to
 *                   each other keep a warp's lanes busy together.  Each orbit's
 *                   result does not depend on the order.
 *   status        : DEVICE int32[N], gala's return code per orbit
 *   stats         : DEVICE int64[4 * N] or NULL: nfcn, nstep, naccpt, nrejct
 *   queue_counter : DEVICE int32 scratch (zeroed by the call)
 * Closed-form components only (SCF -> GX_ERR_UNSUPPORTED). */
int gx_dop853_fp32(const gx_potential* pot, const gx_frame* frame, const double* w0,
                   int64_t n, const double* t, int64_t ntimes, double atol, double rtol,
                   int64_t nmax, double dt_max, int64_t nstiff, int32_t save_all,
                   int64_t out_stride, const int32_t* order, double* w_out, int32_t* status,
                   int64_t* stats, int32_t* queue_counter, void* stream);

/* The processing order of a batch for gx_batch_integrate_fp32 / _fp64, built
 * on the device with no host synchronisation: per integrator the orbits by
 * cost (n_steps x 1 for Leapfrog, x 3 for Ruth4) in 128 bins per octave, the
 * most expensive first, cut into chunks of `chunk` padded with -1; the chunks
 * of both integrators merged by the bin of their first orbit.
 *   n_steps, method  DEVICE (N,) as for gx_batch_integrate_fp32
 *   order            DEVICE int32[n_slots], n_slots >= gx_batch_schedule_slots(N, chunk)
 *                    (every slot written: an orbit index or -1)
 *   work             DEVICE int32[gx_batch_schedule_work_words(N, chunk)] scratch
 * No gala counterpart (gala integrates orbits one after another). */
int64_t gx_batch_schedule_slots(int64_t n, int32_t chunk);
int64_t gx_batch_schedule_work_words(int64_t n, int32_t chunk);
int gx_batch_schedule(const int64_t* n_steps, const int32_t* method, int64_t n, int32_t chunk,
                      int32_t* order, int64_t n_slots, int32_t* work, int64_t work_words, void* stream);

/* ------------------------------------------------------------------------- */
/* Batched FP32 integration with compensated state (no single gala function:  */
/* it runs many leapfrog_integrate_hamiltonian / ruth4_integrate_hamiltonian  */
/* problems of different length, step and integrator in one launch; per-orbit */
/* arithmetic follows leapfrog.pyx:24-51 and ruth4.pyx:24-35 in FP32).         */
/*   w0       (6, N) float64 initial conditions                               */
/*   n_steps  (N,) int64 steps per orbit; dt (N,) float64 step per orbit      */
/*   method   (N,) int32: 0 leapfrog, 1 ruth4                                 */
/*   order    (n_slots,) int32 processing order: orbit indices, -1 = padding; */
/*            n_slots is a multiple of `chunk`; each chunk is one queue item  */
/*   queue_counter  DEVICE int32[GX_BATCH_QUEUE_WORDS] scratch (zeroed by    */
/*                  the call)                                                 */
/*   block, grid    launch shape of the persistent grid                       */
/*   w_out    (6, N) float64 final states (t = n_steps * dt after the start)  */
/* Closed-form components only (SCF -> GX_ERR_UNSUPPORTED).                   */
/* ------------------------------------------------------------------------- */
int gx_batch_integrate_fp32(const gx_potential* pot, const double* w0, int64_t n,
                            const int64_t* n_steps, const double* dt, const int32_t* method,
                            const int32_t* order, int64_t n_slots, int32_t chunk,
                            int32_t block, int32_t grid, int32_t* queue_counter,
                            double* w_out, void* stream);

/* The same with the integrator state in device memory, for checkpoints: a run
 * of k steps that writes its state, then a run of n - k steps that resumes from
 * it, gives the bits of one run of n steps (orbit by orbit; for n = 0 the
 * resumed run returns the state's value, hi + lo, where one run of no steps
 * returns w0 itself).
 *   state_in   DEVICE float[12][N] or NULL: position hi (3), lo (3), velocity
 *              hi (3), lo (3) -- for Leapfrog the half-step velocity v_{1/2},
 *              which the resumed run uses as is (no second c_init_velocity);
 *              w0 then serves only orbits without state (unused here) and may
 *              be the original initial conditions
 *   state_out  DEVICE float[12][N] or NULL: the state after this run's steps
 *              (before the output velocity is synchronised); not aliasing state_in
 * At least one of them is given.  gala keeps no such state: a run started again
 * from an Orbit's last (x, v) forms v_{1/2} again and takes a new rounding path. */
int gx_batch_integrate_fp32_state(const gx_potential* pot, const double* w0, int64_t n,
                                  const int64_t* n_steps, const double* dt, const int32_t* method,
                                  const int32_t* order, int64_t n_slots, int32_t chunk,
                                  int32_t block, int32_t grid, int32_t* queue_counter,
                                  const float* state_in, float* state_out, double* w_out,
                                  void* stream);

/* The plain FP64 form of the same batched workload: identical arguments and
 * queue; per orbit, gala's Leapfrog / Ruth4 arithmetic in FP64 exactly as
 * gx_leapfrog_integrate_hamiltonian / gx_ruth4_integrate_hamiltonian compute it
 * (bit-identical final states).  block <= 128.  SCF components allowed. */
int gx_batch_integrate_fp64(const gx_potential* pot, const double* w0, int64_t n,
                            const int64_t* n_steps, const double* dt, const int32_t* method,
                            const int32_t* order, int64_t n_slots, int32_t chunk,
                            int32_t block, int32_t grid, int32_t* queue_counter,
                            double* w_out, void* stream);

/* Allocation-free form of gx_batch_integrate_fp32.  No counterpart in gala.
 * For callers that cannot allocate device memory (a process whose memory
 * manager owns the GPU, a host that only receives device pointers from another
 * runtime, or a pipeline that cannot afford the device synchronisation of
 * cudaMalloc / cudaFree): only inputs and outputs are passed, and the work
 * queue (counter + processing order) lives in a fixed array inside the library,
 * built on the device by a counting sort (integrator, then cost, longest first).
 *   n <= GX_NOALLOC_MAX_ORBITS, else GX_ERR_CAPACITY and nothing is launched.
 *   Per-orbit results are bit-identical to gx_batch_integrate_fp32.
 *   The first call on a device looks up that array's device address (with
 *   that device current); make that first call before any stream capture.
 *   A call in a new context of the device (after cudaDeviceReset) looks the
 *   address up again.
 *   Every call on a device shares the one array: calls that overlap on the GPU
 *   (different streams, no ordering) race and must not be issued.
 * The library holds the array (about 2.2 MB) on every GPU it is loaded on until
 * the process exits. */
#define GX_NOALLOC_MAX_ORBITS 262144
int gx_batch_integrate_fp32_noalloc(const gx_potential* pot, const double* w0, int64_t n,
                                    const int64_t* n_steps, const double* dt,
                                    const int32_t* method, int32_t block, int32_t grid,
                                    double* w_out, void* stream);

/* ------------------------------------------------------------------------- */
/* Learned potential surrogate.  No counterpart in gala: an MLP             */
/* y(xh), 3 -> 256 -> 256 -> 256 -> 256 -> 1, SiLU, with                        */
/*   Phi(x) = Phi_0(r) + Phi_H(r) y(xh),  Phi_H = -G M / (r + r_s),             */
/*   xh = rho(r) x / r,  rho = 0.1 + 0.9 ln(r / r_min) / ln(r_max / r_min).      */
/* params: FP32 [W1 256x3 | b1 | W2 256x256 | b2 | W3 | b3 | W4 | b4 | w5 | b5]  */
/* (gx_mlp_param_count() floats).  Training runs on the CUDA cores in FP32;      */
/* inference uses BF16 weights [W2, W3, W4, W4^T, W3^T, W2^T] (6 x 256 x 256)    */
/* on the tensor cores with FP32 accumulation.                                   */
/* ------------------------------------------------------------------------- */
int64_t gx_mlp_param_count(void);
/* floats of workspace gx_mlp_train_step / gx_mlp_forward need for a batch */
int64_t gx_mlp_train_workspace_floats(int64_t batch);
/* y (B) and, if G != NULL, dy/dxh (B x 3) for inputs xh (B x 3), FP32 */
int gx_mlp_forward(const float* params, const float* xh, int64_t batch, float* y, float* G,
                   float* workspace, void* stream);
/* gradient of L = alpha mean (y - y*)^2 + beta mean w |dy/dxh - G*|^2 w.r.t. params
 * into grads (w = gweight per sample, or 1 if gweight is NULL); loss[0], loss[1]
 * = the two mean (weighted) squared errors */
int gx_mlp_train_step(const float* params, float* grads, const float* xh, const float* ystar,
                      const float* Gstar, const float* gweight, int64_t batch, float alpha,
                      float beta, float* workspace, float* loss, void* stream);
/* Adam update of params (n floats) with moment buffers m, v; step >= 1 */
int gx_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t n, float lr,
                float beta1, float beta2, float eps, int64_t step, void* stream);
/* grad Phi (3 x n) and Phi (n, may be NULL) at q (3 x n) with
 *   Phi = Phi_0(r) + Phi_H(r) y(xh),
 * Phi_0 the spherical (l = 0) part of the SCF expansion (FP32, exact) and y the
 * network; outside [r_min, r_max] the full analytic SCF force (FP32) is used.
 * scf_params = gala's packed SCF parameters as float.  split = 1: activations
 * rounded to BF16; split = 2: activations as BF16 hi + lo (two MMAs per tile).
 * grid = number of 256-thread CTAs. */
int gx_surrogate_gradient(const float* params, const void* wbf16, const float* scf_params,
                          double r_min, double r_max, double GM, double r_s, int32_t split,
                          const double* q, int64_t n, double* grad, double* phi, int32_t grid,
                          void* stream);
/* FP32 leapfrog (kick-drift-kick, Kahan-compensated state) of n orbits for
 * n_steps of dt in the surrogate potential; w_out = final states (6 x n);
 * *fallbacks += number of force evaluations that used the analytic SCF.
 * analytic != 0: every force is the analytic SCF force in FP32 (the same
 * integrator without the surrogate; params / wbf16 may then be NULL). */
int gx_surrogate_leapfrog(const float* params, const void* wbf16, const float* scf_params,
                          double r_min, double r_max, double GM, double r_s, int32_t split,
                          int32_t analytic, const double* w0, int64_t n, int64_t n_steps,
                          double dt, double* w_out, unsigned long long* fallbacks, int32_t grid,
                          void* stream);
int gx_surrogate_smem_bytes(void);

/* The same surrogate force and leapfrog on the 5th-generation tensor cores
 * (tcgen05.mma, accumulators in tensor memory; 128-position tiles, BF16 hi + lo
 * activations).  `wimg` is the weight image: for each of W2, W3, W4, W4^T,
 * W3^T, W2^T (BF16, [256 out][256 in] row-major) four 32 KB K-chunks of 64
 * columns, each 256 rows x 128 bytes, the 16-byte granule g of row r stored at
 * position g ^ (r & 7) (the 128-byte swizzle); 786,432 bytes, 16-byte aligned.
 * split = 2 multiplies BF16 hi and lo parts of every activation (two MMAs per
 * K step), split = 1 the BF16 activations only.  `status` (DEVICE int32) is set
 * to 1 if a bounded wait inside the kernel ran out (the results are then
 * incomplete); the caller zeroes it. */
int gx_surrogate_gradient_tc(const float* params, const void* wimg, const float* scf_params,
                             double r_min, double r_max, double GM, double r_s, int32_t split,
                             const double* q, int64_t n, double* grad, double* phi, int32_t grid,
                             int32_t* status, void* stream);
int gx_surrogate_leapfrog_tc(const float* params, const void* wimg, const float* scf_params,
                             double r_min, double r_max, double GM, double r_s, int32_t split,
                             const double* w0, int64_t n, int64_t n_steps, double dt, double* w_out,
                             unsigned long long* fallbacks, int32_t grid, int32_t* status,
                             void* stream);
int gx_surrogate_tc_smem_bytes(void);

/* ------------------------------------------------------------------------- */
/* Pipe calibration.  No counterpart in gala: it measures the FP64 / FP32     */
/* multiply-add throughput that bounds the integrators (the roofline          */
/* denominator).  Runs blocks x threads threads, each with 8 independent FMA  */
/* chains of `iters` steps: flops = 16 * iters * blocks * threads.  `sink` is */
/* a DEVICE buffer of blocks * threads doubles (fp64 != 0) or floats.         */
/* ------------------------------------------------------------------------- */
int gx_calibrate_fma(int32_t fp64, int32_t blocks, int32_t threads, int64_t iters,
                     void* sink, void* stream);

/* Numerics self-check of the FP64 forms the DOP853 force uses instead of the
 * library functions (no counterpart in gala): for n DEVICE doubles x, out is
 * (4, n) DEVICE doubles: the table-driven ln x, the library log(x), the
 * seeded-Newton sqrt(x) and 1/x. */
int gx_selfcheck_fast64(const double* x, int64_t n, double* out, void* stream);

/* ------------------------------------------------------------------------- */
/* Direct n-body systems and mock streams                                    */
/* ------------------------------------------------------------------------- */

/* DirectNBody.integrate_orbit with DOPRI853 (src/gala/dynamics/nbody/core.py:
 * 166-260 -> direct_nbody_dop853, nbody.pyx:30-115), for n_systems independent
 * systems at once.  Each system is one gala call: dop853_helper
 * (dop853.pyx:90-193) with Fwrapper_direct_nbody (dop853.cpp:990-1006) on
 * nparticles bodies, the first `nbody` of them massive, uround = eps,
 * h0 = t[1] - t[0], one step size and error norm per system.
 *   bodies  DEVICE gx_body (n_systems, nbody): the massive bodies' potentials
 *           (types NULL, KEPLER, HERNQUIST, PLUMMER, MIYAMOTONAGAI,
 *           SPHERICALNFW; any other type yields NaN forces)
 *   w0      DEVICE (n_systems, nparticles, 6): gala's (nparticles, 6) per system
 *   t       DEVICE (ntimes)
 *   nstiff  gala passes -1 (no stiffness test)
 *   w_out   DEVICE (n_systems, n_out, nparticles, 6) with n_out =
 *           (ntimes - 1) / out_stride + 1 if save_all, else (n_systems,
 *           nparticles, 6)
 *   status  DEVICE int32 (n_systems): gala's dop853() code per system
 *   stats   DEVICE int64 (n_systems, 4) or NULL: nfcn, nstep, naccpt, nrejct
 *   queue_counter  DEVICE int64 scratch (zeroed by the call)
 * 1 <= nparticles <= 32 (wider systems: gx_nbody_dop853_wide). */
int gx_nbody_dop853(const gx_potential* pot, const gx_frame* frame, int64_t n_systems,
                    int32_t nparticles, int32_t nbody, const gx_body* bodies,
                    const double* w0, const double* t, int64_t ntimes, double atol,
                    double rtol, int64_t nmax, double dt_max, int64_t nstiff,
                    int32_t save_all, int64_t out_stride, double* w_out, int32_t* status,
                    int64_t* stats, int64_t* queue_counter, void* stream);

/* The release systems of mockstream_dop853 (src/gala/dynamics/mockstream/
 * mockstream.pyx:176-303) for n_streams progenitor systems that share one
 * release grid.  For stream s and release i with particles, one dop853_step
 * call (dop853.pyx:27-75: uround 2.3e-16, nstiff 1, hmax = t_final - t_i,
 * h0 = dt0, no dense output) integrates [the nbody bodies at release i, the
 * particles released at i] from release_t[i] to t_final.
 *   bodies          DEVICE gx_body (n_streams, nbody): progenitor first
 *   nbody_w         DEVICE (n_streams, n_release, nbody, 6): the bodies at each
 *                   release time (gala's nbody dense output on the release grid)
 *   release_t       DEVICE (n_release): gala's stream_t1
 *   release_offset  DEVICE int64 (n_release + 1): prefix sums of gala's nstream;
 *                   the particles of release i are rows
 *                   [release_offset[i], release_offset[i+1]) of a stream, and
 *                   release_offset[n_release] == n_particles (a release whose
 *                   rows fall outside [0, n_particles) or exceed max_per_release
 *                   is not integrated and gets status -1)
 *   max_per_release largest nstream[i]; nbody + max_per_release <= 32
 *   stream_w0       DEVICE (n_streams, n_particles, 6), gala's stream_w0 per stream
 *   dt0             gala's time[1] - time[0] of the release grid
 *   stream_w_out    DEVICE (n_streams, n_particles, 6): the particles at t_final
 *   nbody_w_out     DEVICE (n_streams, nbody, 6) or NULL: the bodies as the last
 *                   release system leaves them (gala's return_nbody_w)
 *   status          DEVICE int32 (n_streams, n_release): dop853() code of each
 *                   release system, 0 where nothing was released (a NaN step
 *                   size ends a system at once with gala's eventual code, -2)
 *   stats           DEVICE int64 (n_streams, n_release, 4) or NULL
 *   queue_counter   DEVICE int64 scratch (zeroed by the call) */
int gx_mockstream_dop853(const gx_potential* pot, const gx_frame* frame, int64_t n_streams,
                         int32_t nbody, const gx_body* bodies, const double* nbody_w,
                         int64_t n_release, const double* release_t,
                         const int64_t* release_offset, int32_t max_per_release,
                         const double* stream_w0, int64_t n_particles, double t_final,
                         double dt0, double atol, double rtol, int64_t nmax,
                         double* stream_w_out, double* nbody_w_out, int32_t* status,
                         int64_t* stats, int64_t* queue_counter, void* stream);

/* The release systems of gx_mockstream_dop853 by DOP853 with FP32 stages and
 * forces and FP64 step control (the arithmetic of gx_dop853_fp32: double-float
 * state, FP64 time / error-norm combination / accept-reject; the particle-body
 * separations from the double-float parts).  Same arguments as
 * gx_mockstream_dop853 without the frame (static frames only); nbody <= 4.
 * Not bit-compatible with gala; tolerances below ~1e-8 relative only shrink the
 * steps.  No gala counterpart beyond mockstream_dop853 itself
 * (src/gala/dynamics/mockstream/mockstream.pyx:176-303). */
int gx_mockstream_dop853_fp32(const gx_potential* pot, int64_t n_streams, int32_t nbody,
                              const gx_body* bodies, const double* nbody_w, int64_t n_release,
                              const double* release_t, const int64_t* release_offset,
                              int32_t max_per_release, const double* stream_w0,
                              int64_t n_particles, double t_final, double dt0, double atol,
                              double rtol, int64_t nmax, double* stream_w_out,
                              double* nbody_w_out, int32_t* status, int64_t* stats,
                              int64_t* queue_counter, void* stream);

/* Release systems wider than a warp (mockstream.pyx:176-303: gala integrates
 * each release -- the bodies at the release time plus every particle released
 * then -- as one dop853_step system, however many particles it holds).  One
 * CTA per listed system, its state in caller-provided device scratch; the error
 * and stiffness sums are fixed-order CTA sums (gala sums sequentially), so the
 * results agree with gala to rounding.  Arguments as gx_mockstream_dop853, plus
 *   systems      DEVICE int64[n_systems]: ids si * n_streams + ss of the
 *                (release si, stream ss) systems to integrate here
 *   max_members  nbody + the largest release among them
 *   scratch      DEVICE buffer of gx_mockstream_wide_scratch_bytes(n_systems,
 *                max_members) bytes
 * Writes the same outputs (particles, the bodies after the last release,
 * status, stats) for those systems only.  dt0 must be non-zero. */
int64_t gx_mockstream_wide_scratch_bytes(int64_t n_systems, int32_t max_members);
int gx_mockstream_dop853_wide(const gx_potential* pot, const gx_frame* frame, int64_t n_streams,
                              int32_t nbody, const gx_body* bodies, const double* nbody_w,
                              int64_t n_release, const double* release_t,
                              const int64_t* release_offset, const double* stream_w0,
                              int64_t n_particles, double t_final, double dt0, double atol,
                              double rtol, int64_t nmax, const int64_t* systems,
                              int64_t n_systems, int32_t max_members, double* scratch,
                              int64_t scratch_bytes, double* stream_w_out, double* nbody_w_out,
                              int32_t* status, int64_t* stats, void* stream);

/* DirectNBody systems of any size: the same call as gx_nbody_dop853
 * (direct_nbody_dop853, nbody.pyx:30-115 -> dop853_helper, dop853.pyx:90-193)
 * for systems too wide for a warp, one CTA per system, its state and
 * dense-output coefficients in caller-provided device scratch of
 * gx_nbody_wide_scratch_bytes(n_systems, nparticles) bytes.  Arguments and
 * outputs as gx_nbody_dop853 without the queue counter.  The error and
 * stiffness sums are fixed-order CTA sums (gala sums sequentially): results
 * agree with gala to rounding. */
int64_t gx_nbody_wide_scratch_bytes(int64_t n_systems, int32_t nparticles);
int gx_nbody_dop853_wide(const gx_potential* pot, const gx_frame* frame, int64_t n_systems,
                         int32_t nparticles, int32_t nbody, const gx_body* bodies, const double* w0,
                         const double* t, int64_t ntimes, double atol, double rtol, int64_t nmax,
                         double dt_max, int64_t nstiff, int32_t save_all, int64_t out_stride,
                         double* scratch, int64_t scratch_bytes, double* w_out, int32_t* status,
                         int64_t* stats, void* stream);

/* MockStreamGenerator.run with output_every: mockstream_dop853_animate
 * (src/gala/dynamics/mockstream/mockstream.pyx:306-440) for n_streams
 * independent streams, one CTA each.  A stream's state holds its bodies and
 * every particle from the start; interval i (t[i-1] -> t[i]) integrates the
 * bodies plus the particles released at t[0..i-1] as one dop853_step system
 * (h0 = dt0, nstiff 1, whole-system error norm), and the particles released at
 * t[i] join after it.
 *   bodies     DEVICE gx_body[n_streams][nbody] (massive first)
 *   nbody_w0   DEVICE double[n_streams][nbody][6], the bodies at t[0]
 *   t          DEVICE double[ntimes], the whole orbit grid; dt0 = t[1] - t[0]
 *   nstream    DEVICE int32[ntimes], particles released at t[i] (zeros allowed;
 *              they sum to n_particles -- an interval whose count would break
 *              that bound reports -1 and the count is clamped)
 *   stream_w0  DEVICE double[n_streams][n_particles][6] in release order
 *   scratch    DEVICE buffer of gx_mockstream_wide_scratch_bytes(n_streams,
 *              nbody + n_particles) bytes
 *   snap       DEVICE double[n_streams][6][n_output][nbody + n_particles] or NULL:
 *              the state at t[0] and after every interval i with
 *              i % output_every == 0 or i == ntimes - 1 (n_output =
 *              gx_mockstream_animate_snapshots(ntimes, output_every)); members
 *              not yet released are NaN, the fill value of gala's HDF5 datasets
 *   w_out      DEVICE double[n_streams][nbody + n_particles][6], the final state
 *   status     DEVICE int32[n_streams][ntimes]: 1 at [0], gala's idid of every
 *              interval after it
 *   stats      DEVICE int64[n_streams][4] or NULL: {nfcn, nstep, naccpt, nrejct}
 *              summed over the intervals
 * Every interval's error and stiffness sums are fixed-order CTA sums (gala sums
 * sequentially): results agree with gala to rounding. */
int64_t gx_mockstream_animate_snapshots(int64_t ntimes, int64_t output_every);
int gx_mockstream_dop853_animate(const gx_potential* pot, const gx_frame* frame, int64_t n_streams,
                                 int32_t nbody, const gx_body* bodies, const double* nbody_w0,
                                 int64_t ntimes, const double* t, double dt0, const int32_t* nstream,
                                 const double* stream_w0, int64_t n_particles, int64_t output_every,
                                 double atol, double rtol, int64_t nmax, double* scratch,
                                 int64_t scratch_bytes, double* snap, double* w_out, int32_t* status,
                                 int64_t* stats, void* stream);

/* The animate mode with FP32 stages and forces and FP64 step control (the
 * arithmetic of gx_mockstream_dop853_fp32: double-float state, FP64 time,
 * error-norm combination and accept/reject, the particle-body separations
 * from the double-float parts).  Same arguments and outputs as
 * gx_mockstream_dop853_animate without the frame (static frames only), and
 * the same scratch size; nbody <= 32.  Not bit-compatible with gala;
 * tolerances below ~1e-8 relative only shrink the steps. */
int gx_mockstream_dop853_animate_fp32(const gx_potential* pot, int64_t n_streams, int32_t nbody,
                                      const gx_body* bodies, const double* nbody_w0, int64_t ntimes,
                                      const double* t, double dt0, const int32_t* nstream,
                                      const double* stream_w0, int64_t n_particles,
                                      int64_t output_every, double atol, double rtol, int64_t nmax,
                                      double* scratch, int64_t scratch_bytes, double* snap,
                                      double* w_out, int32_t* status, int64_t* stats, void* stream);

/* DirectNBody.integrate_orbit with LeapfrogIntegrator: leapfrog_integrate_nbody
 * (src/gala/integrate/cyintegrators/leapfrog.pyx:161-255) for n_systems
 * independent systems of nparticles <= 8 bodies, the first `nbody` massive.  Within
 * a step the bodies are updated in order, each feeling the others at their
 * current positions (c_nbody_gradient_symplectic, cpotential.cpp:418-442).
 * Static frame.  dt = t[1] - t[0] (read from the device array).
 *   w0     DEVICE (n_systems, nparticles, 6)
 *   w_out  DEVICE (n_systems, ntimes, nparticles, 6) if save_all else
 *          (n_systems, nparticles, 6) */
int gx_nbody_leapfrog(const gx_potential* pot, int64_t n_systems, int32_t nparticles,
                      int32_t nbody, const gx_body* bodies, const double* w0, const double* t,
                      int64_t ntimes, int32_t save_all, double* w_out, void* stream);

/* The release systems of mockstream_leapfrog (src/gala/dynamics/mockstream/
 * mockstream.pyx:442-610) for n_streams progenitor systems on one release grid:
 * release i integrates [bodies at release i, its particles] for
 * (int)((t_final - release_t[i]) / dt + 0.5) steps of dt.  Arguments as
 * gx_mockstream_dop853; nbody_w holds the bodies at each release time (gala takes
 * them from the bodies' Leapfrog trajectory on the full grid).  nbody +
 * max_per_release <= 8.  status: 1, 0 where nothing was released, -1 for a
 * release whose rows fall outside the particle array. */
int gx_mockstream_leapfrog(const gx_potential* pot, int64_t n_streams, int32_t nbody,
                           const gx_body* bodies, const double* nbody_w, int64_t n_release,
                           const double* release_t, const int64_t* release_offset,
                           int32_t max_per_release, const double* stream_w0,
                           int64_t n_particles, double t_final, double dt,
                           double* stream_w_out, double* nbody_w_out, int32_t* status,
                           void* stream);

/* The same release systems in FP32 with compensated (Kahan) positions and
 * velocities and FP32 forces (no gala counterpart: the fast form; closed-form
 * components only).  Identical arguments. */
int gx_mockstream_leapfrog_fp32(const gx_potential* pot, int64_t n_streams, int32_t nbody,
                                const gx_body* bodies, const double* nbody_w, int64_t n_release,
                                const double* release_t, const int64_t* release_offset,
                                int32_t max_per_release, const double* stream_w0,
                                int64_t n_particles, double t_final, double dt,
                                double* stream_w_out, double* nbody_w_out, int32_t* status,
                                void* stream);

/* Orbit.pericenter / apocenter / zmax statistics (src/gala/dynamics/orbit.py:
 * 391-656) of N orbits stored as (6, ntimes, N) snapshots at times t, in one
 * pass: per orbit and kind (0 pericentre, 1 apocentre, 2 z maximum) the number
 * of interior strict extrema of r or |z|, each refined by the vertex of the
 * parabola through its three samples (approximate != 0: the sample itself),
 * and their sum (in increasing time), minimum and maximum.  A grid with
 * t[ntimes-1] < t[0] is scanned from the end, as gala reverses it.
 *   count             DEVICE int32 (3, N)
 *   sum, vmin, vmax   DEVICE double (3, N); vmin and vmax are NaN where
 *                     count is 0
 *   vals, times       DEVICE double (3, N, keep): the first `keep` extrema, or
 *                     NULL with keep = 0
 * ntimes must be below 2^31. */
int gx_orbit_extrema(const double* w, const double* t, int64_t ntimes, int64_t n,
                     int32_t approximate, int32_t keep, int32_t* count, double* sum,
                     double* vmin, double* vmax, double* vals, double* times, void* stream);

/* FardalStreamDF._sample (src/gala/dynamics/mockstream/df.pyx:363-457) with
 * get_rj_vj_R (:61-92) and transform_from_sat (:94-106) for n_streams
 * progenitor orbits on one time grid; the Jacobi radius uses c_d2_dr2
 * (cpotential.cpp:346-371) of `pot`.
 *   prog_w          DEVICE (n_streams, ntimes, row_stride): progenitor x, v in
 *                   the first six entries of each row
 *   prog_m          DEVICE (n_streams, ntimes): progenitor mass
 *   t               DEVICE (ntimes)
 *   release_offset  DEVICE int64 (ntimes + 1): first particle row of each time;
 *                   a time releases (lead + trail) * n_i rows, trailing first
 *   draws           DEVICE (n_streams, n_particles, 4): the four normal draws of
 *                   each particle (kx, kz, kvt, kvz) in gala's order
 *   G               the gravitational constant of `pot`
 *   w_out           DEVICE (n_streams, n_particles, 6) */
int gx_fardal_sample(const gx_potential* pot, int64_t n_streams, int64_t ntimes,
                     const double* prog_w, int64_t row_stride, const double* prog_m,
                     const double* t, const int64_t* release_offset, int64_t n_particles,
                     const double* draws, double G, int32_t lead, int32_t trail,
                     int32_t gala_modified, double* w_out, void* stream);

/* The same release sampler for the other stream DFs of gala (df.pyx): kind 0
 * FardalStreamDF as above (4 draws per particle; the streakline DF is kind 0
 * with draws 1, 0, 1, 0), kind 1 LagrangeCloudStreamDF (df.pyx:460-555; 3
 * draws: the satellite-frame velocity, each normal(0, v_disp)), kind 2
 * ChenStreamDF (df.pyx:557-703; 6 draws: one multivariate_normal sample of
 * r, phi, theta, v, alpha, beta in degrees).  draws is DEVICE (n_streams,
 * n_particles, 4 | 3 | 6); the other arguments are those of gx_fardal_sample. */
int gx_stream_sample(const gx_potential* pot, int64_t n_streams, int64_t ntimes,
                     const double* prog_w, int64_t row_stride, const double* prog_m,
                     const double* t, const int64_t* release_offset, int64_t n_particles,
                     int32_t kind, const double* draws, double G, int32_t lead, int32_t trail,
                     int32_t gala_modified, double* w_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GALA_GB300_H */
