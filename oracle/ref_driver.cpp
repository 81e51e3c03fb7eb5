/*
 * ORACLE (test infrastructure only): a driver around gala's OWN compiled C/C++
 * (cpotential.cpp, builtin_potentials.cpp, builtin_frames.cpp, cframe.cpp,
 * chamiltonian.cpp, dopri/dop853.cpp), built by oracle/Makefile straight from the
 * gala sources into oracle/_ref/libgalaref.so.  It is used to pin the C
 * restatement (gx_oracle.c) and to generate the golden fixtures in tests/golden/.
 *
 * What this file adds is only the glue that gala's Cython layer provides:
 *   - a CPotential built the way CPotentialWrapper.init / CCompositePotentialWrapper
 *     build it (src/gala/potential/potential/cpotential.pyx:57-102,
 *     ccompositepotential.pyx:27-67), from the gx_potential descriptor;
 *   - the Leapfrog and Ruth4 driver loops of leapfrog.pyx:24-121 and
 *     ruth4.pyx:24-113 (Cython that cannot be compiled without gala's Python
 *     package), calling gala's c_gradient;
 *   - dop853_integrate_hamiltonian / dop853_helper (dop853.pyx:90-250): one call
 *     of gala's dop853() per batch of nbatch orbits with exactly that argument
 *     list, Fwrapper_T as the right-hand side and a dense-output state;
 *   - direct_nbody_dop853 (nbody.pyx:30-115) and mockstream_dop853 with
 *     dop853_step (mockstream.pyx:176-303, dop853.pyx:27-75): gala's dop853()
 *     with Fwrapper_direct_nbody and an array of per-body CPotentials built as
 *     the particle potentials are (NullWrapper sets `null = 1`,
 *     builtin/cybuiltin.pyx:365-372);
 *   - leapfrog_integrate_nbody (leapfrog.pyx:126-255) and the release loop of
 *     mockstream_leapfrog (mockstream.pyx:442-610): the Cython loops restated
 *     around gala's c_gradient and c_nbody_gradient_symplectic.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "potential/src/cpotential.h"
#include "frame/src/cframe.h"
#include "hamiltonian/src/chamiltonian.h"
#include "dopri/dop853.h"
#include "potential/builtin/builtin_potentials.h"
#include "frame/builtin/builtin_frames.h"

#include "../include/gala_gb300.h"

namespace {

struct RefPot {
    CPotential *cp;
    CFrameType cf;
    double frame_params[3];
};

bool set_funcs(CPotential *cp, int i, int type) {
    switch (type) {
    case GX_POT_NULL:
        cp->value[i] = null_value; cp->density[i] = null_density;
        cp->gradient[i] = null_gradient; cp->hessian[i] = null_hessian;
        return true;
    case GX_POT_KEPLER:
        cp->value[i] = kepler_value; cp->density[i] = kepler_density;
        cp->gradient[i] = kepler_gradient; cp->hessian[i] = kepler_hessian;
        return true;
    case GX_POT_HERNQUIST:
        cp->value[i] = hernquist_value; cp->density[i] = hernquist_density;
        cp->gradient[i] = hernquist_gradient; cp->hessian[i] = hernquist_hessian;
        return true;
    case GX_POT_PLUMMER:
        cp->value[i] = plummer_value; cp->density[i] = plummer_density;
        cp->gradient[i] = plummer_gradient; cp->hessian[i] = plummer_hessian;
        return true;
    case GX_POT_MIYAMOTONAGAI:
        cp->value[i] = miyamotonagai_value; cp->density[i] = miyamotonagai_density;
        cp->gradient[i] = miyamotonagai_gradient; cp->hessian[i] = miyamotonagai_hessian;
        return true;
    case GX_POT_SPHERICALNFW:
        cp->value[i] = sphericalnfw_value; cp->density[i] = sphericalnfw_density;
        cp->gradient[i] = sphericalnfw_gradient; cp->hessian[i] = sphericalnfw_hessian;
        return true;
    case GX_POT_FLATTENEDNFW:
        cp->value[i] = flattenednfw_value; cp->density[i] = nan_density;
        cp->gradient[i] = flattenednfw_gradient; cp->hessian[i] = flattenednfw_hessian;
        return true;
    case GX_POT_TRIAXIALNFW:
        cp->value[i] = triaxialnfw_value; cp->density[i] = nan_density;
        cp->gradient[i] = triaxialnfw_gradient; cp->hessian[i] = triaxialnfw_hessian;
        return true;
    default:
        return false; /* SCF needs GSL inside gala: not buildable here */
    }
}

bool build(const gx_potential *pot, const gx_frame *fr, RefPot *rp) {
    const int nc = pot->n_components;
    rp->cp = allocate_cpotential(nc > 0 ? nc : 1);
    CPotential *cp = rp->cp;
    cp->n_dim = 3;
    cp->null = 0;
    for (int i = 0; i < nc; i++) {
        const gx_component *c = &pot->components[i];
        if (!set_funcs(cp, i, c->type)) return false;
        cp->n_params[i] = c->n_params;
        cp->parameters[i] = const_cast<double *>(pot->params + c->param_offset);
        cp->q0[i] = const_cast<double *>(c->q0);
        cp->R[i] = const_cast<double *>(c->R);
        cp->state[i] = NULL;
        cp->do_shift_rotate[i] = c->do_shift_rotate;
    }
    if (fr == NULL || fr->type == GX_FRAME_STATIC) {
        rp->cf.energy = (energyfunc)static_frame_hamiltonian;
        rp->cf.gradient = (gradientfunc)static_frame_gradient;
        rp->cf.hessian = (hessianfunc)static_frame_hessian;
        rp->cf.n_params = 0;
        rp->frame_params[0] = rp->frame_params[1] = rp->frame_params[2] = 0.;
    } else {
        rp->cf.energy = (energyfunc)constant_rotating_frame_3d_hamiltonian;
        rp->cf.gradient = (gradientfunc)constant_rotating_frame_3d_gradient;
        rp->cf.hessian = (hessianfunc)constant_rotating_frame_3d_hessian;
        rp->cf.n_params = 3;
        memcpy(rp->frame_params, fr->params, sizeof(rp->frame_params));
    }
    rp->cf.parameters = rp->frame_params;
    return true;
}

void release(RefPot *rp) {
    if (rp->cp) free_cpotential(rp->cp);
    rp->cp = NULL;
}

typedef void (*range_fn)(void *ctx, int64_t lo, int64_t hi);
struct Pool {
    range_fn fn;
    void *ctx;
    int64_t n, chunk, next;
    pthread_mutex_t mu;
};

void *worker(void *arg) {
    Pool *P = (Pool *)arg;
    for (;;) {
        pthread_mutex_lock(&P->mu);
        int64_t lo = P->next;
        P->next += P->chunk;
        pthread_mutex_unlock(&P->mu);
        if (lo >= P->n) break;
        P->fn(P->ctx, lo, lo + P->chunk < P->n ? lo + P->chunk : P->n);
    }
    return NULL;
}

void parallel_for(int nthreads, int64_t n, int64_t chunk, range_fn fn, void *ctx) {
    if (nthreads <= 1 || n <= chunk) {
        fn(ctx, 0, n);
        return;
    }
    Pool P;
    P.fn = fn; P.ctx = ctx; P.n = n; P.chunk = chunk; P.next = 0;
    pthread_mutex_init(&P.mu, NULL);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, worker, &P);
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&P.mu);
}

struct FixedCtx {
    const gx_potential *pot;
    const double *w0, *t;
    int64_t n, ntimes;
    int save_all, method;
    double *w_out;
    int failed;
};

/* leapfrog.pyx:54-121 / ruth4.pyx:37-113 on orbits [lo, hi): the Cython loops,
 * restated, each step calling gala's c_gradient over the chunk. */
void fixed_chunk(void *vctx, int64_t lo, int64_t hi) {
    FixedCtx *C = (FixedCtx *)vctx;
    RefPot rp;
    if (!build(C->pot, NULL, &rp)) { C->failed = 1; release(&rp); return; }
    CPotential *cp = rp.cp;
    const int64_t n = C->n, ntimes = C->ntimes;
    const size_t m = (size_t)(hi - lo);
    const double dt = C->t[1] - C->t[0];
    double *tmp_w = (double *)malloc(sizeof(double) * 6 * m);
    double *v_jm1_2 = (double *)calloc(3 * m, sizeof(double));
    double *grad = (double *)calloc(3 * m, sizeof(double));
    for (int k = 0; k < 6; k++)
        for (size_t i = 0; i < m; i++) tmp_w[k * m + i] = C->w0[k * n + lo + i];
    if (C->save_all)
        for (int k = 0; k < 6; k++)
            for (size_t i = 0; i < m; i++) C->w_out[(k * ntimes + 0) * n + lo + i] = tmp_w[k * m + i];
    if (C->method == 0) {
        double *x = tmp_w, *v = tmp_w + 3 * m;
        c_gradient(cp, m, C->t[0], x, grad);
        for (int k = 0; k < 3; k++)
            for (size_t i = 0; i < m; i++) v_jm1_2[i + k * m] = v[i + k * m] - grad[i + k * m] * dt / 2.;
        for (int64_t j = 1; j < ntimes; j++) {
            memset(grad, 0, sizeof(double) * 3 * m);
            for (int k = 0; k < 3; k++)
                for (size_t i = 0; i < m; i++) x[i + k * m] = x[i + k * m] + v_jm1_2[i + k * m] * dt;
            c_gradient(cp, m, C->t[j], x, grad);
            for (int k = 0; k < 3; k++)
                for (size_t i = 0; i < m; i++) {
                    v[i + k * m] = v_jm1_2[i + k * m] - grad[i + k * m] * dt / 2.;
                    v_jm1_2[i + k * m] = v_jm1_2[i + k * m] - grad[i + k * m] * dt;
                }
            if (C->save_all)
                for (int k = 0; k < 6; k++)
                    for (size_t i = 0; i < m; i++) C->w_out[(k * ntimes + j) * n + lo + i] = tmp_w[k * m + i];
        }
    } else {
        const double two_13 = pow(2., 1. / 3.);
        const double cs[4] = {1. / (2. * (2. - two_13)), (1. - two_13) / (2. * (2. - two_13)),
                              (1. - two_13) / (2. * (2. - two_13)), 1. / (2. * (2. - two_13))};
        const double ds[4] = {0., 1. / (2. - two_13), -two_13 / (2. - two_13), 1. / (2. - two_13)};
        double *w = tmp_w;
        for (int64_t j = 1; j < ntimes; j++) {
            memset(grad, 0, sizeof(double) * 3 * m);
            for (int s = 0; s < 4; s++) {
                c_gradient(cp, m, C->t[j], w, grad);
                for (int k = 0; k < 3; k++)
                    for (size_t i = 0; i < m; i++) {
                        w[(3 + k) * m + i] = w[(3 + k) * m + i] - ds[s] * grad[k * m + i] * dt;
                        w[k * m + i] = w[k * m + i] + cs[s] * w[(3 + k) * m + i] * dt;
                    }
            }
            if (C->save_all)
                for (int k = 0; k < 6; k++)
                    for (size_t i = 0; i < m; i++) C->w_out[(k * ntimes + j) * n + lo + i] = tmp_w[k * m + i];
        }
    }
    if (!C->save_all)
        for (int k = 0; k < 6; k++)
            for (size_t i = 0; i < m; i++) C->w_out[k * n + lo + i] = tmp_w[k * m + i];
    free(tmp_w);
    free(v_jm1_2);
    free(grad);
    release(&rp);
}

struct DopCtx {
    const gx_potential *pot;
    const gx_frame *fr;
    const double *w0, *t;
    int64_t n, ntimes, nmax, nstiff;
    double atol, rtol, dt_max;
    int save_all, nbatch;
    double *w_out;
    int32_t *status;
};

/* dop853_integrate_hamiltonian's batch loop (dop853.pyx:228-245) calling
 * dop853_helper (:90-193) for batches [blo, bhi). */
void dop_chunk(void *vctx, int64_t blo, int64_t bhi) {
    DopCtx *C = (DopCtx *)vctx;
    RefPot rp;
    if (!build(C->pot, C->fr, &rp)) {
        for (int64_t b = blo; b < bhi; b++) C->status[b] = -100;
        release(&rp);
        return;
    }
    const int64_t n = C->n, ntimes = C->ntimes;
    for (int64_t b = blo; b < bhi; b++) {
        const int64_t i0 = b * C->nbatch;
        const unsigned nb = (unsigned)((i0 + C->nbatch <= n) ? C->nbatch : n - i0);
        const unsigned size = 6 * nb;
        double *w = (double *)malloc(sizeof(double) * size);
        for (int k = 0; k < 6; k++)
            for (unsigned j = 0; j < nb; j++) w[k * nb + j] = C->w0[k * n + i0 + j];
        double *output_w = NULL;
        Dop853DenseState *state = NULL;
        unsigned nrdens = 0;
        if (C->save_all) {
            output_w = (double *)malloc(sizeof(double) * size * (size_t)ntimes);
            state = dop853_dense_state_alloc(size, size);
            nrdens = size;
        }
        double rtol = C->rtol, atol = C->atol;
        int res = dop853(size, (FcnEqDiff)Fwrapper_T, rp.cp, &rp.cf, nb, 0, NULL, C->t[0], w,
                         C->t[ntimes - 1], &rtol, &atol, 0, NULL, 0, NULL,
                         2.220446049250313e-16, 0.0, 0.0, 0.0, 0.0, C->dt_max, C->t[1] - C->t[0],
                         (long)C->nmax, 1, (long)C->nstiff, nrdens, NULL, 0, state,
                         const_cast<double *>(C->t), (int)ntimes, output_w);
        C->status[b] = res;
        if (C->save_all) {
            for (int64_t s = 0; s < ntimes; s++)
                for (int k = 0; k < 6; k++)
                    for (unsigned j = 0; j < nb; j++)
                        C->w_out[(k * ntimes + s) * n + i0 + j] = output_w[(s * 6 + k) * nb + j];
            free(output_w);
            dop853_dense_state_free(state, size);
        } else {
            for (int k = 0; k < 6; k++)
                for (unsigned j = 0; j < nb; j++) C->w_out[k * n + i0 + j] = w[k * nb + j];
        }
        free(w);
    }
    release(&rp);
}

/* A body's CPotential: one component with its own parameters (q0 and
 * do_shift_rotate are set by c_nbody_acceleration), or gala's NullPotential. */
struct RefBody {
    CPotential *cp;
    double q0[3];
    double R[9];
    double params[7];
};

bool build_body(const gx_body *b, RefBody *rb) {
    rb->cp = allocate_cpotential(1);
    CPotential *cp = rb->cp;
    cp->n_dim = 3;
    if (!set_funcs(cp, 0, b->type)) return false;
    cp->null = (b->type == GX_POT_NULL) ? 1 : 0;
    memcpy(rb->params, b->params, sizeof(rb->params));
    for (int k = 0; k < 3; k++) rb->q0[k] = 0.;
    for (int k = 0; k < 9; k++) rb->R[k] = (k % 4 == 0) ? 1. : 0.;
    cp->n_params[0] = b->n_params;
    cp->parameters[0] = rb->params;
    cp->q0[0] = rb->q0;
    cp->R[0] = rb->R;
    cp->state[0] = NULL;
    cp->do_shift_rotate[0] = 0;
    return true;
}

/* direct_nbody_dop853's dop853_helper call (nbody.pyx:99-107, dop853.pyx:157-182). */
int nbody_helper(RefPot &rp, CPotential **pots, int nparticles, int nbody, double *w, const double *t,
                 int64_t ntimes, double atol, double rtol, int64_t nmax, double dt_max, int64_t nstiff,
                 int save_all, double *output_w) {
    const unsigned size = 6 * (unsigned)nparticles;
    Dop853DenseState *state = NULL;
    unsigned nrdens = 0;
    if (save_all) {
        state = dop853_dense_state_alloc(size, size);
        nrdens = size;
    }
    int res = dop853(size, (FcnEqDiff)Fwrapper_direct_nbody, rp.cp, &rp.cf, (unsigned)nparticles, (unsigned)nbody,
                     (void *)pots, t[0], w, t[ntimes - 1], &rtol, &atol, 0, NULL, 0, NULL,
                     2.220446049250313e-16, 0.0, 0.0, 0.0, 0.0, dt_max, t[1] - t[0], (long)nmax, 1,
                     (long)nstiff, nrdens, NULL, 0, state, const_cast<double *>(t), (int)ntimes,
                     save_all ? output_w : NULL);
    if (state) dop853_dense_state_free(state, size);
    return res;
}

/* c_init_velocity_nbody / c_leapfrog_step_nbody (leapfrog.pyx:126-158) around
 * gala's c_gradient and c_nbody_gradient_symplectic. */
void ref_lf_init(CPotential *cp, CPotential **pots, int nbody, double *w, int i, double t, double dt, double *vh) {
    double grad[3] = {0., 0., 0.};
    c_gradient(cp, 1, t, w + 6 * i, grad);
    c_nbody_gradient_symplectic(pots, t, w + 6 * i, w, nbody, i, 3, grad);
    for (int k = 0; k < 3; k++) vh[3 * i + k] = w[6 * i + 3 + k] - grad[k] * dt / 2.;
}

void ref_lf_step(CPotential *cp, CPotential **pots, int nbody, double *w, int i, double t, double dt, double *vh) {
    double *x = w + 6 * i, *v = x + 3, *h = vh + 3 * i;
    for (int k = 0; k < 3; k++) x[k] = x[k] + h[k] * dt;
    double grad[3] = {0., 0., 0.};
    c_gradient(cp, 1, t, x, grad);
    c_nbody_gradient_symplectic(pots, t, x, w, nbody, i, 3, grad);
    for (int k = 0; k < 3; k++) {
        v[k] = h[k] - grad[k] * dt / 2.;
        h[k] = h[k] - grad[k] * dt;
    }
}

} // namespace

extern "C" {

/* c_gradient over N points, q (3, N) -> grad (3, N). Returns 0, or -1 when a
 * component type has no gala build here (SCF needs GSL). */
int ref_gradient(const gx_potential *pot, int64_t N, double t, const double *q, double *grad) {
    RefPot rp;
    if (!build(pot, NULL, &rp)) { release(&rp); return -1; }
    c_gradient(rp.cp, (size_t)N, t, const_cast<double *>(q), grad);
    release(&rp);
    return 0;
}

/* c_potential / c_density at each column of q (3, N). */
int ref_potential_value_n(const gx_potential *pot, double t, const double *q, int64_t N, double *out) {
    RefPot rp;
    if (!build(pot, NULL, &rp)) { release(&rp); return -1; }
    for (int64_t i = 0; i < N; i++) {
        double qi[3] = {q[i], q[N + i], q[2 * N + i]};
        out[i] = c_potential(rp.cp, t, qi);
    }
    release(&rp);
    return 0;
}

int ref_potential_density_n(const gx_potential *pot, double t, const double *q, int64_t N, double *out) {
    RefPot rp;
    if (!build(pot, NULL, &rp)) { release(&rp); return -1; }
    for (int64_t i = 0; i < N; i++) {
        double qi[3] = {q[i], q[N + i], q[2 * N + i]};
        out[i] = c_density(rp.cp, t, qi);
    }
    release(&rp);
    return 0;
}

/* hamiltonian_gradient_T over w (6, N) -> f (6, N). */
int ref_hamiltonian_gradient(const gx_potential *pot, const gx_frame *fr, int64_t N, double t,
                             const double *w, double *f) {
    RefPot rp;
    if (!build(pot, fr, &rp)) { release(&rp); return -1; }
    hamiltonian_gradient_T(rp.cp, &rp.cf, (size_t)N, t, const_cast<double *>(w), f);
    release(&rp);
    return 0;
}

/* leapfrog (method 0) / ruth4 (method 1) integrate_hamiltonian. */
int ref_fixed_integrate(const gx_potential *pot, int method, const double *w0, int64_t n,
                        const double *t, int64_t ntimes, int save_all, double *w_out, int nthreads) {
    FixedCtx C = {pot, w0, t, n, ntimes, save_all, method, w_out, 0};
    int64_t chunk = 256;
    if (nthreads > 1 && n / nthreads < chunk) chunk = (n + nthreads - 1) / nthreads;
    if (chunk < 1) chunk = 1;
    parallel_for(nthreads, n, chunk, fixed_chunk, &C);
    return C.failed ? -1 : 0;
}

/* dop853_integrate_hamiltonian with gala's full-grid dense output. */
int ref_dop853_integrate(const gx_potential *pot, const gx_frame *fr, const double *w0, int64_t n,
                         const double *t, int64_t ntimes, double atol, double rtol, int64_t nmax,
                         double dt_max, int64_t nstiff, int save_all, int nbatch, double *w_out,
                         int32_t *status, int nthreads) {
    DopCtx C;
    C.pot = pot; C.fr = fr; C.w0 = w0; C.t = t; C.n = n; C.ntimes = ntimes;
    C.nmax = nmax; C.nstiff = nstiff; C.atol = atol; C.rtol = rtol; C.dt_max = dt_max;
    C.save_all = save_all; C.nbatch = nbatch; C.w_out = w_out; C.status = status;
    parallel_for(nthreads, (n + nbatch - 1) / nbatch, 1, dop_chunk, &C);
    return 0;
}

/* direct_nbody_dop853 on one system: w0 (nparticles, 6), bodies (nparticles)
 * with the massive ones first (nbody of them); w_out (ntimes, nparticles, 6)
 * if save_all, else (nparticles, 6).  Returns gala's idid or -100 when a body
 * type cannot be built. */
int ref_nbody_dop853(const gx_potential *pot, const gx_frame *fr, int nparticles, int nbody, const gx_body *bodies,
                     const double *w0, const double *t, int64_t ntimes, double atol, double rtol, int64_t nmax,
                     double dt_max, int64_t nstiff, int save_all, double *w_out) {
    RefPot rp;
    if (!build(pot, fr, &rp)) { release(&rp); return -100; }
    RefBody *rb = (RefBody *)calloc((size_t)nparticles, sizeof(RefBody));
    CPotential **pots = (CPotential **)malloc(sizeof(CPotential *) * (size_t)nparticles);
    int ok = 1;
    for (int i = 0; i < nparticles; i++) {
        if (!build_body(&bodies[i], &rb[i])) ok = 0;
        pots[i] = rb[i].cp;
    }
    int res = -100;
    if (ok) {
        double *w = (double *)malloc(sizeof(double) * 6 * (size_t)nparticles);
        memcpy(w, w0, sizeof(double) * 6 * (size_t)nparticles);
        res = nbody_helper(rp, pots, nparticles, nbody, w, t, ntimes, atol, rtol, nmax, dt_max, nstiff, save_all,
                           w_out);
        if (!save_all) memcpy(w_out, w, sizeof(double) * 6 * (size_t)nparticles);
        free(w);
    }
    for (int i = 0; i < nparticles; i++)
        if (rb[i].cp) free_cpotential(rb[i].cp);
    free(rb);
    free(pots);
    release(&rp);
    return res;
}

/* mockstream_dop853 (mockstream.pyx:176-303) for one progenitor system, same
 * arguments and outputs as the oracle's orc_mockstream_dop853.  The body
 * potentials of the released particles are gala's NullPotential. */
int ref_mockstream_dop853(const gx_potential *pot, const gx_frame *fr, int nbodies, const gx_body *bodies,
                          const double *nbody_w0, const double *time, int64_t ntimes, const double *stream_w0,
                          const double *stream_t1, double tfinal, const int32_t *nstream, double atol, double rtol,
                          int64_t nmax, double dt_max, int64_t nstiff, double *nbody_w_final,
                          double *stream_w_final, int32_t *status) {
    RefPot rp;
    if (!build(pot, fr, &rp)) { release(&rp); return -100; }
    int64_t total = 0;
    int maxn = 0;
    for (int64_t i = 0; i < ntimes; i++) {
        total += nstream[i];
        maxn = nstream[i] > maxn ? nstream[i] : maxn;
    }
    const int64_t total_bodies = nbodies + total;
    RefBody *rb = (RefBody *)calloc((size_t)nbodies + 1, sizeof(RefBody));
    CPotential **pots = (CPotential **)malloc(sizeof(CPotential *) * (size_t)total_bodies);
    int ok = 1;
    for (int i = 0; i < nbodies; i++) {
        if (!build_body(&bodies[i], &rb[i])) ok = 0;
        pots[i] = rb[i].cp;
    }
    gx_body null_body;
    memset(&null_body, 0, sizeof(null_body));
    null_body.type = GX_POT_NULL;
    if (!build_body(&null_body, &rb[nbodies])) ok = 0;
    for (int64_t i = nbodies; i < total_bodies; i++) pots[i] = rb[nbodies].cp;
    int res = -100;
    if (ok) {
        /* the bodies first, with dense output on `time` (mockstream.pyx:245-255) */
        double *nbody_w = (double *)malloc(sizeof(double) * (size_t)ntimes * 6 * (size_t)nbodies);
        double *w0c = (double *)malloc(sizeof(double) * 6 * (size_t)nbodies);
        memcpy(w0c, nbody_w0, sizeof(double) * 6 * (size_t)nbodies);
        res = nbody_helper(rp, pots, nbodies, nbodies, w0c, time, ntimes, atol, rtol, nmax, dt_max, nstiff, 1,
                           nbody_w);
        free(w0c);
        if (res >= 0) {
            res = 0;
            const double dt0 = time[1] - time[0];
            double *w_tmp = (double *)malloc(sizeof(double) * 6 * (size_t)(nbodies + maxn));
            int64_t n = 0;
            for (int64_t i = 0; i < ntimes; i++) {
                status[i] = 0;
                if (nstream[i] == 0) continue;
                memcpy(w_tmp, nbody_w + (size_t)i * 6 * (size_t)nbodies, sizeof(double) * 6 * (size_t)nbodies);
                memcpy(w_tmp + 6 * nbodies, stream_w0 + 6 * n, sizeof(double) * 6 * (size_t)nstream[i]);
                /* dop853_step (dop853.pyx:27-75): its exact argument list */
                double rt = rtol, at = atol;
                const unsigned nsys = (unsigned)(nbodies + nstream[i]);
                status[i] = dop853(6 * nsys, (FcnEqDiff)Fwrapper_direct_nbody, rp.cp, &rp.cf, nsys,
                                   (unsigned)nbodies, (void *)pots, stream_t1[i], w_tmp, tfinal, &rt, &at, 0, NULL,
                                   0, NULL, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, dt0, (long)nmax, 0, 1, 0, NULL, 0, NULL,
                                   NULL, 0, NULL);
                memcpy(stream_w_final + 6 * n, w_tmp + 6 * nbodies, sizeof(double) * 6 * (size_t)nstream[i]);
                memcpy(nbody_w_final, w_tmp, sizeof(double) * 6 * (size_t)nbodies);
                n += nstream[i];
            }
            free(w_tmp);
        }
        free(nbody_w);
    }
    for (int i = 0; i <= nbodies; i++)
        if (rb[i].cp) free_cpotential(rb[i].cp);
    free(rb);
    free(pots);
    release(&rp);
    return res;
}

/* mockstream_dop853_animate (mockstream.pyx:306-440) for one progenitor system:
 * gala's dop853() on the growing system, interval by interval, with
 * dop853_step's argument list; the same arguments and outputs as the oracle's
 * orc_mockstream_dop853_animate (stats are not kept). */
int ref_mockstream_dop853_animate(const gx_potential *pot, const gx_frame *fr, int nbodies, const gx_body *bodies,
                                  const double *nbody_w0, const double *t, int64_t ntimes, const double *stream_w0,
                                  const int32_t *nstream, int64_t output_every, double atol, double rtol,
                                  int64_t nmax, double *snap, double *snap_t, double *w_final, int32_t *status) {
    if (ntimes < 2 || nbodies < 1 || output_every < 1) return -1;
    RefPot rp;
    if (!build(pot, fr, &rp)) { release(&rp); return -100; }
    int64_t ntot = 0;
    for (int64_t i = 0; i < ntimes; i++) ntot += nstream[i];
    const int64_t all = nbodies + ntot;
    RefBody *rb = (RefBody *)calloc((size_t)nbodies, sizeof(RefBody));
    CPotential **pots = (CPotential **)malloc(sizeof(CPotential *) * (size_t)nbodies);
    int ok = 1;
    for (int i = 0; i < nbodies; i++) {
        if (!build_body(&bodies[i], &rb[i])) ok = 0;
        pots[i] = rb[i].cp;
    }
    int res = -100;
    if (ok) {
        double *w = w_final;
        memcpy(w, nbody_w0, sizeof(double) * 6 * (size_t)nbodies);
        memcpy(w + 6 * nbodies, stream_w0, sizeof(double) * 6 * (size_t)ntot);
        const double dt0 = t[1] - t[0];
        int64_t n = nstream[0], j = 0;
        auto snapshot = [&](int64_t live) {
            double *dst = snap + (size_t)j * 6 * (size_t)all;
            for (int64_t k = 0; k < 6 * all; k++) dst[k] = (k < 6 * live) ? w[k] : NAN;
        };
        snapshot(nbodies + n);
        snap_t[j++] = t[0];
        status[0] = 1;
        for (int64_t i = 1; i < ntimes; i++) {
            double rt = rtol, at = atol;
            const unsigned nsys = (unsigned)(nbodies + n);
            status[i] = dop853(6 * nsys, (FcnEqDiff)Fwrapper_direct_nbody, rp.cp, &rp.cf, nsys, (unsigned)nbodies,
                               (void *)pots, t[i - 1], w, t[i], &rt, &at, 0, NULL, 0, NULL, 0.0, 0.0, 0.0, 0.0,
                               0.0, 0.0, dt0, (long)nmax, 0, 1, 0, NULL, 0, NULL, NULL, 0, NULL);
            n += nstream[i];
            if (i % output_every == 0 || i == ntimes - 1) {
                snapshot(nbodies + n);
                snap_t[j++] = t[i];
            }
        }
        res = (int)j;
    }
    for (int i = 0; i < nbodies; i++)
        if (rb[i].cp) free_cpotential(rb[i].cp);
    free(rb);
    free(pots);
    release(&rp);
    return res;
}

/* c_d2_dr2 (cpotential.cpp:346-371) at N points q (N, 3). */
int ref_d2_dr2_n(const gx_potential *pot, double t, const double *q, int64_t N, double *out) {
    RefPot rp;
    if (!build(pot, NULL, &rp)) { release(&rp); return -1; }
    double eps[3];
    for (int64_t i = 0; i < N; i++) out[i] = c_d2_dr2(rp.cp, t, const_cast<double *>(q + 3 * i), eps);
    release(&rp);
    return 0;
}

/* leapfrog_integrate_nbody (leapfrog.pyx:161-255): bodies (n) with the massive
 * ones first (nbody of them), w0 (n, 6), w_out (ntimes, n, 6) or (n, 6). */
int ref_leapfrog_nbody(const gx_potential *pot, int n, int nbody, const gx_body *bodies, const double *w0,
                       const double *t, int64_t ntimes, int save_all, double *w_out) {
    RefPot rp;
    if (!build(pot, NULL, &rp)) { release(&rp); return -100; }
    RefBody *rb = (RefBody *)calloc((size_t)n, sizeof(RefBody));
    CPotential **pots = (CPotential **)malloc(sizeof(CPotential *) * (size_t)n);
    int ok = 1;
    for (int i = 0; i < n; i++) {
        if (!build_body(&bodies[i], &rb[i])) ok = 0;
        pots[i] = rb[i].cp;
    }
    if (ok) {
        const double dt = t[1] - t[0];
        double *w = (double *)malloc(sizeof(double) * 6 * (size_t)n);
        double *vh = (double *)calloc(3 * (size_t)n, sizeof(double));
        memcpy(w, w0, sizeof(double) * 6 * (size_t)n);
        if (save_all) memcpy(w_out, w0, sizeof(double) * 6 * (size_t)n);
        for (int i = 0; i < n; i++) ref_lf_init(rp.cp, pots, nbody, w, i, t[0], dt, vh);
        for (int64_t j = 1; j < ntimes; j++) {
            for (int i = 0; i < n; i++) ref_lf_step(rp.cp, pots, nbody, w, i, t[j], dt, vh);
            if (save_all) memcpy(w_out + (size_t)j * 6 * (size_t)n, w, sizeof(double) * 6 * (size_t)n);
        }
        if (!save_all) memcpy(w_out, w, sizeof(double) * 6 * (size_t)n);
        free(w);
        free(vh);
    }
    for (int i = 0; i < n; i++)
        if (rb[i].cp) free_cpotential(rb[i].cp);
    free(rb);
    free(pots);
    release(&rp);
    return ok ? 0 : -100;
}

/* mockstream_leapfrog (mockstream.pyx:442-610) for one progenitor system; the
 * same arguments and outputs as the oracle's orc_mockstream_leapfrog. */
int ref_mockstream_leapfrog(const gx_potential *pot, int nbodies, const gx_body *bodies, const double *nbody_w0,
                            const double *full_time, int64_t nfull, const double *stream_w0, const double *stream_t1,
                            int64_t ntimes, double tfinal, const int32_t *nstream, double *nbody_w_final,
                            double *stream_w_final) {
    RefPot rp;
    if (!build(pot, NULL, &rp)) { release(&rp); return -100; }
    int64_t total = 0;
    int maxn = 0;
    for (int64_t i = 0; i < ntimes; i++) {
        total += nstream[i];
        maxn = nstream[i] > maxn ? nstream[i] : maxn;
    }
    const int64_t total_bodies = nbodies + total;
    RefBody *rb = (RefBody *)calloc((size_t)nbodies + 1, sizeof(RefBody));
    CPotential **pots = (CPotential **)malloc(sizeof(CPotential *) * (size_t)total_bodies);
    int ok = 1;
    for (int i = 0; i < nbodies; i++) {
        if (!build_body(&bodies[i], &rb[i])) ok = 0;
        pots[i] = rb[i].cp;
    }
    gx_body null_body;
    memset(&null_body, 0, sizeof(null_body));
    null_body.type = GX_POT_NULL;
    if (!build_body(&null_body, &rb[nbodies])) ok = 0;
    for (int64_t i = nbodies; i < total_bodies; i++) pots[i] = rb[nbodies].cp;
    if (ok) {
        const double dt = full_time[1] - full_time[0];
        double *traj = (double *)malloc(sizeof(double) * (size_t)nfull * 6 * (size_t)nbodies);
        double *w = (double *)malloc(sizeof(double) * 6 * (size_t)(nbodies + maxn));
        double *vh = (double *)calloc(3 * (size_t)(nbodies + maxn), sizeof(double));
        /* the bodies over full_time (leapfrog_integrate_nbody, mockstream.pyx:524-528) */
        memcpy(w, nbody_w0, sizeof(double) * 6 * (size_t)nbodies);
        memcpy(traj, w, sizeof(double) * 6 * (size_t)nbodies);
        for (int i = 0; i < nbodies; i++) ref_lf_init(rp.cp, pots, nbodies, w, i, full_time[0], dt, vh);
        for (int64_t j = 1; j < nfull; j++) {
            for (int i = 0; i < nbodies; i++) ref_lf_step(rp.cp, pots, nbodies, w, i, full_time[j], dt, vh);
            memcpy(traj + (size_t)j * 6 * (size_t)nbodies, w, sizeof(double) * 6 * (size_t)nbodies);
        }
        int64_t n = 0;
        for (int64_t i = 0; i < ntimes; i++) {
            if (nstream[i] == 0) continue;
            const int idx = (int)((stream_t1[i] - full_time[0]) / dt + 0.5);
            memcpy(w, traj + (size_t)idx * 6 * (size_t)nbodies, sizeof(double) * 6 * (size_t)nbodies);
            memcpy(w + 6 * nbodies, stream_w0 + 6 * n, sizeof(double) * 6 * (size_t)nstream[i]);
            const int nsys = nbodies + nstream[i];
            for (int j = 0; j < nsys; j++) ref_lf_init(rp.cp, pots, nbodies, w, j, stream_t1[i], dt, vh);
            const int n_steps = (int)((tfinal - stream_t1[i]) / dt + 0.5);
            for (int j = 0; j < n_steps; j++)
                for (int k = 0; k < nsys; k++)
                    ref_lf_step(rp.cp, pots, nbodies, w, k, stream_t1[i] + (j + 1) * dt, dt, vh);
            memcpy(stream_w_final + 6 * n, w + 6 * nbodies, sizeof(double) * 6 * (size_t)nstream[i]);
            memcpy(nbody_w_final, w, sizeof(double) * 6 * (size_t)nbodies);
            n += nstream[i];
        }
        free(traj);
        free(w);
        free(vh);
    }
    for (int i = 0; i <= nbodies; i++)
        if (rb[i].cp) free_cpotential(rb[i].cp);
    free(rb);
    free(pots);
    release(&rp);
    return ok ? 0 : -100;
}

} // extern "C"
