/* CPU oracle for the Magnus-expansion hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of s-cavalier/magnus-dp's per-Gauss-Legendre-node
 * recursion (src/magnus.hpp, src/grad.hpp, src/graddata.hpp,
 * src/integration/*.hpp, src/linalg/{manual,fixed,spacecurve,generic}.hpp).
 * It is loaded (ctypes) only by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py, as the checker or the
 * timed CPU baseline.  The GB300 product path never calls it.
 *
 * Parity of this restatement is pinned against the reference compiled from
 * its own sources (oracle/build_ref.sh) through the golden fixtures in
 * tests/golden/ (generated by tests/golden/make_golden.py).
 *
 * Scalars: the _f64 entry points compute in double, the _f32 ones in float
 * with the reference's float casts of every double coefficient
 * (generic.hpp:8-15 scalar_as_num).  SpaceCurve data is the reference's
 * padded 4-vector form (composer/backends.hpp:253-357): the caller pads
 * (0, f0, f1, f2) and unpads. */
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdlib.h>

enum { MO_MATRIX = 0, MO_SPACECURVE = 1 };
enum { MO_BOOLE = 0, MO_SIMPSON = 1, MO_TRAPEZOID = 2, MO_RIEMANN = 3 };
enum { MO_ONE = 0, MO_MANY = 1, MO_SUM = 2 };

#define REAL double
#define SFX(name) name##_f64
#include "magnus_oracle_impl.inc"
#undef REAL
#undef SFX

#define REAL float
#define SFX(name) name##_f32
#include "magnus_oracle_impl.inc"
#undef REAL
#undef SFX

/* ---- uniform batches over host threads (CPU baseline) ----
 * Instances are independent; each worker takes instances i = w, w+T, ...
 * and runs the serial per-instance routine, which is how the reference is
 * driven one call per instance (pybind.cpp:146-192). */

typedef struct {
    int is_vjp, is_f32, kind, integ, op;
    size_t n, S, d, Q, count, worker, workers;
    double t0, tf;
    const double *gl_w, *gl_x;
    const void* A;
    const void* cot;
    void* out;
    int status;
} mo_job;

static void* mo_worker(void* arg) {
    mo_job* j = (mo_job*)arg;
    size_t m = (j->kind == MO_SPACECURVE) ? 4 : j->d * j->d;
    size_t nout = (j->op == MO_MANY) ? j->n : 1;
    for (size_t b = j->worker; b < j->count; b += j->workers) {
        int rc;
        if (j->is_f32) {
            const float* A = (const float*)j->A + b * j->S * m;
            if (j->is_vjp)
                rc = mo_vjp_f32(j->kind, j->integ, j->op, j->n, j->S, j->d, j->t0, j->tf, j->Q, j->gl_w, j->gl_x, A,
                                (const float*)j->cot + b * nout * m, NULL, (float*)j->out + b * j->S * m);
            else
                rc = mo_forward_f32(j->kind, j->integ, j->op, j->n, j->S, j->d, j->t0, j->tf, j->Q, j->gl_w, j->gl_x, A,
                                    (float*)j->out + b * nout * m, NULL);
        } else {
            const double* A = (const double*)j->A + b * j->S * m;
            if (j->is_vjp)
                rc = mo_vjp_f64(j->kind, j->integ, j->op, j->n, j->S, j->d, j->t0, j->tf, j->Q, j->gl_w, j->gl_x, A,
                                (const double*)j->cot + b * nout * m, NULL, (double*)j->out + b * j->S * m);
            else
                rc = mo_forward_f64(j->kind, j->integ, j->op, j->n, j->S, j->d, j->t0, j->tf, j->Q, j->gl_w, j->gl_x, A,
                                    (double*)j->out + b * nout * m, NULL);
        }
        if (rc != 0) j->status = rc;
    }
    return NULL;
}

/* Runs `count` instances laid out back to back ((count, S, m) inputs,
 * (count, nout, m) or (count, S, m) outputs) on `threads` host threads.
 * Returns 0 on success. */
int mo_batch(int is_vjp, int is_f32, int kind, int integ, int op, size_t n, size_t S, size_t d,
             double t0, double tf, size_t Q, const double* gl_w, const double* gl_x,
             size_t count, const void* A, const void* cot, void* out, int threads) {
    if (threads < 1) threads = 1;
    if ((size_t)threads > count) threads = (int)count;
    mo_job* jobs = (mo_job*)calloc((size_t)threads, sizeof(mo_job));
    pthread_t* tids = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    if (!jobs || !tids) { free(jobs); free(tids); return -1; }
    for (int w = 0; w < threads; ++w) {
        mo_job j = {is_vjp, is_f32, kind, integ, op, n, S, d, Q, count, (size_t)w, (size_t)threads,
                    t0, tf, gl_w, gl_x, A, cot, out, 0};
        jobs[w] = j;
    }
    for (int w = 1; w < threads; ++w) pthread_create(&tids[w], NULL, mo_worker, &jobs[w]);
    mo_worker(&jobs[0]);
    int status = jobs[0].status;
    for (int w = 1; w < threads; ++w) {
        pthread_join(tids[w], NULL);
        if (jobs[w].status) status = jobs[w].status;
    }
    free(jobs); free(tids);
    return status;
}
