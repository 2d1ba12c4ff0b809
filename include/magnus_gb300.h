/* magnus_gb300.h — C ABI of the GB300 Magnus-expansion engine.
 *
 * The engine computes the Magnus terms Omega_1..Omega_n of a sampled matrix
 * function A(t_i), i = 0..S-1 on [t0, tf] (dt = (tf - t0) / (S - 1)), and
 * their vector-Jacobian products, on one NVIDIA GB300 GPU.  Every entry point
 * takes plain pointers and sizes; none throws; each returns an mgb_status and
 * leaves a message retrievable with mgb_last_error() (per calling thread).
 *
 * Buffer conventions (C-contiguous, row-major, element type = problem dtype):
 *   matrix kind      A   (S, d, d)          out  (d, d) | (n, d, d) for op=many
 *                    dA  (S, d, d)          cot  shape of out
 *   spacecurve kind  A   (S, 3)             out  (3,)   | (n, 3)
 *                    dA  (S, 3)             cot  shape of out
 *   carry (record_vjp) (Q, n-1, S, d, d) with Q = (n+3)/2 (spacecurve: d=2),
 *     element ((q*(n-1) + k-2)*S + i) holds the prefix P_k[i] of GL node q,
 *     exactly the reference's VJP::Data layout.
 *
 * Device entry points (mgb_forward, mgb_vjp, *_batched) take DEVICE pointers
 * and a cudaStream_t (as void*, NULL = legacy default stream); they are
 * stream-ordered and return before the GPU work completes.  Host entry
 * points (*_host) take host pointers and are synchronous.
 *
 * Reference interfaces replaced (paths in s-cavalier/magnus-dp):
 *   mgb_forward      <- Magnus::detail::run_raw_impl            src/composer/backends.hpp:182-220
 *                       and run_spacecurve_raw_impl             src/composer/backends.hpp:253-301
 *                       (KernelPlan::run of make_plan,          src/composer/backends.cpp:65-93)
 *   mgb_vjp          <- Magnus::detail::run_vjp_raw_impl        src/composer/backends.hpp:222-251
 *                       and run_spacecurve_vjp_raw_impl         src/composer/backends.hpp:303-357
 *                       (KernelPlan::run of make_vjp_plan,      src/composer/backends.cpp:95-102)
 *   mgb_*_host       <- _core.compute / compute_sc / compute_vjp / compute_sc_vjp
 *                                                               src/api/pybind.cpp:357-433
 *   mgb_set_gl_table <- Magnus::detail::replace_gl_table        src/api/pybind.cpp:102-116
 *   mgb_max_order    <- Magnus::detail::max_order               src/api/pybind.cpp:57-59
 *   error strings    <- std::invalid_argument messages of       src/composer/backends.hpp:108-180,
 *                                                               src/composer/backends.cpp:37-53,
 *                                                               src/composer/dispatch.hpp:119-183
 */
#ifndef MAGNUS_GB300_H
#define MAGNUS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mgb_status {
    MGB_OK = 0,
    MGB_ERR_INVALID_ARGUMENT = 1, /* maps to ValueError / std::invalid_argument */
    MGB_ERR_TYPE = 2,             /* maps to TypeError */
    MGB_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    MGB_ERR_OUT_OF_MEMORY = 4,
    MGB_ERR_DEVICE_TIMEOUT = 5    /* a bounded device-side wait gave up */
} mgb_status;

enum { MGB_KIND_MATRIX = 0, MGB_KIND_SPACECURVE = 1 };
/* C64 / C128: interleaved (re, im) pairs of float / double.  A complex d x d
 * matrix problem runs as the real 2d x 2d problem on [[Re A, -Im A],
 * [Im A, Re A]]; complex SpaceCurve data as the real 8 x 8 problem on the
 * embedding of the quaternion right-multiplication matrix of (0, f); the VJP
 * is the reference's bilinear one.  Complex problems go through the
 * one-shot entry points (not plans, not mgb_forward_noalloc, not
 * mgb_fwd_vjp_host_batched). */
enum { MGB_DTYPE_F32 = 0, MGB_DTYPE_F64 = 1, MGB_DTYPE_C64 = 2, MGB_DTYPE_C128 = 3 };
/* PLAIN: every product and sum in FP64 (parity form, <=1e-12 vs the reference).
 * MIXED: per-sample products and in-chunk prefixes in FP32, chunk carries,
 *        scans and the final Omega assembly in FP64. */
enum { MGB_PRECISION_PLAIN = 0, MGB_PRECISION_MIXED = 1 };
enum { MGB_OP_ONE = 0, MGB_OP_MANY = 1, MGB_OP_SUM = 2 };
enum { MGB_INTEGRATOR_BOOLE = 0, MGB_INTEGRATOR_SIMPSON = 1, MGB_INTEGRATOR_TRAPEZOID = 2, MGB_INTEGRATOR_RIEMANN = 3 };

typedef struct mgb_problem {
    int32_t kind;          /* MGB_KIND_* */
    int32_t dtype;         /* MGB_DTYPE_* : element type of every buffer */
    int32_t precision;     /* MGB_PRECISION_* */
    int32_t op;            /* MGB_OP_* */
    int32_t integrator;    /* MGB_INTEGRATOR_* */
    uint32_t checkpoint_K; /* samples per checkpoint chunk; 0 = engine default; else a multiple of 4 */
    uint64_t n;            /* Magnus order, >= 1 */
    uint64_t samples;      /* S, >= 2 */
    uint64_t dim;          /* d (ignored for spacecurve) */
    double t0;
    double tf;
} mgb_problem;

/* Forward: out <- op(Omega_1..Omega_n).  carry (nullable): reference-format
 * prefix record.  ckpt (nullable): engine checkpoints (mgb_checkpoint_bytes)
 * that a later mgb_vjp can reuse instead of recomputing the forward scan. */
mgb_status mgb_forward(const mgb_problem* p, const void* A, void* out, void* carry, void* ckpt, void* stream);

/* VJP: dA <- d<cot, op(Omega)>/dA (bilinear pairing, as the reference).
 * ckpt: buffer written by mgb_forward for the same problem and A, or NULL to
 * recompute the forward checkpoints. */
mgb_status mgb_vjp(const mgb_problem* p, const void* A, const void* cot, const void* ckpt, void* dA, void* stream);

/* Bytes of the checkpoint buffer for problem p (0 on invalid p). */
size_t mgb_checkpoint_bytes(const mgb_problem* p);

/* Batched forms: `count` independent instances in one set of launches.
 * Instances may differ in n, samples, dim, op, t0, tf and checkpoint_K; they
 * must share kind, dtype, precision and integrator.  ckpt may be NULL (the
 * array) or hold NULL entries. */
mgb_status mgb_forward_batched(const mgb_problem* probs, size_t count, const void* const* A, void* const* out,
                               void* const* ckpt, void* stream);
mgb_status mgb_vjp_batched(const mgb_problem* probs, size_t count, const void* const* A, const void* const* cot,
                           const void* const* ckpt, void* const* dA, void* stream);

/* Plans.  mgb_plan_create validates `count` problems, binds their device
 * buffers (A; out for the forward; cot and dA for the VJP — either pair may
 * be NULL) and prepares everything the engine needs on the device (one
 * cudaMalloc, descriptors uploaded, instances of equal dimension grouped into
 * segments that run concurrently, each segment's chunk-kernel launch variant
 * picked by timing the variants on a sample of its chunks — once per shape
 * per process, with a temporary allocation; MGB_AUTOTUNE=0 disables, and
 * the one-shot entry points do the same when their stream is not being
 * captured).  mgb_plan_forward / mgb_plan_vjp then only
 * enqueue kernels on `stream`, so they can be captured into a CUDA graph and
 * replayed.  The VJP reuses the checkpoints of the plan's last forward (or
 * recomputes them when the plan has not run forward yet).  Replaces the
 * reference's KernelPlan { divisibility_requirement(); run(alloc) } made by
 * make_plan / make_vjp_plan (src/composer/dispatch.hpp:446-492,
 * src/composer/backends.cpp:65-102). */
typedef struct mgb_plan mgb_plan;
mgb_status mgb_plan_create(const mgb_problem* probs, size_t count, const void* const* A, void* const* out,
                           const void* const* cot, void* const* dA, mgb_plan** plan);
mgb_status mgb_plan_forward(mgb_plan* plan, void* stream);
mgb_status mgb_plan_vjp(mgb_plan* plan, void* stream);
size_t mgb_plan_bytes(const mgb_plan* plan);
/* Engine-specific, no reference counterpart: a JSON description of the plan's
 * segments (dimension, instances, chunks, chunk kernel, the launch variant the
 * autotuner chose and the per-variant times it measured in ms, scan kind)
 * written to buf (truncated to len - 1 bytes, NUL-terminated); returns the
 * length needed including the NUL. */
size_t mgb_plan_describe(const mgb_plan* plan, char* buf, size_t len);
mgb_status mgb_plan_destroy(mgb_plan* plan);

/* Host-pointer forms (synchronous; device staging inside). carry nullable. */
mgb_status mgb_forward_host(const mgb_problem* p, const void* A, void* out, void* carry);
mgb_status mgb_vjp_host(const mgb_problem* p, const void* A, const void* cot, void* dA);

/* Engine-specific (the reference makes one compute(record_vjp=True) and one
 * compute_vjp(vjp_data) call per instance, src/api/pybind.cpp:357-433): the
 * forward (out) and the VJP (dA) of `count` instances from HOST buffers in
 * one synchronous call.  Instances go to the device in sub-batches of at
 * least 256 MB (by default ramped: 1, 3, 4, 4, 3, 1 sixteenths of the input;
 * MGB_HOST_SUBBATCHES = p cuts p equal ones) through three rotating device
 * slots, so the host-to-device copy of one sub-batch, the kernels of the
 * previous one and the device-to-host copy of the one before overlap.  Host
 * buffers should be page-locked (cudaHostAlloc / cudaMallocHost / torch
 * pin_memory) for the copies to overlap; pageable ones are correct but
 * staged by the driver.  With page-locked buffers the inputs of the first
 * two sub-batches and the dA of the last two are moved by a copy kernel
 * through the host mapping (the pipeline's fill and drain, when the copy
 * engines alone were slow on the GB300's host link), the rest by the copy
 * engines.  The slots stay allocated on
 * the device for later calls (calls are serialized inside the library). */
mgb_status mgb_fwd_vjp_host_batched(const mgb_problem* probs, size_t count, const void* const* A,
                                    const void* const* cot, void* const* out, void* const* dA);

/* Forward that allocates no device memory.  For callers that cannot call
 * cudaMalloc during their work — an XLA/JAX custom call, or any framework
 * whose caching allocator already holds the GPU's memory, or a host that must
 * not allocate (or synchronize the device) mid-run.  Same result as
 * mgb_forward(p, A, out, NULL, NULL, stream) (no carry, no checkpoints), but
 * every piece of working memory comes from one array of
 * MGB_NOALLOC_SCRATCH_BYTES compiled into the library, which each GPU that
 * loads the library holds until the process exits.  A problem whose
 * workspace does not fit is rejected with MGB_ERR_INVALID_ARGUMENT and a
 * message giving the bytes it needs.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress with that device current); make
 * that first call before any stream capture.  All calls on a device share the
 * array and it keeps the previous call's contents (nothing needs clearing);
 * calls whose GPU work can overlap race on it, so order them on one stream.
 * No counterpart in the reference (its CPU code allocates on the host heap).
 * A and out are device pointers; the call is stream-ordered and enqueues
 * kernels only: the problem's descriptor and Gauss-Legendre values travel as
 * kernel parameters, so no host-to-device copy makes it wait for the stream. */
#define MGB_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
mgb_status mgb_forward_noalloc(const mgb_problem* p, const void* A, void* out, void* stream);

/* Gauss-Legendre table: weights/nodes on [0, 1] for orders 1..max_order,
 * order q at offset q(q-1)/2 (flattened like the reference).  Copied. */
mgb_status mgb_set_gl_table(size_t max_order, const double* weights, const double* nodes);
size_t mgb_max_order(void);

/* Engine-specific, no reference counterpart.  Synchronizes the current
 * device and returns MGB_ERR_DEVICE_TIMEOUT if a kernel gave up one of its
 * bounded device-side waits since the last check (its outputs are then
 * invalid).  The host entry points check this themselves; callers of the
 * device entry points and plans check it when they synchronize. */
mgb_status mgb_device_check(void);

/* Engine-specific, no reference counterpart: a self-test of the error path
 * above.  Enqueues one small kernel that waits up to limit_ns (at most 2e9)
 * on a device-side barrier nothing arrives at, then gives up the way the
 * engine's kernels do (raises the time-out flag and returns; nothing else is
 * in flight).  The next mgb_device_check() returns MGB_ERR_DEVICE_TIMEOUT and
 * clears the flag; the context stays usable.  Mirrors the error contract of
 * the reference's JAX handlers (src/api/jax_ffi.cpp:280-284): a failure is a
 * status, not an abort. */
mgb_status mgb_selftest_bounded_wait(int64_t limit_ns, void* stream);

/* Kernel timing.  While enabled, every engine kernel launch is bracketed by
 * CUDA events on its stream, and mgb_fwd_vjp_host_batched brackets each
 * sub-batch's stages ("h2d.<b>", "comp.<b>", "d2h.<b>"); mgb_profile_read
 * waits for the recorded events, fills up to `capacity` entries (one per
 * name: launches, total milliseconds, and the first start / last end in
 * milliseconds after the moment timing was switched on) and returns the
 * number of names.  For benchmarking only: the events add a few
 * microseconds per launch.  No reference counterpart (the reference has no
 * tracing). */
typedef struct mgb_kernel_time {
    char name[40];
    uint64_t launches;
    double total_ms;
    double first_start_ms;
    double last_end_ms;
} mgb_kernel_time;
mgb_status mgb_profile_enable(int enable);
size_t mgb_profile_read(mgb_kernel_time* out, size_t capacity, int reset);

/* Message of the last non-OK status on the calling thread ("" if none). */
const char* mgb_last_error(void);
int mgb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MAGNUS_GB300_H */
