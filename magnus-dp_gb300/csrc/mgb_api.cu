// C ABI of the engine (declared in include/magnus_gb300.h): validation with
// the reference's error contract, call planning, a stream-ordered workspace,
// and the kernel launch sequences for forward and VJP.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "magnus_gb300.h"
#include "mgb_kernels.h"
#include "mgb_tuned.h"
#include "gl_table.inc"

namespace {

using namespace mgb;

thread_local std::string g_last_error;

mgb_status fail(mgb_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

// ---------------------------------------------------------------- GL table
struct GLData {
    size_t max_order;
    std::vector<double> w, x;
};

std::mutex g_gl_mutex;
std::shared_ptr<const GLData> g_gl;

std::shared_ptr<const GLData> gl_snapshot() {
    std::lock_guard<std::mutex> lock(g_gl_mutex);
    if (!g_gl) {
        auto t = std::make_shared<GLData>();
        t->max_order = MGB_GL_DEFAULT_MAX_ORDER;
        size_t cnt = sizeof(mgb_gl_default_nodes) / sizeof(double);
        t->x.assign(mgb_gl_default_nodes, mgb_gl_default_nodes + cnt);
        t->w.assign(mgb_gl_default_weights, mgb_gl_default_weights + cnt);
        g_gl = t;
    }
    return g_gl;
}

// ---------------------------------------------------------------- profiler
struct ProfEvent {
    std::string name;
    cudaEvent_t start, stop;
};
struct ProfTotal {
    uint64_t launches = 0;
    double ms = 0.0;
    double first = 1e300, last = -1e300;  // ms from the reference event
};
std::mutex g_prof_mutex;
bool g_prof_enabled = false;
cudaEvent_t g_prof_ref = nullptr;  // recorded when timing is switched on
std::vector<ProfEvent> g_prof_pending;
std::vector<std::pair<std::string, ProfTotal>> g_prof_totals;

bool prof_on() {
    std::lock_guard<std::mutex> lock(g_prof_mutex);
    return g_prof_enabled;
}

template <class F>
cudaError_t timed(const char* name, cudaStream_t st, F&& fn) {
    if (!prof_on()) return fn();
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, st);
    cudaError_t e = fn();
    cudaEventRecord(b, st);
    std::lock_guard<std::mutex> lock(g_prof_mutex);
    g_prof_pending.push_back(ProfEvent{name, a, b});
    return e;
}

// ---------------------------------------------------------------- devices
struct DevInfo {
    int sms = 0;
};

DevInfo device_info() {
    static std::mutex mu;
    static std::vector<DevInfo> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    if ((int)cache.size() <= dev) cache.resize(dev + 1);
    if (cache[dev].sms == 0) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cache[dev].sms = sms > 0 ? sms : 1;
    }
    return cache[dev];
}

// ---------------------------------------------------------------- validation
bool is_complex(int32_t dtype) { return dtype == MGB_DTYPE_C64 || dtype == MGB_DTYPE_C128; }

// The real problem a complex one runs as (dimension 2d, real parts' type).
// Complex SpaceCurve data run as the real 8 x 8 matrix problem with op many
// (mgb_complex.cu); complex matrix data as the real 2d x 2d problem.
mgb_problem real_problem(const mgb_problem& p) {
    mgb_problem r = p;
    if (is_complex(p.dtype)) {
        r.dtype = p.dtype == MGB_DTYPE_C128 ? MGB_DTYPE_F64 : MGB_DTYPE_F32;
        if (p.kind == MGB_KIND_SPACECURVE) {
            r.kind = MGB_KIND_MATRIX;
            r.dim = 8;
            r.op = MGB_OP_MANY;
        } else {
            r.dim = 2 * p.dim;
        }
    }
    return r;
}

struct Derived {
    int m, Q, C, K, div;
    int64_t nm;
};

int rule_divisibility(int integrator) {
    switch (integrator) {
        case MGB_INTEGRATOR_BOOLE: return 4;
        case MGB_INTEGRATOR_SIMPSON: return 2;
        case MGB_INTEGRATOR_TRAPEZOID: return 2;
        default: return 1;
    }
}

// Checkpoint interval.  The mixed form's chunk scans are FP64 (n(n-1)/2
// products per chunk against (n-1)K FP32 products inside it), so it takes
// long chunks at every d; the plain form keeps shorter ones at large d,
// where its slots are twice as large and its scans cost little.
int default_K(const mgb_problem& p) {
    // 4-element algebras (SpaceCurve, 2 x 2) in the mixed form with long
    // sample runs: 1024.  Their FP32 chunk kernel (one thread per chunk) is
    // cheap per sample, while every chunk step of the FP64 scan costs
    // n(n-1)/2 products on the 1/64-rate FP64 pipe; four times fewer steps,
    // and still 64+ chunks per instance for the thread-per-chunk parallelism.
    // (The plain form's FP64 chunk kernel is the larger cost: it keeps 256
    // and the parallelism.)
    if ((p.kind == MGB_KIND_SPACECURVE || p.dim == 2) && p.precision == MGB_PRECISION_MIXED && p.samples - 1 >= 65536)
        return 1024;
    if (p.kind == MGB_KIND_SPACECURVE || p.dim <= 32 || p.precision == MGB_PRECISION_MIXED) return 256;
    if (p.dim <= 64) return 128;
    return 64;
}

// Mirrors Magnus::detail::matrix_input_shape / spacecurve_input_shape
// (src/composer/backends.hpp:108-137) and dispatch_plan's checks
// (src/composer/backends.cpp:37-53).
mgb_status validate(const mgb_problem* p, size_t gl_max, Derived* dv) {
    if (!p) return fail(MGB_ERR_INVALID_ARGUMENT, "problem must not be null");
    if (p->n == 0) return fail(MGB_ERR_INVALID_ARGUMENT, "n must be at least 1");
    if (p->kind != MGB_KIND_MATRIX && p->kind != MGB_KIND_SPACECURVE)
        return fail(MGB_ERR_INVALID_ARGUMENT, "invalid dispatch option (based on params)");
    if (p->dtype != MGB_DTYPE_F32 && p->dtype != MGB_DTYPE_F64 && p->dtype != MGB_DTYPE_C64 &&
        p->dtype != MGB_DTYPE_C128)
        return fail(MGB_ERR_TYPE, "magnus only supports dtypes float32, float64, complex64, and complex128");
    if (is_complex(p->dtype) && p->dim > 2048) return fail(MGB_ERR_INVALID_ARGUMENT, "matrix dimension is too large");
    if (p->precision != MGB_PRECISION_PLAIN && p->precision != MGB_PRECISION_MIXED)
        return fail(MGB_ERR_INVALID_ARGUMENT, "invalid dispatch option (based on params)");
    if (p->op < MGB_OP_ONE || p->op > MGB_OP_SUM)
        return fail(MGB_ERR_INVALID_ARGUMENT,
                    "could not deduce kernel op from str in Magnus::Dispatch::op_from_str(std::string_view)");
    if (p->integrator < MGB_INTEGRATOR_BOOLE || p->integrator > MGB_INTEGRATOR_RIEMANN)
        return fail(MGB_ERR_INVALID_ARGUMENT, "Could not resolve dispatch name option");
    if (p->samples < 2) return fail(MGB_ERR_INVALID_ARGUMENT, "data must contain at least two samples");
    if (p->kind == MGB_KIND_MATRIX && p->dim == 0) return fail(MGB_ERR_INVALID_ARGUMENT, "data must contain square matrices");
    const uint64_t d = (p->kind == MGB_KIND_SPACECURVE) ? 2 : p->dim;
    if (d > 4096) return fail(MGB_ERR_INVALID_ARGUMENT, "matrix dimension is too large");
    if (p->n > 1 && (p->n + 3) / 2 > gl_max)
        return fail(MGB_ERR_INVALID_ARGUMENT, "requested magnus order exceeds GL table. Consider providing a larger table.");
    if (p->n > 4096) return fail(MGB_ERR_INVALID_ARGUMENT, "requested magnus order exceeds GL table. Consider providing a larger table.");
    const int div = rule_divisibility(p->integrator);
    if ((p->samples - 1) % (uint64_t)div != 0)
        return fail(MGB_ERR_INVALID_ARGUMENT,
                    "sample interval count violates integrator divisibility (a power of 2 is recommneded; i.e., total "
                    "samples is 2^k + 1 for some k > 4)");
    if (p->samples > (uint64_t)std::numeric_limits<int64_t>::max() / (d * d + 1))
        return fail(MGB_ERR_INVALID_ARGUMENT, "input shape is too large");
    int K = p->checkpoint_K ? (int)p->checkpoint_K : default_K(*p);
    if (K < 4 || K % 4 != 0 || K > (1 << 20))
        return fail(MGB_ERR_INVALID_ARGUMENT, "checkpoint_K must be a positive multiple of 4");
    dv->m = (int)(d * d);
    dv->Q = p->n > 1 ? (int)((p->n + 3) / 2) : 1;
    dv->K = K;
    dv->C = (int)((p->samples - 1 + K - 1) / K);
    dv->div = div;
    dv->nm = (int64_t)p->n * dv->m;
    return MGB_OK;
}

size_t ckpt_doubles(const mgb_problem&, const Derived& dv) { return (size_t)(2 * dv.C + 1) * dv.nm; }
size_t ws_doubles(const Derived& dv) { return (size_t)dv.C * dv.nm + 3 * (size_t)dv.Q * dv.nm + 6 * (size_t)dv.nm; }

// Step used inside the chunk kernels (see InstDev::dt_k): the plain form
// integrates with dt itself; the mixed form with u * 2^p, u the rule's
// coefficient denominator, so that all FP32 rule weights are exact.
double kernel_step(const mgb_problem& p, double dt) {
    if (p.precision == MGB_PRECISION_PLAIN || !(dt > 0.0) || !std::isfinite(dt)) return dt;
    const double u = p.integrator == MGB_INTEGRATOR_BOOLE ? 90.0
                   : p.integrator == MGB_INTEGRATOR_SIMPSON ? 6.0
                   : p.integrator == MGB_INTEGRATOR_TRAPEZOID ? 2.0 : 1.0;
    return u * std::exp2(std::round(std::log2(dt / u)));
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// ---------------------------------------------------------------- workspace
struct Workspace {
    void* base = nullptr;
    cudaStream_t st = nullptr;
    ~Workspace() {
        if (base) cudaFreeAsync(base, st);
    }
};

#define MGB_CUDA_TRY(expr)                                                                         \
    do {                                                                                           \
        cudaError_t e_ = (expr);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            if (e_ == cudaErrorMemoryAllocation) {                                                 \
                cudaGetLastError();                                                                \
                return fail(MGB_ERR_OUT_OF_MEMORY, std::string("CUDA out of memory: ") + #expr);   \
            }                                                                                      \
            return fail(MGB_ERR_CUDA, std::string(cudaGetErrorString(e_)) + " in " + #expr);       \
        }                                                                                          \
    } while (0)

struct Call {
    bool vjp;
    size_t count;
    const mgb_problem* probs;
    const void* const* A;
    void* const* out;      // forward
    void* const* carry;    // forward, nullable array
    void* const* ckpt_out; // forward, nullable array
    const void* const* cot;      // vjp
    const void* const* ckpt_in;  // vjp, nullable array
    void* const* dA;             // vjp
    cudaStream_t stream;
    int budget_parts = 1;        // plans that will be resident at once (their scratch budgets share the memory)
};

// ---------------------------------------------------------------- plans
// A plan holds everything a call needs on the device: per-instance
// descriptors, chunk work lists, Gauss-Legendre values, checkpoints, small
// algebra workspace and per-CTA scratch, in one buffer.  Instances are sorted
// by matrix dimension and cut into segments; each segment runs the fastest
// chunk kernel that covers its shape (mgb_tuned.cu) or the generic kernel,
// on its own stream when there are several segments.  After the one-time
// upload, launching a plan only enqueues kernels (so it can be captured into
// a CUDA graph).  This is the engine's counterpart of the reference's
// KernelPlan made by make_plan / make_vjp_plan
// (src/composer/dispatch.hpp:446-492, src/composer/backends.cpp:65-102).
int env_int(const char* name, int dflt);

struct Segment {
    int32_t first = 0, count = 0;  // instance range (sorted order)
    int64_t work_off = 0, nwork = 0;
    TunedChoice tc;
    int64_t slot_elems = 0, grid = 0;
    size_t scr_off = 0;
    std::vector<InstDev> hi;
    // chunk scans spread over the GPU (matrix, d a multiple of 16):
    // active[c] = instances of the segment with more than c chunks
    bool tiled_scan = false;
    // mixed form at d = 16 / 32: both scans in one double-FP32 launch each
    bool df_scan = false;
    int d = 0, nmax = 0;
    std::vector<int32_t> active;
    // chunk-kernel launch variant (autotuner) and the times it measured
    int variant = 0;
    std::vector<float> tune_ms;
    bool tuned_here = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

struct PlanCore {
    int kind = 0, rule = 0, f64io = 0;
    bool plain = true;
    size_t count = 0;
    bool has_out = false, has_vjp = false, any_carry = false, all_ck_in = false;
    std::vector<InstDev> hi;       // sorted order
    std::vector<int32_t> order;    // sorted position -> caller index
    std::vector<ChunkRef> work;
    std::vector<double> gl;
    std::vector<Segment> segs;
    size_t off_inst = 0, off_work = 0, off_gl = 0, off_ck = 0, off_ws = 0, off_gscr = 0, bytes = 0;
    int64_t gslot_elems = 0, ggrid = 0;  // generic scratch (carry record)
    char* base = nullptr;
    bool async_alloc = false;
    cudaStream_t alloc_stream = nullptr;
    cudaEvent_t fork = nullptr;
    int sms = 1;

    void release_streams() {
        for (Segment& sg : segs) {
            if (sg.stream) cudaStreamDestroy(sg.stream);
            if (sg.done) cudaEventDestroy(sg.done);
            sg.stream = nullptr;
            sg.done = nullptr;
        }
        if (fork) cudaEventDestroy(fork);
        fork = nullptr;
    }
};

// Validate, sort, cut segments and compute the layout (no device work).
mgb_status plan_layout(const Call& call, PlanCore& pc, std::vector<Derived>& dv) {
    if (call.count == 0) return fail(MGB_ERR_INVALID_ARGUMENT, "no problems given");
    if (!call.probs || !call.A) return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
    auto gl = gl_snapshot();
    dv.resize(call.count);
    const mgb_problem& p0 = call.probs[0];
    for (size_t i = 0; i < call.count; ++i) {
        mgb_status st = validate(&call.probs[i], gl->max_order, &dv[i]);
        if (st != MGB_OK) return st;
        if (is_complex(call.probs[i].dtype))
            return fail(MGB_ERR_INVALID_ARGUMENT,
                        "complex problems run through mgb_forward / mgb_vjp and their batched and host forms");
        const mgb_problem& p = call.probs[i];
        if (p.kind != p0.kind || p.dtype != p0.dtype || p.precision != p0.precision || p.integrator != p0.integrator)
            return fail(MGB_ERR_INVALID_ARGUMENT, "batched instances must share kind, dtype, precision and integrator");
        if (!call.A[i]) return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
        if (call.out && !call.out[i]) return fail(MGB_ERR_INVALID_ARGUMENT, "output buffer must not be null");
        if (call.cot && !call.cot[i]) return fail(MGB_ERR_INVALID_ARGUMENT, "cotangent buffer must not be null");
        if (call.dA && !call.dA[i]) return fail(MGB_ERR_INVALID_ARGUMENT, "output buffer must not be null");
    }
    if (!call.out && !call.dA) return fail(MGB_ERR_INVALID_ARGUMENT, "output buffer must not be null");
    if ((call.cot == nullptr) != (call.dA == nullptr))
        return fail(MGB_ERR_INVALID_ARGUMENT, "cotangent and dA buffers must be given together");
    pc.kind = p0.kind;
    pc.rule = p0.integrator;
    pc.plain = p0.precision == MGB_PRECISION_PLAIN;
    pc.f64io = p0.dtype == MGB_DTYPE_F64;
    pc.count = call.count;
    pc.has_out = call.out != nullptr;
    pc.has_vjp = call.dA != nullptr;
    pc.sms = device_info().sms;
    const size_t tsz = pc.plain ? sizeof(double) : sizeof(float);

    // sort by dimension (largest first: heavy segments start first), then by
    // chunk count (the tiled scans launch each step over a prefix)
    pc.order.resize(call.count);
    for (size_t i = 0; i < call.count; ++i) pc.order[i] = (int32_t)i;
    std::stable_sort(pc.order.begin(), pc.order.end(), [&](int32_t a, int32_t b) {
        return dv[a].m != dv[b].m ? dv[a].m > dv[b].m : dv[a].C > dv[b].C;
    });

    size_t nwork = 0, gl_doubles = 0, ck_doubles = 0, wsd = 0;
    pc.all_ck_in = call.ckpt_in != nullptr;
    for (size_t i = 0; i < call.count; ++i) {
        nwork += (size_t)dv[i].C;
        gl_doubles += 2 * (size_t)dv[i].Q;
        const bool user_ck = (call.ckpt_in && call.ckpt_in[i]) || (call.ckpt_out && call.ckpt_out[i]);
        if (!user_ck) ck_doubles += ckpt_doubles(call.probs[i], dv[i]);
        if (call.ckpt_in && !call.ckpt_in[i]) pc.all_ck_in = false;
        wsd += ws_doubles(dv[i]);
        if (call.carry && call.carry[i]) pc.any_carry = true;
    }
    if (nwork > (size_t)std::numeric_limits<int32_t>::max()) return fail(MGB_ERR_INVALID_ARGUMENT, "input shape is too large");

    // segments: runs of equal dimension
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    // up to half the free memory, at most 96 GB (a two-CTA d = 128 segment asks
    // ~51 GB at n = 6), shared by the plans resident at once
    size_t budget = std::max<size_t>((size_t)256 << 20,
                                     std::min<size_t>(free_b / 2, (size_t)96 << 30) / (size_t)std::max(1, call.budget_parts));
    // MGB_SCRATCH_MB: a fixed scratch budget in MiB (tests use it to make the
    // segments' slot counts shrink below their asks)
    if (const char* ev = std::getenv("MGB_SCRATCH_MB"))
        if (std::atoll(ev) > 0) budget = (size_t)std::atoll(ev) << 20;
    int64_t wpos = 0;
    for (size_t a = 0; a < call.count;) {
        size_t b = a;
        while (b < call.count && dv[pc.order[b]].m == dv[pc.order[a]].m) ++b;
        Segment sg;
        sg.first = (int32_t)a;
        sg.count = (int32_t)(b - a);
        sg.work_off = wpos;
        for (size_t k = a; k < b; ++k) {
            const int32_t i = pc.order[k];
            const mgb_problem& p = call.probs[i];
            sg.nwork += dv[i].C;
            InstDev I{};  // the fields the kernel choice looks at
            I.A = call.A[i];
            I.dA = call.dA ? call.dA[i] : nullptr;
            I.S = (int64_t)p.samples;
            I.d = (p.kind == MGB_KIND_SPACECURVE) ? 2 : (int32_t)p.dim;
            I.m = dv[i].m;
            I.n = (int32_t)p.n;
            I.K = dv[i].K;
            sg.hi.push_back(I);
            sg.nmax = std::max<int>(sg.nmax, (int)p.n);
        }
        sg.d = sg.hi[0].d;
        sg.tiled_scan = scan_tiled_ok(pc.kind, sg.d);
        sg.df_scan = sg.tiled_scan && !pc.plain && env_int("MGB_DF_SCAN", 1) != 0 && scan_df_ok(pc.kind, sg.d, sg.nmax);
        if (sg.tiled_scan) {
            sg.active.assign((size_t)dv[pc.order[a]].C, 0);
            for (size_t k = a; k < b; ++k)
                for (int c = 0; c < dv[pc.order[k]].C; ++c) ++sg.active[(size_t)c];
        }
        wpos += sg.nwork;
        pc.segs.push_back(std::move(sg));
        a = b;
    }
    // scratch budget shared by the segments in proportion to their work
    size_t off = 0;
    pc.off_inst = off; off = align_up(off + call.count * sizeof(InstDev), 256);
    pc.off_work = off; off = align_up(off + nwork * sizeof(ChunkRef), 256);
    pc.off_gl = off; off = align_up(off + gl_doubles * sizeof(double), 256);
    pc.off_ck = off; off = align_up(off + ck_doubles * sizeof(double), 256);
    pc.off_ws = off; off = align_up(off + wsd * sizeof(double), 256);
    // every segment asks for one slot per resident CTA; when the asks exceed
    // the budget, all are cut in the same proportion
    std::vector<SegSizing> want(pc.segs.size());
    double asked = 0.0;
    for (size_t s = 0; s < pc.segs.size(); ++s) {
        const Segment& sg = pc.segs[s];
        want[s] = size_segment(pc.plain, pc.kind, pc.rule, pc.f64io != 0, sg.hi, sg.nwork, pc.sms,
                               std::numeric_limits<size_t>::max());
        asked += (double)want[s].grid * (double)want[s].slot_elems * (double)tsz;
    }
    const double cut = asked > (double)budget ? (double)budget / asked : 1.0;
    for (size_t s = 0; s < pc.segs.size(); ++s) {
        Segment& sg = pc.segs[s];
        sg.slot_elems = want[s].slot_elems;
        sg.grid = std::max<int64_t>(1, (int64_t)((double)want[s].grid * cut));
        sg.scr_off = off;
        off = align_up(off + (size_t)sg.grid * (size_t)sg.slot_elems * tsz, 256);
    }
    if (pc.any_carry) {
        // the carry record runs the generic kernel over all instances
        for (size_t i = 0; i < call.count; ++i) {
            const mgb_problem& p = call.probs[i];
            const int64_t L = std::min<int64_t>((int64_t)dv[i].K, (int64_t)p.samples - 1) + 1;
            pc.gslot_elems = std::max<int64_t>(pc.gslot_elems, (int64_t)(p.n + 4) * L * dv[i].m + 3 * (int64_t)p.n * dv[i].m);
        }
        const size_t slot_bytes = (size_t)pc.gslot_elems * tsz;
        pc.ggrid = std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>((int64_t)nwork, (int64_t)pc.sms * 8),
                                                          (int64_t)(budget / std::max<size_t>(slot_bytes, 1))));
        pc.off_gscr = off;
        off = align_up(off + (size_t)pc.ggrid * slot_bytes, 256);
    }
    pc.bytes = off;
    return MGB_OK;
}

// Fill the host descriptors for a device buffer at `base`.
void plan_fill(const Call& call, PlanCore& pc, const std::vector<Derived>& dv) {
    auto gl = gl_snapshot();
    char* base = pc.base;
    pc.hi.assign(call.count, InstDev{});
    pc.work.clear();
    pc.work.reserve((size_t)pc.segs.back().work_off + (size_t)pc.segs.back().nwork);
    pc.gl.clear();
    size_t ckpos = 0, wspos = 0;
    for (size_t k = 0; k < call.count; ++k) {
        const int32_t i = pc.order[k];
        const mgb_problem& p = call.probs[i];
        const Derived& v = dv[i];
        InstDev& I = pc.hi[k];
        std::memset(&I, 0, sizeof(I));
        I.A = call.A[i];
        I.out = call.out ? call.out[i] : nullptr;
        I.carry = (call.carry && call.carry[i]) ? call.carry[i] : nullptr;
        I.cot = call.cot ? call.cot[i] : nullptr;
        I.dA = call.dA ? call.dA[i] : nullptr;
        double* ck;
        if (call.ckpt_in && call.ckpt_in[i]) {
            ck = static_cast<double*>(const_cast<void*>(call.ckpt_in[i]));
        } else if (call.ckpt_out && call.ckpt_out[i]) {
            ck = static_cast<double*>(call.ckpt_out[i]);
        } else {
            ck = reinterpret_cast<double*>(base + pc.off_ck) + ckpos;
            ckpos += ckpt_doubles(p, v);
        }
        I.pi = ck;
        I.lam = ck + (size_t)(v.C + 1) * v.nm;
        double* w = reinterpret_cast<double*>(base + pc.off_ws) + wspos;
        wspos += ws_doubles(v);
        I.rho = w; w += (size_t)v.C * v.nm;
        I.dq = w; w += (size_t)v.Q * v.nm;
        I.ee = w; w += v.nm;
        I.tau = w; w += v.nm;
        I.ob = w; w += v.nm;
        I.eb = w; w += v.nm;
        I.db = w; w += v.nm;
        I.tt = w; w += v.nm;
        I.dbq = w; w += (size_t)v.Q * v.nm;
        I.tauq = w; w += (size_t)v.Q * v.nm;
        double* g = reinterpret_cast<double*>(base + pc.off_gl) + pc.gl.size();
        const size_t go = (size_t)v.Q * (v.Q - 1) / 2;
        for (int q = 0; q < v.Q; ++q) pc.gl.push_back(gl->w[go + q]);
        for (int q = 0; q < v.Q; ++q) pc.gl.push_back(gl->x[go + q]);
        I.glw = g;
        I.glx = g + v.Q;
        I.dt = (p.tf - p.t0) / (double)(p.samples - 1);
        I.dt_k = kernel_step(p, I.dt);
        fill_rule_coefs(I);
        I.sig = (I.dt_k != 0.0) ? I.dt / I.dt_k : 1.0;
        I.S = (int64_t)p.samples;
        I.d = (p.kind == MGB_KIND_SPACECURVE) ? 2 : (int32_t)p.dim;
        I.m = v.m;
        I.n = (int32_t)p.n;
        I.C = v.C;
        I.Q = v.Q;
        I.K = v.K;
        I.op = p.op;
        for (int c = 0; c < v.C; ++c) pc.work.push_back(ChunkRef{(int32_t)k, c});
    }
    for (Segment& sg : pc.segs) {
        // double-FP32 scans read the chunk kernels' transfer pairs directly
        for (int32_t k = sg.first; k < sg.first + sg.count; ++k) pc.hi[k].lam_pair = sg.df_scan ? 1 : 0;
        sg.hi.assign(pc.hi.begin() + sg.first, pc.hi.begin() + sg.first + sg.count);
        sg.tc = TunedChoice{};
    }
}

mgb_status plan_upload(PlanCore& pc, cudaStream_t st, bool synchronous) {
    char* base = pc.base;
    if (synchronous) {
        MGB_CUDA_TRY(cudaMemcpy(base + pc.off_inst, pc.hi.data(), pc.hi.size() * sizeof(InstDev), cudaMemcpyHostToDevice));
        MGB_CUDA_TRY(cudaMemcpy(base + pc.off_work, pc.work.data(), pc.work.size() * sizeof(ChunkRef), cudaMemcpyHostToDevice));
        MGB_CUDA_TRY(cudaMemcpy(base + pc.off_gl, pc.gl.data(), pc.gl.size() * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        MGB_CUDA_TRY(cudaMemcpyAsync(base + pc.off_inst, pc.hi.data(), pc.hi.size() * sizeof(InstDev), cudaMemcpyHostToDevice, st));
        MGB_CUDA_TRY(cudaMemcpyAsync(base + pc.off_work, pc.work.data(), pc.work.size() * sizeof(ChunkRef), cudaMemcpyHostToDevice, st));
        MGB_CUDA_TRY(cudaMemcpyAsync(base + pc.off_gl, pc.gl.data(), pc.gl.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        MGB_CUDA_TRY(cudaStreamSynchronize(st));  // the host vectors may change after this
    }
    return MGB_OK;
}

mgb_status plan_streams(PlanCore& pc) {
    for (const Segment& sg : pc.segs) {
        for (int mode : {MODE_LOCAL, MODE_VJP})
            MGB_CUDA_TRY(prepare_tuned(choose_tuned(pc.plain, pc.kind, pc.rule, mode, pc.f64io != 0, sg.hi, sg.variant),
                                       pc.rule, mode));
        if (sg.df_scan)
            for (bool rev : {false, true})
                MGB_CUDA_TRY(launch_scan_df(nullptr, 0, sg.d, sg.nmax, rev, pc.f64io, nullptr, true));
    }
    if (pc.segs.size() < 2 || pc.fork) return MGB_OK;
    MGB_CUDA_TRY(cudaEventCreateWithFlags(&pc.fork, cudaEventDisableTiming));
    for (Segment& sg : pc.segs) {
        MGB_CUDA_TRY(cudaStreamCreateWithFlags(&sg.stream, cudaStreamNonBlocking));
        MGB_CUDA_TRY(cudaEventCreateWithFlags(&sg.done, cudaEventDisableTiming));
    }
    return MGB_OK;
}

LaunchArgs seg_args(const PlanCore& pc, const Segment& sg, cudaStream_t st) {
    LaunchArgs la;
    la.insts = reinterpret_cast<const InstDev*>(pc.base + pc.off_inst);
    la.work = reinterpret_cast<const ChunkRef*>(pc.base + pc.off_work) + sg.work_off;
    la.nwork = sg.nwork;
    la.scratch = pc.base + sg.scr_off;
    la.slot_elems = sg.slot_elems;
    la.grid = sg.grid;
    la.f64io = pc.f64io;
    la.stream = st;
    return la;
}

// ---------------------------------------------------------------- autotuner
// Each chunk-kernel family has launch variants (mgb_tuned.h): k-block and CTAs
// per SM of the tensor-core kernel, CTAs per SM (register budget) of the
// group-tiled kernel, CTAs per SM of the generic kernel.  Before a plan's
// first use, every variant of each segment's kernel runs the forward local
// pass over a sample of the segment's chunks (two waves of resident CTAs,
// spread over its instances, chunk totals written to a private buffer so no
// caller buffer is touched) and the fastest is kept.  Results are cached for
// the process by (family, d, rule, order bound, form).  MGB_AUTOTUNE=0 turns
// tuning off (variant 0 everywhere); MGB_FORCE_VARIANT=k forces variant k
// (tests use it to check every variant against the oracle).
struct TuneKey {
    int family, D, rule, nmax, plain, kind, f64io;
    bool operator<(const TuneKey& o) const {
        return std::tie(family, D, rule, nmax, plain, kind, f64io) <
               std::tie(o.family, o.D, o.rule, o.nmax, o.plain, o.kind, o.f64io);
    }
};
struct TuneResult {
    int variant = 0;
    std::vector<float> ms;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneResult> g_tune;

int env_int(const char* name, int dflt) {
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    return std::atoi(v);
}

mgb_status plan_autotune(PlanCore& pc, cudaStream_t st) {
    const int forced = env_int("MGB_FORCE_VARIANT", -1);
    const bool enabled = env_int("MGB_AUTOTUNE", 1) != 0;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (st) cudaStreamIsCapturing(st, &cap);
    for (Segment& sg : pc.segs) {
        const TunedChoice tc0 = choose_tuned(pc.plain, pc.kind, pc.rule, MODE_LOCAL, pc.f64io != 0, sg.hi, 0);
        const int nv = tc0.use ? (tc0.family == 1 ? 1 : tc0.nvariants) : GENERIC_VARIANTS;
        if (forced >= 0) {
            sg.variant = forced < nv ? forced : 0;
            continue;
        }
        if (nv <= 1 || !enabled) continue;
        const TuneKey key{tc0.use ? tc0.family : 0, sg.d, pc.rule, sg.nmax, pc.plain ? 1 : 0, pc.kind, pc.f64io};
        {
            std::lock_guard<std::mutex> lock(g_tune_mu);
            auto it = g_tune.find(key);
            if (it != g_tune.end()) {
                sg.variant = it->second.variant;
                sg.tune_ms = it->second.ms;
                continue;
            }
        }
        if (cap != cudaStreamCaptureStatusNone) continue;  // no timing inside a capture
        // sample: up to two waves of the most resident CTAs, round-robin over
        // the segment's instances, chunk indices below csub per instance
        const int maxctas = tc0.use ? std::max(tc0.ctas_per_sm, 2) : 8;
        const int64_t target = std::min<int64_t>(sg.nwork, 2LL * pc.sms * maxctas);
        const int nsub = (int)std::min<int64_t>(sg.count, target);
        const int csub = (int)((target + nsub - 1) / nsub);
        std::vector<InstDev> sub(pc.hi.begin() + sg.first, pc.hi.begin() + sg.first + nsub);
        std::vector<ChunkRef> work;
        size_t lam_doubles = 0;
        std::vector<size_t> lam_off(nsub);
        for (int k = 0; k < nsub; ++k) {
            lam_off[k] = lam_doubles;
            lam_doubles += (size_t)std::min(csub, sub[k].C) * (size_t)sub[k].n * (size_t)sub[k].m;
        }
        for (int c = 0; c < csub && (int64_t)work.size() < target; ++c)
            for (int k = 0; k < nsub && (int64_t)work.size() < target; ++k)
                if (c < sub[k].C) work.push_back(ChunkRef{k, c});
        char* tmp = nullptr;
        const size_t b_inst = align_up(sub.size() * sizeof(InstDev), 256);
        const size_t b_work = align_up(work.size() * sizeof(ChunkRef), 256);
        const size_t bytes = b_inst + b_work + lam_doubles * sizeof(double);
        if (cudaMalloc(&tmp, bytes) != cudaSuccess) {
            cudaGetLastError();
            continue;  // no room to tune: keep variant 0
        }
        double* lam = reinterpret_cast<double*>(tmp + b_inst + b_work);
        for (int k = 0; k < nsub; ++k) sub[k].lam = lam + lam_off[k];
        cudaError_t e = cudaMemcpy(tmp, sub.data(), sub.size() * sizeof(InstDev), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(tmp + b_inst, work.data(), work.size() * sizeof(ChunkRef), cudaMemcpyHostToDevice);
        LaunchArgs la = seg_args(pc, sg, st);
        la.insts = reinterpret_cast<const InstDev*>(tmp);
        la.work = reinterpret_cast<const ChunkRef*>(tmp + b_inst);
        la.nwork = (int64_t)work.size();
        std::vector<float> ms(nv, -1.f);
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (e == cudaSuccess) e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        for (int v = 0; v < nv && e == cudaSuccess; ++v) {
            cudaError_t r = launch_chunk_any(pc.plain, pc.kind, pc.rule, MODE_LOCAL, la, sg.hi, pc.sms, v);  // warm-up
            if (r == cudaSuccess) r = cudaEventRecord(e0, st);
            for (int rep = 0; rep < 2 && r == cudaSuccess; ++rep)
                r = launch_chunk_any(pc.plain, pc.kind, pc.rule, MODE_LOCAL, la, sg.hi, pc.sms, v);
            if (r == cudaSuccess) r = cudaEventRecord(e1, st);
            if (r == cudaSuccess) r = cudaEventSynchronize(e1);
            float t = 0.f;
            if (r == cudaSuccess && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess) ms[v] = t / 2.f;
            else cudaGetLastError();
            if (r != cudaSuccess && r != cudaErrorInvalidValue && r != cudaErrorInvalidConfiguration &&
                r != cudaErrorLaunchOutOfResources)
                e = r;  // a sticky error: stop
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFree(tmp);
        if (e != cudaSuccess) return fail(MGB_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
        if (read_clear_device_timeout()) return fail(MGB_ERR_DEVICE_TIMEOUT, "autotune: a device-side wait timed out");
        int best = 0;
        for (int v = 0; v < nv; ++v)
            if (ms[v] >= 0.f && (ms[best] < 0.f || ms[v] < ms[best])) best = v;
        sg.variant = best;
        sg.tune_ms = ms;
        sg.tuned_here = true;
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune[key] = TuneResult{best, ms};
    }
    return MGB_OK;
}

// Run f(segment, stream) for every segment: on `st` when there is one, else
// each on its own stream, forked from and joined back into `st`.
template <class F>
mgb_status for_segments(PlanCore& pc, cudaStream_t st, F&& f) {
    if (pc.segs.size() == 1) return f(pc.segs[0], st);
    MGB_CUDA_TRY(cudaEventRecord(pc.fork, st));
    for (Segment& sg : pc.segs) {
        MGB_CUDA_TRY(cudaStreamWaitEvent(sg.stream, pc.fork, 0));
        mgb_status s = f(sg, sg.stream);
        if (s != MGB_OK) return s;
        MGB_CUDA_TRY(cudaEventRecord(sg.done, sg.stream));
    }
    for (Segment& sg : pc.segs) MGB_CUDA_TRY(cudaStreamWaitEvent(st, sg.done, 0));
    return MGB_OK;
}

mgb_status seg_chunks(PlanCore& pc, Segment& sg, int mode, cudaStream_t s, const char* name) {
    const LaunchArgs la = seg_args(pc, sg, s);
    MGB_CUDA_TRY(timed(name, s, [&] { return launch_chunk_any(pc.plain, pc.kind, pc.rule, mode, la, sg.hi, pc.sms, sg.variant); }));
    return MGB_OK;
}

// Largest n d^2 of a segment's instances (SpaceCurves: d = 2, 4-vectors).
int64_t seg_nm(const Segment& sg) { return (int64_t)sg.nmax * sg.d * sg.d; }

// Forward scan over a segment's chunks: pi^0..pi^C.
mgb_status seg_scan(PlanCore& pc, Segment& sg, cudaStream_t s) {
    const InstDev* di = reinterpret_cast<const InstDev*>(pc.base + pc.off_inst) + sg.first;
    if (sg.df_scan)
        MGB_CUDA_TRY(timed("scan", s, [&] { return launch_scan_df(di, sg.count, sg.d, sg.nmax, false, pc.f64io, s); }));
    else if (sg.tiled_scan)
        MGB_CUDA_TRY(timed("scan", s, [&] { return launch_scan_tiled(di, sg.count, sg.d, sg.nmax, sg.active, false, pc.f64io, s); }));
    else
        MGB_CUDA_TRY(timed("scan", s, [&] { return launch_small(true, pc.kind, SMALL_SCAN, di, sg.count, pc.f64io, 0, seg_nm(sg), s); }));
    return MGB_OK;
}

mgb_status seg_small(PlanCore& pc, Segment& sg, int which, int write_out, cudaStream_t s, const char* name) {
    const InstDev* di = reinterpret_cast<const InstDev*>(pc.base + pc.off_inst) + sg.first;
    if (which == SMALL_RSCAN && sg.df_scan)
        MGB_CUDA_TRY(timed(name, s, [&] { return launch_scan_df(di, sg.count, sg.d, sg.nmax, true, pc.f64io, s); }));
    else if (which == SMALL_RSCAN && sg.tiled_scan)
        MGB_CUDA_TRY(timed(name, s, [&] { return launch_scan_tiled(di, sg.count, sg.d, sg.nmax, sg.active, true, pc.f64io, s); }));
    else if ((which == SMALL_FIN_FWD || which == SMALL_FIN_VJP) && sg.tiled_scan)
        MGB_CUDA_TRY(timed(name, s, [&] {
            return launch_fin_tiled(di, sg.count, sg.d, sg.nmax, which == SMALL_FIN_VJP, write_out, pc.f64io, s);
        }));
    else
        MGB_CUDA_TRY(timed(name, s, [&] { return launch_small(true, pc.kind, which, di, sg.count, pc.f64io, write_out, seg_nm(sg), s); }));
    return MGB_OK;
}

mgb_status plan_forward(PlanCore& pc, cudaStream_t st) {
    if (!pc.has_out) return fail(MGB_ERR_INVALID_ARGUMENT, "output buffer must not be null");
    const InstDev* d_inst = reinterpret_cast<const InstDev*>(pc.base + pc.off_inst);
    mgb_status s = for_segments(pc, st, [&](Segment& sg, cudaStream_t ss) {
        mgb_status r = seg_chunks(pc, sg, MODE_LOCAL, ss, "chunk_local");
        if (r == MGB_OK) r = seg_scan(pc, sg, ss);
        if (r == MGB_OK) r = seg_small(pc, sg, SMALL_FIN_FWD, 1, ss, "fin_fwd");
        return r;
    });
    if (s != MGB_OK) return s;
    if (pc.any_carry) {
        LaunchArgs la;
        la.insts = d_inst;
        la.work = reinterpret_cast<const ChunkRef*>(pc.base + pc.off_work);
        la.nwork = (int64_t)pc.work.size();
        la.scratch = pc.base + pc.off_gscr;
        la.slot_elems = pc.gslot_elems;
        la.grid = pc.ggrid;
        la.f64io = pc.f64io;
        la.stream = st;
        MGB_CUDA_TRY(timed("chunk_carry", st, [&] { return launch_generic_chunk(pc.plain, pc.kind, pc.rule, MODE_CARRY, la); }));
    }
    return MGB_OK;
}

mgb_status plan_vjp(PlanCore& pc, cudaStream_t st, bool recompute) {
    if (!pc.has_vjp) return fail(MGB_ERR_INVALID_ARGUMENT, "cotangent and dA buffers were not given to this plan");
    return for_segments(pc, st, [&](Segment& sg, cudaStream_t ss) {
        mgb_status r = MGB_OK;
        if (recompute) {
            r = seg_chunks(pc, sg, MODE_LOCAL, ss, "chunk_local");
            if (r == MGB_OK) r = seg_scan(pc, sg, ss);
        }
        if (r == MGB_OK) r = seg_small(pc, sg, SMALL_FIN_FWD, 0, ss, "fin_fwd");
        if (r == MGB_OK) r = seg_small(pc, sg, SMALL_FIN_VJP, 0, ss, "fin_vjp");
        if (r == MGB_OK) r = seg_small(pc, sg, SMALL_RSCAN, 0, ss, "rscan");
        if (r == MGB_OK) r = seg_chunks(pc, sg, MODE_VJP, ss, "chunk_vjp");
        return r;
    });
}

// One-shot call: plan in stream-ordered memory, run, release.
mgb_status run_complex(const Call& call);

mgb_status run(const Call& call) {
    if (call.count == 0) return MGB_OK;
    if (call.probs && is_complex(call.probs[0].dtype)) return run_complex(call);
    PlanCore pc;
    std::vector<Derived> dv;
    mgb_status st = plan_layout(call, pc, dv);
    if (st != MGB_OK) return st;
    Workspace ws;
    ws.st = call.stream;
    MGB_CUDA_TRY(cudaMallocAsync(&ws.base, pc.bytes, call.stream));
    pc.base = static_cast<char*>(ws.base);
    plan_fill(call, pc, dv);
    st = plan_upload(pc, call.stream, false);
    if (st == MGB_OK) st = plan_autotune(pc, call.stream);
    if (st == MGB_OK) st = plan_streams(pc);
    if (st == MGB_OK) st = call.vjp ? plan_vjp(pc, call.stream, !pc.all_ck_in) : plan_forward(pc, call.stream);
    pc.release_streams();
    return st;
}

// Complex problems: expand the inputs to the real 2d x 2d form
// (launch_cplx_embed), run the real problems, and read the outputs back
// (launch_cplx_extract).  Checkpoint buffers are the real problems' own.
mgb_status run_complex(const Call& call) {
    const size_t count = call.count;
    for (size_t i = 0; i < count; ++i) {
        Derived dv;
        mgb_status st = validate(&call.probs[i], gl_snapshot()->max_order, &dv);
        if (st != MGB_OK) return st;
        if (call.probs[i].dtype != call.probs[0].dtype)
            return fail(MGB_ERR_INVALID_ARGUMENT, "batched instances must share kind, dtype, precision and integrator");
    }
    if (!call.A) return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
    const bool f64 = call.probs[0].dtype == MGB_DTYPE_C128;
    const size_t es = f64 ? 8 : 4;  // bytes per real part
    std::vector<mgb_problem> rp(count);
    std::vector<size_t> off_a(count), off_o(count), off_c(count), off_k(count), off_g(count);
    size_t bytes = 0;
    for (size_t i = 0; i < count; ++i) {
        const mgb_problem& p = call.probs[i];
        if (!call.A[i]) return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
        rp[i] = real_problem(p);
        const size_t m4 = (size_t)rp[i].dim * rp[i].dim;  // real elements of one matrix of the real problem
        const size_t nout = rp[i].op == MGB_OP_MANY ? (size_t)p.n : 1;
        const size_t Q = p.n > 1 ? (size_t)(p.n + 3) / 2 : 1;
        off_a[i] = bytes; bytes = align_up(bytes + (size_t)p.samples * m4 * es, 256);
        off_o[i] = bytes; bytes = align_up(bytes + nout * m4 * es, 256);
        off_c[i] = bytes;
        if (!call.vjp && call.carry && call.carry[i] && p.n > 1)
            bytes = align_up(bytes + Q * (size_t)(p.n - 1) * (size_t)p.samples * m4 * es, 256);
        off_k[i] = bytes;
        if (call.vjp) bytes = align_up(bytes + nout * m4 * es, 256);
        off_g[i] = bytes;
        if (call.vjp) bytes = align_up(bytes + (size_t)p.samples * m4 * es, 256);
    }
    cudaStream_t st = call.stream;
    Workspace ws;
    ws.st = st;
    MGB_CUDA_TRY(cudaMallocAsync(&ws.base, bytes, st));
    char* base = static_cast<char*>(ws.base);
    std::vector<const void*> rA(count), rcot(count);
    std::vector<void*> rout(count), rcarry(count, nullptr), rdA(count);
    for (size_t i = 0; i < count; ++i) {
        const mgb_problem& p = call.probs[i];
        const bool sc = p.kind == MGB_KIND_SPACECURVE;
        const int d = (int)p.dim;
        const size_t nout = p.op == MGB_OP_MANY ? (size_t)p.n : 1;
        rA[i] = base + off_a[i];
        rout[i] = base + off_o[i];
        if (sc) MGB_CUDA_TRY(launch_sc_complex(SC_EMBED, f64, call.A[i], base + off_a[i], (int64_t)p.samples, (int)p.n, p.op, st));
        else MGB_CUDA_TRY(launch_cplx_embed(f64, call.A[i], base + off_a[i], (int64_t)p.samples, d, false, st));
        if (call.vjp) {
            if (!call.cot || !call.cot[i] || !call.dA || !call.dA[i])
                return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
            rcot[i] = base + off_k[i];
            rdA[i] = base + off_g[i];
            if (sc) MGB_CUDA_TRY(launch_sc_complex(SC_COT, f64, call.cot[i], base + off_k[i], 0, (int)p.n, p.op, st));
            else MGB_CUDA_TRY(launch_cplx_embed(f64, call.cot[i], base + off_k[i], (int64_t)nout, d, true, st));
        } else if (call.carry && call.carry[i] && p.n > 1) {
            rcarry[i] = base + off_c[i];
        }
    }
    Call rc = call;
    rc.probs = rp.data();
    rc.A = rA.data();
    rc.out = call.vjp ? nullptr : rout.data();
    rc.carry = (!call.vjp && call.carry) ? rcarry.data() : nullptr;
    rc.cot = call.vjp ? rcot.data() : nullptr;
    rc.dA = call.vjp ? rdA.data() : nullptr;
    mgb_status s = run(rc);
    if (s != MGB_OK) return s;
    for (size_t i = 0; i < count; ++i) {
        const mgb_problem& p = call.probs[i];
        const int d = (int)p.dim;
        const size_t nout = p.op == MGB_OP_MANY ? (size_t)p.n : 1;
        const size_t Q = p.n > 1 ? (size_t)(p.n + 3) / 2 : 1;
        const bool sc = p.kind == MGB_KIND_SPACECURVE;
        if (call.vjp) {
            if (sc) MGB_CUDA_TRY(launch_sc_complex(SC_GRAD, f64, rdA[i], call.dA[i], (int64_t)p.samples, (int)p.n, p.op, st));
            else MGB_CUDA_TRY(launch_cplx_extract(f64, rdA[i], call.dA[i], (int64_t)p.samples, d, true, st));
        } else {
            if (!call.out || !call.out[i]) return fail(MGB_ERR_INVALID_ARGUMENT, "output buffer must not be null");
            if (sc) MGB_CUDA_TRY(launch_sc_complex(SC_OUT, f64, rout[i], call.out[i], 0, (int)p.n, p.op, st));
            else MGB_CUDA_TRY(launch_cplx_extract(f64, rout[i], call.out[i], (int64_t)nout, d, false, st));
            if (rcarry[i]) {
                if (sc) MGB_CUDA_TRY(launch_sc_complex(SC_CARRY, f64, rcarry[i], call.carry[i], (int64_t)p.samples, (int)p.n, p.op, st));
                else MGB_CUDA_TRY(launch_cplx_extract(f64, rcarry[i], call.carry[i],
                                                      (int64_t)(Q * (size_t)(p.n - 1) * (size_t)p.samples), d, false, st));
            }
        }
    }
    return MGB_OK;
}

}  // namespace

namespace mgb {
// Chooses the fastest chunk kernel available for the call: the tuned
// family when every instance has a shape it covers, else the generic one.
int generic_ctas_per_sm(int variant) { return variant == 1 ? 4 : variant == 2 ? 2 : 8; }

cudaError_t launch_chunk_any(bool plain, int kind, int rule, int mode, const LaunchArgs& a,
                             const std::vector<InstDev>& hi, int sms, int variant) {
    TunedChoice tc = choose_tuned(plain, kind, rule, mode, a.f64io != 0, hi, variant);
    if (tc.use) return launch_tuned(tc, plain, kind, rule, mode, a, sms);
    LaunchArgs g = a;
    g.grid = std::max<int64_t>(1, std::min<int64_t>(a.grid, (int64_t)sms * generic_ctas_per_sm(variant % GENERIC_VARIANTS)));
    return launch_generic_chunk(plain, kind, rule, mode, g);
}
}  // namespace mgb

// ============================================================================
// C ABI
// ============================================================================
struct mgb_plan {
    PlanCore pc;
    bool forward_done = false;
};

// ---------------------------------------------------------------- host staging
namespace {

// SM-driven copy of n4 16-byte words (host side through its device mapping).
__global__ void k_stage_copy(const float4* __restrict__ src, float4* __restrict__ dst, size_t n4) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// Device address of a page-locked host buffer (nullptr for pageable memory).
const void* mapped_host(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Host <-> device copy on stream s: through the copy engines (asynchronous
// for page-locked host buffers, staged by the driver for pageable ones), or,
// with sm and a page-locked, 16-byte aligned host buffer, by a copy kernel
// reading or writing the host memory through its mapping.  On the GB300 host
// link the copy engines moved 14-65 GB/s while no kernel was running (the
// pipeline's fill and drain) against about 210 GB/s beside the kernels; the
// copy kernel keeps about 120-210 GB/s there, at the cost of SM slots, so the
// pipeline uses it only at its two ends.
cudaError_t stage_copy(void* dst, const void* src, size_t bytes, bool to_device, int sms, cudaStream_t s,
                       bool sm = false) {
    if (bytes == 0) return cudaSuccess;
    if (sm && bytes % 16 == 0 && (uintptr_t)src % 16 == 0 && (uintptr_t)dst % 16 == 0) {
        const void* hp = mapped_host(to_device ? src : dst);
        if (hp) {
            const float4* from = static_cast<const float4*>(to_device ? hp : src);
            float4* to = static_cast<float4*>(to_device ? dst : const_cast<void*>(hp));
            k_stage_copy<<<(unsigned)std::max(sms, 1), 512, 0, s>>>(from, to, bytes / 16);
            return cudaGetLastError();
        }
    }
    return cudaMemcpyAsync(dst, src, bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, s);
}

// Staging slots kept per device across calls (grown on demand, held until
// the process exits): the first copy into freshly allocated device memory
// measured 17-35 GB/s on the GB300 against 210 GB/s into memory written
// before, so a fresh allocation per call would put that cost in every call.
struct StageCache {
    std::mutex mu;
    std::vector<std::pair<char*, size_t>> per_dev;
};
StageCache& stage_cache() {
    static StageCache c;
    return c;
}
cudaError_t stage_buffer(size_t bytes, char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    StageCache& c = stage_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    if ((int)c.per_dev.size() <= dev) c.per_dev.resize(dev + 1, {nullptr, 0});
    auto& slot = c.per_dev[dev];
    if (slot.second < bytes) {
        if (slot.first) cudaFree(slot.first);
        slot = {nullptr, 0};
        e = cudaMalloc(&slot.first, bytes);
        if (e != cudaSuccess) {
            slot.first = nullptr;
            return e;
        }
        slot.second = bytes;
    }
    *out = slot.first;
    return cudaSuccess;
}

}  // namespace

extern "C" {

mgb_status mgb_plan_create(const mgb_problem* probs, size_t count, const void* const* A, void* const* out,
                           const void* const* cot, void* const* dA, mgb_plan** plan) {
    g_last_error.clear();
    if (!plan) return fail(MGB_ERR_INVALID_ARGUMENT, "plan pointer must not be null");
    *plan = nullptr;
    Call c{};
    c.count = count;
    c.probs = probs;
    c.A = A;
    c.out = out;
    c.cot = cot;
    c.dA = dA;
    std::unique_ptr<mgb_plan> P(new mgb_plan());
    std::vector<Derived> dv;
    mgb_status st = plan_layout(c, P->pc, dv);
    if (st != MGB_OK) return st;
    void* base = nullptr;
    cudaError_t e = cudaMalloc(&base, P->pc.bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? MGB_ERR_OUT_OF_MEMORY : MGB_ERR_CUDA,
                    std::string("plan workspace: ") + cudaGetErrorString(e));
    }
    P->pc.base = static_cast<char*>(base);
    plan_fill(c, P->pc, dv);
    st = plan_upload(P->pc, nullptr, true);
    if (st == MGB_OK) st = plan_autotune(P->pc, nullptr);
    if (st == MGB_OK) st = plan_streams(P->pc);
    if (st != MGB_OK) {
        P->pc.release_streams();
        cudaFree(base);
        return st;
    }
    *plan = P.release();
    return MGB_OK;
}

mgb_status mgb_plan_forward(mgb_plan* plan, void* stream) {
    g_last_error.clear();
    if (!plan) return fail(MGB_ERR_INVALID_ARGUMENT, "plan must not be null");
    mgb_status st = plan_forward(plan->pc, static_cast<cudaStream_t>(stream));
    if (st == MGB_OK) plan->forward_done = true;
    return st;
}

mgb_status mgb_plan_vjp(mgb_plan* plan, void* stream) {
    g_last_error.clear();
    if (!plan) return fail(MGB_ERR_INVALID_ARGUMENT, "plan must not be null");
    return plan_vjp(plan->pc, static_cast<cudaStream_t>(stream), !plan->forward_done);
}

size_t mgb_plan_bytes(const mgb_plan* plan) { return plan ? plan->pc.bytes : 0; }

size_t mgb_plan_describe(const mgb_plan* plan, char* buf, size_t len) {
    if (!plan) return 0;
    const PlanCore& pc = plan->pc;
    std::string o = "{\"segments\": [";
    char tmp[256];
    for (size_t i = 0; i < pc.segs.size(); ++i) {
        const Segment& sg = pc.segs[i];
        const TunedChoice tc = choose_tuned(pc.plain, pc.kind, pc.rule, MODE_LOCAL, pc.f64io != 0, sg.hi, sg.variant);
        // the forward local pass's kernel; at d = 32 variants 2 and 3 run the
        // VJP on the warp-MMA kernel
        const char* kernel = !tc.use ? "k_chunk" : tc.family == 1 ? "k_small" : tc.family == 3 ? "k_bigtc"
                             : (tc.D == 32 && sg.variant == 2) ? "k_tiletc"
                             : (tc.D == 32 && sg.variant == 3) ? "k_mma32" : "k_tile";
        const int ctas = !tc.use ? generic_ctas_per_sm(sg.variant % GENERIC_VARIANTS) : tc.ctas_per_sm;
        std::snprintf(tmp, sizeof(tmp),
                      "%s{\"d\": %d, \"instances\": %d, \"chunks\": %lld, \"kernel\": \"%s\", \"variant\": %d, "
                      "\"ctas_per_sm\": %d, \"slots\": %lld, \"scan\": \"%s\", \"tuned_ms\": [",
                      i ? ", " : "", sg.d, sg.count, (long long)sg.nwork, kernel, sg.variant, ctas, (long long)sg.grid,
                      sg.tiled_scan ? "tiled" : "per-instance");
        o += tmp;
        for (size_t v = 0; v < sg.tune_ms.size(); ++v) {
            std::snprintf(tmp, sizeof(tmp), "%s%.9g", v ? ", " : "", (double)sg.tune_ms[v]);
            o += tmp;
        }
        o += "]}";
    }
    o += "]}";
    if (buf && len) {
        const size_t n = std::min(len - 1, o.size());
        std::memcpy(buf, o.data(), n);
        buf[n] = 0;
    }
    return o.size() + 1;
}

mgb_status mgb_plan_destroy(mgb_plan* plan) {
    g_last_error.clear();
    if (!plan) return MGB_OK;
    plan->pc.release_streams();
    cudaError_t e = plan->pc.base ? cudaFree(plan->pc.base) : cudaSuccess;
    delete plan;
    if (e != cudaSuccess) return fail(MGB_ERR_CUDA, cudaGetErrorString(e));
    return MGB_OK;
}


mgb_status mgb_forward(const mgb_problem* p, const void* A, void* out, void* carry, void* ckpt, void* stream) {
    g_last_error.clear();
    void* outs[1] = {out};
    void* carries[1] = {carry};
    void* cks[1] = {ckpt};
    Call c{};
    c.vjp = false;
    c.count = 1;
    c.probs = p;
    c.A = &A;
    c.out = outs;
    c.carry = carries;
    c.ckpt_out = cks;
    c.stream = static_cast<cudaStream_t>(stream);
    return run(c);
}

mgb_status mgb_vjp(const mgb_problem* p, const void* A, const void* cot, const void* ckpt, void* dA, void* stream) {
    g_last_error.clear();
    const void* cots[1] = {cot};
    const void* cks[1] = {ckpt};
    void* das[1] = {dA};
    Call c{};
    c.vjp = true;
    c.count = 1;
    c.probs = p;
    c.A = &A;
    c.cot = cots;
    c.ckpt_in = cks;
    c.dA = das;
    c.stream = static_cast<cudaStream_t>(stream);
    return run(c);
}

size_t mgb_checkpoint_bytes(const mgb_problem* p) {
    Derived dv;
    std::string saved = g_last_error;
    mgb_status st = validate(p, gl_snapshot()->max_order, &dv);
    if (st == MGB_OK && is_complex(p->dtype)) {  // the checkpoints of the real problem it runs as
        const mgb_problem r = real_problem(*p);
        st = validate(&r, gl_snapshot()->max_order, &dv);
        g_last_error = saved;
        return st == MGB_OK ? ckpt_doubles(r, dv) * sizeof(double) : 0;
    }
    g_last_error = saved;
    if (st != MGB_OK) return 0;
    return ckpt_doubles(*p, dv) * sizeof(double);
}

mgb_status mgb_forward_batched(const mgb_problem* probs, size_t count, const void* const* A, void* const* out,
                               void* const* ckpt, void* stream) {
    g_last_error.clear();
    Call c{};
    c.vjp = false;
    c.count = count;
    c.probs = probs;
    c.A = A;
    c.out = out;
    c.carry = nullptr;
    c.ckpt_out = ckpt;
    c.stream = static_cast<cudaStream_t>(stream);
    return run(c);
}

mgb_status mgb_vjp_batched(const mgb_problem* probs, size_t count, const void* const* A, const void* const* cot,
                           const void* const* ckpt, void* const* dA, void* stream) {
    g_last_error.clear();
    Call c{};
    c.vjp = true;
    c.count = count;
    c.probs = probs;
    c.A = A;
    c.cot = cot;
    c.ckpt_in = ckpt;
    c.dA = dA;
    c.stream = static_cast<cudaStream_t>(stream);
    return run(c);
}

static size_t elem_size(const mgb_problem* p) {
    return p->dtype == MGB_DTYPE_C128 ? 16 : (p->dtype == MGB_DTYPE_F64 || p->dtype == MGB_DTYPE_C64) ? 8 : 4;
}

static void sizes_of(const mgb_problem* p, size_t* in_elems, size_t* out_elems, size_t* carry_elems) {
    const size_t m = p->kind == MGB_KIND_SPACECURVE ? 4 : (size_t)(p->dim * p->dim);
    const size_t mi = p->kind == MGB_KIND_SPACECURVE ? 3 : m;
    *in_elems = (size_t)p->samples * mi;
    *out_elems = (p->op == MGB_OP_MANY ? (size_t)p->n : 1) * mi;
    const size_t Q = p->n > 1 ? (size_t)(p->n + 3) / 2 : 1;
    *carry_elems = p->n > 1 ? Q * (size_t)(p->n - 1) * (size_t)p->samples * m : 0;
}

mgb_status mgb_forward_host(const mgb_problem* p, const void* A, void* out, void* carry) {
    g_last_error.clear();
    Derived dv;
    mgb_status st = validate(p, gl_snapshot()->max_order, &dv);
    if (st != MGB_OK) return st;
    if (!A) return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
    if (!out) return fail(MGB_ERR_INVALID_ARGUMENT, "output buffer must not be null");
    size_t ni, no, nc;
    sizes_of(p, &ni, &no, &nc);
    const size_t es = elem_size(p);
    void *dA_ = nullptr, *dO = nullptr, *dC = nullptr;
    auto cleanup = [&]() {
        if (dA_) cudaFree(dA_);
        if (dO) cudaFree(dO);
        if (dC) cudaFree(dC);
    };
    cudaError_t e = cudaMalloc(&dA_, ni * es);
    if (e == cudaSuccess) e = cudaMalloc(&dO, no * es);
    if (e == cudaSuccess && carry && nc) e = cudaMalloc(&dC, nc * es);
    if (e == cudaSuccess) e = cudaMemcpy(dA_, A, ni * es, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cleanup();
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? MGB_ERR_OUT_OF_MEMORY : MGB_ERR_CUDA, cudaGetErrorString(e));
    }
    st = mgb_forward(p, dA_, dO, dC, nullptr, nullptr);
    if (st == MGB_OK) {
        e = cudaMemcpy(out, dO, no * es, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && dC) e = cudaMemcpy(carry, dC, nc * es, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = fail(MGB_ERR_CUDA, cudaGetErrorString(e));
        else if (read_clear_device_timeout()) st = fail(MGB_ERR_DEVICE_TIMEOUT, "a device-side wait timed out");
    }
    cleanup();
    return st;
}

mgb_status mgb_vjp_host(const mgb_problem* p, const void* A, const void* cot, void* dA) {
    g_last_error.clear();
    Derived dv;
    mgb_status st = validate(p, gl_snapshot()->max_order, &dv);
    if (st != MGB_OK) return st;
    if (!A || !cot) return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
    if (!dA) return fail(MGB_ERR_INVALID_ARGUMENT, "output buffer must not be null");
    size_t ni, no, nc;
    sizes_of(p, &ni, &no, &nc);
    const size_t es = elem_size(p);
    void *dIn = nullptr, *dCot = nullptr, *dOut = nullptr;
    auto cleanup = [&]() {
        if (dIn) cudaFree(dIn);
        if (dCot) cudaFree(dCot);
        if (dOut) cudaFree(dOut);
    };
    cudaError_t e = cudaMalloc(&dIn, ni * es);
    if (e == cudaSuccess) e = cudaMalloc(&dCot, no * es);
    if (e == cudaSuccess) e = cudaMalloc(&dOut, ni * es);
    if (e == cudaSuccess) e = cudaMemcpy(dIn, A, ni * es, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dCot, cot, no * es, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cleanup();
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? MGB_ERR_OUT_OF_MEMORY : MGB_ERR_CUDA, cudaGetErrorString(e));
    }
    st = mgb_vjp(p, dIn, dCot, nullptr, dOut, nullptr);
    if (st == MGB_OK) {
        e = cudaMemcpy(dA, dOut, ni * es, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = fail(MGB_ERR_CUDA, cudaGetErrorString(e));
        else if (read_clear_device_timeout()) st = fail(MGB_ERR_DEVICE_TIMEOUT, "a device-side wait timed out");
    }
    cleanup();
    return st;
}

mgb_status mgb_fwd_vjp_host_batched(const mgb_problem* probs, size_t count, const void* const* A,
                                    const void* const* cot, void* const* out, void* const* dA) {
    g_last_error.clear();
    if (count == 0) return MGB_OK;
    if (!probs || !A || !cot || !out || !dA) return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
    const int sms = device_info().sms;
    // per-instance byte sizes; sub-batches of 1/parts of the input (>= 256 MB, >= 1 instance)
    std::vector<size_t> bin(count), bout(count), bck(count);
    size_t total = 0;
    for (size_t i = 0; i < count; ++i) {
        Derived dv;
        mgb_status st = validate(&probs[i], gl_snapshot()->max_order, &dv);
        if (st != MGB_OK) return st;
        if (!A[i] || !cot[i] || !out[i] || !dA[i]) return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
        size_t ni, no, nc;
        sizes_of(&probs[i], &ni, &no, &nc);
        bin[i] = ni * elem_size(&probs[i]);
        bout[i] = no * elem_size(&probs[i]);
        bck[i] = mgb_checkpoint_bytes(&probs[i]);
        total += bin[i];
    }
    // Sub-batches: MGB_HOST_SUBBATCHES = p > 0 cuts p equal parts; by default
    // the sizes ramp up and down (1, 3, 4, 4, 3, 1 sixteenths of the input),
    // so that the kernels start after a short first copy and the last copy
    // out is short (the pipeline's fill and drain); each part >= 256 MB.
    const int parts = env_int("MGB_HOST_SUBBATCHES", 0);
    std::vector<double> weights;
    if (parts > 0) weights.assign((size_t)parts, 1.0);
    else weights = {1, 3, 4, 4, 3, 1};
    double wsum = 0.0;
    for (double w : weights) wsum += w;
    std::vector<size_t> cut{0};
    {
        const size_t minb = (size_t)256 << 20;
        double bound = 0.0;
        size_t k = 0, acc = 0, in_part = 0;
        bound = (double)total * weights[0] / wsum;
        for (size_t i = 0; i < count; ++i) {
            acc += bin[i];
            in_part += bin[i];
            if (i + 1 < count && k + 1 < weights.size() && (double)acc >= bound && in_part >= minb) {
                cut.push_back(i + 1);
                in_part = 0;
                ++k;
                bound += (double)total * weights[k] / wsum;
            }
        }
    }
    cut.push_back(count);
    const size_t nb = cut.size() - 1;
    // Three rotating device slots (data: A, dA, out, cot, checkpoints; then
    // the sub-batch's plan).  The H2D copy of one sub-batch, the kernels of
    // the previous one and the D2H copy of the one before overlap; a slot's
    // plan descriptors are written (a synchronous copy on the legacy stream,
    // which does not wait for the pipeline's non-blocking streams) only after
    // the kernels that last used the slot have finished.
    constexpr int NS = 3;
    constexpr size_t kPlaceholder = (size_t)1 << 20;
    struct Sub {
        std::vector<const void*> in, cot;
        std::vector<void*> out, dA, ck;
        Call call{};
        PlanCore pc;
        std::vector<Derived> dv;
        size_t data_bytes = 0;
    };
    std::vector<Sub> sub(nb);
    size_t data_slot = 0;
    for (size_t b = 0; b < nb; ++b) {
        for (size_t i = cut[b]; i < cut[b + 1]; ++i)
            sub[b].data_bytes += 2 * align_up(bin[i], 256) + 2 * align_up(bout[i], 256) + align_up(bck[i], 256);
        data_slot = std::max(data_slot, sub[b].data_bytes);
    }
    char* dev = nullptr;
    cudaError_t e = cudaSuccess;
    auto cuda_fail = [&](cudaError_t err) {
        cudaGetLastError();
        return fail(err == cudaErrorMemoryAllocation ? MGB_ERR_OUT_OF_MEMORY : MGB_ERR_CUDA, cudaGetErrorString(err));
    };
    // lay out every sub-batch's plan against its slot's data addresses
    // (known once the data area size is fixed; the plan area follows it)
    mgb_status st = MGB_OK;
    size_t plan_slot = 0;
    for (size_t b = 0; b < nb && st == MGB_OK; ++b) {
        Sub& u = sub[b];
        const size_t i0 = cut[b], cnt = cut[b + 1] - cut[b];
        u.in.resize(cnt); u.cot.resize(cnt); u.out.resize(cnt); u.dA.resize(cnt); u.ck.resize(cnt);
        // offsets from the slot base, tagged with a non-null placeholder base
        // (the layout only checks presence and alignment); rebased below
        size_t off = kPlaceholder;
        for (size_t j = 0; j < cnt; ++j) {
            const size_t i = i0 + j;
            u.in[j] = reinterpret_cast<const void*>(off); off += align_up(bin[i], 256);
            u.dA[j] = reinterpret_cast<void*>(off); off += align_up(bin[i], 256);
            u.out[j] = reinterpret_cast<void*>(off); off += align_up(bout[i], 256);
            u.cot[j] = reinterpret_cast<const void*>(off); off += align_up(bout[i], 256);
            u.ck[j] = reinterpret_cast<void*>(off); off += align_up(bck[i], 256);
        }
        u.call.vjp = false;
        u.call.count = cnt;
        u.call.probs = probs + i0;
        u.call.A = u.in.data();
        u.call.out = u.out.data();
        u.call.cot = u.cot.data();
        u.call.dA = u.dA.data();
        u.call.ckpt_out = u.ck.data();
        u.call.budget_parts = NS;
        st = plan_layout(u.call, u.pc, u.dv);
        plan_slot = std::max(plan_slot, u.pc.bytes);
    }
    if (st != MGB_OK) return st;
    const size_t slot_bytes = align_up(data_slot, 256) + plan_slot;
    cudaStream_t sin = nullptr, scomp = nullptr, sout = nullptr;
    cudaEvent_t ev_in[NS] = {}, ev_comp[NS] = {}, ev_out[NS] = {};
    bool used[NS] = {false, false, false};
    // one call at a time per process uses the cached staging slots
    static std::mutex call_mu;
    std::lock_guard<std::mutex> call_lock(call_mu);
    e = stage_buffer((size_t)NS * slot_bytes, &dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sin, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&scomp, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sout, cudaStreamNonBlocking);
    for (int k = 0; k < NS && e == cudaSuccess; ++k) {
        e = cudaEventCreateWithFlags(&ev_in[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_comp[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_out[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) st = cuda_fail(e);
    for (size_t b = 0; b < nb && st == MGB_OK; ++b) {
        Sub& u = sub[b];
        const int k = (int)(b % NS);
        const size_t i0 = cut[b], cnt = cut[b + 1] - cut[b];
        char* base = dev + (size_t)k * slot_bytes;
        auto at = [&](const void* rel) { return base + (reinterpret_cast<uintptr_t>(rel) - kPlaceholder); };
        for (size_t j = 0; j < cnt; ++j) {
            u.in[j] = at(u.in[j]);
            u.dA[j] = at(u.dA[j]);
            u.out[j] = at(u.out[j]);
            u.cot[j] = at(u.cot[j]);
            u.ck[j] = at(u.ck[j]);
        }
        // the slot's previous kernels must be done before its plan area is
        // rewritten (host wait), its previous output copy before new inputs land
        if (used[k]) e = cudaEventSynchronize(ev_comp[k]);
        if (e != cudaSuccess) {
            st = cuda_fail(e);
            break;
        }
        u.pc.base = base + align_up(data_slot, 256);
        plan_fill(u.call, u.pc, u.dv);
        st = plan_upload(u.pc, nullptr, true);
        if (st == MGB_OK) st = plan_autotune(u.pc, nullptr);
        if (st == MGB_OK) st = plan_streams(u.pc);
        if (st != MGB_OK) break;
        if (used[k]) e = cudaStreamWaitEvent(sin, ev_out[k], 0);
        char nm_in[32], nm_comp[32], nm_out[32];
        std::snprintf(nm_in, sizeof nm_in, "h2d.%zu", b);
        std::snprintf(nm_comp, sizeof nm_comp, "comp.%zu", b);
        std::snprintf(nm_out, sizeof nm_out, "d2h.%zu", b);
        if (e == cudaSuccess)
            e = timed(nm_in, sin, [&] {
                cudaError_t r = cudaSuccess;
                for (size_t j = 0; j < cnt && r == cudaSuccess; ++j) {
                    r = stage_copy(const_cast<void*>(u.in[j]), A[i0 + j], bin[i0 + j], true, sms, sin, b < 2);
                    if (r == cudaSuccess) r = stage_copy(const_cast<void*>(u.cot[j]), cot[i0 + j], bout[i0 + j], true, sms, sin);
                }
                return r;
            });
        if (e == cudaSuccess) e = cudaEventRecord(ev_in[k], sin);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(scomp, ev_in[k], 0);
        if (e != cudaSuccess) {
            st = cuda_fail(e);
            break;
        }
        e = timed(nm_comp, scomp, [&] {
            st = plan_forward(u.pc, scomp);
            if (st == MGB_OK) st = plan_vjp(u.pc, scomp, false);
            return cudaSuccess;
        });
        if (st != MGB_OK) break;
        if (e != cudaSuccess) {
            st = cuda_fail(e);
            break;
        }
        e = cudaEventRecord(ev_comp[k], scomp);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sout, ev_comp[k], 0);
        if (e == cudaSuccess)
            e = timed(nm_out, sout, [&] {
                cudaError_t r = cudaSuccess;
                for (size_t j = 0; j < cnt && r == cudaSuccess; ++j) {
                    r = stage_copy(out[i0 + j], u.out[j], bout[i0 + j], false, sms, sout);
                    if (r == cudaSuccess) r = stage_copy(dA[i0 + j], u.dA[j], bin[i0 + j], false, sms, sout, b + 2 >= nb);
                }
                return r;
            });
        if (e == cudaSuccess) e = cudaEventRecord(ev_out[k], sout);
        if (e != cudaSuccess) st = cuda_fail(e);
        used[k] = true;
    }
    for (cudaStream_t s2 : {sin, scomp, sout})
        if (s2) {
            e = cudaStreamSynchronize(s2);
            if (e != cudaSuccess && st == MGB_OK) st = cuda_fail(e);
        }
    if (st == MGB_OK && read_clear_device_timeout()) st = fail(MGB_ERR_DEVICE_TIMEOUT, "a device-side wait timed out");
    for (Sub& u : sub) u.pc.release_streams();
    for (int k = 0; k < NS; ++k) {
        if (ev_in[k]) cudaEventDestroy(ev_in[k]);
        if (ev_comp[k]) cudaEventDestroy(ev_comp[k]);
        if (ev_out[k]) cudaEventDestroy(ev_out[k]);
    }
    for (cudaStream_t s2 : {sin, scomp, sout})
        if (s2) cudaStreamDestroy(s2);
    return st;
}

mgb_status mgb_set_gl_table(size_t max_order, const double* weights, const double* nodes) {
    g_last_error.clear();
    if (max_order == 0) return fail(MGB_ERR_INVALID_ARGUMENT, "max_order must be at least 1");
    if (max_order > 4096) return fail(MGB_ERR_INVALID_ARGUMENT, "max_order is too large");
    if (!weights || !nodes) return fail(MGB_ERR_INVALID_ARGUMENT, "GL data must not be null");
    const size_t cnt = max_order * (max_order + 1) / 2;
    auto t = std::make_shared<GLData>();
    t->max_order = max_order;
    t->w.assign(weights, weights + cnt);
    t->x.assign(nodes, nodes + cnt);
    std::lock_guard<std::mutex> lock(g_gl_mutex);
    g_gl = t;
    return MGB_OK;
}

size_t mgb_max_order(void) { return gl_snapshot()->max_order; }

mgb_status mgb_device_check(void) {
    g_last_error.clear();
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail(MGB_ERR_CUDA, cudaGetErrorString(e));
    if (read_clear_device_timeout()) return fail(MGB_ERR_DEVICE_TIMEOUT, "a device-side wait timed out");
    return MGB_OK;
}

mgb_status mgb_selftest_bounded_wait(int64_t limit_ns, void* stream) {
    g_last_error.clear();
    if (limit_ns <= 0 || limit_ns > 2000000000LL)
        return fail(MGB_ERR_INVALID_ARGUMENT, "limit_ns must be in (0, 2e9]");
    MGB_CUDA_TRY(launch_wait_selftest((uint64_t)limit_ns, static_cast<cudaStream_t>(stream)));
    return MGB_OK;
}

const char* mgb_last_error(void) { return g_last_error.c_str(); }

mgb_status mgb_profile_enable(int enable) {
    std::lock_guard<std::mutex> lock(g_prof_mutex);
    if (enable && !g_prof_enabled) {
        if (!g_prof_ref && cudaEventCreate(&g_prof_ref) != cudaSuccess) g_prof_ref = nullptr;
        if (g_prof_ref) cudaEventRecord(g_prof_ref, nullptr);
    }
    g_prof_enabled = enable != 0;
    return MGB_OK;
}

size_t mgb_profile_read(mgb_kernel_time* out, size_t capacity, int reset) {
    std::lock_guard<std::mutex> lock(g_prof_mutex);
    for (auto& ev : g_prof_pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(ev.stop) == cudaSuccess && cudaEventElapsedTime(&ms, ev.start, ev.stop) == cudaSuccess) {
            auto it = std::find_if(g_prof_totals.begin(), g_prof_totals.end(),
                                   [&](const std::pair<std::string, ProfTotal>& t) { return t.first == ev.name; });
            if (it == g_prof_totals.end()) {
                g_prof_totals.push_back({ev.name, ProfTotal{}});
                it = g_prof_totals.end() - 1;
            }
            it->second.launches += 1;
            it->second.ms += ms;
            float t0 = 0.f, t1 = 0.f;
            if (g_prof_ref && cudaEventElapsedTime(&t0, g_prof_ref, ev.start) == cudaSuccess &&
                cudaEventElapsedTime(&t1, g_prof_ref, ev.stop) == cudaSuccess) {
                it->second.first = std::min(it->second.first, (double)t0);
                it->second.last = std::max(it->second.last, (double)t1);
            }
        }
        cudaEventDestroy(ev.start);
        cudaEventDestroy(ev.stop);
    }
    g_prof_pending.clear();
    size_t count = g_prof_totals.size();
    for (size_t i = 0; i < count && i < capacity && out; ++i) {
        std::memset(out[i].name, 0, sizeof(out[i].name));
        std::strncpy(out[i].name, g_prof_totals[i].first.c_str(), sizeof(out[i].name) - 1);
        out[i].launches = g_prof_totals[i].second.launches;
        out[i].total_ms = g_prof_totals[i].second.ms;
        out[i].first_start_ms = g_prof_totals[i].second.first;
        out[i].last_end_ms = g_prof_totals[i].second.last;
    }
    if (reset) g_prof_totals.clear();
    return count;
}

int mgb_version(void) { return 1; }

}  // extern "C"

// ============================================================================
// Forward that allocates no device memory: mgb_forward_noalloc.
//
// Some callers cannot call cudaMalloc in the middle of their work: an XLA /
// JAX custom call or another framework whose caching allocator already owns
// (nearly) all of the GPU's memory, or a host that forbids device-memory
// allocation while it is running (a real-time loop, a callback that must not
// synchronize the device).  For them this entry point keeps all of its
// working memory — the call's descriptors, chunk work list, Gauss-Legendre
// values, chunk checkpoints, per-instance small-math buffers and the chunk
// kernels' per-CTA slots — in one fixed array compiled into this library,
// g_noalloc_scratch below.  The array's size is fixed (MGB_NOALLOC_SCRATCH_BYTES,
// 64 MiB), so every GPU that loads the library holds it until the process
// exits, and problems whose workspace does not fit are rejected.
//
// Sharing: every call on a device uses the same array and leaves its contents
// behind for the next call.  No part of it has to start at zero (each kernel
// writes what it reads first), so nothing is cleared between calls.  Calls
// whose GPU work can overlap (different streams without ordering between
// them) race on the array; order them on one stream or synchronize between
// them.
// ============================================================================
namespace {

constexpr size_t kNoAllocBytes = (size_t)64 << 20;
static_assert(kNoAllocBytes == MGB_NOALLOC_SCRATCH_BYTES, "keep the header constant in sync");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// The call's descriptor and Gauss-Legendre values travel as kernel
// parameters, so the entry point enqueues kernels only: a host-to-device copy
// from pageable host memory would make the driver wait for the stream.
constexpr int kNoAllocGLSlice = 32;
struct NoAllocGL {
    double w[kNoAllocGLSlice];
    double x[kNoAllocGLSlice];
};

__global__ void k_noalloc_setup(InstDev I, InstDev* dst, NoAllocGL gl, int q0, int nq, double* glw, double* glx,
                                ChunkRef* work, int C) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid == 0 && dst) *dst = I;
    if (tid < nq) {
        glw[q0 + tid] = gl.w[tid];
        glx[q0 + tid] = gl.x[tid];
    }
    for (int c = tid; c < C; c += gridDim.x * blockDim.x) work[c] = ChunkRef{0, c};
}

std::mutex g_noalloc_mutex;
std::vector<void*> g_noalloc_base;  // device address of g_noalloc_scratch, per device ordinal

// Device address of the array on the current device.  The first call on a
// device looks it up with cudaGetSymbolAddress (with that device current);
// later calls reuse the cached address.
mgb_status noalloc_base(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(MGB_ERR_CUDA, std::string(cudaGetErrorString(e)) + " in cudaGetDevice");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if ((int)g_noalloc_base.size() <= dev) g_noalloc_base.resize(dev + 1, nullptr);
    if (!g_noalloc_base[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(MGB_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch) failed: ") + cudaGetErrorString(e));
        g_noalloc_base[dev] = ptr;
    }
    *out = g_noalloc_base[dev];
    return MGB_OK;
}

}  // namespace

extern "C" mgb_status mgb_forward_noalloc(const mgb_problem* p, const void* A, void* out, void* stream) {
    g_last_error.clear();
    auto gl = gl_snapshot();
    Derived v;
    mgb_status st = validate(p, gl->max_order, &v);
    if (st != MGB_OK) return st;
    if (is_complex(p->dtype))
        return fail(MGB_ERR_INVALID_ARGUMENT, "complex problems run through mgb_forward / mgb_vjp and their batched and host forms");
    if (!A) return fail(MGB_ERR_INVALID_ARGUMENT, "input buffer must not be null");
    if (!out) return fail(MGB_ERR_INVALID_ARGUMENT, "output buffer must not be null");
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    const bool plain = p->precision == MGB_PRECISION_PLAIN;
    const int f64io = p->dtype == MGB_DTYPE_F64;
    const size_t tsz = plain ? sizeof(double) : sizeof(float);

    // layout inside the fixed array (same pieces as a regular call)
    const int64_t L = std::min<int64_t>((int64_t)v.K, (int64_t)p->samples - 1) + 1;
    const int64_t slot_elems = (int64_t)(p->n + 4) * L * v.m + 3 * (int64_t)p->n * v.m;
    size_t off = 0;
    const size_t off_inst = off; off = align_up(off + sizeof(InstDev), 256);
    const size_t off_work = off; off = align_up(off + (size_t)v.C * sizeof(ChunkRef), 256);
    const size_t off_gl = off; off = align_up(off + 2 * (size_t)v.Q * sizeof(double), 256);
    const size_t off_ck = off; off = align_up(off + ckpt_doubles(*p, v) * sizeof(double), 256);
    const size_t off_ws = off; off = align_up(off + ws_doubles(v) * sizeof(double), 256);
    const size_t off_scr = off;
    const size_t slot_bytes = (size_t)slot_elems * tsz;
    if (off_scr + slot_bytes > kNoAllocBytes)
        return fail(MGB_ERR_INVALID_ARGUMENT,
                    "problem needs " + std::to_string(off_scr + slot_bytes) +
                        " bytes of workspace; mgb_forward_noalloc is limited to MGB_NOALLOC_SCRATCH_BYTES (" +
                        std::to_string(kNoAllocBytes) + ")");
    const DevInfo di = device_info();

    void* basev = nullptr;
    st = noalloc_base(&basev);
    if (st != MGB_OK) return st;
    char* base = static_cast<char*>(basev);

    InstDev I;
    std::memset(&I, 0, sizeof(I));
    double* ck = reinterpret_cast<double*>(base + off_ck);
    double* w = reinterpret_cast<double*>(base + off_ws);
    I.A = A;
    I.out = out;
    I.pi = ck;
    I.lam = ck + (size_t)(v.C + 1) * v.nm;
    I.rho = w; w += (size_t)v.C * v.nm;
    I.dq = w; w += (size_t)v.Q * v.nm;
    I.ee = w; w += v.nm;
    I.tau = w; w += v.nm;
    I.ob = w; w += v.nm;
    I.eb = w; w += v.nm;
    I.db = w; w += v.nm;
    I.tt = w; w += v.nm;
    double* g = reinterpret_cast<double*>(base + off_gl);
    I.glw = g;
    I.glx = g + v.Q;
    I.dt = (p->tf - p->t0) / (double)(p->samples - 1);
    I.dt_k = kernel_step(*p, I.dt);
    fill_rule_coefs(I);
    I.sig = (I.dt_k != 0.0) ? I.dt / I.dt_k : 1.0;
    I.S = (int64_t)p->samples;
    I.d = (p->kind == MGB_KIND_SPACECURVE) ? 2 : (int32_t)p->dim;
    I.m = v.m;
    I.n = (int32_t)p->n;
    I.C = v.C;
    I.Q = v.Q;
    I.K = v.K;
    I.op = p->op;
    const size_t go = (size_t)v.Q * (v.Q - 1) / 2;
    InstDev* d_inst = reinterpret_cast<InstDev*>(base + off_inst);
    ChunkRef* d_work = reinterpret_cast<ChunkRef*>(base + off_work);
    for (int q0 = 0; q0 < v.Q || q0 == 0; q0 += kNoAllocGLSlice) {
        NoAllocGL sl;
        std::memset(&sl, 0, sizeof(sl));
        const int nq = std::min(kNoAllocGLSlice, v.Q - q0);
        for (int q = 0; q < nq; ++q) {
            sl.w[q] = gl->w[go + q0 + q];
            sl.x[q] = gl->x[go + q0 + q];
        }
        const int C = q0 == 0 ? v.C : 0;
        const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(((int64_t)C + 255) / 256, 1024));
        k_noalloc_setup<<<blocks, 256, 0, cs>>>(I, q0 == 0 ? d_inst : nullptr, sl, q0, nq, g, g + v.Q, d_work, C);
        MGB_CUDA_TRY(cudaGetLastError());
    }

    // Grid: as many CTAs (threads, for the one-thread-per-chunk kernel of
    // 2 x 2 and SpaceCurve data) as a regular call would run, cut to the
    // slots that fit in the array.  The thread-per-chunk kernel touches its
    // slot only in the VJP, so its forward slots are the minimum it lays out.
    const std::vector<InstDev> hi(1, I);
    const TunedChoice tc = choose_tuned(plain, p->kind, p->integrator, MODE_LOCAL, f64io != 0, hi, 0);
    int64_t slot_use = slot_elems;
    if (tc.use && tc.family == 1) slot_use = 16 * (int64_t)small_family_max_levels();
    const SegSizing sz = size_segment(plain, p->kind, p->integrator, f64io != 0, hi, v.C, di.sms, ~(size_t)0 >> 1);
    const int64_t grid = std::max<int64_t>(
        1, std::min<int64_t>(sz.grid, (int64_t)((kNoAllocBytes - off_scr) / ((size_t)slot_use * tsz))));

    LaunchArgs la;
    la.insts = d_inst;
    la.work = d_work;
    la.nwork = v.C;
    la.scratch = base + off_scr;
    la.slot_elems = slot_use;
    la.grid = grid;
    la.f64io = f64io;
    la.stream = cs;
    MGB_CUDA_TRY(launch_chunk_any(plain, p->kind, p->integrator, MODE_LOCAL, la, hi, di.sms, 0));
    MGB_CUDA_TRY(launch_small(true, p->kind, SMALL_SCAN, d_inst, 1, f64io, 0, (int64_t)p->n * v.m, cs));
    MGB_CUDA_TRY(launch_small(true, p->kind, SMALL_FIN_FWD, d_inst, 1, f64io, 1, (int64_t)p->n * v.m, cs));
    return MGB_OK;
}
