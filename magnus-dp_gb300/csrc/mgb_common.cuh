// Device-side building blocks shared by all engine kernels.
//
// Algorithm (one instance; S samples A_i, order n, dt = (tf-t0)/(S-1)):
//   The reference runs, for each of Q = (n+3)/2 Gauss-Legendre nodes x_q,
//   Y_1 = A, Y_k[i] = A[i] (P_k[i] + s T_k) with P_k = prefix(Y_{k-1}),
//   T_k = P_k[S-1], s = x_q - 1 (src/magnus.hpp:60-84).  Because prefix is
//   linear and commutes with right-multiplication by constants, every Y_k is
//   Y_k = sum_j W_j D_{k-j+1} with node-independent "levels"
//       W_1 = A,  P_j = prefix(W_j),  W_{j+1}[i] = A[i] P_j[i],
//   and small per-node coefficients D_1 = 1, D_m = s sum_{j<m} T_j D_{m-j}.
//   For all four block rules the rule's weighted sum equals its prefix total,
//   dt * sum_w(W_j) = P_j[S-1] = T_j, so
//       Omega_1 = T_1,  Omega_k = sum_{j<=k} T_j E_{k-j+1},  E_m = sum_q w_q D_m^(q).
//   The GPU work is therefore the nested prefix totals T_1..T_n: n-1 products
//   per sample instead of Q(n-1).
//
//   The sample axis is cut into chunks [b_c, e_c] (e_c = b_{c+1}, b_c a
//   multiple of 4 so every rule block lies inside one chunk).  With the
//   chunk's zero-carry local prefixes L_j, Chen's identity gives
//       P_j[i] = sum_{m=0..j} L_{j-m}[i] pi_m     (pi_0 = 1, L_0 = 1)
//   so chunks run in parallel and a scan over chunk summaries
//   Lambda^c_j = L_j[e_c] carries pi (FP64) from chunk to chunk.  The adjoint
//   runs the same structure backwards: a reverse scan of Lambda^T gives the
//   cotangent rho on each chunk's end state, and each chunk then replays its
//   forward (from the checkpoint pi^c) and its reverse locally.
//
// SpaceCurve data (a 3-vector f padded to (0, f), src/composer/backends.hpp:
// 253-301) uses the reference product c = (a.b, -b0 a + a x b)
// (src/linalg/spacecurve.hpp:8-18), which equals -qmul(a, b) for the
// associative product qmul(a, b) = b (x) a (Hamilton).  With the level
// variables scaled by (-1)^(k-1) the recursion becomes the same associative
// recursion under qmul; outputs, cotangents and carries pick up the signs
// (-1)^(k-1) (Omega_k) and (-1)^k (carry P_k).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mgb {

enum Kind : int { KIND_MATRIX = 0, KIND_SC = 1 };
enum Rule : int { R_BOOLE = 0, R_SIMPSON = 1, R_TRAP = 2, R_RIEMANN = 3 };
enum OpKind : int { OP_ONE = 0, OP_MANY = 1, OP_SUM = 2 };

// Per-instance descriptor, resident in device memory for the duration of a
// call.  Level j (1..n) of an n*m block sits at offset (j-1)*m.
struct InstDev {
    const void* A;     // (S, d, d) or (S, 3), problem dtype
    void* out;         // forward output, problem dtype (nullable in VJP runs)
    void* carry;       // reference-format carry (nullable)
    const void* cot;   // VJP cotangent (nullable in forward runs)
    void* dA;          // VJP output (nullable in forward runs)
    double* pi;        // (C+1) * n*m  : chunk start states, pi[C] = totals T
    double* lam;       // C * n*m      : chunk transfer Lambda^c
    double* rho;       // C * n*m      : cotangent on chunk c's end state
    double* dq;        // Q * n*m      : D_k^(q), k = 1..n
    double* ee;        // n*m          : E_k
    double* tau;       // n*m          : cotangent on T_k
    double* ob;        // n*m          : Omega / Omega-bar scratch
    double* eb;        // n*m          : E-bar scratch
    double* db;        // n*m          : D-bar scratch
    double* tt;        // n*m          : totals T_j = sig^j * pi[C]_j
    double* dbq;       // Q * n*m      : D-bar per node (GPU-wide adjoint)
    double* tauq;      // Q * n*m      : tau contributions per node (GPU-wide adjoint)
    const double* glw; // Q weights on [0, 1]
    const double* glx; // Q nodes on [0, 1]
    double dt;
    // The chunk kernels integrate with step dt_k and the totals are rescaled
    // by sig^j = (dt/dt_k)^j in FP64 (prefix level j is homogeneous of degree
    // j in the step).  Plain form: dt_k = dt, sig = 1.  Mixed form: dt_k is a
    // power of two times the rule's coefficient denominator (90 Boole, 6
    // Simpson, 2 Trapezoid, 1 Riemann), so every rule weight is exact in FP32.
    double dt_k;
    double sig;
    int64_t S;
    int32_t d, m, n, C, Q, K, op;
    // 1: lam holds each transfer element as the chunk kernel's unevaluated
    // FP32 pair (hi, lo) in its 8 bytes (segments whose scans run in
    // double-FP32 read the pair as it is, with no FP64 conversions); 0: FP64
    int32_t lam_pair;
    // The rule coefficients of dt_k (RuleCoef's order), computed once on the
    // host by rule_coefs(): FP64 divisions in every thread of every chunk
    // took a large share of the 1/64-rate FP64 pipe.
    double rcd[9];
    float rcf[9];
    int32_t pad2_;
};

// Store element idx of the chunk transfers (a local prefix total hi + lo).
// Every chunk kernel of a segment goes through this (the scans of a
// double-FP32 segment read pairs whichever kernel ran); FP64 totals (the
// plain form, whose scans are FP64) are stored as they are.
__device__ __forceinline__ void store_lam(const InstDev& I, int64_t idx, float hi, float lo) {
    if (I.lam_pair) reinterpret_cast<float2*>(I.lam)[idx] = make_float2(hi, lo);
    else I.lam[idx] = (double)hi + (double)lo;
}
__device__ __forceinline__ void store_lam(const InstDev& I, int64_t idx, double hi, double lo) {
    I.lam[idx] = hi + lo;
}

// h, t3, c38, c98, c4_3, b14, b64, b24, dt of a step (host and device).
__host__ __device__ inline void rule_coefs(double dtd, double* c) {
    c[0] = dtd / 2;
    c[1] = dtd / 3;
    c[2] = 3 * dtd / 8;
    c[3] = 9 * dtd / 8;
    c[4] = 4 * dtd / 3;
    c[5] = 14 * dtd / 45;
    c[6] = 64 * dtd / 45;
    c[7] = 24 * dtd / 45;
    c[8] = dtd;
}
inline void fill_rule_coefs(InstDev& I) {
    rule_coefs(I.dt_k, I.rcd);
    for (int i = 0; i < 9; ++i) I.rcf[i] = (float)I.rcd[i];
}

// Chunk c of an instance: samples [b, e], e = min(b + K, S - 1).
struct ChunkRef {
    int32_t inst;
    int32_t chunk;
};

// ---------------------------------------------------------------------
// Input / output element access (problem dtype -> compute type T)
// ---------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T load_in(const void* p, int64_t idx, bool f64) {
    return f64 ? (T)__ldg(static_cast<const double*>(p) + idx) : (T)__ldg(static_cast<const float*>(p) + idx);
}
template <class T>
__device__ __forceinline__ void store_out(void* p, int64_t idx, T v, bool f64) {
    if (f64) static_cast<double*>(p)[idx] = (double)v;
    else static_cast<float*>(p)[idx] = (float)v;
}
template <class T>
__device__ __forceinline__ void atomic_add_out(void* p, int64_t idx, T v, bool f64) {
    if (f64) atomicAdd(static_cast<double*>(p) + idx, (double)v);
    else atomicAdd(static_cast<float*>(p) + idx, (float)v);
}

// Sample i, element el of the algebra element (m = d*d, or 4 for
// SpaceCurve where component 0 is the zero padding).
template <class T, int KIND>
__device__ __forceinline__ T load_sample(const void* A, int64_t i, int el, int m, bool f64) {
    if (KIND == KIND_SC) return el == 0 ? T(0) : load_in<T>(A, i * 3 + (el - 1), f64);
    return load_in<T>(A, i * (int64_t)m + el, f64);
}

// ---------------------------------------------------------------------
// Algebra: one output element of the products used by the recursion.
//   mul(a, b)      : level product a (x) b
//   adjL(a, g)[X]  : d<g, a (x) X>/dX   (cotangent to the right factor)
//   adjR(g, b)[X]  : d<g, X (x) b>/dX   (cotangent to the left factor)
// Operands may be of different storage types; accumulation is in T.
// ---------------------------------------------------------------------
template <class T, int KIND>
struct Alg;

template <class T>
struct Alg<T, KIND_MATRIX> {
    __device__ __forceinline__ static T one(int d, int el) { return (el / d == el % d) ? T(1) : T(0); }
    template <class PA, class PB>
    __device__ __forceinline__ static T mul(const PA* a, const PB* b, int d, int el) {
        const int r = el / d, c = el - r * d;
        T s = T(0);
        for (int k = 0; k < d; ++k) s += (T)a[r * d + k] * (T)b[k * d + c];
        return s;
    }
    template <class PA, class PB>
    __device__ __forceinline__ static T adjL(const PA* a, const PB* g, int d, int el) {
        const int r = el / d, c = el - r * d;
        T s = T(0);
        for (int k = 0; k < d; ++k) s += (T)a[k * d + r] * (T)g[k * d + c];
        return s;
    }
    template <class PA, class PB>
    __device__ __forceinline__ static T adjR(const PA* g, const PB* b, int d, int el) {
        const int r = el / d, c = el - r * d;
        T s = T(0);
        for (int k = 0; k < d; ++k) s += (T)g[r * d + k] * (T)b[c * d + k];
        return s;
    }
};

// qmul(a, b) = b (x) a (Hamilton).  Component el of each product is
// sum_k sign(el, k) x[k] y[el ^ k]; the signs are bit masks (bit 4 el + k
// set: negative), so that the lanes of a warp holding different components
// run the same instructions (a switch on el diverged four ways).
//   mul  (a, b): sum_k +-b[k] a[el ^ k]
//   adjL (a, g): sum_k +-g[k] a[el ^ k]
//   adjR (g, b): sum_k +-g[k] b[el ^ k]
template <class T>
struct Alg<T, KIND_SC> {
    static constexpr unsigned kMul = 0x428Eu, kAdjL = 0x3950u, kAdjR = 0x5390u;
    // x with its sign flipped when `neg` is 1 (an integer XOR: the sign
    // differs between lanes, and a negation through the FP64 pipe would cost
    // as much as the fused multiply-add it feeds)
    __device__ __forceinline__ static double flip(double v, unsigned neg) {
        return __longlong_as_double(__double_as_longlong(v) ^ ((long long)neg << 63));
    }
    __device__ __forceinline__ static float flip(float v, unsigned neg) {
        return __int_as_float(__float_as_int(v) ^ (int)(neg << 31));
    }
    template <class PX, class PY>
    __device__ __forceinline__ static T signed_sum(unsigned mask, const PX* x, const PY* y, int el) {
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 4; ++k) s = fma(flip((T)x[k], (mask >> (4 * el + k)) & 1u), (T)y[el ^ k], s);
        return s;
    }
    __device__ __forceinline__ static T one(int, int el) { return el == 0 ? T(1) : T(0); }
    template <class PA, class PB>
    __device__ __forceinline__ static T mul(const PA* pa, const PB* pb, int, int el) {
        return signed_sum(kMul, pb, pa, el);
    }
    template <class PA, class PB>
    __device__ __forceinline__ static T adjL(const PA* pa, const PB* pg, int, int el) {
        return signed_sum(kAdjL, pg, pa, el);
    }
    template <class PA, class PB>
    __device__ __forceinline__ static T adjR(const PA* pg, const PB* pb, int, int el) {
        return signed_sum(kAdjR, pg, pb, el);
    }
};

// ---------------------------------------------------------------------
// Block rules as streaming state machines over one element.
// Position li is the sample index relative to the chunk start b (b is a
// multiple of 4), so li & 3 / li & 1 give the place inside a Boole block /
// Simpson pair.  Coefficients follow the reference's prefix rules:
//   Boole     src/integration/boole.hpp:24-74
//   Simpson   src/integration/simpson.hpp:24-58
//   Trapezoid src/integration/trapezoid.hpp:23-33 (textbook increments; the
//             reference's differencing recurrence equals them up to rounding)
//   Riemann   src/integration/default.hpp:23-26 (inclusive: P_0 = dt f_0)
// ---------------------------------------------------------------------
template <class T>
struct RuleCoef {
    T h, t3, c38, c98, c4_3, b14, b64, b24, dt;
    __device__ __forceinline__ explicit RuleCoef(const T* c)
        : h(c[0]), t3(c[1]), c38(c[2]), c98(c[3]), c4_3(c[4]), b14(c[5]), b64(c[6]), b24(c[7]), dt(c[8]) {}
};
// The instance's coefficients in the compute type (precomputed on the host).
template <class T>
__device__ __forceinline__ RuleCoef<T> rule_coef(const InstDev& I);
template <>
__device__ __forceinline__ RuleCoef<float> rule_coef<float>(const InstDev& I) { return RuleCoef<float>(I.rcf); }
template <>
__device__ __forceinline__ RuleCoef<double> rule_coef<double>(const InstDev& I) { return RuleCoef<double>(I.rcd); }

// A chunk carry (FP64 on the host side) as an unevaluated sum hi + lo in the
// compute type: exact for double, ~2x float precision for float.  Running
// prefix states stay LOCAL to the chunk (they start at zero) and the carry is
// added only when a value is emitted, so FP32 rounding in the mixed form
// scales with the chunk's own increments, not with the carried total.
template <class T>
struct Carry {
    T hi, lo;
};
template <class T>
__device__ __forceinline__ Carry<T> split_carry(double v) {
    Carry<T> c;
    c.hi = (T)v;
    c.lo = (T)(v - (double)c.hi);
    return c;
}
template <class T>
__device__ __forceinline__ T add_carry(T local, const Carry<T>& c) {
    return (local + c.lo) + c.hi;
}

// Error-free sum a + b = s + err (Knuth's TwoSum), used to carry the local
// prefix accumulators at twice the working precision in FP32.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& err) {
    s = a + b;
    const float bb = s - a;
    err = (a - (s - bb)) + (b - bb);
}

// acc (+ lo) += inc.  FP32: compensated, the rounding error kept in lo.
// FP64: plain addition (lo stays 0).
template <class T>
__device__ __forceinline__ void acc_add(T& acc, T& lo, T inc);
template <>
__device__ __forceinline__ void acc_add<float>(float& acc, float& lo, float inc) {
    float s, err;
    two_sum(acc, inc + lo, s, err);
    acc = s;
    lo = err;
}
template <>
__device__ __forceinline__ void acc_add<double>(double& acc, double&, double inc) {
    acc += inc;
}

template <class T>
struct FwdState {
    T base, blo, f0, f1, f2, f3;  // base (+ blo): local prefix at the last anchor
};

// Returns P at position li (carry included) given f at li; updates the state.
// CY = false: the caller's carry is zero (local passes), P is the local value.
template <class T, int RULE, bool CY = true>
__device__ __forceinline__ T fwd_step(FwdState<T>& s, T f, int li, const RuleCoef<T>& k, const Carry<T>& cy) {
    auto add_carry = [&](T local, const Carry<T>& c) { return CY ? mgb::add_carry(local, c) : local; };
    if (RULE == R_BOOLE) {
        switch (li & 3) {
            case 1: s.f1 = f; return add_carry((f * k.h + s.f0 * k.h + s.blo) + s.base, cy);
            case 2: s.f2 = f; return add_carry((f * k.t3 + s.f0 * k.t3 + s.f1 * k.c4_3 + s.blo) + s.base, cy);
            case 3:
                s.f3 = f;
                return add_carry((f * k.c38 + s.f0 * k.c38 + s.f1 * k.c98 + s.f2 * k.c98 + s.blo) + s.base, cy);
            default: {
                const T inc = f * k.b14 + s.f0 * k.b14 + s.f1 * k.b64 + s.f2 * k.b24 + s.f3 * k.b64;
                acc_add(s.base, s.blo, inc);
                s.f0 = f;
                return add_carry(s.base + s.blo, cy);
            }
        }
    } else if (RULE == R_SIMPSON) {
        if (li & 1) {
            s.f1 = f;
            return add_carry((f * k.h + s.f0 * k.h + s.blo) + s.base, cy);
        }
        const T inc = f * k.t3 + s.f0 * k.t3 + s.f1 * (T(4) * k.t3);
        acc_add(s.base, s.blo, inc);
        s.f0 = f;
        return add_carry(s.base + s.blo, cy);
    } else if (RULE == R_TRAP) {
        acc_add(s.base, s.blo, f * k.h + s.f0 * k.h);
        s.f0 = f;
        return add_carry(s.base + s.blo, cy);
    } else {
        acc_add(s.base, s.blo, f * k.dt);
        return add_carry(s.base + s.blo, cy);
    }
}

// Adjoint of the block rules, processing positions from the chunk end
// downwards.  Rb (+ rlo): LOCAL cotangent on the current anchor prefix from
// later samples of the chunk (the cotangent rho from beyond the chunk is the
// carry cy, added where totals are used); pend: cotangent on the anchor's f
// from its use as the first sample of the later block.  Input H: local
// cotangent on P[li]; returns the cotangent on f[li].
template <class T>
struct RevState {
    T Rb, rlo, pend, R4l, R4, H2, H3;
};

template <class T, int RULE>
__device__ __forceinline__ T rev_step(RevState<T>& s, T H, int li, const RuleCoef<T>& k, const Carry<T>& cy) {
    if (RULE == R_BOOLE) {
        switch (li & 3) {
            case 0: {
                s.R4l = H;  // block-local part; the anchor total is Rb + rlo + H
                s.R4 = add_carry((H + s.rlo) + s.Rb, cy);
                return s.R4 * k.b14 + s.pend;
            }
            case 3: s.H3 = H; return H * k.c38 + s.R4 * k.b64;
            case 2: s.H2 = H; return H * k.t3 + s.H3 * k.c98 + s.R4 * k.b24;
            default: {
                const T G = H * k.h + s.H2 * k.c4_3 + s.H3 * k.c98 + s.R4 * k.b64;
                s.pend = H * k.h + s.H2 * k.t3 + s.H3 * k.c38 + s.R4 * k.b14;
                acc_add(s.Rb, s.rlo, H + s.H2 + s.H3 + s.R4l);
                return G;
            }
        }
    } else if (RULE == R_SIMPSON) {
        if ((li & 1) == 0) {
            s.R4l = H;
            s.R4 = add_carry((H + s.rlo) + s.Rb, cy);
            return s.R4 * k.t3 + s.pend;
        }
        const T G = H * k.h + s.R4 * (T(4) * k.t3);
        s.pend = H * k.h + s.R4 * k.t3;
        acc_add(s.Rb, s.rlo, H + s.R4l);
        return G;
    } else if (RULE == R_TRAP) {
        acc_add(s.Rb, s.rlo, H);
        const T Rt = add_carry(s.Rb + s.rlo, cy);
        const T G = Rt * k.h + s.pend;
        s.pend = Rt * k.h;
        return G;
    } else {
        acc_add(s.Rb, s.rlo, H);
        return add_carry(s.Rb + s.rlo, cy) * k.dt;
    }
}

}  // namespace mgb
