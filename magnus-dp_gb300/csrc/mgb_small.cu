// Chunk kernel for the 4-element algebras — 2x2 matrices (the reference's
// Fixed2 policy, src/linalg/fixed.hpp) and SpaceCurve 4-vectors
// (src/linalg/spacecurve.hpp) — with one thread per chunk and every level's
// prefix state in registers.  Used by both precision forms (T = double for
// plain, float for mixed).  Samples are processed one rule block at a time
// (Boole 4, Simpson 2, Trapezoid / Riemann 1) with all levels per block; the
// VJP replays the chunk from its checkpoint into a per-thread tape of the
// prefix values in global memory and then runs the adjoint over the blocks in
// reverse.  Orders up to NMAX = 6 levels stay in registers; larger orders use
// the generic kernel.
#include <cstdint>
#include <vector>

#include "mgb_common.cuh"
#include "mgb_tuned.h"

namespace mgb {
namespace {

constexpr int SNT = 128;   // threads per block
constexpr int NMAX = 6;    // levels kept in registers

template <class T, int KIND>
struct Small;

// 2x2 row-major: mul = a b, adjL = a^T g, adjR = g p^T
template <class T>
struct Small<T, KIND_MATRIX> {
    __device__ __forceinline__ static void mul(const T* a, const T* b, T* c) {
        c[0] = a[0] * b[0] + a[1] * b[2];
        c[1] = a[0] * b[1] + a[1] * b[3];
        c[2] = a[2] * b[0] + a[3] * b[2];
        c[3] = a[2] * b[1] + a[3] * b[3];
    }
    __device__ __forceinline__ static void adjL(const T* a, const T* g, T* c) {
        c[0] = a[0] * g[0] + a[2] * g[2];
        c[1] = a[0] * g[1] + a[2] * g[3];
        c[2] = a[1] * g[0] + a[3] * g[2];
        c[3] = a[1] * g[1] + a[3] * g[3];
    }
    __device__ __forceinline__ static void adjR(const T* g, const T* p, T* c) {
        c[0] = g[0] * p[0] + g[1] * p[1];
        c[1] = g[0] * p[2] + g[1] * p[3];
        c[2] = g[2] * p[0] + g[3] * p[1];
        c[3] = g[2] * p[2] + g[3] * p[3];
    }
    // products with a sample of the input as left factor (general here)
    __device__ __forceinline__ static void mul_in(const T* a, const T* b, T* c) { mul(a, b, c); }
    __device__ __forceinline__ static void adjL_in(const T* a, const T* g, T* c) { adjL(a, g, c); }
    __device__ __forceinline__ static void load(const void* A, int64_t i, bool f64, T* v) {
        if (f64) {
            const double2* p = reinterpret_cast<const double2*>(static_cast<const double*>(A) + i * 4);
            const double2 x = __ldg(p), y = __ldg(p + 1);
            v[0] = (T)x.x; v[1] = (T)x.y; v[2] = (T)y.x; v[3] = (T)y.y;
        } else {
            const float4 x = __ldg(reinterpret_cast<const float4*>(static_cast<const float*>(A) + i * 4));
            v[0] = (T)x.x; v[1] = (T)x.y; v[2] = (T)x.z; v[3] = (T)x.w;
        }
    }
};

// SpaceCurve as the associative algebra qmul(a, b) = b (x) a (Hamilton).
template <class T>
struct Small<T, KIND_SC> {
    __device__ __forceinline__ static void mul(const T* a, const T* b, T* c) {
        c[0] = b[0] * a[0] - b[1] * a[1] - b[2] * a[2] - b[3] * a[3];
        c[1] = b[0] * a[1] + b[1] * a[0] + b[2] * a[3] - b[3] * a[2];
        c[2] = b[0] * a[2] - b[1] * a[3] + b[2] * a[0] + b[3] * a[1];
        c[3] = b[0] * a[3] + b[1] * a[2] - b[2] * a[1] + b[3] * a[0];
    }
    __device__ __forceinline__ static void adjL(const T* a, const T* g, T* c) {
        c[0] = a[0] * g[0] + a[1] * g[1] + a[2] * g[2] + a[3] * g[3];
        c[1] = -a[1] * g[0] + a[0] * g[1] - a[3] * g[2] + a[2] * g[3];
        c[2] = -a[2] * g[0] + a[3] * g[1] + a[0] * g[2] - a[1] * g[3];
        c[3] = -a[3] * g[0] - a[2] * g[1] + a[1] * g[2] + a[0] * g[3];
    }
    __device__ __forceinline__ static void adjR(const T* g, const T* p, T* c) {
        c[0] = p[0] * g[0] + p[1] * g[1] + p[2] * g[2] + p[3] * g[3];
        c[1] = -p[1] * g[0] + p[0] * g[1] + p[3] * g[2] - p[2] * g[3];
        c[2] = -p[2] * g[0] - p[3] * g[1] + p[0] * g[2] + p[1] * g[3];
        c[3] = -p[3] * g[0] + p[2] * g[1] - p[1] * g[2] + p[0] * g[3];
    }
    // mul / adjL with a curve sample (0, f) as left factor: a[0] = 0, so its
    // four terms drop out (12 multiply-adds instead of 16)
    __device__ __forceinline__ static void mul_in(const T* a, const T* b, T* c) {
        c[0] = -b[1] * a[1] - b[2] * a[2] - b[3] * a[3];
        c[1] = b[0] * a[1] + b[2] * a[3] - b[3] * a[2];
        c[2] = b[0] * a[2] - b[1] * a[3] + b[3] * a[1];
        c[3] = b[0] * a[3] + b[1] * a[2] - b[2] * a[1];
    }
    __device__ __forceinline__ static void adjL_in(const T* a, const T* g, T* c) {
        c[0] = a[1] * g[1] + a[2] * g[2] + a[3] * g[3];
        c[1] = -a[1] * g[0] - a[3] * g[2] + a[2] * g[3];
        c[2] = -a[2] * g[0] + a[3] * g[1] - a[1] * g[3];
        c[3] = -a[3] * g[0] - a[2] * g[1] + a[1] * g[2];
    }
    __device__ __forceinline__ static void load(const void* A, int64_t i, bool f64, T* v) {
        v[0] = T(0);
        if (f64) {
            const double* p = static_cast<const double*>(A) + i * 3;
            v[1] = (T)__ldg(p); v[2] = (T)__ldg(p + 1); v[3] = (T)__ldg(p + 2);
        } else {
            const float* p = static_cast<const float*>(A) + i * 3;
            v[1] = (T)__ldg(p); v[2] = (T)__ldg(p + 1); v[3] = (T)__ldg(p + 2);
        }
    }
};

template <int RULE>
struct Block {
    static constexpr int BS = RULE == R_BOOLE ? 4 : (RULE == R_SIMPSON ? 2 : 1);
};

template <class T, int KIND>
__device__ __forceinline__ void write_dA(const InstDev& I, int64_t i, const T* v, bool shared, bool f64) {
    if (KIND == KIND_SC) {
        for (int e = 1; e < 4; ++e) {
            if (shared) atomic_add_out<T>(I.dA, i * 3 + e - 1, v[e], f64);
            else store_out<T>(I.dA, i * 3 + e - 1, v[e], f64);
        }
    } else {
        for (int e = 0; e < 4; ++e) {
            if (shared) atomic_add_out<T>(I.dA, i * 4 + e, v[e], f64);
            else store_out<T>(I.dA, i * 4 + e, v[e], f64);
        }
    }
}

template <class T, int KIND, int RULE, int MODE>
__global__ void __launch_bounds__(SNT) k_small(const InstDev* __restrict__ insts, const ChunkRef* __restrict__ work,
                                               int64_t nwork, T* __restrict__ scratch, int64_t slot_elems, int64_t nslots,
                                               int f64io) {
    using Al = Small<T, KIND>;
    constexpr int BS = Block<RULE>::BS;
    const bool f64 = f64io != 0;
    // one tape slot per working thread: the last block's threads beyond the
    // slot count (the scratch budget need not be a multiple of the block
    // size) take no work
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nslots) return;
    T* const tape = scratch + tid * slot_elems;  // [L][NMAX-1][4] prefix values P_j
    // VJP: the chunk carries pi^c and rho^c split into hi + lo once per chunk,
    // [4][NMAX][4] at the slot's end (a split in every rule block ran FP64
    // conversions on the 1/64-rate pipe for every sample)
    T* const cya = scratch + tid * slot_elems + slot_elems - 16 * NMAX;

    for (int64_t w = tid; w < nwork; w += nslots) {
        const ChunkRef wk = work[w];
        const InstDev& I = insts[wk.inst];
        const int c = wk.chunk, n = I.n;
        const int64_t b = (int64_t)c * I.K;
        const int64_t e = (b + I.K < I.S - 1) ? b + I.K : I.S - 1;
        const int Kp = (int)(e - b);
        const bool riem0 = (RULE == R_RIEMANN) && c == 0;
        const int first = riem0 ? 0 : 1;
        const RuleCoef<T> kc = rule_coef<T>(I);
        const double* pic = I.pi + (int64_t)c * n * 4;
        const int NL = (MODE == MODE_LOCAL) ? n : n - 1;
        if (MODE == MODE_VJP) {
            const double* rcc = I.rho + (int64_t)c * n * 4;
            for (int jq = 0; jq < n * 4; ++jq) {
                const Carry<T> f = split_carry<T>(riem0 ? 0.0 : pic[jq]);
                const Carry<T> r = split_carry<T>(rcc[jq]);
                cya[jq] = f.hi;
                cya[4 * NMAX + jq] = f.lo;
                cya[8 * NMAX + jq] = r.hi;
                cya[12 * NMAX + jq] = r.lo;
            }
        }

        // ---------------- forward over the chunk ----------------
        T base[NMAX][4], blo[NMAX][4], f0[NMAX][4];
        {
            T a0[4];
            Al::load(I.A, b, f64, a0);
#pragma unroll
            for (int j = 0; j < NMAX; ++j) {
#pragma unroll
                for (int q = 0; q < 4; ++q) base[j][q] = blo[j][q] = f0[j][q] = T(0);
                if (j == 0) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) f0[0][q] = a0[q];
                } else if (MODE == MODE_VJP && j < NL && !riem0) {
                    T p[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) p[q] = (T)pic[(j - 1) * 4 + q];
                    Al::mul(a0, p, f0[j]);
                }
            }
        }
        for (int li = first; li <= Kp; li += BS) {
            T f[BS][4], a[BS][4];
#pragma unroll
            for (int s = 0; s < BS; ++s) {
                Al::load(I.A, b + li + s, f64, a[s]);
#pragma unroll
                for (int q = 0; q < 4; ++q) f[s][q] = a[s][q];
            }
#pragma unroll
            for (int j = 0; j < NMAX; ++j) {
                if (j < NL) {
                    T P[BS][4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        Carry<T> cy{T(0), T(0)};
                        if (MODE == MODE_VJP) {
                            cy.hi = cya[j * 4 + q];
                            cy.lo = cya[4 * NMAX + j * 4 + q];
                        }
                        FwdState<T> st;
                        st.base = base[j][q];
                        st.blo = blo[j][q];
                        st.f0 = f0[j][q];
                        st.f1 = st.f2 = st.f3 = T(0);
#pragma unroll
                        for (int s = 0; s < BS; ++s) P[s][q] = fwd_step<T, RULE, MODE != MODE_LOCAL>(st, f[s][q], 1 + s, kc, cy);
                        base[j][q] = st.base;
                        blo[j][q] = st.blo;
                        f0[j][q] = st.f0;
                    }
                    if (MODE == MODE_VJP) {
#pragma unroll
                        for (int s = 0; s < BS; ++s)
#pragma unroll
                            for (int q = 0; q < 4; ++q) tape[((int64_t)(li + s) * (NMAX - 1) + j) * 4 + q] = P[s][q];
                    }
                    if (j + 1 < NL) {
#pragma unroll
                        for (int s = 0; s < BS; ++s) Al::mul_in(a[s], P[s], f[s]);
                    }
                }
            }
        }
        if (MODE == MODE_LOCAL) {
#pragma unroll
            for (int j = 0; j < NMAX; ++j)
                if (j < n)
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        I.lam[(int64_t)c * n * 4 + j * 4 + q] = (double)base[j][q] + (double)blo[j][q];
        }

        if (MODE == MODE_VJP) {
            T Rb[NMAX][4], rlo[NMAX][4], pend[NMAX][4];
#pragma unroll
            for (int j = 0; j < NMAX; ++j)
#pragma unroll
                for (int q = 0; q < 4; ++q) Rb[j][q] = rlo[j][q] = pend[j][q] = T(0);
            const int last0 = first + ((Kp - first) / BS) * BS;
            for (int li = last0; li >= first; li -= BS) {
                T a[BS][4], Gup[BS][4], dacc[BS][4];
#pragma unroll
                for (int s = 0; s < BS; ++s) {
                    Al::load(I.A, b + li + s, f64, a[s]);
#pragma unroll
                    for (int q = 0; q < 4; ++q) dacc[s][q] = Gup[s][q] = T(0);
                }
#pragma unroll
                for (int j = NMAX - 1; j >= 0; --j) {
                    if (j < n) {
                        T H[BS][4];
                        if (j + 1 < n) {
#pragma unroll
                            for (int s = 0; s < BS; ++s) {
                                Al::adjL_in(a[s], Gup[s], H[s]);
                                T p[4], t[4];
#pragma unroll
                                for (int q = 0; q < 4; ++q) p[q] = tape[((int64_t)(li + s) * (NMAX - 1) + j) * 4 + q];
                                Al::adjR(Gup[s], p, t);
#pragma unroll
                                for (int q = 0; q < 4; ++q) dacc[s][q] += t[q];
                            }
                        } else {
#pragma unroll
                            for (int s = 0; s < BS; ++s)
#pragma unroll
                                for (int q = 0; q < 4; ++q) H[s][q] = T(0);
                        }
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const Carry<T> cy{cya[8 * NMAX + j * 4 + q], cya[12 * NMAX + j * 4 + q]};
                            RevState<T> st;
                            st.Rb = Rb[j][q];
                            st.rlo = rlo[j][q];
                            st.pend = pend[j][q];
                            st.R4l = st.R4 = st.H2 = st.H3 = T(0);
#pragma unroll
                            for (int s = BS - 1; s >= 0; --s) Gup[s][q] = rev_step<T, RULE>(st, H[s][q], 1 + s, kc, cy);
                            Rb[j][q] = st.Rb;
                            rlo[j][q] = st.rlo;
                            pend[j][q] = st.pend;
                        }
                    }
                }
#pragma unroll
                for (int s = 0; s < BS; ++s) {
                    T v[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) v[q] = dacc[s][q] + Gup[s][q];
                    const int lis = li + s;
                    write_dA<T, KIND>(I, b + lis, v, lis == Kp && c < I.C - 1, f64);
                }
            }
            if (!riem0 && RULE != R_RIEMANN) {
                // this chunk's copy of W_j[b]: dA[b] += pend_1 + sum_{j<n} pend_{j+1} pi_j^T
                T v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) v[q] = pend[0][q];
#pragma unroll
                for (int j = 1; j < NMAX; ++j) {
                    if (j < n) {
                        T p[4], t[4];
#pragma unroll
                        for (int q = 0; q < 4; ++q) p[q] = (T)pic[(j - 1) * 4 + q];
                        Al::adjR(pend[j], p, t);
#pragma unroll
                        for (int q = 0; q < 4; ++q) v[q] += t[q];
                    }
                }
                write_dA<T, KIND>(I, b, v, c > 0, f64);
            }
        }
    }
}

template <class T, int KIND, int RULE>
cudaError_t launch_small_t(int mode, const LaunchArgs& a, int64_t threads) {
    const int blocks = (int)((threads + SNT - 1) / SNT);
    T* scr = static_cast<T*>(a.scratch);
    if (mode == MODE_LOCAL)
        k_small<T, KIND, RULE, MODE_LOCAL><<<blocks, SNT, 0, a.stream>>>(a.insts, a.work, a.nwork, scr,
                                                                          a.slot_elems, threads, a.f64io);
    else
        k_small<T, KIND, RULE, MODE_VJP><<<blocks, SNT, 0, a.stream>>>(a.insts, a.work, a.nwork, scr,
                                                                        a.slot_elems, threads, a.f64io);
    return cudaGetLastError();
}

template <class T, int KIND>
cudaError_t launch_small_r(int rule, int mode, const LaunchArgs& a, int64_t threads) {
    switch (rule) {
        case R_BOOLE: return launch_small_t<T, KIND, R_BOOLE>(mode, a, threads);
        case R_SIMPSON: return launch_small_t<T, KIND, R_SIMPSON>(mode, a, threads);
        case R_TRAP: return launch_small_t<T, KIND, R_TRAP>(mode, a, threads);
        default: return launch_small_t<T, KIND, R_RIEMANN>(mode, a, threads);
    }
}

}  // namespace

// a.grid = number of threads, a.slot_elems = per-thread tape [L][NMAX-1][4]
// (both sized by size_segment).
cudaError_t launch_small_family(bool plain, int kind, int rule, int mode, const LaunchArgs& a) {
    const int64_t threads = std::max<int64_t>(1, a.grid);
    if (plain) return kind == KIND_SC ? launch_small_r<double, KIND_SC>(rule, mode, a, threads)
                                      : launch_small_r<double, KIND_MATRIX>(rule, mode, a, threads);
    return kind == KIND_SC ? launch_small_r<float, KIND_SC>(rule, mode, a, threads)
                           : launch_small_r<float, KIND_MATRIX>(rule, mode, a, threads);
}

int small_family_max_levels() { return NMAX; }

}  // namespace mgb
