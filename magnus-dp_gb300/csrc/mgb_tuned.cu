// Shape-specialised chunk kernel for the mixed form (FP32 products, FP64
// carries) at d = 16 and d = 32: one CTA per chunk, samples processed in
// groups of G (G = 256 / (d/4)^2, so every thread owns one 4x4 output tile
// of one sample), all Magnus levels per group, per-level prefix state in
// shared memory.
//
// Per group and level: a prefix pass (thread per element, FP32 local
// accumulators, FP64 chunk carry added at emission) and a batched
// 4x4-register-tiled product pass with operands in shared memory:
//   forward  W = A P        A^T and P staged with a 16-byte row pitch (float4 loads)
//   adjoint  H = A^T G      A (float4 rows) x G (odd pitch, conflict-free scalars)
//            dA += G P^T    G (odd pitch) x P^T (float4 rows, from the tape)
// The VJP replays the chunk forward from its checkpoint, writing the prefix
// values of levels 1..n-1 to a per-CTA tape in global memory, then runs the
// adjoint over the groups in reverse order with dA accumulated in registers.
#include <cstdint>
#include <mutex>
#include <vector>

#include "mgb_common.cuh"
#include "mgb_tuned.h"

namespace mgb {
namespace {

constexpr int TNT = 256;

template <int D>
struct TileCfg {
    static constexpr int m = D * D;
    static constexpr int TPS = (D / 4) * (D / 4);  // threads per sample
    static constexpr int G = TNT / TPS;           // samples per group
    static constexpr int P4 = D + 4;              // 16-byte aligned pitch
    static constexpr int P1 = D + 1;              // odd pitch (column reads)
    static constexpr int EPT = m / TNT;           // prefix elements per thread
    static constexpr int OPND = (3 * G * D * P4 > 2 * G * D * P4 + 2 * G * D * P1) ? 3 * G * D * P4
                                                                                   : 2 * G * D * P4 + 2 * G * D * P1;
    static_assert(G * TPS == TNT, "tile mapping");
    static_assert(EPT >= 1 && EPT * TNT == m, "prefix mapping");
};

// acc += X Y with X given transposed (XT[k][r], pitch px) and Y row-major
// (pitch py); both 16-byte aligned rows.
template <int D>
__device__ __forceinline__ void mma_tv(float (&acc)[4][4], const float* __restrict__ XT, int px,
                                       const float* __restrict__ Y, int py, int r0, int c0) {
#pragma unroll 8
    for (int k = 0; k < D; ++k) {
        const float4 a = *reinterpret_cast<const float4*>(XT + k * px + r0);
        const float4 b = *reinterpret_cast<const float4*>(Y + k * py + c0);
        const float av[4] = {a.x, a.y, a.z, a.w};
        const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int t = 0; t < 4; ++t)
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[t][u] = fmaf(av[t], bv[u], acc[t][u]);
    }
}

// acc += A^T G : A row-major (pitch P4, float4), G row-major odd pitch P1.
template <int D>
__device__ __forceinline__ void mma_adjL(float (&acc)[4][4], const float* __restrict__ A,
                                         const float* __restrict__ G, int r0, int c0) {
    constexpr int P4 = D + 4, P1 = D + 1;
#pragma unroll 8
    for (int k = 0; k < D; ++k) {
        const float4 a = *reinterpret_cast<const float4*>(A + k * P4 + r0);
        const float av[4] = {a.x, a.y, a.z, a.w};
        float bv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) bv[u] = G[k * P1 + c0 + u];
#pragma unroll
        for (int t = 0; t < 4; ++t)
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[t][u] = fmaf(av[t], bv[u], acc[t][u]);
    }
}

// acc += G P^T : G row-major odd pitch P1 (column reads), P^T row-major P4.
template <int D>
__device__ __forceinline__ void mma_adjR(float (&acc)[4][4], const float* __restrict__ G,
                                         const float* __restrict__ PT, int r0, int c0) {
    constexpr int P4 = D + 4, P1 = D + 1;
#pragma unroll 8
    for (int k = 0; k < D; ++k) {
        float av[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) av[t] = G[(r0 + t) * P1 + k];
        const float4 b = *reinterpret_cast<const float4*>(PT + k * P4 + c0);
        const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int t = 0; t < 4; ++t)
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[t][u] = fmaf(av[t], bv[u], acc[t][u]);
    }
}

// MINB: resident CTAs per SM the register allocation targets (2, or 1 with
// up to 255 registers per thread); the autotuner picks.
template <int D, int RULE, int MODE, int MINB>
__global__ void __launch_bounds__(TNT, MINB) k_tile(const InstDev* __restrict__ insts, const ChunkRef* __restrict__ work,
                                                 int64_t nwork, float* __restrict__ scratch, int64_t slot_elems) {
    using Cf = TileCfg<D>;
    constexpr int m = Cf::m, G = Cf::G, P4 = Cf::P4, P1 = Cf::P1, TPS = Cf::TPS, EPT = Cf::EPT;
    extern __shared__ __align__(16) float sm[];
    float* const sAT = sm;               // forward: A^T   [G][D][P4]
    float* const sP = sAT + G * D * P4;  // forward: P     [G][D][P4]
    float* const sF = sP + G * D * P4;   // forward: f     [G][D][P4]
    float* const sA = sm;                // reverse: A     [G][D][P4]
    float* const sPT = sA + G * D * P4;  // reverse: P^T   [G][D][P4]
    float* const sG = sPT + G * D * P4;  // reverse: G     [G][D][P1]
    float* const sH = sG + G * D * P1;   // reverse: H     [G][D][P1]
    float* const slot = scratch + (int64_t)blockIdx.x * slot_elems;

    const int tid = threadIdx.x;
    const int tl = tid / TPS, tu = tid % TPS;
    const int r0 = (tu / (D / 4)) * 4, c0 = (tu % (D / 4)) * 4;

    for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        const ChunkRef wk = work[w];
        const InstDev& I = insts[wk.inst];
        const int c = wk.chunk, n = I.n;
        const int64_t b = (int64_t)c * I.K;
        const int64_t e = (b + I.K < I.S - 1) ? b + I.K : I.S - 1;
        const int Kp = (int)(e - b), L = Kp + 1;
        const bool riem0 = (RULE == R_RIEMANN) && c == 0;
        const int first = riem0 ? 0 : 1;
        const int64_t nm = (int64_t)n * m;
        const RuleCoef<float> kc = rule_coef<float>(I);
        const double* pic = I.pi + (int64_t)c * nm;
        const float* Ag = static_cast<const float*>(I.A) + b * m;
        const int NLf = (MODE == MODE_LOCAL) ? n : n - 1;  // levels with a forward prefix
        // per-level prefix state [n][3][m] (L2-resident), the tape [n-1][L][m],
        // then (VJP) the chunk carries pi^c and rho^c split into FP32 hi / lo
        // once per chunk, [2][n][2][m] (FP64 conversions cost a 1/64-rate pipe)
        float* const st = slot;
        float* const tape = slot + (int64_t)3 * n * m;
        float* const cyt = tape + (int64_t)(n - 1) * L * m;
        if (MODE == MODE_VJP) {
            const double* rcc = I.rho + (int64_t)c * nm;
            for (int j = 1; j <= n; ++j)
#pragma unroll
                for (int q = 0; q < EPT; ++q) {
                    const int el = tid + q * TNT;
                    const Carry<float> a = split_carry<float>(riem0 ? 0.0 : pic[(int64_t)(j - 1) * m + el]);
                    const Carry<float> r = split_carry<float>(rcc[(int64_t)(j - 1) * m + el]);
                    cyt[((int64_t)(j - 1) * 2) * m + el] = a.hi;
                    cyt[((int64_t)(j - 1) * 2 + 1) * m + el] = a.lo;
                    cyt[((int64_t)(n + j - 1) * 2) * m + el] = r.hi;
                    cyt[((int64_t)(n + j - 1) * 2 + 1) * m + el] = r.lo;
                }
        }

        // ---------------- forward state at the chunk start ----------------
        for (int j = 1; j <= NLf; ++j)
            for (int q = 0; q < EPT; ++q) {
                const int el = tid + q * TNT;
                st[(j - 1) * 3 * m + el] = 0.f;
                st[(j - 1) * 3 * m + m + el] = 0.f;
                st[(j - 1) * 3 * m + 2 * m + el] = (j == 1) ? __ldg(Ag + el) : 0.f;
            }
        if (MODE == MODE_VJP && !riem0 && NLf >= 2) {
            // f0_j = A[b] P_{j-1}[b] = A[b] pi_{j-1} for j = 2..NLf
            for (int el = tid; el < m; el += TNT) sAT[(el % D) * P4 + el / D] = __ldg(Ag + el);
            for (int j0 = 2; j0 <= NLf; j0 += G) {
                for (int idx = tid; idx < G * m; idx += TNT) {
                    const int l = idx / m, el = idx % m;
                    if (j0 + l <= NLf) sP[l * D * P4 + (el / D) * P4 + el % D] = (float)pic[(int64_t)(j0 + l - 2) * m + el];
                }
                __syncthreads();
                if (j0 + tl <= NLf) {
                    float acc[4][4] = {};
                    mma_tv<D>(acc, sAT, P4, sP + tl * D * P4, P4, r0, c0);
                    float* f0 = st + (j0 + tl - 1) * 3 * m + 2 * m;
#pragma unroll
                    for (int t = 0; t < 4; ++t)
#pragma unroll
                        for (int u = 0; u < 4; ++u) f0[(r0 + t) * D + c0 + u] = acc[t][u];
                }
                __syncthreads();
            }
        }
        __syncthreads();

        // ---------------- forward over the groups ----------------
        // Global loads run one step ahead of their use: the next group's A
        // during this group's levels, the next level's prefix state (and
        // carry) during this level's product.
        constexpr int NV = G * m / 4 / TNT;  // float4 per thread per group
        float4 va[NV];
        // A is read-only for the launch (non-coherent path); the tape is
        // written by this kernel (plain loads)
        auto load_group = [&](float4 (&v)[NV], const float* src, int nvalid, bool ro) {
#pragma unroll
            for (int q = 0; q < NV; ++q) {
                const int i4 = tid + q * TNT;
                const float4* p = reinterpret_cast<const float4*>(src) + i4;
                v[q] = (i4 * 4 < nvalid) ? (ro ? __ldg(p) : *p) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        };
        FwdState<float> fs[EPT];
        Carry<float> fcy[EPT];
        auto load_fstate = [&](int j) {
            const float* sj = st + (j - 1) * 3 * m;
#pragma unroll
            for (int q = 0; q < EPT; ++q) {
                const int el = tid + q * TNT;
                fs[q].base = sj[el];
                fs[q].blo = sj[m + el];
                fs[q].f0 = sj[2 * m + el];
                fs[q].f1 = fs[q].f2 = fs[q].f3 = 0.f;
                if (MODE == MODE_LOCAL) {
                    fcy[q].hi = fcy[q].lo = 0.f;
                } else {
                    fcy[q].hi = cyt[((int64_t)(j - 1) * 2) * m + el];
                    fcy[q].lo = cyt[((int64_t)(j - 1) * 2 + 1) * m + el];
                }
            }
        };
        load_group(va, Ag + (int64_t)first * m, min(G, Kp - first + 1) * m, true);
        for (int li0 = first; li0 <= Kp; li0 += G) {
            const int ge = min(G, Kp - li0 + 1);
#pragma unroll
            for (int q = 0; q < NV; ++q) {
                const int i4 = tid + q * TNT;
                const int l = (i4 * 4) / m, el = (i4 * 4) % m, r = el / D, cc = el % D;
                *reinterpret_cast<float4*>(sF + l * D * P4 + r * P4 + cc) = va[q];
                float* at = sAT + l * D * P4 + r;
                at[(cc + 0) * P4] = va[q].x;
                at[(cc + 1) * P4] = va[q].y;
                at[(cc + 2) * P4] = va[q].z;
                at[(cc + 3) * P4] = va[q].w;
            }
            if (li0 + G <= Kp) load_group(va, Ag + (int64_t)(li0 + G) * m, min(G, Kp - li0 - G + 1) * m, true);
            load_fstate(1);
            __syncthreads();
            for (int j = 1; j <= NLf; ++j) {
                {
                    // samples outer, the thread's EPT elements inner: EPT
                    // independent dependency chains interleave
                    float* sj = st + (j - 1) * 3 * m;
                    // groups start at positions = 1 mod 4 (G is a multiple
                    // of 4), so a sample's place in its rule block is 1 + l
                    // mod 4 (Riemann, the only rule starting at 0, has none)
#pragma unroll
                    for (int l = 0; l < G; ++l) {
                        if (l < ge) {
#pragma unroll
                            for (int q = 0; q < EPT; ++q) {
                                const int el = tid + q * TNT, r = el / D, cc = el % D;
                                const float P = fwd_step<float, RULE, MODE != MODE_LOCAL>(fs[q], sF[l * D * P4 + r * P4 + cc], 1 + l, kc, fcy[q]);
                                sP[l * D * P4 + r * P4 + cc] = P;
                                if (MODE == MODE_VJP) tape[((int64_t)(j - 1) * L + li0 + l) * m + el] = P;
                            }
                        }
                    }
#pragma unroll
                    for (int q = 0; q < EPT; ++q) {
                        const int el = tid + q * TNT;
                        sj[el] = fs[q].base;
                        sj[m + el] = fs[q].blo;
                        sj[2 * m + el] = fs[q].f0;
                    }
                }
                __syncthreads();
                if (j < NLf) {
                    load_fstate(j + 1);
                    if (tl < ge) {
                        float acc[4][4] = {};
                        mma_tv<D>(acc, sAT + tl * D * P4, P4, sP + tl * D * P4, P4, r0, c0);
#pragma unroll
                        for (int t = 0; t < 4; ++t)
                            *reinterpret_cast<float4*>(sF + tl * D * P4 + (r0 + t) * P4 + c0) =
                                make_float4(acc[t][0], acc[t][1], acc[t][2], acc[t][3]);
                    }
                    __syncthreads();
                }
            }
        }

        if (MODE == MODE_LOCAL) {
            for (int j = 1; j <= n; ++j)
                for (int q = 0; q < EPT; ++q) {
                    const int el = tid + q * TNT;
                    store_lam(I, (int64_t)c * nm + (int64_t)(j - 1) * m + el, st[(j - 1) * 3 * m + el],
                              st[(j - 1) * 3 * m + m + el]);
                }
        }

        if (MODE == MODE_VJP) {
            __syncthreads();
            for (int j = 1; j <= n; ++j)
                for (int q = 0; q < EPT; ++q) {
                    const int el = tid + q * TNT;
                    st[(j - 1) * 3 * m + el] = 0.f;          // Rb (local)
                    st[(j - 1) * 3 * m + m + el] = 0.f;      // its compensation
                    st[(j - 1) * 3 * m + 2 * m + el] = 0.f;  // pend
                }
            float* dAg = static_cast<float*>(I.dA) + b * m;
            const int last0 = first + ((Kp - first) / G) * G;
            // the tape of the next level and that level's reverse state (and
            // carry) are loaded one level ahead of their use
            float4 vt[NV];
            RevState<float> rs[EPT];
            Carry<float> rcy[EPT];
            auto load_rstate = [&](int j) {
                const float* sj = st + (j - 1) * 3 * m;
#pragma unroll
                for (int q = 0; q < EPT; ++q) {
                    const int el = tid + q * TNT;
                    rs[q].Rb = sj[el];
                    rs[q].rlo = sj[m + el];
                    rs[q].pend = sj[2 * m + el];
                    rs[q].R4l = rs[q].R4 = rs[q].H2 = rs[q].H3 = 0.f;
                    rcy[q].hi = cyt[((int64_t)(n + j - 1) * 2) * m + el];
                    rcy[q].lo = cyt[((int64_t)(n + j - 1) * 2 + 1) * m + el];
                }
            };
            for (int li0 = last0; li0 >= first; li0 -= G) {
                const int ge = min(G, Kp - li0 + 1);
                load_group(va, Ag + (int64_t)li0 * m, ge * m, true);
                if (n > 1) load_group(vt, tape + ((int64_t)(n - 2) * L + li0) * m, ge * m, false);
                load_rstate(n);
#pragma unroll
                for (int q = 0; q < NV; ++q) {
                    const int i4 = tid + q * TNT;
                    const int l = (i4 * 4) / m, el = (i4 * 4) % m, r = el / D, cc = el % D;
                    *reinterpret_cast<float4*>(sA + l * D * P4 + r * P4 + cc) = va[q];
                }
                float dacc[4][4] = {};
                // two barriers per level: P^T of the next level is staged in
                // this level's prefix phase (its products have finished
                // reading sPT at the first barrier)
                for (int j = n; j >= 1; --j) {
                    if (j < n) {
                        load_rstate(j);
                        if (tl < ge) {
                            float hacc[4][4] = {};
                            mma_adjL<D>(hacc, sA + tl * D * P4, sG + tl * D * P1, r0, c0);
                            mma_adjR<D>(dacc, sG + tl * D * P1, sPT + tl * D * P4, r0, c0);
#pragma unroll
                            for (int t = 0; t < 4; ++t)
#pragma unroll
                                for (int u = 0; u < 4; ++u) sH[tl * D * P1 + (r0 + t) * P1 + c0 + u] = hacc[t][u];
                        }
                    }
                    __syncthreads();
                    {
                        float* sj = st + (j - 1) * 3 * m;
#pragma unroll
                        for (int l = G - 1; l >= 0; --l) {
                            if (l < ge) {
#pragma unroll
                                for (int q = 0; q < EPT; ++q) {
                                    const int el = tid + q * TNT, r = el / D, cc = el % D;
                                    const float H = (j < n) ? sH[l * D * P1 + r * P1 + cc] : 0.f;
                                    sG[l * D * P1 + r * P1 + cc] = rev_step<float, RULE>(rs[q], H, 1 + l, kc, rcy[q]);
                                }
                            }
                        }
#pragma unroll
                        for (int q = 0; q < EPT; ++q) {
                            const int el = tid + q * TNT;
                            sj[el] = rs[q].Rb;
                            sj[m + el] = rs[q].rlo;
                            sj[2 * m + el] = rs[q].pend;
                        }
                    }
                    if (j > 1) {
                        // P_{j-1} (row-major on the tape) -> P^T in shared
                        // memory for the next level; then the tape of the
                        // level after it
#pragma unroll
                        for (int q = 0; q < NV; ++q) {
                            const int i4 = tid + q * TNT;
                            const int l = (i4 * 4) / m, el = (i4 * 4) % m, r = el / D, cc = el % D;
                            float* pt = sPT + l * D * P4 + r;
                            pt[(cc + 0) * P4] = vt[q].x;
                            pt[(cc + 1) * P4] = vt[q].y;
                            pt[(cc + 2) * P4] = vt[q].z;
                            pt[(cc + 3) * P4] = vt[q].w;
                        }
                        if (j > 2) load_group(vt, tape + ((int64_t)(j - 3) * L + li0) * m, ge * m, false);
                    }
                    __syncthreads();
                }
                if (tl < ge) {
                    const int li = li0 + tl;
                    const bool shared = (li == Kp && c < I.C - 1);
                    float* row = dAg + (int64_t)li * m;
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        float v[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) v[u] = dacc[t][u] + sG[tl * D * P1 + (r0 + t) * P1 + c0 + u];
                        float* dst = row + (r0 + t) * D + c0;
                        if (shared) {
#pragma unroll
                            for (int u = 0; u < 4; ++u) atomicAdd(dst + u, v[u]);
                        } else {
                            *reinterpret_cast<float4*>(dst) = make_float4(v[0], v[1], v[2], v[3]);
                        }
                    }
                }
                __syncthreads();
            }
            // chunk start sample: cotangent pend_j on this chunk's copy of
            // W_j[b]; dA[b] += pend_1 + sum_{j<n} pend_{j+1} pi_j^T
            if (!riem0 && RULE != R_RIEMANN) {
                float bacc[4][4] = {};
                for (int j = 1; j < n; ++j) {
                    for (int el = tid; el < m; el += TNT) {
                        const int r = el / D, cc = el % D;
                        sG[r * P1 + cc] = st[j * 3 * m + 2 * m + el];
                        sPT[cc * P4 + r] = (float)pic[(int64_t)(j - 1) * m + el];
                    }
                    __syncthreads();
                    if (tl == 0) mma_adjR<D>(bacc, sG, sPT, r0, c0);
                    __syncthreads();
                }
                if (tl == 0) {
                    float* row = dAg;
#pragma unroll
                    for (int t = 0; t < 4; ++t)
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const int el = (r0 + t) * D + c0 + u;
                            const float v = bacc[t][u] + st[2 * m + el];
                            if (c > 0) atomicAdd(row + el, v);
                            else row[el] = v;
                        }
                }
            }
        }
        __syncthreads();
    }
}

template <int D>
size_t tile_smem_bytes(int) {
    return (size_t)TileCfg<D>::OPND * sizeof(float);
}

// The dynamic shared-memory opt-in is a per-kernel, per-device setting; it is
// made once (and can be made ahead of a stream capture by prepare_tuned).
template <int D, int RULE, int MODE, int MINB>
cudaError_t set_tile_attr() {
    static std::mutex mu;
    static std::vector<bool> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, false);
    if (done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(k_tile<D, RULE, MODE, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tile_smem_bytes<D>(0));
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

template <int D, int RULE, int MODE, int MINB>
cudaError_t launch_tile_t(const LaunchArgs& a, int grid, bool prepare_only) {
    const size_t smem = tile_smem_bytes<D>(0);
    cudaError_t e = set_tile_attr<D, RULE, MODE, MINB>();
    if (e != cudaSuccess || prepare_only) return e;
    k_tile<D, RULE, MODE, MINB><<<grid, TNT, smem, a.stream>>>(a.insts, a.work, a.nwork, static_cast<float*>(a.scratch),
                                                              a.slot_elems);
    return cudaGetLastError();
}

template <int D, int MODE, int MINB>
cudaError_t launch_tile_r(int rule, const LaunchArgs& a, int grid, bool prepare_only) {
    switch (rule) {
        case R_BOOLE: return launch_tile_t<D, R_BOOLE, MODE, MINB>(a, grid, prepare_only);
        case R_SIMPSON: return launch_tile_t<D, R_SIMPSON, MODE, MINB>(a, grid, prepare_only);
        case R_TRAP: return launch_tile_t<D, R_TRAP, MODE, MINB>(a, grid, prepare_only);
        default: return launch_tile_t<D, R_RIEMANN, MODE, MINB>(a, grid, prepare_only);
    }
}

template <int D, int MINB>
cudaError_t launch_tile_m(int rule, int mode, const LaunchArgs& a, int grid, bool prepare_only) {
    return mode == MODE_LOCAL ? launch_tile_r<D, MODE_LOCAL, MINB>(rule, a, grid, prepare_only)
                              : launch_tile_r<D, MODE_VJP, MINB>(rule, a, grid, prepare_only);
}

}  // namespace

// variant 0: two CTAs per SM (if shared memory allows), 1: one; at d = 32
// variant 2: the tcgen05 forward local pass with the warp-MMA VJP, 3: the
// warp-MMA kernel (mgb_mma32.cu) for both
cudaError_t launch_tile(int D, int rule, int mode, const LaunchArgs& a, int grid, int variant, bool prepare_only) {
    if (D == 32 && variant >= 2) {
        if (variant == 2 && mode == MODE_LOCAL) return launch_tiletc(rule, a, grid, prepare_only);
        return launch_mma32(rule, mode, a, grid, prepare_only);
    }
    if (variant >= 2) variant = 0;
    if (D == 32) return variant == 0 ? launch_tile_m<32, 2>(rule, mode, a, grid, prepare_only)
                                     : launch_tile_m<32, 1>(rule, mode, a, grid, prepare_only);
    return variant == 0 ? launch_tile_m<16, 2>(rule, mode, a, grid, prepare_only)
                        : launch_tile_m<16, 1>(rule, mode, a, grid, prepare_only);
}

TunedChoice choose_tuned(bool plain, int kind, int rule, int mode, bool f64io, const std::vector<InstDev>& hi,
                         int variant) {
    TunedChoice tc;
    (void)rule;
    if (hi.empty() || (mode != MODE_LOCAL && mode != MODE_VJP)) return tc;
    if (hi[0].m == 4) {  // 2x2 matrices and SpaceCurve: thread-per-chunk, both precisions
        for (const InstDev& I : hi) {
            if (I.m != 4 || I.n > small_family_max_levels()) return tc;
            if (kind == KIND_MATRIX && reinterpret_cast<uintptr_t>(I.A) % 16 != 0) return tc;
        }
        tc.use = true;
        tc.family = 1;
        tc.D = 2;
        return tc;
    }
    if (plain || f64io || kind != KIND_MATRIX) return tc;
    const int D = hi[0].d;
    if (D == 64 || D == 128) {
        for (const InstDev& I : hi) {
            if (I.d != D || reinterpret_cast<uintptr_t>(I.A) % 16 != 0) return tc;
            if (mode == MODE_VJP && reinterpret_cast<uintptr_t>(I.dA) % 16 != 0) return tc;
        }
        tc.use = true;
        tc.family = 3;
        tc.D = D;
        tc.nvariants = big_variants(D);
        tc.variant = variant < tc.nvariants ? variant : 0;
        tc.ctas_per_sm = big_ctas_per_sm(D, tc.variant);
        return tc;
    }
    if (D != 16 && D != 32) return tc;
    int nmax = 0;
    for (const InstDev& I : hi) {
        if (I.d != D || I.n < 1) return tc;
        if (reinterpret_cast<uintptr_t>(I.A) % 16 != 0) return tc;
        if (mode == MODE_VJP && reinterpret_cast<uintptr_t>(I.dA) % 16 != 0) return tc;
        nmax = I.n > nmax ? I.n : nmax;
    }
    const size_t smem = D == 32 ? tile_smem_bytes<32>(nmax) : tile_smem_bytes<16>(nmax);
    if (smem > 227 * 1024) return tc;
    tc.use = true;
    tc.family = 2;
    tc.D = D;
    tc.nmax = nmax;
    tc.nvariants = smem <= 113 * 1024 ? (D == 32 ? 4 : 2) : 1;
    tc.variant = variant < tc.nvariants ? variant : 0;
    if (tc.nvariants == 1) tc.variant = 1;  // one CTA per SM only
    tc.ctas_per_sm = tc.variant == 1 ? 1 : 2;
    return tc;
}

cudaError_t prepare_tuned(const TunedChoice& tc, int rule, int mode) {
    if (!tc.use) return cudaSuccess;
    LaunchArgs none{};
    if (tc.family == 3) return launch_big(tc.D, rule, mode, none, 1, tc.variant, true);
    if (tc.family == 2) return launch_tile(tc.D, rule, mode, none, 1, tc.variant, true);
    return cudaSuccess;
}

SegSizing size_segment(bool plain, int kind, int rule, bool f64io, const std::vector<InstDev>& hi, int64_t nwork,
                       int sms, size_t budget_bytes) {
    SegSizing sz;
    const size_t tsz = plain ? sizeof(double) : sizeof(float);
    int64_t Lmax = 1, generic = 0;
    for (const InstDev& I : hi) {
        const int64_t L = std::min<int64_t>((int64_t)I.K, I.S - 1) + 1;
        Lmax = std::max(Lmax, L);
        generic = std::max<int64_t>(generic, (int64_t)(I.n + 4) * L * I.m + 7 * (int64_t)I.n * I.m);
        // the warp-MMA VJP at d = 32: reverse and unwind states, the group
        // buffer of P_1..P_{n-1} (pieces), the split carries and the group
        // buffer's exponents, (14 n - 4) m floats + 4 (n - 1) ints
        generic = std::max<int64_t>(generic, 14 * (int64_t)I.n * I.m);
    }
    // slots for the most resident CTAs any variant of the segment's kernel has
    TunedChoice tc = choose_tuned(plain, kind, rule, MODE_VJP, f64io, hi, 0);
    int64_t want;
    if (tc.use && tc.family == 1) {
        // one thread's tape, then its chunk carries split to hi + lo (VJP)
        sz.slot_elems = Lmax * (small_family_max_levels() - 1) * 4 + 16 * small_family_max_levels();
        want = std::min<int64_t>(nwork, (int64_t)sms * 1024);
    } else if (tc.use) {
        int cps = tc.ctas_per_sm;
        if (tc.family == 3)
            for (int v = 0; v < tc.nvariants; ++v) cps = std::max(cps, big_ctas_per_sm(tc.D, v));
        sz.slot_elems = generic;
        want = std::min<int64_t>(nwork, (int64_t)sms * cps);
    } else {
        sz.slot_elems = generic;
        want = std::min<int64_t>(nwork, (int64_t)sms * 8);
    }
    const size_t slot_bytes = (size_t)sz.slot_elems * tsz;
    sz.grid = std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)(budget_bytes / std::max<size_t>(slot_bytes, 1))));
    return sz;
}

cudaError_t launch_tuned(const TunedChoice& tc, bool plain, int kind, int rule, int mode, const LaunchArgs& a, int sms) {
    if (tc.family == 1) return launch_small_family(plain, kind, rule, mode, a);
    if (tc.family == 3) return launch_big(tc.D, rule, mode, a, sms, tc.variant, false);
    int grid = (int)std::min<int64_t>(a.grid, (int64_t)sms * tc.ctas_per_sm);
    if (grid < 1) grid = 1;
    return launch_tile(tc.D, rule, mode, a, grid, tc.variant, false);
}

}  // namespace mgb
