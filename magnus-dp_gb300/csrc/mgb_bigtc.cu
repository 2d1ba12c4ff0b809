// Chunk kernel for the mixed form (FP32 products, FP64 carries) at d = 64 and
// d = 128, with the products on the tensor cores.
//
// Level-major over one chunk per CTA (chunk buffers in a per-CTA global
// slot): per level a prefix pass (elementwise over the chunk's samples, each
// thread four adjacent elements with eight samples of loads in flight, FP32
// local accumulators with compensation, the FP64 chunk carry added when a
// value is emitted) and a product pass over the chunk's samples:
//   forward  W = A P
//   adjoint  H = A^T G,  dA += G P^T
// Products are tcgen05.mma kind::f16 on BF16 pieces: every FP32 operand is
// split exactly into three BF16 values, x = x0 + x1 + x2, and X Y is the sum
// of the six piece products with i + j <= 2, accumulated in FP32 in tensor
// memory (neglected terms ~2^-27 relative: FP32 accuracy at the tensor-core
// cost of a TF32 three-term split).  The tensor core rounds each
// accumulation step toward zero, so the main product X0 Y0 and the five
// small ones go to separate accumulators, summed in FP32 by the epilogue:
// the main accumulator takes one step per 16 of K instead of six.  All threads stage the operands from global memory (splitting
// on the way) into shared memory in the K-major, no-swizzle core-matrix
// layout: core matrix = 8 rows x 16 bytes, 8-row groups 128 bytes apart
// (SBO), 16-byte K chunks D*16 bytes apart (LBO).  K goes in blocks of 32
// through two stages; one thread issues the MMAs (M = N = D, K = 16 each) and
// tcgen05.commit arrives on a per-stage
// and a per-accumulator mbarrier; accumulators for two samples (4 D columns
// of tensor memory) let the epilogue of one sample overlap the MMAs of the
// next.
// Accumulator layout: M = 128 puts row r in lane r; M = 64 puts row r in lane
// 32 (r / 16) + r % 16.
//
// Every mbarrier wait is bounded (about two seconds of the global timer).
// On time-out the CTA stops issuing work, waits (bounded) for its MMAs in
// flight, frees its tensor memory, raises a device flag and returns; the
// host reports MGB_ERR_DEVICE_TIMEOUT.
#include <cstdint>
#include <mutex>
#include <vector>

#include <cuda_bf16.h>

#include "mgb_common.cuh"
#include "mgb_tc.cuh"
#include "mgb_tuned.h"

namespace mgb {

__device__ int g_device_timeout;

namespace {

constexpr int TNT = 256;

// KB: k-block per stage (32 or 64); NACC: accumulator pairs (2: the
// epilogue of one sample overlaps the MMAs of the next; 1: half the tensor
// memory, so that two d = 128 CTAs share an SM).  The autotuner picks.
template <int D, int KB, int NACC = 2>
struct TcCfg {
    static constexpr int m = D * D;
    static constexpr uint32_t TILE = D * KB * 2;              // bytes per operand piece (bf16)
    static constexpr uint32_t STAGE = 6 * TILE;               // X0 X1 X2 Y0 Y1 Y2
    static constexpr uint32_t LBO = D * 16, SBO = 128;        // bytes
    static constexpr uint32_t NCOL = 2 * NACC * D;            // NACC samples x (main, small) accumulators
    // D = 128 with two accumulator pairs takes 4 x 128 columns, all of an
    // SM's tensor memory: its shared memory request is padded so that no
    // other CTA of these kernels fits on the SM beside it.
    static constexpr size_t SMEM = (D == 128 && NACC == 2) ? (size_t)200 * 1024 : 2 * (size_t)STAGE + 64;
    static constexpr size_t BAR_OFF = 2 * (size_t)STAGE;
    static constexpr int NKB = D / KB;
    // kind::f16 instruction descriptor: F32 accumulator (bits 4-5 = 1), BF16 A
    // and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at 24
    static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(D >> 3) << 17) |
                                      ((uint32_t)(D >> 4) << 24);
};

// tcgen05 / mbarrier helpers and the BF16 split: mgb_tc.cuh
using namespace tc;

// byte offset of element (row, 8-wide k chunk kc) in a K-major BF16 tile
template <int D>
__device__ __forceinline__ uint32_t core_off(int row, int kc) {
    return (uint32_t)kc * (D * 16) + (uint32_t)(row >> 3) * 128 + (uint32_t)(row & 7) * 16;
}

// One k-block of an operand tile, element (row, k) = TRANS ? src[k][row] :
// src[row][k] (src row-major D x D in global memory), held in registers
// between its load and its store to shared memory so that the loads of the
// next block overlap the MMAs and the epilogue.  Item = (row, 8 consecutive
// k): direct loads are one 32-byte sector per thread, transposed loads eight
// 4-byte loads coalesced across the warp; the stores are one 16-byte chunk
// per piece, consecutive rows at consecutive 16 bytes (no bank conflicts).
// Plain loads: the chunk buffers are written by this kernel.
template <int D, int KB>
struct TileRegs {
    static constexpr int NI = D * (KB / 8) / TNT;  // items per thread
    float v[NI][8];
};

template <int D, int KB, bool TRANS>
__device__ __forceinline__ void load_tile(TileRegs<D, KB>& r, const float* __restrict__ src, int kb) {
#pragma unroll
    for (int i = 0; i < TileRegs<D, KB>::NI; ++i) {
        const int it = threadIdx.x + i * TNT, row = it % D, s8 = it / D;
        if (!TRANS) {
            const float* p = src + (int64_t)row * D + kb * KB + s8 * 8;
            const float4 a = *reinterpret_cast<const float4*>(p);
            const float4 b = *reinterpret_cast<const float4*>(p + 4);
            r.v[i][0] = a.x; r.v[i][1] = a.y; r.v[i][2] = a.z; r.v[i][3] = a.w;
            r.v[i][4] = b.x; r.v[i][5] = b.y; r.v[i][6] = b.z; r.v[i][7] = b.w;
        } else {
            const float* p = src + (int64_t)(kb * KB + s8 * 8) * D + row;
#pragma unroll
            for (int u = 0; u < 8; ++u) r.v[i][u] = p[(int64_t)u * D];
        }
    }
}

// Split the held block into three BF16 pieces at t, t + TILE, t + 2 TILE.
template <int D, int KB>
__device__ __forceinline__ void store_tile(uint8_t* t, const TileRegs<D, KB>& r) {
    constexpr uint32_t TL = TcCfg<D, KB>::TILE;
#pragma unroll
    for (int i = 0; i < TileRegs<D, KB>::NI; ++i) {
        const int it = threadIdx.x + i * TNT, row = it % D, s8 = it / D;
        uint32_t w[3][4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            uint16_t l0, l1, l2, h0, h1, h2;
            split3(r.v[i][2 * h], l0, l1, l2);
            split3(r.v[i][2 * h + 1], h0, h1, h2);
            w[0][h] = (uint32_t)l0 | ((uint32_t)h0 << 16);
            w[1][h] = (uint32_t)l1 | ((uint32_t)h1 << 16);
            w[2][h] = (uint32_t)l2 | ((uint32_t)h2 << 16);
        }
        const uint32_t o = core_off<D>(row, s8);
#pragma unroll
        for (int q = 0; q < 3; ++q) *reinterpret_cast<uint4*>(t + q * TL + o) = make_uint4(w[q][0], w[q][1], w[q][2], w[q][3]);
    }
}

// ------------------------------------------------------------ product pipeline
struct Pipe {
    uint32_t kt, ns;         // stages and samples issued so far (uniform)
    uint32_t tbase;          // tensor memory base
    uint32_t mb;             // mbarriers: [0,1] stages, [2,3] accumulators (NACC = 1: [2]), [4] final
    uint8_t* stg;            // two stages
    bool ok;                 // this thread saw no time-out
};

// Accumulator of sample counter s -> out (row-major D x D), stored or added.
template <int D, int NACC>
__device__ __forceinline__ void epilogue(Pipe& pp, uint32_t s, float* __restrict__ out, bool add) {
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, q = warp & 3, h = warp >> 2;
    const uint32_t a = NACC == 2 ? (s & 1) : 0u;
    const uint32_t par = NACC == 2 ? ((s >> 1) & 1) : (s & 1);
    if (pp.ok && !mbar_wait(pp.mb + 8 * (2 + a), par)) pp.ok = false;
    pp.ok = __all_sync(0xffffffffu, pp.ok);  // tcgen05.ld is warp-collective
    fence_after();
    if (!pp.ok) return;
    constexpr int CW = D / 2;  // columns per warp
    const int row = (D == 128) ? 32 * q + lane : 16 * q + (lane & 15);
    const bool valid = (D == 128) || lane < 16;
#pragma unroll
    for (int c0 = 0; c0 < CW; c0 += 16) {
        const int col = h * CW + c0;
        float v[16], u[16];
        const uint32_t ta = pp.tbase + ((uint32_t)(32 * q) << 16) + a * 2 * D + (uint32_t)col;
        tmem_ld16(ta, v);
        tmem_ld16(ta + D, u);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += u[i];
        if (valid) {
            float4* o = reinterpret_cast<float4*>(out + (int64_t)row * D + col);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                float4 w = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
                if (add) {
                    const float4 p = o[i];
                    w.x += p.x; w.y += p.y; w.z += p.z; w.w += p.w;
                }
                o[i] = w;
            }
        }
    }
    fence_before();
}

// out[li] (=|+=) op(X[li]) op(Y[li]) for li in [l0, l1]; X, Y, out advance by
// D*D per sample.  XT / YT: the operand's K-major tile is the transpose of
// the stored matrix (X: element (r, k) = X[k][r]; Y: B^T element (n, k) =
// Y[k][n] for YT, Y[n][k] otherwise).  Returns false on a time-out (uniform).
template <int D, int KB, int NACC, bool XT, bool YT>
__device__ bool tc_pass(Pipe& pp, const float* __restrict__ X, const float* __restrict__ Y, float* __restrict__ out,
                        bool add, int l0, int l1) {
    using Cf = TcCfg<D, KB, NACC>;
    constexpr int m = Cf::m;
    const int cnt = l1 - l0 + 1;
    if (cnt <= 0) return true;
    TileRegs<D, KB> rx, ry;
    load_tile<D, KB, XT>(rx, X + (int64_t)l0 * m, 0);
    load_tile<D, KB, YT>(ry, Y + (int64_t)l0 * m, 0);
    for (int idx = 0; idx <= cnt; ++idx) {
        if (idx < cnt) {
            const int li = l0 + idx;
            const uint32_t a = NACC == 2 ? (pp.ns & 1) : 0u;
            for (int kb = 0; kb < Cf::NKB; ++kb) {
                // one accumulator pair: the previous sample's epilogue frees
                // it before this sample's first MMA (the barrier below orders
                // its tensor-memory loads before the issue)
                if (NACC == 1 && kb == 0 && idx > 0) epilogue<D, NACC>(pp, pp.ns - 1, out + (int64_t)(li - 1) * m, add);
                const uint32_t b = pp.kt & 1;
                if (pp.kt >= 2 && pp.ok && !mbar_wait(pp.mb + 8 * b, ((pp.kt - 2) >> 1) & 1)) pp.ok = false;
                uint8_t* xs = pp.stg + (size_t)b * Cf::STAGE;
                uint8_t* ys = xs + 3 * Cf::TILE;
                if (pp.ok) {
                    store_tile<D, KB>(xs, rx);
                    store_tile<D, KB>(ys, ry);
                }
                fence_async_smem();
                if (__syncthreads_or(!pp.ok)) return false;
                if (threadIdx.x == 0) {
                    fence_after();
                    // main term X0 Y0 and the five small terms in separate
                    // accumulators (each tensor-core accumulation step rounds
                    // toward zero; keeping the main accumulator to one step per
                    // 16 of K keeps that bias at FP32 level)
                    const uint32_t dmain = pp.tbase + a * 2 * D, dsmall = dmain + D;
                    const uint32_t x0 = su32(xs), y0 = su32(ys);
                    constexpr int PI[5] = {2, 0, 1, 1, 0}, PJ[5] = {0, 2, 1, 0, 1};
#pragma unroll
                    for (int ks = 0; ks < KB / 16; ++ks) {
                        const uint32_t o = (uint32_t)ks * 2 * Cf::LBO;  // K = 16: two 8-wide chunks
                        const uint32_t fresh = (kb == 0 && ks == 0) ? 0u : 1u;
#pragma unroll
                        for (int t = 0; t < 5; ++t)
                            mma_bf16(dsmall, smem_desc(x0 + PI[t] * Cf::TILE + o, Cf::LBO, Cf::SBO),
                                     smem_desc(y0 + PJ[t] * Cf::TILE + o, Cf::LBO, Cf::SBO), Cf::IDESC,
                                     t == 0 ? fresh : 1u);
                        mma_bf16(dmain, smem_desc(x0 + o, Cf::LBO, Cf::SBO), smem_desc(y0 + o, Cf::LBO, Cf::SBO),
                                 Cf::IDESC, fresh);
                    }
                    mma_commit(pp.mb + 8 * b);
                    if (kb == Cf::NKB - 1) mma_commit(pp.mb + 8 * (2 + a));
                }
                ++pp.kt;
                // operands of the next k-block (this sample's or the next one's)
                const int nkb = kb + 1 < Cf::NKB ? kb + 1 : 0;
                const int nli = kb + 1 < Cf::NKB ? li : li + 1;
                if (nli <= l1) {
                    load_tile<D, KB, XT>(rx, X + (int64_t)nli * m, nkb);
                    load_tile<D, KB, YT>(ry, Y + (int64_t)nli * m, nkb);
                }
                if (NACC == 2 && kb == 0 && idx > 0) epilogue<D, NACC>(pp, pp.ns - 1, out + (int64_t)(li - 1) * m, add);
            }
            ++pp.ns;
        } else {
            epilogue<D, NACC>(pp, pp.ns - 1, out + (int64_t)(l1)*m, add);
        }
    }
    return !__syncthreads_or(!pp.ok);
}

// ------------------------------------------------------------ prefix passes
// PF: samples of loads in flight per thread (8; 4 in the three-CTA variant,
// whose register budget is smaller).  A sample's place in its rule block is
// a compile-time constant: the forward sweep starts at position 1 and the
// reverse one at Kp (a multiple of 4 for Boole, of 2 for Simpson; Trapezoid
// and Riemann have no blocks), and both advance PF (a multiple of 4) at a time.

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, const float4& v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float comp(const float4& v, int u) { return u == 0 ? v.x : u == 1 ? v.y : u == 2 ? v.z : v.w; }

// P_j over the chunk from f (F) for levels with a carry row pic_j (nullptr:
// zero); keep: write P to the tape; lam_j (MODE_LOCAL): the chunk total.
template <int RULE, int PF, bool CY>
__device__ __forceinline__ void prefix_fwd(const float* __restrict__ F, float* __restrict__ Pj, bool keep,
                                           const double* __restrict__ pic_j, double* __restrict__ lam_j, int m, int Kp,
                                           int first, bool riem0, const RuleCoef<float>& kc) {
    for (int e4 = threadIdx.x * 4; e4 < m; e4 += TNT * 4) {
        Carry<float> cy[4];
        FwdState<float> s[4];
        const float4 f0 = ld4(F + e4);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            cy[u] = split_carry<float>(pic_j ? pic_j[e4 + u] : 0.0);
            s[u].base = s[u].blo = 0.f;
            s[u].f0 = comp(f0, u);
            s[u].f1 = s[u].f2 = s[u].f3 = 0.f;
        }
        if (!riem0 && keep)
            st4(Pj + e4, make_float4(add_carry(0.f, cy[0]), add_carry(0.f, cy[1]), add_carry(0.f, cy[2]),
                                     add_carry(0.f, cy[3])));
        float4 nx[PF];
#pragma unroll
        for (int u = 0; u < PF; ++u) nx[u] = (first + u <= Kp) ? ld4(F + (int64_t)(first + u) * m + e4) : f0;
        for (int l0 = first; l0 <= Kp; l0 += PF) {
            float4 cur[PF];
#pragma unroll
            for (int u = 0; u < PF; ++u) cur[u] = nx[u];
#pragma unroll
            for (int u = 0; u < PF; ++u) {
                const int ln = l0 + PF + u;
                if (ln <= Kp) nx[u] = ld4(F + (int64_t)ln * m + e4);
            }
#pragma unroll
            for (int u = 0; u < PF; ++u) {
                const int li = l0 + u;
                if (li <= Kp) {
                    float4 P;
                    P.x = fwd_step<float, RULE, CY>(s[0], cur[u].x, 1 + u, kc, cy[0]);
                    P.y = fwd_step<float, RULE, CY>(s[1], cur[u].y, 1 + u, kc, cy[1]);
                    P.z = fwd_step<float, RULE, CY>(s[2], cur[u].z, 1 + u, kc, cy[2]);
                    P.w = fwd_step<float, RULE, CY>(s[3], cur[u].w, 1 + u, kc, cy[3]);
                    if (keep) st4(Pj + (int64_t)li * m + e4, P);
                }
            }
        }
        if (lam_j)
#pragma unroll
            for (int u = 0; u < 4; ++u) lam_j[e4 + u] = (double)s[u].base + (double)s[u].blo;
    }
}

// G over the chunk (positions Kp..first) from H (nullptr: zero) and the
// carry row rc_j; G[0] = pend unless riem0.
template <int RULE, int PF>
__device__ __forceinline__ void prefix_rev(const float* __restrict__ H, float* __restrict__ G,
                                           const double* __restrict__ rc_j, int m, int Kp, int first, bool riem0,
                                           const RuleCoef<float>& kc) {
    for (int e4 = threadIdx.x * 4; e4 < m; e4 += TNT * 4) {
        Carry<float> cy[4];
        RevState<float> s[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            cy[u] = split_carry<float>(rc_j[e4 + u]);
            s[u].Rb = s[u].rlo = s[u].pend = s[u].R4l = s[u].R4 = s[u].H2 = s[u].H3 = 0.f;
        }
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        float4 nx[PF];
#pragma unroll
        for (int u = 0; u < PF; ++u) nx[u] = (H && Kp - u >= first) ? ld4(H + (int64_t)(Kp - u) * m + e4) : z;
        for (int l0 = Kp; l0 >= first; l0 -= PF) {
            float4 cur[PF];
#pragma unroll
            for (int u = 0; u < PF; ++u) cur[u] = nx[u];
#pragma unroll
            for (int u = 0; u < PF; ++u) {
                const int ln = l0 - PF - u;
                if (H && ln >= first) nx[u] = ld4(H + (int64_t)ln * m + e4);
            }
#pragma unroll
            for (int u = 0; u < PF; ++u) {
                const int li = l0 - u;
                if (li >= first) {
                    float4 g;
                    g.x = rev_step<float, RULE>(s[0], cur[u].x, 4 * PF - u, kc, cy[0]);
                    g.y = rev_step<float, RULE>(s[1], cur[u].y, 4 * PF - u, kc, cy[1]);
                    g.z = rev_step<float, RULE>(s[2], cur[u].z, 4 * PF - u, kc, cy[2]);
                    g.w = rev_step<float, RULE>(s[3], cur[u].w, 4 * PF - u, kc, cy[3]);
                    st4(G + (int64_t)li * m + e4, g);
                }
            }
        }
        if (!riem0) st4(G + e4, make_float4(s[0].pend, s[1].pend, s[2].pend, s[3].pend));
    }
}

// ------------------------------------------------------------ the kernel
template <int D, int KB, int RULE, int MODE, int MINB, int NACC>
__global__ void __launch_bounds__(TNT, MINB)
    k_bigtc(const InstDev* __restrict__ insts, const ChunkRef* __restrict__ work, int64_t nwork,
            float* __restrict__ scratch, int64_t slot_elems) {
    using Cf = TcCfg<D, KB, NACC>;
    constexpr int m = Cf::m;
    constexpr int PF = MINB >= 3 ? 4 : 8;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + Cf::BAR_OFF);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 5);
    const int tid = threadIdx.x, warp = tid / 32;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                     "r"(Cf::NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < 5; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(bars + i)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    Pipe pp;
    pp.kt = pp.ns = 0;
    pp.tbase = *tslot;
    pp.mb = su32(bars);
    pp.stg = smem;
    pp.ok = true;
    float* const slot = scratch + (int64_t)blockIdx.x * slot_elems;
    bool alive = true;

    for (int64_t w = blockIdx.x; w < nwork && alive; w += gridDim.x) {
        const ChunkRef wk = work[w];
        const InstDev& I = insts[wk.inst];
        const int c = wk.chunk, n = I.n;
        const int64_t b = (int64_t)c * I.K;
        const int64_t e = (b + I.K < I.S - 1) ? b + I.K : I.S - 1;
        const int Kp = (int)(e - b), L = Kp + 1;
        const bool riem0 = (RULE == R_RIEMANN) && c == 0;
        const int first = riem0 ? 0 : 1;
        const int64_t Lm = (int64_t)L * m, nm = (int64_t)n * m;
        const RuleCoef<float> kc = rule_coef<float>(I);
        const float* Ag = static_cast<const float*>(I.A) + b * m;
        float* const tape = slot;               // [n-1][L][m] P_j
        float* const Wb = tape + (n - 1) * Lm;  // [L][m] level values
        float* const Gb = Wb + Lm;              // [L][m] cotangents on W_j
        float* const Hb = Gb + Lm;              // [L][m] cotangents on P_j
        float* const dAb = Hb + Lm;             // [L][m] dA from the products
        const double* pic = I.pi + (int64_t)c * nm;
        const int NL = (MODE == MODE_LOCAL) ? n : n - 1;

        // ---------------- forward over the chunk ----------------
        const float* F = Ag;
        for (int j = 1; j <= NL && alive; ++j) {
            const bool keep = j < n;
            float* Pj = tape + (int64_t)((j < n ? j : 1) - 1) * Lm;
            const double* carry = (MODE == MODE_LOCAL || riem0) ? nullptr : pic + (int64_t)(j - 1) * m;
            double* lam = (MODE == MODE_LOCAL) ? I.lam + (int64_t)c * nm + (int64_t)(j - 1) * m : nullptr;
            prefix_fwd<RULE, PF, MODE != MODE_LOCAL>(F, Pj, keep, carry, lam, m, Kp, first, riem0, kc);
            __syncthreads();
            if (j < NL) {
                alive = tc_pass<D, KB, NACC, false, true>(pp, Ag, Pj, Wb, false, 0, Kp);  // W = A P
                F = Wb;
            }
        }

        if (MODE == MODE_VJP && alive) {
            const double* rc = I.rho + (int64_t)c * nm;
            for (int j = n; j >= 1 && alive; --j) {
                if (j < n) {
                    const float* Pj = tape + (int64_t)(j - 1) * Lm;
                    alive = tc_pass<D, KB, NACC, true, true>(pp, Ag, Gb, Hb, false, first, Kp);         // H = A^T G
                    if (alive) alive = tc_pass<D, KB, NACC, false, false>(pp, Gb, Pj, dAb, j < n - 1, 0, Kp);  // dA += G P^T
                    if (!alive) break;
                }
                prefix_rev<RULE, PF>(j < n ? Hb : nullptr, Gb, rc + (int64_t)(j - 1) * m, m, Kp, first, riem0, kc);
                __syncthreads();
            }
            if (alive) {
                float* dAg = static_cast<float*>(I.dA) + b * m;
                for (int64_t i4 = (int64_t)tid * 4; i4 < Lm; i4 += TNT * 4) {
                    const int li = (int)(i4 / m);
                    if (RULE == R_RIEMANN && li == 0 && c > 0) continue;  // f_b unused by Riemann
                    float4 v = ld4(Gb + i4);
                    if (n > 1) {
                        const float4 p = ld4(dAb + i4);
                        v.x += p.x; v.y += p.y; v.z += p.z; v.w += p.w;
                    }
                    const bool shared = (li == 0 && c > 0) || (li == Kp && c < I.C - 1);
                    if (shared) {
                        atomicAdd(dAg + i4, v.x);
                        atomicAdd(dAg + i4 + 1, v.y);
                        atomicAdd(dAg + i4 + 2, v.z);
                        atomicAdd(dAg + i4 + 3, v.w);
                    } else {
                        st4(dAg + i4, v);
                    }
                }
            }
        }
        __syncthreads();
    }

    // ---------------- teardown ----------------
    if (!alive && tid == 0) {
        // wait (bounded) for every MMA this CTA issued, then report
        fence_after();
        mma_commit(pp.mb + 8 * 4);
        mbar_wait(pp.mb + 8 * 4, 0);
        atomicExch(&g_device_timeout, 1);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(pp.tbase), "r"(Cf::NCOL) : "memory");
}

template <int D, int KB, int RULE, int MODE, int MINB, int NACC>
cudaError_t set_attr() {
    static std::mutex mu;
    static std::vector<bool> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, false);
    if (done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(k_bigtc<D, KB, RULE, MODE, MINB, NACC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)TcCfg<D, KB, NACC>::SMEM);
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

template <int D, int KB, int RULE, int MODE, int MINB, int NACC>
cudaError_t launch_t(const LaunchArgs& a, int grid, bool prepare_only) {
    cudaError_t e = set_attr<D, KB, RULE, MODE, MINB, NACC>();
    if (e != cudaSuccess || prepare_only) return e;
    k_bigtc<D, KB, RULE, MODE, MINB, NACC><<<grid, TNT, TcCfg<D, KB, NACC>::SMEM, a.stream>>>(
        a.insts, a.work, a.nwork, static_cast<float*>(a.scratch), a.slot_elems);
    return cudaGetLastError();
}

template <int D, int KB, int MODE, int MINB, int NACC>
cudaError_t launch_r(int rule, const LaunchArgs& a, int grid, bool prepare_only) {
    switch (rule) {
        case R_BOOLE: return launch_t<D, KB, R_BOOLE, MODE, MINB, NACC>(a, grid, prepare_only);
        case R_SIMPSON: return launch_t<D, KB, R_SIMPSON, MODE, MINB, NACC>(a, grid, prepare_only);
        case R_TRAP: return launch_t<D, KB, R_TRAP, MODE, MINB, NACC>(a, grid, prepare_only);
        default: return launch_t<D, KB, R_RIEMANN, MODE, MINB, NACC>(a, grid, prepare_only);
    }
}

template <int D, int KB, int MINB, int NACC = 2>
cudaError_t launch_m(int rule, int mode, const LaunchArgs& a, int grid, bool prepare_only) {
    return mode == MODE_LOCAL ? launch_r<D, KB, MODE_LOCAL, MINB, NACC>(rule, a, grid, prepare_only)
                              : launch_r<D, KB, MODE_VJP, MINB, NACC>(rule, a, grid, prepare_only);
}

}  // namespace

int big_variants(int D) { return D == 64 ? 5 : 3; }
int big_ctas_per_sm(int D, int variant) {
    if (D == 64) return variant == 4 ? 3 : (variant < 2 ? 2 : 1);
    return variant == 2 ? 2 : 1;
}

// variant: D = 64: 0 KB 32 / 2 CTAs per SM, 1 KB 64 / 2, 2 KB 32 / 1, 3 KB 64 / 1,
//                  4 KB 32 with one accumulator pair / 3;
//          D = 128: 0 KB 32, 1 KB 64 (one CTA per SM, two accumulator pairs),
//          2 KB 32 with one accumulator pair, two CTAs per SM.
cudaError_t launch_big(int D, int rule, int mode, const LaunchArgs& a, int sms, int variant, bool prepare_only) {
    const int ctas = sms * big_ctas_per_sm(D, variant);
    int grid = (int)std::min<int64_t>(a.grid, (int64_t)ctas);
    if (grid < 1) grid = 1;
    if (D == 128) {
        if (variant == 2) return launch_m<128, 32, 2, 1>(rule, mode, a, grid, prepare_only);
        return variant == 1 ? launch_m<128, 64, 1>(rule, mode, a, grid, prepare_only)
                            : launch_m<128, 32, 1>(rule, mode, a, grid, prepare_only);
    }
    switch (variant) {
        case 1: return launch_m<64, 64, 2>(rule, mode, a, grid, prepare_only);
        case 2: return launch_m<64, 32, 1>(rule, mode, a, grid, prepare_only);
        case 3: return launch_m<64, 64, 1>(rule, mode, a, grid, prepare_only);
        case 4: return launch_m<64, 32, 3, 1>(rule, mode, a, grid, prepare_only);
        default: return launch_m<64, 32, 2>(rule, mode, a, grid, prepare_only);
    }
}

int* device_timeout_ptr() {
    static std::mutex mu;
    static std::vector<int*> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)cache.size() <= dev) cache.resize(dev + 1, nullptr);
    if (!cache[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_device_timeout) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        cache[dev] = static_cast<int*>(p);
    }
    return cache[dev];
}

int read_clear_device_timeout() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_device_timeout, sizeof(int)) != cudaSuccess) return 0;
    if (v) {
        const int z = 0;
        cudaMemcpyToSymbol(g_device_timeout, &z, sizeof(int));
    }
    return v;
}

}  // namespace mgb
