// Chunk kernel for the mixed form at d = 32 with every per-sample product on
// the tensor cores through warp-level MMA (mma.sync m16n8k16, BF16 operands,
// FP32 accumulators): the forward local pass and the VJP (replay + adjoint).
//
// Why warp MMA at d = 32: the per-sample products W = A P, H = A^T G and
// G P^T share no operand between samples, so a tcgen05 MMA (M >= 64) can only
// hold them as a block-diagonal batch with 50-75 % of it wasted.  On the
// GB300 the m16n8k16 warp MMA measured 607 TFLOP/s dense (BF16 or FP16), so
// a 32 x 32 x 32 product runs as 2 x 4 x 2 of them with no waste, against
// 483 TFLOP/s of useful work for the block-diagonal tcgen05 batch and
// 74 TFLOP/s on the FP32 FMA pipes.
//
// Precision: every FP32 operand is split exactly into three BF16 pieces
// (x = x0 + x1 + x2) once, by the thread that produces it, and each product
// is the sum of the six piece products with i + j <= 2.  X0 Y0 accumulates
// alone and the five small terms together (the tensor core truncates each
// accumulation step): measured 4.7e-8 relative per 32^3 product, against
// 1.0e-7 for FP32 FMA (3.2e-7 with a single accumulator).
//
// Layout (one CTA of NW = 4 warps per chunk, samples in groups of G = 4 = a
// Boole block; warp s owns sample s of the group in the product phases):
//   xa  A of the group as BF16 pieces             [G][3][32 x 32], swizzled
//   xb  P_j (forward) or G_{j+1} (adjoint) pieces [G][3][32 x 32]
//   xc  P_j from the replay tape (adjoint)         [G][3][32 x 32]
//   sw  FP32 product outputs (prefix input)        [G][32][40]
//   sg  FP32 staging of a bulk copy (A of a group or a tape level)
// Piece tiles hold 64-byte rows with the 16-byte chunk c stored at c ^
// ((row >> 1) & 3): ldmatrix of 8 rows and the prefix threads' row stores are
// both free of bank conflicts.
//
// A of each group and (adjoint) each tape level arrive by TMA bulk copies
// (cp.async.bulk, completion on an mbarrier), one copy ahead of their use.
// Prefix passes are the shared block-rule state machines (fwd_step /
// rev_step) with FP32 compensated local accumulators and the FP64 chunk
// carries added as hi + lo, per-level state in the CTA's global slot as in
// the SIMT kernel.  Every mbarrier wait is bounded; on time-out the CTA
// waits (bounded) for its copy in flight, stops and raises the device flag.
#include <cstdint>
#include <cuda_bf16.h>
#include <mutex>
#include <vector>

#include "mgb_common.cuh"
#include "mgb_tc.cuh"
#include "mgb_tuned.h"

namespace mgb {
namespace {

constexpr int D = 32, m = D * D;
constexpr int NW = 4, NT = 32 * NW, G = NW;
constexpr int NP = m / 2 / NT;        // element pairs per thread per sample (4)
constexpr int WP = 40;                // FP32 row pitch of sw (conflict-free float2 epilogue stores)
constexpr uint32_t PT = 32 * 64;      // bytes per piece tile (32 rows x 64 B)
constexpr uint32_t SX = G * 3 * PT;   // bytes per operand set
constexpr size_t OFF_XA = 0, OFF_XB = SX, OFF_XC = 2 * (size_t)SX, OFF_W = 3 * (size_t)SX;
constexpr size_t OFF_SG = OFF_W + (size_t)G * 32 * WP * 4;
constexpr size_t OFF_BAR = OFF_SG + (size_t)G * m * 4;
constexpr size_t SMEM = OFF_BAR + 64;
static_assert(NP * 2 * NT == m, "pair mapping");

// byte offset of (row, col) in a piece tile; col a multiple of 8 for ldmatrix rows
__device__ __forceinline__ uint32_t toff(int r, int c) {
    return (uint32_t)r * 64u + ((uint32_t)((c >> 3) ^ ((r >> 1) & 3)) << 4) + (uint32_t)(c & 7) * 2u;
}

__device__ __forceinline__ void ldsm4(uint32_t a, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void ldsm4t(uint32_t a, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Exact three-piece BF16 split of two values, packed per piece (low half =
// the first value).
__device__ __forceinline__ void split2(float x, float y, uint32_t& p0, uint32_t& p1, uint32_t& p2) {
    const __nv_bfloat162 b0 = __floats2bfloat162_rn(x, y);
    const float2 f0 = __bfloat1622float2(b0);
    const float rx = x - f0.x, ry = y - f0.y;
    const __nv_bfloat162 b1 = __floats2bfloat162_rn(rx, ry);
    const float2 f1 = __bfloat1622float2(b1);
    const __nv_bfloat162 b2 = __floats2bfloat162_rn(rx - f1.x, ry - f1.y);
    p0 = *reinterpret_cast<const uint32_t*>(&b0);
    p1 = *reinterpret_cast<const uint32_t*>(&b1);
    p2 = *reinterpret_cast<const uint32_t*>(&b2);
}

// Store a pair (row r, columns c, c+1) of FP32 values as pieces of tile set t.
__device__ __forceinline__ void put_pair(uint8_t* t, int r, int c, float x, float y) {
    uint32_t p0, p1, p2;
    split2(x, y, p0, p1, p2);
    const uint32_t o = toff(r, c);
    *reinterpret_cast<uint32_t*>(t + o) = p0;
    *reinterpret_cast<uint32_t*>(t + PT + o) = p1;
    *reinterpret_cast<uint32_t*>(t + 2 * PT + o) = p2;
}

// Store four consecutive FP32 values (row r, columns c..c+3, c % 4 == 0).
__device__ __forceinline__ void put_quad(uint8_t* t, int r, int c, float4 v) {
    uint32_t a0, a1, a2, b0, b1, b2;
    split2(v.x, v.y, a0, a1, a2);
    split2(v.z, v.w, b0, b1, b2);
    const uint32_t o = toff(r, c);
    *reinterpret_cast<uint2*>(t + o) = make_uint2(a0, b0);
    *reinterpret_cast<uint2*>(t + PT + o) = make_uint2(a1, b1);
    *reinterpret_cast<uint2*>(t + 2 * PT + o) = make_uint2(a2, b2);
}

// One warp: acc (main, small) [mt][nt] += X Y for one sample, X and Y 32 x 32
// given as BF16 piece tiles (3 tiles, PT bytes apart) in row-major storage S:
//   XT = false: X = S_x (rows m, cols k);  XT = true: X = S_x^T
//   YT = false: Y = S_y (rows k, cols n);  YT = true: Y = S_y^T
// The MMAs are issued piece pair by piece pair over all eight output tiles,
// so that consecutive MMAs never feed the same accumulator (an accumulator's
// next MMA waits out the previous one's latency).
template <bool XT, bool YT>
__device__ __forceinline__ void warp_product(uint32_t xs, uint32_t ys, float (&am)[2][4][4], float (&as)[2][4][4],
                                             int lane) {
    const int l8 = lane & 7, lb = (lane >> 3) & 1, lh = lane >> 4;
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        uint32_t bf[3][4][2];  // [piece][n-tile][reg]
        uint32_t af[3][2][4];  // [piece][m-tile][reg]
#pragma unroll
        for (int ntp = 0; ntp < 2; ++ntp) {
            uint32_t o;
            if (!YT) o = toff(ks * 16 + l8 + 8 * lb, (2 * ntp + lh) * 8);   // trans: rows k, cols n
            else o = toff((2 * ntp + lh) * 8 + l8, ks * 16 + 8 * lb);        // rows n, cols k
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                uint32_t r[4];
                if (!YT) ldsm4t(ys + p * PT + o, r);
                else ldsm4(ys + p * PT + o, r);
                bf[p][2 * ntp][0] = r[0];
                bf[p][2 * ntp][1] = r[1];
                bf[p][2 * ntp + 1][0] = r[2];
                bf[p][2 * ntp + 1][1] = r[3];
            }
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            uint32_t o;
            if (!XT) o = toff(mt * 16 + l8 + 8 * lb, ks * 16 + 8 * lh);   // rows m, cols k
            else o = toff(ks * 16 + l8 + 8 * lh, mt * 16 + 8 * lb);       // trans: rows k, cols m
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                if (!XT) ldsm4(xs + p * PT + o, af[p][mt]);
                else ldsm4t(xs + p * PT + o, af[p][mt]);
            }
        }
        // small terms (smallest first), then the main term
        constexpr int PI[6] = {0, 2, 1, 0, 1, 0}, PJ[6] = {2, 0, 1, 1, 0, 0};
#pragma unroll
        for (int q = 0; q < 6; ++q)
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt)
                    mma16816(q == 5 ? am[mt][nt] : as[mt][nt], af[PI[q]][mt], bf[PJ[q]][nt][0], bf[PJ[q]][nt][1]);
    }
}

__device__ __forceinline__ void zero_acc(float (&a)[2][4][4]) {
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) a[i][j][k] = 0.f;
}

// FP32 output tile of one warp's product (main + small) into sw (pitch WP)
__device__ __forceinline__ void store_acc(float* o, const float (&am)[2][4][4], const float (&as)[2][4][4], int g8,
                                          int t4) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const int r = mt * 16 + g8, cc = nt * 8 + 2 * t4;
            *reinterpret_cast<float2*>(o + r * WP + cc) =
                make_float2(am[mt][nt][0] + as[mt][nt][0], am[mt][nt][1] + as[mt][nt][1]);
            *reinterpret_cast<float2*>(o + (r + 8) * WP + cc) =
                make_float2(am[mt][nt][2] + as[mt][nt][2], am[mt][nt][3] + as[mt][nt][3]);
        }
}

// Bulk copy of `bytes` (a multiple of 16) from global to shared memory,
// completing on the mbarrier.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    const uint32_t b = tc::su32(bar);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(tc::su32(dst)),
        "l"(src), "r"(bytes), "r"(b)
        : "memory");
}

template <int RULE, int MODE>
__global__ void __launch_bounds__(NT, 2)
    k_mma32(const InstDev* __restrict__ insts, const ChunkRef* __restrict__ work, int64_t nwork,
            float* __restrict__ scratch, int64_t slot_elems, int* __restrict__ tflag) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* const xa = smem + OFF_XA;
    uint8_t* const xb = smem + OFF_XB;
    uint8_t* const xc = smem + OFF_XC;
    float* const sw = reinterpret_cast<float*>(smem + OFF_W);
    float* const sg = reinterpret_cast<float*>(smem + OFF_SG);
    uint64_t* const bar = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g8 = lane >> 2, t4 = lane & 3;
    const uint32_t sxa = tc::su32(xa), sxb = tc::su32(xb), sxc = tc::su32(xc);

    if (tid == 0) {
        tc::mbar_init(bar);
        tc::mbar_init_fence();
    }
    __syncthreads();
    uint32_t phase = 0;  // completed copies on bar
    bool alive = true;
    float* const slot = scratch + (int64_t)blockIdx.x * slot_elems;

    // the copy issued last has landed; false after the bounded wait (the
    // copy then stays pending at this parity)
    auto wait_copy = [&]() -> bool {
        const bool ok = __syncthreads_and(tc::mbar_wait(tc::su32(bar), phase & 1)) != 0;
        if (ok) ++phase;
        return ok;
    };
    // thread tid's element pairs: pair p = tid + NT q, elements 2p, 2p + 1
    auto prow = [&](int q) { return (tid + NT * q) >> 4; };
    auto pcol = [&](int q) { return ((tid + NT * q) & 15) * 2; };

    for (int64_t w = blockIdx.x; w < nwork && alive; w += gridDim.x) {
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
        const int NLf = (MODE == MODE_LOCAL) ? n : n - 1;
        float* const st = slot;                              // [n][3][m] prefix state
        float* const tape = slot + (int64_t)3 * n * m;       // [n-1][L][m]
        float* const cyt = tape + (int64_t)(n - 1) * L * m;  // [2][n][2][m] carries hi / lo
        if (MODE == MODE_VJP) {
            const double* rcc = I.rho + (int64_t)c * nm;
            for (int el = tid; el < (int)nm; el += NT) {
                const int j = el / m, e2 = el % m;
                const Carry<float> a = split_carry<float>(riem0 ? 0.0 : pic[el]);
                const Carry<float> r = split_carry<float>(rcc[el]);
                cyt[((int64_t)j * 2) * m + e2] = a.hi;
                cyt[((int64_t)j * 2 + 1) * m + e2] = a.lo;
                cyt[((int64_t)(n + j) * 2) * m + e2] = r.hi;
                cyt[((int64_t)(n + j) * 2 + 1) * m + e2] = r.lo;
            }
        }

        // ---------------- forward state at the chunk start ----------------
        for (int j = 1; j <= NLf; ++j)
            for (int el = tid; el < m; el += NT) {
                st[(j - 1) * 3 * m + el] = 0.f;
                st[(j - 1) * 3 * m + m + el] = 0.f;
                st[(j - 1) * 3 * m + 2 * m + el] = (j == 1) ? __ldg(Ag + el) : 0.f;
            }
        if (MODE == MODE_VJP && !riem0 && NLf >= 2) {
            // f0_j = A[b] P_{j-1}[b] = A[b] pi_{j-1} for j = 2..NLf (FP32 FMA, once per chunk)
            float* sA0 = sw;            // A[b], row pitch WP
            float* sPi = sw + 32 * WP;  // pi_{j-1}
            for (int el = tid; el < m; el += NT) sA0[(el >> 5) * WP + (el & 31)] = __ldg(Ag + el);
            for (int j = 2; j <= NLf; ++j) {
                __syncthreads();
                for (int el = tid; el < m; el += NT)
                    sPi[(el >> 5) * WP + (el & 31)] = (float)pic[(int64_t)(j - 2) * m + el];
                __syncthreads();
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const int r = prow(q), cc = pcol(q);
                    float s0 = 0.f, s1 = 0.f;
                    for (int k = 0; k < D; ++k) {
                        const float a = sA0[r * WP + k];
                        const float2 pv = *reinterpret_cast<const float2*>(sPi + k * WP + cc);
                        s0 = fmaf(a, pv.x, s0);
                        s1 = fmaf(a, pv.y, s1);
                    }
                    *reinterpret_cast<float2*>(st + (j - 1) * 3 * m + 2 * m + r * D + cc) = make_float2(s0, s1);
                }
            }
        }
        __syncthreads();

        // ---------------- forward over the groups ----------------
        // group staging: A of the group by bulk copy into sg, then FP32 into
        // sw (the level-1 prefix input) and BF16 pieces into xa
        auto issue_group = [&](int l0g) {
            if (tid == 0) {
                const int geg = min(G, Kp - l0g + 1);
                tc::fence_async_smem();
                bulk_load(sg, Ag + (int64_t)l0g * m, (uint32_t)geg * m * 4u, bar);
            }
        };
        FwdState<float> fs[NP][2];
        Carry<float> fcy[NP][2];
        auto load_fstate = [&](int j) {
            const float* sj = st + (j - 1) * 3 * m;
#pragma unroll
            for (int q = 0; q < NP; ++q) {
                const int el = 2 * (tid + NT * q);
                const float2 bs = *reinterpret_cast<const float2*>(sj + el);
                const float2 bl = *reinterpret_cast<const float2*>(sj + m + el);
                const float2 f0 = *reinterpret_cast<const float2*>(sj + 2 * m + el);
                fs[q][0].base = bs.x; fs[q][1].base = bs.y;
                fs[q][0].blo = bl.x; fs[q][1].blo = bl.y;
                fs[q][0].f0 = f0.x; fs[q][1].f0 = f0.y;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    fs[q][h].f1 = fs[q][h].f2 = fs[q][h].f3 = 0.f;
                    if (MODE == MODE_LOCAL) {
                        fcy[q][h].hi = fcy[q][h].lo = 0.f;
                    } else {
                        fcy[q][h].hi = cyt[((int64_t)(j - 1) * 2) * m + el + h];
                        fcy[q][h].lo = cyt[((int64_t)(j - 1) * 2 + 1) * m + el + h];
                    }
                }
            }
        };
        if (first <= Kp) issue_group(first);
        for (int li0 = first; li0 <= Kp && alive; li0 += G) {
            const int ge = min(G, Kp - li0 + 1);
            if (!wait_copy()) {
                alive = false;
                break;
            }
            for (int i4 = tid; i4 < ge * m / 4; i4 += NT) {
                const float4 v = reinterpret_cast<const float4*>(sg)[i4];
                const int s = (i4 * 4) / m, el = (i4 * 4) % m, r = el >> 5, cc = el & 31;
                *reinterpret_cast<float4*>(sw + (s * 32 + r) * WP + cc) = v;
                put_quad(xa + s * 3 * PT, r, cc, v);
            }
            load_fstate(1);
            __syncthreads();
            if (li0 + G <= Kp) issue_group(li0 + G);
            for (int j = 1; j <= NLf; ++j) {
                // prefix pass of level j over the group's samples
                {
                    float* sj = st + (j - 1) * 3 * m;
#pragma unroll
                    for (int l = 0; l < G; ++l) {
                        if (l < ge) {
#pragma unroll
                            for (int q = 0; q < NP; ++q) {
                                const int r = prow(q), cc = pcol(q);
                                const float2 f = *reinterpret_cast<const float2*>(sw + (l * 32 + r) * WP + cc);
                                const float P0 = fwd_step<float, RULE, MODE != MODE_LOCAL>(fs[q][0], f.x, 1 + l, kc, fcy[q][0]);
                                const float P1 = fwd_step<float, RULE, MODE != MODE_LOCAL>(fs[q][1], f.y, 1 + l, kc, fcy[q][1]);
                                if (j < NLf) put_pair(xb + l * 3 * PT, r, cc, P0, P1);
                                if (MODE == MODE_VJP)
                                    *reinterpret_cast<float2*>(tape + ((int64_t)(j - 1) * L + li0 + l) * m + r * D + cc) =
                                        make_float2(P0, P1);
                            }
                        }
                    }
#pragma unroll
                    for (int q = 0; q < NP; ++q) {
                        const int el = 2 * (tid + NT * q);
                        *reinterpret_cast<float2*>(sj + el) = make_float2(fs[q][0].base, fs[q][1].base);
                        *reinterpret_cast<float2*>(sj + m + el) = make_float2(fs[q][0].blo, fs[q][1].blo);
                        *reinterpret_cast<float2*>(sj + 2 * m + el) = make_float2(fs[q][0].f0, fs[q][1].f0);
                    }
                }
                __syncthreads();
                if (j < NLf) {
                    load_fstate(j + 1);
                    if (warp < ge) {
                        float am[2][4][4], as[2][4][4];
                        zero_acc(am);
                        zero_acc(as);
                        warp_product<false, false>(sxa + warp * 3 * PT, sxb + warp * 3 * PT, am, as, lane);
                        store_acc(sw + warp * 32 * WP, am, as, g8, t4);
                    }
                    __syncthreads();
                }
            }
        }

        if (MODE == MODE_LOCAL && alive) {
            for (int j = 1; j <= n; ++j)
                for (int el = tid; el < m; el += NT)
                    I.lam[(int64_t)c * nm + (int64_t)(j - 1) * m + el] =
                        (double)st[(j - 1) * 3 * m + el] + (double)st[(j - 1) * 3 * m + m + el];
        }

        if (MODE == MODE_VJP && alive) {
            // the tape written above is read back by bulk copies (async proxy)
            asm volatile("fence.proxy.async.global;" ::: "memory");
            __syncthreads();
            for (int j = 1; j <= n; ++j)
                for (int el = tid; el < m; el += NT) {
                    st[(j - 1) * 3 * m + el] = 0.f;          // Rb (local)
                    st[(j - 1) * 3 * m + m + el] = 0.f;      // its compensation
                    st[(j - 1) * 3 * m + 2 * m + el] = 0.f;  // pend
                }
            float* dAg = static_cast<float*>(I.dA) + b * m;
            const int last0 = first + ((Kp - first) / G) * G;
            RevState<float> rs[NP][2];
            Carry<float> rcy[NP][2];
            auto load_rstate = [&](int j) {
                const float* sj = st + (j - 1) * 3 * m;
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const int el = 2 * (tid + NT * q);
                    const float2 rb = *reinterpret_cast<const float2*>(sj + el);
                    const float2 rl = *reinterpret_cast<const float2*>(sj + m + el);
                    const float2 pd = *reinterpret_cast<const float2*>(sj + 2 * m + el);
                    rs[q][0].Rb = rb.x; rs[q][1].Rb = rb.y;
                    rs[q][0].rlo = rl.x; rs[q][1].rlo = rl.y;
                    rs[q][0].pend = pd.x; rs[q][1].pend = pd.y;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        rs[q][h].R4l = rs[q][h].R4 = rs[q][h].H2 = rs[q][h].H3 = 0.f;
                        rcy[q][h].hi = cyt[((int64_t)(n + j - 1) * 2) * m + el + h];
                        rcy[q][h].lo = cyt[((int64_t)(n + j - 1) * 2 + 1) * m + el + h];
                    }
                }
            };
            // staging uses, in order: A(group), P_{n-1}, ..., P_1 of the group, A(next group), ...
            auto issue_tape = [&](int jt, int l0g) {
                if (tid == 0) {
                    const int geg = min(G, Kp - l0g + 1);
                    tc::fence_async_smem();
                    bulk_load(sg, tape + ((int64_t)(jt - 1) * L + l0g) * m, (uint32_t)geg * m * 4u, bar);
                }
            };
            __syncthreads();
            issue_group(last0);
            for (int li0 = last0; li0 >= first && alive; li0 -= G) {
                const int ge = min(G, Kp - li0 + 1);
                if (!wait_copy()) {
                    alive = false;
                    break;
                }
                for (int i4 = tid; i4 < ge * m / 4; i4 += NT) {
                    const float4 v = reinterpret_cast<const float4*>(sg)[i4];
                    const int s = (i4 * 4) / m, el = (i4 * 4) % m;
                    put_quad(xa + s * 3 * PT, el >> 5, el & 31, v);
                }
                __syncthreads();
                if (n > 1) issue_tape(n - 1, li0);
                else if (li0 - G >= first) issue_group(li0 - G);
                load_rstate(n);
                // dA of the warp's sample: each level's product accumulates
                // in fresh (main, small) accumulators, added here in FP32
                float da[2][4][4];
                zero_acc(da);
                for (int j = n; j >= 1; --j) {
                    if (j < n) {
                        load_rstate(j);
                        if (warp < ge) {
                            // H_j = A^T G_{j+1} -> sw;  dA += G_{j+1} P_j^T
                            float hm[2][4][4], hs[2][4][4];
                            zero_acc(hm);
                            zero_acc(hs);
                            warp_product<true, false>(sxa + warp * 3 * PT, sxb + warp * 3 * PT, hm, hs, lane);
                            store_acc(sw + warp * 32 * WP, hm, hs, g8, t4);
                            float tm[2][4][4], ts[2][4][4];
                            zero_acc(tm);
                            zero_acc(ts);
                            warp_product<false, true>(sxb + warp * 3 * PT, sxc + warp * 3 * PT, tm, ts, lane);
#pragma unroll
                            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                                for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                                    for (int k = 0; k < 4; ++k) da[mt][nt][k] += tm[mt][nt][k] + ts[mt][nt][k];
                        }
                    }
                    __syncthreads();
                    // reverse prefix pass of level j: G_j -> pieces in xb (and
                    // FP32 into sw at level 1, for the final dA)
                    {
                        float* sj = st + (j - 1) * 3 * m;
#pragma unroll
                        for (int l = G - 1; l >= 0; --l) {
                            if (l < ge) {
#pragma unroll
                                for (int q = 0; q < NP; ++q) {
                                    const int r = prow(q), cc = pcol(q);
                                    float2 h = make_float2(0.f, 0.f);
                                    if (j < n) h = *reinterpret_cast<const float2*>(sw + (l * 32 + r) * WP + cc);
                                    const float G0 = rev_step<float, RULE>(rs[q][0], h.x, 1 + l, kc, rcy[q][0]);
                                    const float G1 = rev_step<float, RULE>(rs[q][1], h.y, 1 + l, kc, rcy[q][1]);
                                    if (j > 1) put_pair(xb + l * 3 * PT, r, cc, G0, G1);
                                    else *reinterpret_cast<float2*>(sw + (l * 32 + r) * WP + cc) = make_float2(G0, G1);
                                }
                            }
                        }
#pragma unroll
                        for (int q = 0; q < NP; ++q) {
                            const int el = 2 * (tid + NT * q);
                            *reinterpret_cast<float2*>(sj + el) = make_float2(rs[q][0].Rb, rs[q][1].Rb);
                            *reinterpret_cast<float2*>(sj + m + el) = make_float2(rs[q][0].rlo, rs[q][1].rlo);
                            *reinterpret_cast<float2*>(sj + 2 * m + el) = make_float2(rs[q][0].pend, rs[q][1].pend);
                        }
                    }
                    if (j > 1) {
                        // P_{j-1} from the tape (landed in sg) -> pieces in xc;
                        // then the next copy: P_{j-2}, or A of the next group
                        if (!wait_copy()) {
                            alive = false;
                            break;
                        }
                        for (int i4 = tid; i4 < ge * m / 4; i4 += NT) {
                            const float4 v = reinterpret_cast<const float4*>(sg)[i4];
                            const int s = (i4 * 4) / m, el = (i4 * 4) % m;
                            put_quad(xc + s * 3 * PT, el >> 5, el & 31, v);
                        }
                        __syncthreads();
                        if (j > 2) issue_tape(j - 2, li0);
                        else if (li0 - G >= first) issue_group(li0 - G);
                    } else {
                        __syncthreads();
                    }
                }
                if (!alive) break;
                if (warp < ge) {
                    const int li = li0 + warp;
                    const bool shared = (li == Kp && c < I.C - 1);
                    float* row = dAg + (int64_t)li * m;
                    const float* g1 = sw + warp * 32 * WP;
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                            for (int hh = 0; hh < 2; ++hh) {
                                const int r = mt * 16 + g8 + 8 * hh, cc = nt * 8 + 2 * t4;
                                const float2 gv = *reinterpret_cast<const float2*>(g1 + r * WP + cc);
                                const float v0 = da[mt][nt][2 * hh] + gv.x;
                                const float v1 = da[mt][nt][2 * hh + 1] + gv.y;
                                float* dst = row + r * D + cc;
                                if (shared) {
                                    atomicAdd(dst, v0);
                                    atomicAdd(dst + 1, v1);
                                } else {
                                    *reinterpret_cast<float2*>(dst) = make_float2(v0, v1);
                                }
                            }
                }
                __syncthreads();
            }
            // chunk start sample: cotangent pend_j on this chunk's copy of
            // W_j[b]; dA[b] += pend_1 + sum_{j<n} pend_{j+1} pi_j^T (FP32 FMA)
            if (alive && !riem0 && RULE != R_RIEMANN) {
                float* sPd = sw;            // pend_{j+1}, row-major
                float* sPT = sw + 32 * WP;  // pi_j transposed
                float acc[NP][2];
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const int el = 2 * (tid + NT * q);
                    acc[q][0] = st[2 * m + el];
                    acc[q][1] = st[2 * m + el + 1];
                }
                for (int j = 1; j < n; ++j) {
                    __syncthreads();
                    for (int el = tid; el < m; el += NT) {
                        const int r = el >> 5, cc = el & 31;
                        sPd[r * WP + cc] = st[j * 3 * m + 2 * m + el];
                        sPT[cc * WP + r] = (float)pic[(int64_t)(j - 1) * m + el];
                    }
                    __syncthreads();
#pragma unroll
                    for (int q = 0; q < NP; ++q) {
                        const int r = prow(q), cc = pcol(q);
                        for (int k = 0; k < D; ++k) {
                            const float a = sPd[r * WP + k];
                            const float2 pv = *reinterpret_cast<const float2*>(sPT + k * WP + cc);
                            acc[q][0] = fmaf(a, pv.x, acc[q][0]);
                            acc[q][1] = fmaf(a, pv.y, acc[q][1]);
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                    const int el = 2 * (tid + NT * q);
                    if (c > 0) {
                        atomicAdd(dAg + el, acc[q][0]);
                        atomicAdd(dAg + el + 1, acc[q][1]);
                    } else {
                        *reinterpret_cast<float2*>(dAg + el) = make_float2(acc[q][0], acc[q][1]);
                    }
                }
            }
        }
        __syncthreads();
    }

    if (!alive && tid == 0) {
        // a copy may still be in flight: wait for it (bounded) before exiting
        tc::mbar_wait(tc::su32(bar), phase & 1);
        atomicExch(tflag, 1);
    }
}

template <int RULE, int MODE>
cudaError_t launch_rm(const LaunchArgs& a, int grid, bool prepare_only) {
    static std::mutex mu;
    static std::vector<bool> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    {
        std::lock_guard<std::mutex> lock(mu);
        if ((int)done.size() <= dev) done.resize(dev + 1, false);
        if (!done[dev]) {
            e = cudaFuncSetAttribute(k_mma32<RULE, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
            if (e != cudaSuccess) return e;
            done[dev] = true;
        }
    }
    if (prepare_only) return cudaSuccess;
    int* flag = device_timeout_ptr();
    if (!flag) return cudaErrorInvalidValue;
    k_mma32<RULE, MODE><<<grid, NT, SMEM, a.stream>>>(a.insts, a.work, a.nwork, static_cast<float*>(a.scratch),
                                                      a.slot_elems, flag);
    return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_r(int rule, const LaunchArgs& a, int grid, bool prepare_only) {
    switch (rule) {
        case R_BOOLE: return launch_rm<R_BOOLE, MODE>(a, grid, prepare_only);
        case R_SIMPSON: return launch_rm<R_SIMPSON, MODE>(a, grid, prepare_only);
        case R_TRAP: return launch_rm<R_TRAP, MODE>(a, grid, prepare_only);
        default: return launch_rm<R_RIEMANN, MODE>(a, grid, prepare_only);
    }
}

}  // namespace

cudaError_t launch_mma32(int rule, int mode, const LaunchArgs& a, int grid, bool prepare_only) {
    return mode == MODE_LOCAL ? launch_r<MODE_LOCAL>(rule, a, grid, prepare_only)
                              : launch_r<MODE_VJP>(rule, a, grid, prepare_only);
}

}  // namespace mgb
