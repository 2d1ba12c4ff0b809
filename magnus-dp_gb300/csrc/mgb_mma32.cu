// Chunk kernel for the mixed form at d = 32 with every per-sample product on
// the tensor cores through warp-level MMA (mma.sync m16n8k16, FP16 operands,
// FP32 accumulators): the forward local pass and the VJP.
//
// Why warp MMA at d = 32: the per-sample products W = A P, H = A^T G and
// G P^T share no operand between samples, so a tcgen05 MMA (M >= 64) can only
// hold them as a block-diagonal batch with 50-75 % of it wasted.  On the
// GB300 the m16n8k16 warp MMA measured 607 TFLOP/s dense (BF16 or FP16), so
// a 32 x 32 x 32 product runs as 2 x 4 x 2 of them with no waste, against
// 483 TFLOP/s of useful work for the block-diagonal tcgen05 batch and
// 74 TFLOP/s on the FP32 FMA pipes.
//
// Precision: every FP32 operand matrix is scaled by a power of two from its
// largest element and split exactly into two FP16 pieces once, by the
// threads that produce it (mgb_mma.cuh); a product is the sum of three piece
// products, X0 Y0 in its own accumulator and X0 Y1 + X1 Y0 in a second (the
// tensor core truncates each accumulation step), rescaled in FP32.  The
// scale needs the matrix's maximum before the split: each producing pass
// reduces it per sample (warp max + one shared atomic per warp) and splits
// after a barrier.
//
// Layout (one CTA of NW = 8 warps per chunk, samples in groups of G = 4 = a
// Boole block; in the product phases warps 2s and 2s + 1 own sample s, each
// one 32 x 16 column half of it, so that sixteen warps per SM (two CTAs)
// hide the latency of the prefix and split work):
//   xa  A as FP16 pieces, five sample slots        [5][2][32 x 32], swizzled
//   xb  P_j (forward) or G_{j+1} (adjoint) pieces [G][2][32 x 32]
//   xc  P_j of the group (adjoint), copied in as pieces from the group
//       buffer                                     [G][2][32 x 32]
//   sw  FP32 product outputs (prefix input)        [G][32][36]
//   sg  FP32 staging of a bulk copy of A (a group's samples)
//   mx / sk  per-sample maxima being reduced / scale exponents of the piece
//       sets (A slots 0..4, xb 8..11; the group buffer's in the CTA's slot)
// Piece tiles hold 64-byte rows with the 16-byte chunk c stored at c ^
// ((row >> 1) & 3): ldmatrix of 8 rows and the prefix threads' row stores are
// both free of bank conflicts.
//
// A of each group and (adjoint) each level of the group's P buffer (written
// as scaled pieces by the backward rebuild) arrive by TMA bulk copies
// (cp.async.bulk, completion on an mbarrier), one copy ahead of their use.  The adjoint needs every P_j at every sample in reverse
// order; instead of replaying the chunk forward into a chunk-long tape (4 KB
// per sample and level through HBM, twice), each group's P_j are rebuilt
// backwards from the group end (the chunk end holds P_j = pi^{c+1}_j) by the
// inverse block rules on compensated FP32 pairs, with W_j = A P_{j-1}
// recomputed on the tensor cores.
// Prefix passes are the shared block-rule state machines (fwd_step /
// rev_step) with FP32 compensated local accumulators and the FP64 chunk
// carries added as hi + lo, per-level state in the CTA's global slot as in
// the SIMT kernel.  Every mbarrier wait is bounded; on time-out the CTA
// waits (bounded) for its copy in flight, stops and raises the device flag.
#include <cstdint>
#include <mutex>
#include <type_traits>
#include <vector>

#include "mgb_common.cuh"
#include "mgb_mma.cuh"
#include "mgb_tc.cuh"
#include "mgb_tuned.h"

namespace mgb {
namespace {

using namespace wm;

constexpr int D = 32, m = D * D;
constexpr int NW = 8, NT = 32 * NW, G = 4;
constexpr int NP = m / 2 / NT;        // element pairs per thread per sample (2)
constexpr int WP = 36;                // FP32 row pitch of sw
constexpr uint32_t SET = NPC * PT;    // bytes of one sample's pieces
constexpr uint32_t SX = G * SET;      // bytes per operand set
// xa holds five sample sets: the VJP keeps A of a group's anchor and of its
// four samples (a ring indexed by sample % 5)
constexpr size_t OFF_XA = 0, OFF_XB = 5 * (size_t)SET, OFF_XC = OFF_XB + SX, OFF_W = OFF_XC + SX;
constexpr size_t OFF_SG = OFF_W + (size_t)G * 32 * WP * 4;
constexpr size_t OFF_MX = OFF_SG + (size_t)G * m * 4;  // uint32 [2][8]
constexpr size_t OFF_SK = OFF_MX + 64;                  // int [16]
constexpr size_t OFF_BAR = OFF_SK + 64;
constexpr size_t SMEM = OFF_BAR + 64;
constexpr int SK_B = 8;  // scale-exponent slots of xb (A: 0..4)
static_assert(NP * 2 * NT == m, "pair mapping");
static_assert(m / 4 == NT, "one quad of every sample per thread");
static_assert(SMEM + 1024 <= 114 * 1024, "two CTAs per SM");

// One warp: acc (main, small) [mt][nt] = (X Y)[:, 16 nh .. 16 nh + 15] for
// one sample (scaled), X and Y 32 x 32 given as FP16 piece tiles (NPC tiles,
// PT bytes apart) in row-major storage S:
//   XT = false: X = S_x (rows m, cols k);  XT = true: X = S_x^T
//   YT = false: Y = S_y (rows k, cols n);  YT = true: Y = S_y^T
// The MMAs are issued piece pair by piece pair over the four output tiles,
// so that consecutive MMAs never feed the same accumulator (an accumulator's
// next MMA waits out the previous one's latency).
template <bool XT, bool YT>
__device__ __forceinline__ void warp_product(uint32_t xs, uint32_t ys, float (&am)[2][2][4], float (&as)[2][2][4],
                                             int lane, int nh) {
    const int l8 = lane & 7, lb = (lane >> 3) & 1, lh = lane >> 4;
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        uint32_t bf[NPC][2][2];  // [piece][n-tile][reg]
        uint32_t af[NPC][2][4];  // [piece][m-tile][reg]
        {
            uint32_t o;
            if (!YT) o = toff(ks * 16 + l8 + 8 * lb, (2 * nh + lh) * 8);   // trans: rows k, cols n
            else o = toff((2 * nh + lh) * 8 + l8, ks * 16 + 8 * lb);        // rows n, cols k
#pragma unroll
            for (int p = 0; p < NPC; ++p) {
                uint32_t r[4];
                if (!YT) ldsm4t(ys + p * PT + o, r);
                else ldsm4(ys + p * PT + o, r);
                bf[p][0][0] = r[0];
                bf[p][0][1] = r[1];
                bf[p][1][0] = r[2];
                bf[p][1][1] = r[3];
            }
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            uint32_t o;
            if (!XT) o = toff(mt * 16 + l8 + 8 * lb, ks * 16 + 8 * lh);   // rows m, cols k
            else o = toff(ks * 16 + l8 + 8 * lh, mt * 16 + 8 * lb);       // trans: rows k, cols m
#pragma unroll
            for (int p = 0; p < NPC; ++p) {
                if (!XT) ldsm4(xs + p * PT + o, af[p][mt]);
                else ldsm4t(xs + p * PT + o, af[p][mt]);
            }
        }
        // the two small terms, then the main term
        constexpr int PI[3] = {0, 1, 0}, PJ[3] = {1, 0, 0};
#pragma unroll
        for (int q = 0; q < 3; ++q)
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 2; ++nt) {
                    // each accumulator's first MMA (k-step 0: the first small
                    // term, the main term) starts from zero
                    if (ks == 0 && q != 1)
                        mma16816_first(q == 2 ? am[mt][nt] : as[mt][nt], af[PI[q]][mt], bf[PJ[q]][nt][0],
                                       bf[PJ[q]][nt][1]);
                    else
                        mma16816(q == 2 ? am[mt][nt] : as[mt][nt], af[PI[q]][mt], bf[PJ[q]][nt][0], bf[PJ[q]][nt][1]);
                }
    }
}

// Factors undoing the operand scales 2^kx, 2^ky: v * u.a, then * u.b when
// kx + ky is outside the normal exponent range (u.b != 1; two factors keep
// each one a normal float).  u.b is the same for a whole warp.
struct Unscale {
    float a, b;
};
__device__ __forceinline__ Unscale unscale(int kx, int ky) {
    const int k = kx + ky, k1 = min(126, max(-126, k));
    return Unscale{pow2f(-k1), pow2f(k1 - k)};
}
__device__ __forceinline__ float apply(float v, const Unscale& u, bool two) { return two ? v * u.a * u.b : v * u.a; }

__device__ __forceinline__ void zero_acc(float (&a)[2][2][4]) {
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) a[i][j][k] = 0.f;
}

// FP32 output half-tile of one warp's product (main + small, unscaled) into
// sw (pitch WP)
__device__ __forceinline__ void store_acc(float* o, const float (&am)[2][2][4], const float (&as)[2][2][4], int g8,
                                          int t4, int nh, Unscale u) {
    const bool two = u.b != 1.f;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
            const int r = mt * 16 + g8, cc = (2 * nh + nt) * 8 + 2 * t4;
            *reinterpret_cast<float2*>(o + r * WP + cc) =
                make_float2(apply(am[mt][nt][0] + as[mt][nt][0], u, two), apply(am[mt][nt][1] + as[mt][nt][1], u, two));
            *reinterpret_cast<float2*>(o + (r + 8) * WP + cc) =
                make_float2(apply(am[mt][nt][2] + as[mt][nt][2], u, two), apply(am[mt][nt][3] + as[mt][nt][3], u, two));
        }
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
    uint32_t* const mx = reinterpret_cast<uint32_t*>(smem + OFF_MX);
    int* const sk = reinterpret_cast<int*>(smem + OFF_SK);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g8 = lane >> 2, t4 = lane & 3;
    const int ws = warp >> 1, nh = warp & 1;  // product phases: sample ws, column half nh
    const uint32_t sxa = tc::su32(xa), sxb = tc::su32(xb), sxc = tc::su32(xc);

    if (tid == 0) {
        tc::mbar_init(bar);
        tc::mbar_init_fence();
    }
    if (tid < 16) mx[tid] = 0u;
    __syncthreads();
    // Scaled passes: every thread adds |value| bits of entry i (a sample of
    // the pass) with mx_put (all lanes of every warp, uniformly), then after
    // a barrier reads the entry's scale exponent with mx_get and splits; the
    // pass ends with mx_done (the buffer of the following pass is cleared;
    // a barrier always separates two scaled passes).
    int par = 0;
    auto mx_put = [&](int i, uint32_t u) { max_into(mx + par * 8 + i, u); };
    auto mx_get = [&](int i) { return scale_exp(mx[par * 8 + i]); };
    auto mx_done = [&]() {
        if (tid < 8) mx[(par ^ 1) * 8 + tid] = 0u;
        par ^= 1;
    };
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
    // Scaled pass over up to G samples of FP32 data, quad tid of each
    // (elements 4 tid .. 4 tid + 3): v[s] for s < cnt; sample s's pieces go
    // to the set dst(s) (skipped when null), its exponent to sk[ski(s)].
    auto stage_quads = [&](const float4 (&v)[G], int cnt, auto dst, auto ski) {
#pragma unroll
        for (int s2 = 0; s2 < G; ++s2) mx_put(s2, (s2 < cnt && dst(s2)) ? max4(v[s2]) : 0u);
        __syncthreads();
        const int r = (tid * 4) >> 5, cc = (tid * 4) & 31;
#pragma unroll
        for (int s2 = 0; s2 < G; ++s2) {
            uint8_t* t = s2 < cnt ? dst(s2) : nullptr;
            if (t) {
                const int k = mx_get(s2);
                put_quad(t, r, cc, v[s2], pow2f(k));
                if (tid == 0) sk[ski(s2)] = k;
            }
        }
        mx_done();
    };

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
        const int NLf = n;  // forward local pass: levels with a prefix
        // slot: [n][3][m] prefix state (forward) / reverse state (VJP); VJP:
        // then [n][3][m] unwind state, the group's P_1..P_{n-1} as scaled
        // piece sets [n-1][G][SET bytes], [2][n][2][m] the carries pi^{c+1}
        // and rho^c split into hi / lo, the piece sets' exponents [n-1][G]
        float* const st = slot;
        float* const ust = slot + (int64_t)3 * n * m;
        uint8_t* const gtp = reinterpret_cast<uint8_t*>(ust + (int64_t)3 * n * m);
        float* const cyt = reinterpret_cast<float*>(gtp + (int64_t)(n - 1) * G * SET);
        int* const gtk = reinterpret_cast<int*>(cyt + (int64_t)4 * n * m);
        (void)L;
        if (MODE == MODE_VJP) {
            const double* rcc = I.rho + (int64_t)c * nm;
            const double* pnx = I.pi + (int64_t)(c + 1) * nm;
            for (int el = tid; el < (int)nm; el += NT) {
                const int j = el / m, e2 = el % m;
                const Carry<float> a = split_carry<float>(pnx[el]);
                const Carry<float> r = split_carry<float>(rcc[el]);
                cyt[((int64_t)j * 2) * m + e2] = a.hi;
                cyt[((int64_t)j * 2 + 1) * m + e2] = a.lo;
                cyt[((int64_t)(n + j) * 2) * m + e2] = r.hi;
                cyt[((int64_t)(n + j) * 2 + 1) * m + e2] = r.lo;
            }
        }

        if (MODE == MODE_LOCAL) {
        // ---------------- forward state at the chunk start ----------------
        for (int j = 1; j <= NLf; ++j)
            for (int el = tid; el < m; el += NT) {
                st[(j - 1) * 3 * m + el] = 0.f;
                st[(j - 1) * 3 * m + m + el] = 0.f;
                st[(j - 1) * 3 * m + 2 * m + el] = (j == 1) ? __ldg(Ag + el) : 0.f;
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
            {
                // A of the group: FP32 into sw (the level-1 prefix input),
                // scaled pieces into xa
                float4 v[G];
#pragma unroll
                for (int s2 = 0; s2 < G; ++s2) {
                    v[s2] = s2 < ge ? reinterpret_cast<const float4*>(sg)[s2 * NT + tid] : make_float4(0.f, 0.f, 0.f, 0.f);
                    if (s2 < ge) *reinterpret_cast<float4*>(sw + (s2 * 32 + ((tid * 4) >> 5)) * WP + ((tid * 4) & 31)) = v[s2];
                }
                stage_quads(v, ge, [&](int s2) { return xa + s2 * SET; }, [](int s2) { return s2; });
            }
            load_fstate(1);
            __syncthreads();
            if (li0 + G <= Kp) issue_group(li0 + G);
            for (int j = 1; j <= NLf; ++j) {
                // prefix pass of level j over the group's samples
                {
                    float* sj = st + (j - 1) * 3 * m;
                    float P[G][NP][2];
                    // all of the group's inputs are loaded before any output
                    // is computed, and full groups take a branch-free body, so
                    // the element chains interleave
                    auto pass = [&](auto fullc) {
                        constexpr bool FULL = decltype(fullc)::value;
                        float2 f[G][NP];
#pragma unroll
                        for (int l = 0; l < G; ++l)
#pragma unroll
                            for (int q = 0; q < NP; ++q)
                                f[l][q] = (FULL || l < ge)
                                              ? *reinterpret_cast<const float2*>(sw + (l * 32 + prow(q)) * WP + pcol(q))
                                              : make_float2(0.f, 0.f);
#pragma unroll
                        for (int l = 0; l < G; ++l)
#pragma unroll
                            for (int q = 0; q < NP; ++q) {
                                if (FULL || l < ge) {
                                    P[l][q][0] = fwd_step<float, RULE, false>(fs[q][0], f[l][q].x, 1 + l, kc, fcy[q][0]);
                                    P[l][q][1] = fwd_step<float, RULE, false>(fs[q][1], f[l][q].y, 1 + l, kc, fcy[q][1]);
                                } else {
                                    P[l][q][0] = P[l][q][1] = 0.f;
                                }
                            }
                    };
                    if (ge == G) pass(std::true_type{});
                    else pass(std::false_type{});
#pragma unroll
                    for (int q = 0; q < NP; ++q) {
                        const int el = 2 * (tid + NT * q);
                        *reinterpret_cast<float2*>(sj + el) = make_float2(fs[q][0].base, fs[q][1].base);
                        *reinterpret_cast<float2*>(sj + m + el) = make_float2(fs[q][0].blo, fs[q][1].blo);
                        *reinterpret_cast<float2*>(sj + 2 * m + el) = make_float2(fs[q][0].f0, fs[q][1].f0);
                    }
                    if (j < NLf) {
                        // P_j of the group as scaled pieces (the next level's products)
#pragma unroll
                        for (int l = 0; l < G; ++l) {
                            uint32_t u = 0u;
#pragma unroll
                            for (int q = 0; q < NP; ++q) u = max(u, max(absbits(P[l][q][0]), absbits(P[l][q][1])));
                            mx_put(l, u);
                        }
                        __syncthreads();
#pragma unroll
                        for (int l = 0; l < G; ++l) {
                            if (l < ge) {
                                const int k = mx_get(l);
                                const float sc = pow2f(k);
#pragma unroll
                                for (int q = 0; q < NP; ++q)
                                    put_pair(xb + l * SET, prow(q), pcol(q), P[l][q][0], P[l][q][1], sc);
                                if (tid == 0) sk[SK_B + l] = k;
                            }
                        }
                        mx_done();
                    }
                }
                __syncthreads();
                if (j < NLf) {
                    load_fstate(j + 1);
                    if (ws < ge) {
                        float am[2][2][4], as[2][2][4];
                        warp_product<false, false>(sxa + ws * SET, sxb + ws * SET, am, as, lane, nh);
                        store_acc(sw + ws * 32 * WP, am, as, g8, t4, nh, unscale(sk[ws], sk[SK_B + ws]));
                    }
                    __syncthreads();
                }
            }
        }

        if (alive) {
            for (int j = 1; j <= n; ++j)
                for (int el = tid; el < m; el += NT)
                    store_lam(I, (int64_t)c * nm + (int64_t)(j - 1) * m + el, st[(j - 1) * 3 * m + el],
                              st[(j - 1) * 3 * m + m + el]);
        }
        }  // MODE_LOCAL

        if (MODE == MODE_VJP && alive) {
            // ============ VJP: per group, backwards from the chunk end ============
            // The prefix values P_j of the group's samples are rebuilt from the
            // values at the group's end (at the chunk end: P_j[e] = pi^{c+1}_j)
            // by running each block rule backwards (compensated), with
            // W_j = A P_{j-1} recomputed on the tensor cores; they go through
            // a small per-CTA buffer (L2) to the adjoint.  No replay of the
            // chunk and no chunk-long tape through HBM.
            const RuleCoef<float> kr = kc;
            float* dAg = static_cast<float*>(I.dA) + b * m;
            const float* Ae = Ag + (int64_t)Kp * m;  // the chunk end sample
            auto ring = [](int li) { return li % 5; };
            // reverse state zero, unwind state at the chunk end
            for (int j = 1; j <= n; ++j)
                for (int el = tid; el < m; el += NT) {
                    st[(j - 1) * 3 * m + el] = 0.f;
                    st[(j - 1) * 3 * m + m + el] = 0.f;
                    st[(j - 1) * 3 * m + 2 * m + el] = 0.f;
                }
            for (int j = 1; j < n; ++j)
                for (int el = tid; el < m; el += NT) {
                    ust[(j - 1) * 3 * m + el] = cyt[((int64_t)(j - 1) * 2) * m + el];
                    ust[(j - 1) * 3 * m + m + el] = cyt[((int64_t)(j - 1) * 2 + 1) * m + el];
                    if (j == 1) ust[2 * m + el] = __ldg(Ae + el);
                }
            {
                // A at the chunk end as scaled pieces
                float4 v[G];
                v[0] = __ldg(reinterpret_cast<const float4*>(Ae) + tid);
#pragma unroll
                for (int s2 = 1; s2 < G; ++s2) v[s2] = make_float4(0.f, 0.f, 0.f, 0.f);
                stage_quads(v, 1, [&](int) { return xa + ring(Kp) * SET; }, [&](int) { return ring(Kp); });
            }
            if (n > 2) {
                // W_j[e] = A[e] pi^{c+1}_{j-1} for j = 2..n-1 (FP32 FMA, once per chunk)
                float* sA0 = sw;
                float* sPi = sw + 32 * WP;
                for (int el = tid; el < m; el += NT) sA0[(el >> 5) * WP + (el & 31)] = __ldg(Ae + el);
                for (int j = 2; j < n; ++j) {
                    __syncthreads();
                    for (int el = tid; el < m; el += NT)
                        sPi[(el >> 5) * WP + (el & 31)] =
                            cyt[((int64_t)(j - 2) * 2) * m + el] + cyt[((int64_t)(j - 2) * 2 + 1) * m + el];
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
                        *reinterpret_cast<float2*>(ust + (j - 1) * 3 * m + 2 * m + r * D + cc) = make_float2(s0, s1);
                    }
                }
            }
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
            // bulk copies, one in flight, in order: a group's new samples
            // into sg (its anchor a = li0 - 1 through li0 + ge - 2, sg offset
            // s holding sample a + s; the group end is staged already), then
            // P_{n-1}, ..., P_1 of the group as pieces into xc, then the next
            // group's new samples ...
            auto issue_new = [&](int l0g) {
                if (tid == 0) {
                    const int geg = min(G, Kp - l0g + 1);
                    const int s0 = max(l0g - 1, 0);  // Riemann's first chunk has no anchor sample
                    const int cnt = l0g + geg - 1 - s0;
                    tc::fence_async_smem();
                    bulk_load(sg + (s0 - (l0g - 1)) * m, Ag + (int64_t)s0 * m, (uint32_t)cnt * m * 4u, bar);
                }
            };
            // P_jt of the group, as pieces, straight into xc
            auto issue_tape = [&](int jt, int geg) {
                if (tid == 0) {
                    tc::fence_async_smem();
                    bulk_load(xc, gtp + (int64_t)(jt - 1) * G * SET, (uint32_t)geg * SET, bar);
                }
            };
            __syncthreads();
            issue_new(last0);
            for (int li0 = last0; li0 >= first && alive; li0 -= G) {
                const int ge = min(G, Kp - li0 + 1);
                const int a = li0 - 1;
                const bool noa = riem0 && li0 == 0;
                if (!wait_copy()) {
                    alive = false;
                    break;
                }
                {
                    // A of the anchor and the new samples (sg offset so holds
                    // sample a + so) as scaled pieces into the ring
                    float4 v[G];
#pragma unroll
                    for (int s2 = 0; s2 < G; ++s2)
                        v[s2] = s2 < ge ? reinterpret_cast<const float4*>(sg)[s2 * NT + tid] : make_float4(0.f, 0.f, 0.f, 0.f);
                    stage_quads(
                        v, ge, [&](int so) -> uint8_t* { return (noa && so == 0) ? nullptr : xa + ring(a + so) * SET; },
                        [&](int so) { return ring(a + so); });
                }
                __syncthreads();
                // ---- unwind levels 1..n-1: P_j at the group's samples
                for (int j = 1; j < n; ++j) {
                    if (j > 1) {
                        // W_j = A P_{j-1} at offsets 0..ge-1 (samples a .. a + ge - 1)
                        if (ws < ge && !(noa && ws == 0)) {
                            float am[2][2][4], as[2][2][4];
                            warp_product<false, false>(sxa + ring(a + ws) * SET, sxb + ws * SET, am, as, lane, nh);
                            store_acc(sw + ws * 32 * WP, am, as, g8, t4, nh, unscale(sk[ring(a + ws)], sk[SK_B + ws]));
                        }
                        __syncthreads();
                    }
                    float* uj = ust + (j - 1) * 3 * m;
                    uint8_t* gj = gtp + (int64_t)(j - 1) * G * SET;
                    float Pk[NP][2][G + 1];  // P_j at offsets 0..G (gg: the group end)
                    auto pass = [&](auto fullc) {
                        constexpr bool FULL = decltype(fullc)::value;
                        const int gg = FULL ? G : ge;
#pragma unroll
                        for (int q = 0; q < NP; ++q) {
                            const int r = prow(q), cc = pcol(q), el = 2 * (tid + NT * q);
                            // W at offsets 0..G (G: the group end, carried)
                            float W[2][G + 1];
                            const float2 ph = *reinterpret_cast<const float2*>(uj + el);
                            const float2 pl = *reinterpret_cast<const float2*>(uj + m + el);
                            const float2 we = *reinterpret_cast<const float2*>(uj + 2 * m + el);
#pragma unroll
                            for (int so = 0; so < G; ++so) {
                                float2 v = make_float2(0.f, 0.f);
                                if (FULL || so < ge)
                                    v = (j == 1) ? *reinterpret_cast<const float2*>(sg + so * m + el)
                                                 : *reinterpret_cast<const float2*>(sw + (so * 32 + r) * WP + cc);
                                W[0][so] = v.x;
                                W[1][so] = v.y;
                            }
#pragma unroll
                            for (int so = 0; so <= G; ++so)
                                if (so == gg) {
                                    W[0][so] = we.x;
                                    W[1][so] = we.y;
                                }
                            float P[2][G] = {};
                            float hi[2] = {ph.x, ph.y}, lo[2] = {pl.x, pl.y};
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
                                const float* w = W[h];
                                if (RULE == R_BOOLE) {
                                    // one block (a, a + 4]
                                    const float inc = w[0] * kr.b14 + w[1] * kr.b64 + w[2] * kr.b24 + w[3] * kr.b64 + w[4] * kr.b14;
                                    acc_add(hi[h], lo[h], -inc);
                                    P[h][0] = hi[h] + lo[h];
                                    P[h][1] = (w[1] * kr.h + w[0] * kr.h + lo[h]) + hi[h];
                                    P[h][2] = (w[2] * kr.t3 + w[0] * kr.t3 + w[1] * kr.c4_3 + lo[h]) + hi[h];
                                    P[h][3] = (w[3] * kr.c38 + w[0] * kr.c38 + w[1] * kr.c98 + w[2] * kr.c98 + lo[h]) + hi[h];
                                } else if (RULE == R_SIMPSON) {
                                    // blocks (a + 2, a + 4] (full groups) and (a, a + 2]
                                    if (FULL || gg == 4) {
                                        const float inc = w[4] * kr.t3 + w[2] * kr.t3 + w[3] * (4.f * kr.t3);
                                        acc_add(hi[h], lo[h], -inc);
                                        P[h][2] = hi[h] + lo[h];
                                        P[h][3] = (w[3] * kr.h + w[2] * kr.h + lo[h]) + hi[h];
                                    }
                                    const float inc = w[2] * kr.t3 + w[0] * kr.t3 + w[1] * (4.f * kr.t3);
                                    acc_add(hi[h], lo[h], -inc);
                                    P[h][0] = hi[h] + lo[h];
                                    P[h][1] = (w[1] * kr.h + w[0] * kr.h + lo[h]) + hi[h];
                                } else {
#pragma unroll
                                    for (int so = G; so >= 1; --so) {
                                        if (FULL || so <= gg) {
                                            const float inc = (RULE == R_TRAP) ? w[so] * kr.h + w[so - 1] * kr.h : w[so] * kr.dt;
                                            acc_add(hi[h], lo[h], -inc);
                                            P[h][so - 1] = hi[h] + lo[h];
                                        }
                                    }
                                }
                            }
                            // P_j at offsets 0..gg (gg: the previous group-end
                            // value), the new group-end state
#pragma unroll
                            for (int so = 0; so <= G; ++so) {
                                Pk[q][0][so] = so < gg ? P[0][so < G ? so : 0] : so == gg ? ph.x + pl.x : 0.f;
                                Pk[q][1][so] = so < gg ? P[1][so < G ? so : 0] : so == gg ? ph.y + pl.y : 0.f;
                            }
                            *reinterpret_cast<float2*>(uj + el) = make_float2(hi[0], hi[1]);
                            *reinterpret_cast<float2*>(uj + m + el) = make_float2(lo[0], lo[1]);
                            *reinterpret_cast<float2*>(uj + 2 * m + el) = make_float2(W[0][0], W[1][0]);
                        }
                    };
                    if (ge == G) pass(std::true_type{});
                    else pass(std::false_type{});
                    {
                        // P_j as scaled pieces: offsets 0..ge-1 into xb (the
                        // next level's products), the group's samples (offsets
                        // 1..gg) to the group buffer (the adjoint's G P^T),
                        // one exponent per offset
                        const int gg = ge;
                        const bool nxt = j + 1 < n;
#pragma unroll
                        for (int so = 0; so <= G; ++so) {
                            uint32_t u = 0u;
                            if (so <= gg && !(noa && so == 0)) {
#pragma unroll
                                for (int q = 0; q < NP; ++q)
                                    u = max(u, max(absbits(Pk[q][0][so]), absbits(Pk[q][1][so])));
                            }
                            mx_put(so, u);
                        }
                        __syncthreads();
#pragma unroll
                        for (int so = 0; so <= G; ++so) {
                            if (so <= gg) {
                                const int k = mx_get(so);
                                const float sc = pow2f(k);
                                const bool tox = nxt && so < gg && !(noa && so == 0), tot = so >= 1;
                                // one split, stored to both destinations
#pragma unroll
                                for (int q = 0; q < NP; ++q) {
                                    if (!tox && !tot) break;
                                    uint32_t p0, p1;
                                    split2(Pk[q][0][so], Pk[q][1][so], sc, p0, p1);
                                    const uint32_t o = toff(prow(q), pcol(q));
                                    if (tox) {
                                        *reinterpret_cast<uint32_t*>(xb + so * SET + o) = p0;
                                        *reinterpret_cast<uint32_t*>(xb + so * SET + PT + o) = p1;
                                    }
                                    if (tot) {
                                        *reinterpret_cast<uint32_t*>(gj + (so - 1) * SET + o) = p0;
                                        *reinterpret_cast<uint32_t*>(gj + (so - 1) * SET + PT + o) = p1;
                                    }
                                }
                                if (tid == 0 && tox) sk[SK_B + so] = k;
                                if (tid == 0 && tot) gtk[(j - 1) * G + so - 1] = k;
                            }
                        }
                        mx_done();
                    }
                    __syncthreads();
                }
                // the group buffer was written by threads, is read by bulk copies
                asm volatile("fence.proxy.async.global;" ::: "memory");
                __syncthreads();
                if (n > 1) issue_tape(n - 1, ge);
                else if (li0 - G >= first) issue_new(li0 - G);
                load_rstate(n);
                // dA of the warp's sample: each level's product accumulates
                // in fresh (main, small) accumulators, added here in FP32
                float da[2][2][4];
                zero_acc(da);
                const uint32_t xas = sxa + ring(li0 + ws) * SET;
                for (int j = n; j >= 1; --j) {
                    if (j < n) {
                        load_rstate(j);
                        if (ws < ge) {
                            // H_j = A^T G_{j+1} -> sw;  dA += G_{j+1} P_j^T
                            const int kp = gtk[(j - 1) * G + ws];
                            float hm[2][2][4], hs[2][2][4];
                            warp_product<true, false>(xas, sxb + ws * SET, hm, hs, lane, nh);
                            store_acc(sw + ws * 32 * WP, hm, hs, g8, t4, nh, unscale(sk[ring(li0 + ws)], sk[SK_B + ws]));
                            float tm[2][2][4], ts[2][2][4];
                            warp_product<false, true>(sxb + ws * SET, sxc + ws * SET, tm, ts, lane, nh);
                            const Unscale u = unscale(sk[SK_B + ws], kp);
                            if (u.b == 1.f) {
#pragma unroll
                                for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                                    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                                        for (int k = 0; k < 4; ++k)
                                            da[mt][nt][k] = fmaf(tm[mt][nt][k] + ts[mt][nt][k], u.a, da[mt][nt][k]);
                            } else {
#pragma unroll
                                for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                                    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                                        for (int k = 0; k < 4; ++k)
                                            da[mt][nt][k] += (tm[mt][nt][k] + ts[mt][nt][k]) * u.a * u.b;
                            }
                        }
                    }
                    __syncthreads();
                    // the products above were the last readers of xc: P_{j-1}
                    // of the group lands there during the reverse pass
                    if (j < n && j > 1) issue_tape(j - 1, ge);
                    // reverse prefix pass of level j: G_j -> scaled pieces in
                    // xb (and FP32 into sw at level 1, for the final dA)
                    {
                        float* sj = st + (j - 1) * 3 * m;
                        float Gv[G][NP][2];
                        auto pass = [&](auto fullc) {
                            constexpr bool FULL = decltype(fullc)::value;
                            float2 h[G][NP];
#pragma unroll
                            for (int l = 0; l < G; ++l)
#pragma unroll
                                for (int q = 0; q < NP; ++q)
                                    h[l][q] = ((FULL || l < ge) && j < n)
                                                  ? *reinterpret_cast<const float2*>(sw + (l * 32 + prow(q)) * WP + pcol(q))
                                                  : make_float2(0.f, 0.f);
#pragma unroll
                            for (int l = G - 1; l >= 0; --l)
#pragma unroll
                                for (int q = 0; q < NP; ++q) {
                                    if (FULL || l < ge) {
                                        Gv[l][q][0] = rev_step<float, RULE>(rs[q][0], h[l][q].x, 1 + l, kc, rcy[q][0]);
                                        Gv[l][q][1] = rev_step<float, RULE>(rs[q][1], h[l][q].y, 1 + l, kc, rcy[q][1]);
                                    } else {
                                        Gv[l][q][0] = Gv[l][q][1] = 0.f;
                                    }
                                }
                        };
                        if (ge == G) pass(std::true_type{});
                        else pass(std::false_type{});
#pragma unroll
                        for (int q = 0; q < NP; ++q) {
                            const int el = 2 * (tid + NT * q);
                            *reinterpret_cast<float2*>(sj + el) = make_float2(rs[q][0].Rb, rs[q][1].Rb);
                            *reinterpret_cast<float2*>(sj + m + el) = make_float2(rs[q][0].rlo, rs[q][1].rlo);
                            *reinterpret_cast<float2*>(sj + 2 * m + el) = make_float2(rs[q][0].pend, rs[q][1].pend);
                        }
                        if (j > 1) {
#pragma unroll
                            for (int l = 0; l < G; ++l) {
                                uint32_t u = 0u;
#pragma unroll
                                for (int q = 0; q < NP; ++q) u = max(u, max(absbits(Gv[l][q][0]), absbits(Gv[l][q][1])));
                                mx_put(l, u);
                            }
                            __syncthreads();
#pragma unroll
                            for (int l = 0; l < G; ++l) {
                                if (l < ge) {
                                    const int k = mx_get(l);
                                    const float sc = pow2f(k);
#pragma unroll
                                    for (int q = 0; q < NP; ++q)
                                        put_pair(xb + l * SET, prow(q), pcol(q), Gv[l][q][0], Gv[l][q][1], sc);
                                    if (tid == 0) sk[SK_B + l] = k;
                                }
                            }
                            mx_done();
                        } else {
#pragma unroll
                            for (int l = 0; l < G; ++l)
                                if (l < ge) {
#pragma unroll
                                    for (int q = 0; q < NP; ++q)
                                        *reinterpret_cast<float2*>(sw + (l * 32 + prow(q)) * WP + pcol(q)) =
                                            make_float2(Gv[l][q][0], Gv[l][q][1]);
                                }
                        }
                    }
                    if (j > 1) {
                        // P_{j-1} of the group has landed in xc; after P_1 the
                        // next group's samples follow
                        if (!wait_copy()) {
                            alive = false;
                            break;
                        }
                        if (j == 2 && li0 - G >= first) issue_new(li0 - G);
                    } else {
                        __syncthreads();
                    }
                }
                if (!alive) break;
                if (ws < ge) {
                    const int li = li0 + ws;
                    const bool shared = (li == Kp && c < I.C - 1);
                    float* row = dAg + (int64_t)li * m;
                    const float* g1 = sw + ws * 32 * WP;
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                            for (int hh = 0; hh < 2; ++hh) {
                                const int r = mt * 16 + g8 + 8 * hh, cc = (2 * nh + nt) * 8 + 2 * t4;
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
