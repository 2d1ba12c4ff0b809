// Warp-tile form of the d = 32 warp-MMA chunk kernel (mixed form, forward
// local pass and VJP): each warp owns one 16 x 16 output tile of every
// sample of a group, runs its MMAs for all the group's samples and then the
// block-rule prefix pass directly on its accumulators, in registers.
//
// Against the sample-per-warp form (mgb_mma32.cu) this removes the FP32
// round trip of every product through shared memory and one CTA barrier per
// level: a warp goes from its MMAs to its prefix steps to the next level's
// operand stores with no wait on the other warps, so one warp's MMAs overlap
// another's FMA work.  The price is that each operand tile is read by two
// warps (half of it each time), the same shared-memory traffic as the FP32
// round trip it replaces.
//
// Layout (one CTA of NW = 4 warps per chunk, samples in groups of G = 4):
//   warp w: output rows 16 (w >> 1) .. +15, columns 16 (w & 1) .. +15
//   lane (g, t): rows R0 + g (+8), columns C0 + 8 nt + 2 t (+1): 8 elements
//   xa      A of the group as BF16 pieces (A^T by ldmatrix.trans)
//   xb[2]   P_j (forward) or G_j (adjoint) pieces, double-buffered by level
//   xc      P_j from the replay tape (adjoint)
//   sg      FP32 staging of a bulk copy (A of a group or a tape level)
// Products are exact three-piece BF16 splits, six MMAs per piece pair with
// X0 Y0 in its own accumulator, as in the sample-per-warp form.
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
constexpr int NW = 4, NT = 32 * NW, G = NW;
constexpr int NPC = m / 2 / NT;         // element pairs per thread for CTA-wide loops (4)
constexpr uint32_t SET = 3 * PT;        // bytes of one sample's three pieces
constexpr uint32_t SX = G * SET;        // bytes per operand set
constexpr size_t OFF_XA = 0, OFF_XB = SX, OFF_XC = 3 * (size_t)SX, OFF_SG = 4 * (size_t)SX;
constexpr size_t OFF_BAR = OFF_SG + (size_t)G * m * 4;
constexpr size_t SMEM = OFF_BAR + 64;
constexpr int SP = 40;                  // FP32 row pitch of the chunk-boundary scratch (in xc)

// acc[s][nt] (main, small) += X_s[R0.., :] Y_s[:, C0..] for the group's G
// samples, X_s / Y_s as BF16 piece tiles (sample s at +s SET) in row-major
// storage S:  XT: X = S_x^T;  YT: Y = S_y^T.  Two samples' fragments at a
// time; consecutive MMAs feed different accumulators.
template <bool XT, bool YT>
__device__ __forceinline__ void tile_product(uint32_t xs, uint32_t ys, float (&am)[G][2][4], float (&as)[G][2][4],
                                             int lane, int R0, int C0) {
    const int l8 = lane & 7, lb = (lane >> 3) & 1, lh = lane >> 4;
    constexpr int PI[6] = {0, 2, 1, 0, 1, 0}, PJ[6] = {2, 0, 1, 1, 0, 0};
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        const uint32_t oa = !XT ? toff(R0 + l8 + 8 * lb, ks * 16 + 8 * lh) : toff(ks * 16 + l8 + 8 * lh, R0 + 8 * lb);
        const uint32_t ob = !YT ? toff(ks * 16 + l8 + 8 * lb, C0 + 8 * lh) : toff(C0 + 8 * lh + l8, ks * 16 + 8 * lb);
#pragma unroll
        for (int sp = 0; sp < G / 2; ++sp) {
            uint32_t af[2][3][4], bf[2][3][4];
#pragma unroll
            for (int ss = 0; ss < 2; ++ss) {
                const uint32_t so = (uint32_t)(2 * sp + ss) * SET;
#pragma unroll
                for (int p = 0; p < 3; ++p) {
                    if (!XT) ldsm4(xs + so + p * PT + oa, af[ss][p]);
                    else ldsm4t(xs + so + p * PT + oa, af[ss][p]);
                    if (!YT) ldsm4t(ys + so + p * PT + ob, bf[ss][p]);
                    else ldsm4(ys + so + p * PT + ob, bf[ss][p]);
                }
            }
#pragma unroll
            for (int q = 0; q < 6; ++q)
#pragma unroll
                for (int ss = 0; ss < 2; ++ss)
#pragma unroll
                    for (int nt = 0; nt < 2; ++nt) {
                        const int s = 2 * sp + ss;
                        mma16816(q == 5 ? am[s][nt] : as[s][nt], af[ss][PI[q]], bf[ss][PJ[q]][2 * nt],
                                 bf[ss][PJ[q]][2 * nt + 1]);
                    }
        }
    }
}

__device__ __forceinline__ void zero_tile(float (&a)[G][2][4]) {
#pragma unroll
    for (int s = 0; s < G; ++s)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int k = 0; k < 4; ++k) a[s][nt][k] = 0.f;
}

template <int RULE, int MODE>
__global__ void __launch_bounds__(NT, 2)
    k_mma32t(const InstDev* __restrict__ insts, const ChunkRef* __restrict__ work, int64_t nwork,
             float* __restrict__ scratch, int64_t slot_elems, int* __restrict__ tflag) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* const xa = smem + OFF_XA;
    uint8_t* const xb = smem + OFF_XB;  // two sets
    uint8_t* const xc = smem + OFF_XC;
    float* const sg = reinterpret_cast<float*>(smem + OFF_SG);
    float* const scr = reinterpret_cast<float*>(smem + OFF_XC);  // chunk-boundary scratch (xc idle then)
    uint64_t* const bar = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g8 = lane >> 2, t4 = lane & 3;
    const int R0 = 16 * (warp >> 1), C0 = 16 * (warp & 1);
    const uint32_t sxa = tc::su32(xa), sxb = tc::su32(xb), sxc = tc::su32(xc);
    // element (hh, nt, cc) of this lane: row R0 + g8 + 8 hh, column C0 + 8 nt + 2 t4 + cc
    auto erow = [&](int hh) { return R0 + g8 + 8 * hh; };
    auto ecol = [&](int nt) { return C0 + 8 * nt + 2 * t4; };
    auto eidx = [&](int hh, int nt) { return erow(hh) * D + ecol(nt); };

    if (tid == 0) {
        tc::mbar_init(bar);
        tc::mbar_init_fence();
    }
    __syncthreads();
    uint32_t phase = 0;
    bool alive = true;
    float* const slot = scratch + (int64_t)blockIdx.x * slot_elems;
    auto wait_copy = [&]() -> bool {
        const bool ok = __syncthreads_and(tc::mbar_wait(tc::su32(bar), phase & 1)) != 0;
        if (ok) ++phase;
        return ok;
    };
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
        float* const st = slot;
        float* const tape = slot + (int64_t)3 * n * m;
        float* const cyt = tape + (int64_t)(n - 1) * L * m;
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
            // f0_j = A[b] pi_{j-1} for j = 2..NLf (FP32 FMA, once per chunk)
            float* sA0 = scr;
            float* sPi = scr + 32 * SP;
            for (int el = tid; el < m; el += NT) sA0[(el >> 5) * SP + (el & 31)] = __ldg(Ag + el);
            for (int j = 2; j <= NLf; ++j) {
                __syncthreads();
                for (int el = tid; el < m; el += NT)
                    sPi[(el >> 5) * SP + (el & 31)] = (float)pic[(int64_t)(j - 2) * m + el];
                __syncthreads();
#pragma unroll
                for (int q = 0; q < NPC; ++q) {
                    const int r = prow(q), cc = pcol(q);
                    float s0 = 0.f, s1 = 0.f;
                    for (int k = 0; k < D; ++k) {
                        const float a = sA0[r * SP + k];
                        const float2 pv = *reinterpret_cast<const float2*>(sPi + k * SP + cc);
                        s0 = fmaf(a, pv.x, s0);
                        s1 = fmaf(a, pv.y, s1);
                    }
                    *reinterpret_cast<float2*>(st + (j - 1) * 3 * m + 2 * m + r * D + cc) = make_float2(s0, s1);
                }
            }
        }
        __syncthreads();

        auto issue_group = [&](int l0g) {
            if (tid == 0) {
                const int geg = min(G, Kp - l0g + 1);
                tc::fence_async_smem();
                bulk_load(sg, Ag + (int64_t)l0g * m, (uint32_t)geg * m * 4u, bar);
            }
        };
        // this lane's prefix state of a level (8 elements), from the slot
        FwdState<float> fs[2][2][2];
        Carry<float> fcy[2][2][2];
        auto load_fstate = [&](int j) {
            const float* sj = st + (j - 1) * 3 * m;
#pragma unroll
            for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                for (int nt = 0; nt < 2; ++nt) {
                    const int el = eidx(hh, nt);
                    const float2 bs = *reinterpret_cast<const float2*>(sj + el);
                    const float2 bl = *reinterpret_cast<const float2*>(sj + m + el);
                    const float2 f0 = *reinterpret_cast<const float2*>(sj + 2 * m + el);
                    fs[hh][nt][0].base = bs.x; fs[hh][nt][1].base = bs.y;
                    fs[hh][nt][0].blo = bl.x; fs[hh][nt][1].blo = bl.y;
                    fs[hh][nt][0].f0 = f0.x; fs[hh][nt][1].f0 = f0.y;
#pragma unroll
                    for (int cc = 0; cc < 2; ++cc) {
                        fs[hh][nt][cc].f1 = fs[hh][nt][cc].f2 = fs[hh][nt][cc].f3 = 0.f;
                        if (MODE == MODE_LOCAL) {
                            fcy[hh][nt][cc].hi = fcy[hh][nt][cc].lo = 0.f;
                        } else {
                            fcy[hh][nt][cc].hi = cyt[((int64_t)(j - 1) * 2) * m + el + cc];
                            fcy[hh][nt][cc].lo = cyt[((int64_t)(j - 1) * 2 + 1) * m + el + cc];
                        }
                    }
                }
        };
        auto store_fstate = [&](int j) {
            float* sj = st + (j - 1) * 3 * m;
#pragma unroll
            for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                for (int nt = 0; nt < 2; ++nt) {
                    const int el = eidx(hh, nt);
                    *reinterpret_cast<float2*>(sj + el) = make_float2(fs[hh][nt][0].base, fs[hh][nt][1].base);
                    *reinterpret_cast<float2*>(sj + m + el) = make_float2(fs[hh][nt][0].blo, fs[hh][nt][1].blo);
                    *reinterpret_cast<float2*>(sj + 2 * m + el) = make_float2(fs[hh][nt][0].f0, fs[hh][nt][1].f0);
                }
        };
        // prefix of level j over the group from this lane's inputs W[s][hh][nt][cc];
        // P to the pieces of set `pset` (if any), the tape (VJP), the state slot
        auto fwd_level_g = [&](auto fullc, int j, int li0, int ge, const float (&W)[G][2][2][2], uint8_t* pset) {
            constexpr bool FULL = decltype(fullc)::value;
#pragma unroll
            for (int s = 0; s < G; ++s) {
                if (FULL || s < ge) {
#pragma unroll
                    for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                        for (int nt = 0; nt < 2; ++nt) {
                            float P[2];
#pragma unroll
                            for (int cc = 0; cc < 2; ++cc)
                                P[cc] = fwd_step<float, RULE, MODE != MODE_LOCAL>(fs[hh][nt][cc], W[s][hh][nt][cc], 1 + s,
                                                                                   kc, fcy[hh][nt][cc]);
                            if (pset) put_pair(pset + s * SET, erow(hh), ecol(nt), P[0], P[1]);
                            if (MODE == MODE_VJP)
                                *reinterpret_cast<float2*>(tape + ((int64_t)(j - 1) * L + li0 + s) * m + eidx(hh, nt)) =
                                    make_float2(P[0], P[1]);
                        }
                }
            }
            store_fstate(j);
        };
        // full groups take a branch-free body
        auto fwd_level = [&](int j, int li0, int ge, const float (&W)[G][2][2][2], uint8_t* pset) {
            if (ge == G) fwd_level_g(std::true_type{}, j, li0, ge, W, pset);
            else fwd_level_g(std::false_type{}, j, li0, ge, W, pset);
        };

        // ---------------- forward over the groups ----------------
        if (first <= Kp) issue_group(first);
        for (int li0 = first; li0 <= Kp && alive; li0 += G) {
            const int ge = min(G, Kp - li0 + 1);
            if (!wait_copy()) {
                alive = false;
                break;
            }
            for (int i4 = tid; i4 < ge * m / 4; i4 += NT) {
                const float4 v = reinterpret_cast<const float4*>(sg)[i4];
                const int s = (i4 * 4) / m, el = (i4 * 4) % m;
                put_quad(xa + s * SET, el >> 5, el & 31, v);
            }
            load_fstate(1);
            {
                // level 1: W_1 = A, from the staging buffer
                float W[G][2][2][2];
#pragma unroll
                for (int s = 0; s < G; ++s)
#pragma unroll
                    for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                        for (int nt = 0; nt < 2; ++nt) {
                            float2 v = make_float2(0.f, 0.f);
                            if (s < ge) v = *reinterpret_cast<const float2*>(sg + s * m + eidx(hh, nt));
                            W[s][hh][nt][0] = v.x;
                            W[s][hh][nt][1] = v.y;
                        }
                fwd_level(1, li0, ge, W, NLf > 1 ? xb : nullptr);
            }
            __syncthreads();  // xa, P_1 complete; sg free
            if (li0 + G <= Kp) issue_group(li0 + G);
            for (int j = 1; j < NLf; ++j) {
                if (j > 1) __syncthreads();  // P_j complete
                load_fstate(j + 1);
                float am[G][2][4], as[G][2][4];
                zero_tile(am);
                zero_tile(as);
                tile_product<false, false>(sxa, sxb + ((j - 1) & 1) * SX, am, as, lane, R0, C0);
                float W[G][2][2][2];
#pragma unroll
                for (int s = 0; s < G; ++s)
#pragma unroll
                    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                        for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                            for (int cc = 0; cc < 2; ++cc)
                                W[s][hh][nt][cc] = am[s][nt][2 * hh + cc] + as[s][nt][2 * hh + cc];
                fwd_level(j + 1, li0, ge, W, j + 1 < NLf ? xb + (j & 1) * SX : nullptr);
            }
        }

        if (MODE == MODE_LOCAL && alive) {
            __syncthreads();
            for (int j = 1; j <= n; ++j)
                for (int el = tid; el < m; el += NT)
                    I.lam[(int64_t)c * nm + (int64_t)(j - 1) * m + el] =
                        (double)st[(j - 1) * 3 * m + el] + (double)st[(j - 1) * 3 * m + m + el];
        }

        if (MODE == MODE_VJP && alive) {
            asm volatile("fence.proxy.async.global;" ::: "memory");
            __syncthreads();
            for (int j = 1; j <= n; ++j)
                for (int el = tid; el < m; el += NT) {
                    st[(j - 1) * 3 * m + el] = 0.f;
                    st[(j - 1) * 3 * m + m + el] = 0.f;
                    st[(j - 1) * 3 * m + 2 * m + el] = 0.f;
                }
            float* dAg = static_cast<float*>(I.dA) + b * m;
            const int last0 = first + ((Kp - first) / G) * G;
            RevState<float> rs[2][2][2];
            Carry<float> rcy[2][2][2];
            auto load_rstate = [&](int j) {
                const float* sj = st + (j - 1) * 3 * m;
#pragma unroll
                for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                    for (int nt = 0; nt < 2; ++nt) {
                        const int el = eidx(hh, nt);
                        const float2 rb = *reinterpret_cast<const float2*>(sj + el);
                        const float2 rl = *reinterpret_cast<const float2*>(sj + m + el);
                        const float2 pd = *reinterpret_cast<const float2*>(sj + 2 * m + el);
                        rs[hh][nt][0].Rb = rb.x; rs[hh][nt][1].Rb = rb.y;
                        rs[hh][nt][0].rlo = rl.x; rs[hh][nt][1].rlo = rl.y;
                        rs[hh][nt][0].pend = pd.x; rs[hh][nt][1].pend = pd.y;
#pragma unroll
                        for (int cc = 0; cc < 2; ++cc) {
                            RevState<float>& r = rs[hh][nt][cc];
                            r.R4l = r.R4 = r.H2 = r.H3 = 0.f;
                            rcy[hh][nt][cc].hi = cyt[((int64_t)(n + j - 1) * 2) * m + el + cc];
                            rcy[hh][nt][cc].lo = cyt[((int64_t)(n + j - 1) * 2 + 1) * m + el + cc];
                        }
                    }
            };
            auto store_rstate = [&](int j) {
                float* sj = st + (j - 1) * 3 * m;
#pragma unroll
                for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                    for (int nt = 0; nt < 2; ++nt) {
                        const int el = eidx(hh, nt);
                        *reinterpret_cast<float2*>(sj + el) = make_float2(rs[hh][nt][0].Rb, rs[hh][nt][1].Rb);
                        *reinterpret_cast<float2*>(sj + m + el) = make_float2(rs[hh][nt][0].rlo, rs[hh][nt][1].rlo);
                        *reinterpret_cast<float2*>(sj + 2 * m + el) = make_float2(rs[hh][nt][0].pend, rs[hh][nt][1].pend);
                    }
            };
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
                    put_quad(xa + s * SET, el >> 5, el & 31, v);
                }
                __syncthreads();
                if (n > 1) issue_tape(n - 1, li0);
                else if (li0 - G >= first) issue_group(li0 - G);
                float da[G][2][4];  // this lane's dA elements of every sample
                zero_tile(da);
                for (int j = n; j >= 1; --j) {
                    load_rstate(j);
                    float H[G][2][2][2];
                    if (j < n) {
                        // H_j = A^T G_{j+1}
                        float hm[G][2][4], hs[G][2][4];
                        zero_tile(hm);
                        zero_tile(hs);
                        tile_product<true, false>(sxa, sxb + ((j + 1) & 1) * SX, hm, hs, lane, R0, C0);
#pragma unroll
                        for (int s = 0; s < G; ++s)
#pragma unroll
                            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                                for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                                    for (int cc = 0; cc < 2; ++cc)
                                        H[s][hh][nt][cc] = hm[s][nt][2 * hh + cc] + hs[s][nt][2 * hh + cc];
                    } else {
#pragma unroll
                        for (int s = 0; s < G; ++s)
#pragma unroll
                            for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                                for (int nt = 0; nt < 2; ++nt) H[s][hh][nt][0] = H[s][hh][nt][1] = 0.f;
                    }
                    // reverse prefix of level j over the group, in registers:
                    // G_j to pieces (set j & 1), or kept in H for the final dA
                    auto rev_pass = [&](auto fullc) {
                        constexpr bool FULL = decltype(fullc)::value;
#pragma unroll
                    for (int s = G - 1; s >= 0; --s) {
                        if (FULL || s < ge) {
#pragma unroll
                            for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                                for (int nt = 0; nt < 2; ++nt) {
#pragma unroll
                                    for (int cc = 0; cc < 2; ++cc)
                                        H[s][hh][nt][cc] = rev_step<float, RULE>(rs[hh][nt][cc], H[s][hh][nt][cc], 1 + s,
                                                                                 kc, rcy[hh][nt][cc]);
                                    if (j > 1)
                                        put_pair(xb + (j & 1) * SX + s * SET, erow(hh), ecol(nt), H[s][hh][nt][0],
                                                 H[s][hh][nt][1]);
                                }
                        }
                    }
                    };
                    if (ge == G) rev_pass(std::true_type{});
                    else rev_pass(std::false_type{});
                    store_rstate(j);
                    if (j < n) {
                        // dA += G_{j+1} P_j^T
                        float tm[G][2][4], ts[G][2][4];
                        zero_tile(tm);
                        zero_tile(ts);
                        tile_product<false, true>(sxb + ((j + 1) & 1) * SX, sxc, tm, ts, lane, R0, C0);
#pragma unroll
                        for (int s = 0; s < G; ++s)
#pragma unroll
                            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                                for (int k = 0; k < 4; ++k) da[s][nt][k] += tm[s][nt][k] + ts[s][nt][k];
                    }
                    if (j > 1) {
                        // P_{j-1} from the tape -> xc; then the next copy
                        if (!wait_copy()) {
                            alive = false;
                            break;
                        }
                        for (int i4 = tid; i4 < ge * m / 4; i4 += NT) {
                            const float4 v = reinterpret_cast<const float4*>(sg)[i4];
                            const int s = (i4 * 4) / m, el = (i4 * 4) % m;
                            put_quad(xc + s * SET, el >> 5, el & 31, v);
                        }
                        __syncthreads();
                        if (j > 2) issue_tape(j - 2, li0);
                        else if (li0 - G >= first) issue_group(li0 - G);
                    } else {
                        // dA of the group: the level products + G_1 (in H)
#pragma unroll
                        for (int s = 0; s < G; ++s) {
                            if (s < ge) {
                                const int li = li0 + s;
                                const bool shared = (li == Kp && c < I.C - 1);
                                float* row = dAg + (int64_t)li * m;
#pragma unroll
                                for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                                    for (int nt = 0; nt < 2; ++nt) {
                                        const float v0 = da[s][nt][2 * hh] + H[s][hh][nt][0];
                                        const float v1 = da[s][nt][2 * hh + 1] + H[s][hh][nt][1];
                                        float* dst = row + eidx(hh, nt);
                                        if (shared) {
                                            atomicAdd(dst, v0);
                                            atomicAdd(dst + 1, v1);
                                        } else {
                                            *reinterpret_cast<float2*>(dst) = make_float2(v0, v1);
                                        }
                                    }
                            }
                        }
                    }
                }
            }
            // chunk start sample: dA[b] += pend_1 + sum_{j<n} pend_{j+1} pi_j^T (FP32 FMA)
            if (alive && !riem0 && RULE != R_RIEMANN) {
                float* sPd = scr;
                float* sPT = scr + 32 * SP;
                float acc[NPC][2];
                __syncthreads();
#pragma unroll
                for (int q = 0; q < NPC; ++q) {
                    const int el = 2 * (tid + NT * q);
                    acc[q][0] = st[2 * m + el];
                    acc[q][1] = st[2 * m + el + 1];
                }
                for (int j = 1; j < n; ++j) {
                    __syncthreads();
                    for (int el = tid; el < m; el += NT) {
                        const int r = el >> 5, cc = el & 31;
                        sPd[r * SP + cc] = st[j * 3 * m + 2 * m + el];
                        sPT[cc * SP + r] = (float)pic[(int64_t)(j - 1) * m + el];
                    }
                    __syncthreads();
#pragma unroll
                    for (int q = 0; q < NPC; ++q) {
                        const int r = prow(q), cc = pcol(q);
                        for (int k = 0; k < D; ++k) {
                            const float a = sPd[r * SP + k];
                            const float2 pv = *reinterpret_cast<const float2*>(sPT + k * SP + cc);
                            acc[q][0] = fmaf(a, pv.x, acc[q][0]);
                            acc[q][1] = fmaf(a, pv.y, acc[q][1]);
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < NPC; ++q) {
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
            e = cudaFuncSetAttribute(k_mma32t<RULE, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
            if (e != cudaSuccess) return e;
            done[dev] = true;
        }
    }
    if (prepare_only) return cudaSuccess;
    int* flag = device_timeout_ptr();
    if (!flag) return cudaErrorInvalidValue;
    k_mma32t<RULE, MODE><<<grid, NT, SMEM, a.stream>>>(a.insts, a.work, a.nwork, static_cast<float*>(a.scratch),
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

cudaError_t launch_mma32t(int rule, int mode, const LaunchArgs& a, int grid, bool prepare_only) {
    return mode == MODE_LOCAL ? launch_r<MODE_LOCAL>(rule, a, grid, prepare_only)
                              : launch_r<MODE_VJP>(rule, a, grid, prepare_only);
}

}  // namespace mgb
