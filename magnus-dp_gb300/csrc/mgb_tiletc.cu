// Forward chunk kernel for the mixed form at d = 32 with the products on the
// tensor cores (a launch variant of the group-tiled kernel k_tile; the
// autotuner picks between them).
//
// One CTA per chunk, samples in groups of G = 4 (a Boole block).  The four
// samples' 32 x 32 products W_{j+1} = A P_j share no operand, so they go in
// one M = N = 128 MMA as a block-diagonal batch: X = the four A stacked (rows
// 32 s + i), Y = the four P side by side (columns 32 s + c); only the
// diagonal 32 x 32 blocks of the 128 x 128 result are read.  Three quarters
// of each MMA are wasted, but the products leave the FP32 pipes free for the
// prefix passes, which the SIMT kernel interleaves with its products.
// Operands are split exactly into three BF16 pieces and the six piece
// products with i + j <= 2 accumulate in two tensor-memory accumulators
// (X0 Y0 alone, the five small terms together; the tensor core rounds each
// accumulation step toward zero), summed in FP32 by the epilogue.
//
// Per group and level: prefix pass (thread per (4 rows, 1 column) of every
// sample: four independent chains; FP32 local accumulators with the FP64
// chunk carry as hi + lo) -> P_j written as the Y operand's BF16 pieces ->
// one thread issues the MMAs -> the epilogue reads each warp's diagonal block
// (warp q & 3: sample q's rows are its TMEM lanes) into shared memory -> the
// next level's prefix.  Per-level prefix state lives in a per-CTA global
// slot as in k_tile.  Every mbarrier wait is bounded; on time-out the CTA
// stops, waits (bounded) for its MMAs, frees its tensor memory and raises the
// device flag (MGB_ERR_DEVICE_TIMEOUT on the host).
#include <cstdint>
#include <mutex>
#include <vector>

#include "mgb_common.cuh"
#include "mgb_tc.cuh"
#include "mgb_tuned.h"

namespace mgb {
namespace {

using namespace tc;

constexpr int TT = 256;
constexpr int D = 32, m = D * D, G = 4;
constexpr int PF = D + 4;                        // FP32 W rows in shared memory (16-byte aligned, spread banks)
constexpr uint32_t TILE = 128 * D * 2;          // bytes per BF16 piece of a 128 x 32 operand
constexpr uint32_t LBO = 128 * 16, SBO = 128;   // K chunks of 8 columns; 8-row groups
constexpr uint32_t NCOL = 256;                  // accumulators: main (128 columns) + small (128)
// kind::f16, F32 accumulator, BF16 A and B, both K-major, N = M = 128
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
constexpr size_t OFF_X = 0, OFF_Y = 3 * TILE, OFF_F = 6 * TILE;
constexpr size_t OFF_BAR = OFF_F + (size_t)G * D * PF * sizeof(float);
// Padded so that at most two CTAs fit on an SM whatever the register count:
// two take all of its tensor memory, and a third would wait in
// tcgen05.alloc until one of them finished its whole work list.
constexpr size_t SMEM = (OFF_BAR + 64) > 80 * 1024 ? OFF_BAR + 64 : 80 * 1024;

// byte offset of element (row r, column k) of a 128 x 32 K-major BF16 tile
__device__ __forceinline__ uint32_t off128(int r, int k) {
    return (uint32_t)(k >> 3) * LBO + (uint32_t)(r >> 3) * SBO + (uint32_t)(r & 7) * 16 + (uint32_t)(k & 7) * 2;
}

template <int RULE>
__global__ void __launch_bounds__(TT, 2)
    k_tiletc(const InstDev* __restrict__ insts, const ChunkRef* __restrict__ work, int64_t nwork,
             float* __restrict__ scratch, int64_t slot_elems, int* __restrict__ tflag) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* const xs = sm + OFF_X;
    uint8_t* const ys = sm + OFF_Y;
    float* const sF = reinterpret_cast<float*>(sm + OFF_F);
    uint64_t* const bar = reinterpret_cast<uint64_t*>(sm + OFF_BAR);
    uint32_t* const tslot = reinterpret_cast<uint32_t*>(bar + 2);
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    // prefix ownership: column c of rows 4 ig .. 4 ig + 3 of every sample
    const int pc = tid % 32, pig = tid / 32;

    if (warp == 0) tmem_alloc(tslot, NCOL);
    if (tid == 0) {
        mbar_init(bar);
        mbar_init(bar + 1);
        mbar_init_fence();
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tbase = *tslot;
    uint32_t uses = 0;  // completed MMA batches (mbarrier phase)
    bool alive = true;
    float* const slot = scratch + (int64_t)blockIdx.x * slot_elems;

    for (int64_t w = blockIdx.x; w < nwork && alive; w += gridDim.x) {
        const ChunkRef wk = work[w];
        const InstDev& I = insts[wk.inst];
        const int c = wk.chunk, n = I.n;
        const int64_t b = (int64_t)c * I.K;
        const int64_t e = (b + I.K < I.S - 1) ? b + I.K : I.S - 1;
        const int Kp = (int)(e - b);
        const bool riem0 = (RULE == R_RIEMANN) && c == 0;
        const int first = riem0 ? 0 : 1;
        const int64_t nm = (int64_t)n * m;
        const RuleCoef<float> kc = rule_coef<float>(I);
        const float* Ag = static_cast<const float*>(I.A) + b * m;
        float* const st = slot;  // [n][3][m] prefix state

        // state at the chunk start: zero local prefixes, f0 = A[b] on level 1
        for (int j = 1; j <= n; ++j)
            for (int q = 0; q < m / TT; ++q) {
                const int el = tid + q * TT;
                st[(j - 1) * 3 * m + el] = 0.f;
                st[(j - 1) * 3 * m + m + el] = 0.f;
                st[(j - 1) * 3 * m + 2 * m + el] = (j == 1) ? __ldg(Ag + el) : 0.f;
            }
        __syncthreads();

        // A of a group, (row r of the stacked 128 x 32 operand, 8-wide k
        // chunk) items, NIT per thread, held in registers: the next group's
        // loads are issued once this group is staged and land while its
        // levels run
        constexpr int NIT = 128 * (D / 8) / TT;
        float av[NIT][8];
        auto load_group = [&](int l0g) {
            const int geg = min(G, Kp - l0g + 1);
#pragma unroll
            for (int ii = 0; ii < NIT; ++ii) {
                const int it = tid + ii * TT, r = it % 128, k8 = it / 128, s = r / D, i = r % D;
                float4 x0 = make_float4(0.f, 0.f, 0.f, 0.f), x1 = x0;
                if (s < geg) {
                    const float4* p = reinterpret_cast<const float4*>(Ag + (int64_t)(l0g + s) * m + i * D + k8 * 8);
                    x0 = __ldg(p);
                    x1 = __ldg(p + 1);
                }
                av[ii][0] = x0.x; av[ii][1] = x0.y; av[ii][2] = x0.z; av[ii][3] = x0.w;
                av[ii][4] = x1.x; av[ii][5] = x1.y; av[ii][6] = x1.z; av[ii][7] = x1.w;
            }
        };
        if (first <= Kp) load_group(first);
        for (int li0 = first; li0 <= Kp && alive; li0 += G) {
            const int ge = min(G, Kp - li0 + 1);
            // ---- group operands: A of the ge samples -> X pieces and W_1 (FP32)
#pragma unroll
            for (int ii = 0; ii < NIT; ++ii) {
                const int it = tid + ii * TT, r = it % 128, k8 = it / 128, s = r / D, i = r % D;
                const float* v = av[ii];
                float* f = sF + (s * D + i) * PF + k8 * 8;
                reinterpret_cast<float4*>(f)[0] = make_float4(v[0], v[1], v[2], v[3]);
                reinterpret_cast<float4*>(f)[1] = make_float4(v[4], v[5], v[6], v[7]);
                uint32_t wv[3][4];
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    uint16_t a0, a1, a2, b0, b1, b2;
                    split3(v[2 * h], a0, a1, a2);
                    split3(v[2 * h + 1], b0, b1, b2);
                    wv[0][h] = (uint32_t)a0 | ((uint32_t)b0 << 16);
                    wv[1][h] = (uint32_t)a1 | ((uint32_t)b1 << 16);
                    wv[2][h] = (uint32_t)a2 | ((uint32_t)b2 << 16);
                }
                const uint32_t o = off128(r, k8 * 8);
#pragma unroll
                for (int pcs = 0; pcs < 3; ++pcs)
                    *reinterpret_cast<uint4*>(xs + pcs * TILE + o) = make_uint4(wv[pcs][0], wv[pcs][1], wv[pcs][2], wv[pcs][3]);
            }
            if (li0 + G <= Kp) load_group(li0 + G);
            __syncthreads();

            // prefix state of a level (this thread's elements; it alone
            // reads and writes them), loaded one level ahead: level j + 1's
            // loads are in flight while level j's MMAs run
            FwdState<float> fs[4];
            auto load_state = [&](int j) {
                const float* sj = st + (j - 1) * 3 * m;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int el = (4 * pig + q) * D + pc;
                    fs[q].base = sj[el];
                    fs[q].blo = sj[m + el];
                    fs[q].f0 = sj[2 * m + el];
                    fs[q].f1 = fs[q].f2 = fs[q].f3 = 0.f;
                }
            };
            load_state(1);
            for (int j = 1; j <= n; ++j) {
                // ---- prefix pass of level j over the group's samples
                float* sj = st + (j - 1) * 3 * m;
                const Carry<float> zc{0.f, 0.f};
                float P[G][4];
#pragma unroll
                for (int l = 0; l < G; ++l)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        P[l][q] = 0.f;
                        if (l < ge) P[l][q] = fwd_step<float, RULE, false>(fs[q], sF[(l * D + 4 * pig + q) * PF + pc], 1 + l, kc, zc);
                    }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int el = (4 * pig + q) * D + pc;
                    sj[el] = fs[q].base;
                    sj[m + el] = fs[q].blo;
                    sj[2 * m + el] = fs[q].f0;
                }
                if (j == n) break;
                // ---- P_j as the Y operand: element (n = 32 l + c, k = 4 ig + q)
#pragma unroll
                for (int l = 0; l < G; ++l) {
                    uint16_t p0[4], p1[4], p2[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) split3(P[l][q], p0[q], p1[q], p2[q]);
                    const uint32_t o = off128(l * D + pc, 4 * pig);
                    *reinterpret_cast<uint2*>(ys + o) =
                        make_uint2((uint32_t)p0[0] | ((uint32_t)p0[1] << 16), (uint32_t)p0[2] | ((uint32_t)p0[3] << 16));
                    *reinterpret_cast<uint2*>(ys + TILE + o) =
                        make_uint2((uint32_t)p1[0] | ((uint32_t)p1[1] << 16), (uint32_t)p1[2] | ((uint32_t)p1[3] << 16));
                    *reinterpret_cast<uint2*>(ys + 2 * TILE + o) =
                        make_uint2((uint32_t)p2[0] | ((uint32_t)p2[1] << 16), (uint32_t)p2[2] | ((uint32_t)p2[3] << 16));
                }
                fence_async_smem();
                __syncthreads();
                // ---- W_{j+1} = A P_j (block-diagonal MMA batch)
                if (tid == 0) {
                    fence_after();
                    const uint32_t x0 = su32(xs), y0 = su32(ys), dmain = tbase, dsmall = tbase + 128;
                    constexpr int PI[5] = {2, 0, 1, 1, 0}, PJ[5] = {0, 2, 1, 0, 1};
#pragma unroll
                    for (int ks = 0; ks < D / 16; ++ks) {
                        const uint32_t o = (uint32_t)ks * 2 * LBO;
                        const uint32_t fresh = ks == 0 ? 0u : 1u;
#pragma unroll
                        for (int t = 0; t < 5; ++t)
                            mma_bf16(dsmall, smem_desc(x0 + PI[t] * TILE + o, LBO, SBO),
                                     smem_desc(y0 + PJ[t] * TILE + o, LBO, SBO), IDESC, t == 0 ? fresh : 1u);
                        mma_bf16(dmain, smem_desc(x0 + o, LBO, SBO), smem_desc(y0 + o, LBO, SBO), IDESC, fresh);
                    }
                    mma_commit(su32(bar));
                }
                load_state(j + 1);
                bool ok = mbar_wait(su32(bar), uses & 1);
                ++uses;
                ok = __all_sync(0xffffffffu, ok);
                fence_after();
                if (ok) {
                    // warp w: sample q = w & 3 (its rows are TMEM lanes 32 q ..), columns
                    // 32 q + 16 h .. + 15 of its diagonal block
                    const int q = warp & 3, h = warp >> 2;
                    float v[16], u[16];
                    const uint32_t ta = tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * q + 16 * h);
                    tmem_ld16(ta, v);
                    tmem_ld16(ta + 128, u);
                    float* f = sF + (q * D + lane) * PF + 16 * h;
#pragma unroll
                    for (int k4 = 0; k4 < 4; ++k4)
                        reinterpret_cast<float4*>(f)[k4] = make_float4(v[4 * k4] + u[4 * k4], v[4 * k4 + 1] + u[4 * k4 + 1],
                                                                       v[4 * k4 + 2] + u[4 * k4 + 2], v[4 * k4 + 3] + u[4 * k4 + 3]);
                }
                fence_before();
                if (__syncthreads_or(!ok)) {
                    alive = false;
                    break;
                }
            }
            __syncthreads();
        }
        if (alive) {
            for (int j = 1; j <= n; ++j)
                for (int q = 0; q < m / TT; ++q) {
                    const int el = tid + q * TT;
                    store_lam(I, (int64_t)c * nm + (int64_t)(j - 1) * m + el, st[(j - 1) * 3 * m + el],
                              st[(j - 1) * 3 * m + m + el]);
                }
        }
        __syncthreads();
    }

    if (!alive && tid == 0) {
        fence_after();
        mma_commit(su32(bar + 1));
        mbar_wait(su32(bar + 1), 0);
        atomicExch(tflag, 1);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_dealloc(tbase, NCOL);
}

template <int RULE>
cudaError_t launch_rule(const LaunchArgs& a, int grid, bool prepare_only) {
    static std::mutex mu;
    static std::vector<bool> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    {
        std::lock_guard<std::mutex> lock(mu);
        if ((int)done.size() <= dev) done.resize(dev + 1, false);
        if (!done[dev]) {
            e = cudaFuncSetAttribute(k_tiletc<RULE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
            if (e != cudaSuccess) return e;
            done[dev] = true;
        }
    }
    if (prepare_only) return cudaSuccess;
    int* flag = device_timeout_ptr();
    if (!flag) return cudaErrorInvalidValue;
    k_tiletc<RULE><<<grid, TT, SMEM, a.stream>>>(a.insts, a.work, a.nwork, static_cast<float*>(a.scratch), a.slot_elems,
                                                 flag);
    return cudaGetLastError();
}

}  // namespace

size_t tiletc_slot_elems(int n) { return (size_t)3 * n * m; }

cudaError_t launch_tiletc(int rule, const LaunchArgs& a, int grid, bool prepare_only) {
    switch (rule) {
        case R_BOOLE: return launch_rule<R_BOOLE>(a, grid, prepare_only);
        case R_SIMPSON: return launch_rule<R_SIMPSON>(a, grid, prepare_only);
        case R_TRAP: return launch_rule<R_TRAP>(a, grid, prepare_only);
        default: return launch_rule<R_RIEMANN>(a, grid, prepare_only);
    }
}

}  // namespace mgb
