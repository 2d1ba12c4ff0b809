// Chunk kernel for the mixed form (FP32 products, FP64 carries) at d = 64
// and d = 128.  Same level-major structure as the generic kernel (a prefix
// pass, one thread per element over the chunk's samples, alternating with a
// product pass; chunk buffers in a per-CTA global slot), but every product
// pass stages one sample's operands in shared memory and computes a TRxTR
// register tile per thread (TR = d/16: 4x4 at d=64, 8x8 at d=128; 256
// threads cover the d x d output).  At these sizes a sample's product
// (2 d^3 flop) dwarfs its operand traffic (a few d^2 words), so streaming the
// chunk buffers through L2/HBM costs little.
#include <cstdint>
#include <mutex>
#include <vector>

#include "mgb_common.cuh"
#include "mgb_tuned.h"

namespace mgb {
namespace {

constexpr int BNT = 256;

template <int D>
struct BigCfg {
    static constexpr int m = D * D;
    static constexpr int TR = D / 16;   // tile edge per thread
    static constexpr int PD = D + 4;    // 16-byte aligned pitch
    static constexpr int SMEM = 2 * D * PD;  // floats: two staged operands
    static_assert(TR % 4 == 0, "float4 tiles");
};

// Stage a d x d row-major source (global) into shared memory, either as is
// (dst[r][c]) or transposed (dst[c][r]), pitch PD.
template <int D, bool TRANSPOSE>
__device__ __forceinline__ void stage(float* __restrict__ dst, const float* __restrict__ src) {
    constexpr int PD = D + 4, NV = D * D / 4 / BNT;
    float4 v[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = reinterpret_cast<const float4*>(src)[threadIdx.x + q * BNT];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const int e = (threadIdx.x + q * BNT) * 4, r = e / D, c = e % D;
        if (TRANSPOSE) {
            dst[(c + 0) * PD + r] = v[q].x;
            dst[(c + 1) * PD + r] = v[q].y;
            dst[(c + 2) * PD + r] = v[q].z;
            dst[(c + 3) * PD + r] = v[q].w;
        } else {
            *reinterpret_cast<float4*>(dst + r * PD + c) = v[q];
        }
    }
}

// acc[t][u] = sum_k XT[k][r0+t] * Y[k][c0+u]   (X given transposed)
template <int D>
__device__ __forceinline__ void tile_mm(float (&acc)[BigCfg<D>::TR][BigCfg<D>::TR], const float* __restrict__ XT,
                                       const float* __restrict__ Y, int r0, int c0) {
    constexpr int TR = BigCfg<D>::TR, PD = BigCfg<D>::PD;
#pragma unroll
    for (int t = 0; t < TR; ++t)
#pragma unroll
        for (int u = 0; u < TR; ++u) acc[t][u] = 0.f;
#pragma unroll 4
    for (int k = 0; k < D; ++k) {
        float av[TR], bv[TR];
#pragma unroll
        for (int q = 0; q < TR / 4; ++q) {
            const float4 a = *reinterpret_cast<const float4*>(XT + k * PD + r0 + 4 * q);
            const float4 b = *reinterpret_cast<const float4*>(Y + k * PD + c0 + 4 * q);
            av[4 * q] = a.x; av[4 * q + 1] = a.y; av[4 * q + 2] = a.z; av[4 * q + 3] = a.w;
            bv[4 * q] = b.x; bv[4 * q + 1] = b.y; bv[4 * q + 2] = b.z; bv[4 * q + 3] = b.w;
        }
#pragma unroll
        for (int t = 0; t < TR; ++t)
#pragma unroll
            for (int u = 0; u < TR; ++u) acc[t][u] = fmaf(av[t], bv[u], acc[t][u]);
    }
}

template <int D, bool ACCUMULATE>
__device__ __forceinline__ void tile_store(float* __restrict__ dst, const float (&acc)[BigCfg<D>::TR][BigCfg<D>::TR],
                                           int r0, int c0) {
    constexpr int TR = BigCfg<D>::TR;
#pragma unroll
    for (int t = 0; t < TR; ++t)
#pragma unroll
        for (int q = 0; q < TR / 4; ++q) {
            float4* p = reinterpret_cast<float4*>(dst + (r0 + t) * D + c0 + 4 * q);
            float4 v = make_float4(acc[t][4 * q], acc[t][4 * q + 1], acc[t][4 * q + 2], acc[t][4 * q + 3]);
            if (ACCUMULATE) {
                const float4 o = *p;
                v.x += o.x; v.y += o.y; v.z += o.z; v.w += o.w;
            }
            *p = v;
        }
}

template <int D, int RULE, int MODE>
__global__ void __launch_bounds__(BNT, 1) k_big(const InstDev* __restrict__ insts, const ChunkRef* __restrict__ work,
                                                int64_t nwork, float* __restrict__ scratch, int64_t slot_elems) {
    using Cf = BigCfg<D>;
    constexpr int m = Cf::m, TR = Cf::TR, PD = Cf::PD;
    extern __shared__ __align__(16) float sb[];
    float* const sX = sb;           // staged left operand (transposed form)
    float* const sY = sb + D * PD;  // staged right operand
    float* const slot = scratch + (int64_t)blockIdx.x * slot_elems;
    const int tid = threadIdx.x;
    const int r0 = (tid / (D / TR)) * TR, c0 = (tid % (D / TR)) * TR;

    for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        const ChunkRef wk = work[w];
        const InstDev& I = insts[wk.inst];
        const int c = wk.chunk, n = I.n;
        const int64_t b = (int64_t)c * I.K;
        const int64_t e = (b + I.K < I.S - 1) ? b + I.K : I.S - 1;
        const int Kp = (int)(e - b), L = Kp + 1;
        const bool riem0 = (RULE == R_RIEMANN) && c == 0;
        const int first = riem0 ? 0 : 1;
        const int64_t Lm = (int64_t)L * m, nm = (int64_t)n * m;
        const RuleCoef<float> kc(I.dt_k);
        const float* Ag = static_cast<const float*>(I.A) + b * m;  // the chunk's samples, read in place
        float* const tape = slot;                 // [n-1][L][m] P_j
        float* const Wb = tape + (n - 1) * Lm;    // [L][m] level values
        float* const Gb = Wb + Lm;                // [L][m] cotangents on W_j
        float* const Hb = Gb + Lm;                // [L][m] cotangents on P_j
        float* const dAb = Hb + Lm;               // [L][m] dA accumulator
        const double* pic = I.pi + (int64_t)c * nm;
        const int NL = (MODE == MODE_LOCAL) ? n : n - 1;

        // ---------------- forward over the chunk ----------------
        const float* F = Ag;
        for (int j = 1; j <= NL; ++j) {
            float* Pj = tape + (int64_t)((j < n ? j : 1) - 1) * Lm;
            const bool keep = j < n;
            for (int el = tid; el < m; el += BNT) {
                const double pij = (MODE == MODE_LOCAL || riem0) ? 0.0 : pic[(int64_t)(j - 1) * m + el];
                const Carry<float> cy = split_carry<float>(pij);
                FwdState<float> s;
                s.base = s.blo = 0.f;
                s.f0 = F[el];
                s.f1 = s.f2 = s.f3 = 0.f;
                if (!riem0 && keep) Pj[el] = add_carry(0.f, cy);
                for (int li = first; li <= Kp; ++li) {
                    const float P = fwd_step<float, RULE>(s, F[(int64_t)li * m + el], li, kc, cy);
                    if (keep) Pj[(int64_t)li * m + el] = P;
                }
                if (MODE == MODE_LOCAL)
                    I.lam[(int64_t)c * nm + (int64_t)(j - 1) * m + el] = (double)s.base + (double)s.blo;
            }
            __syncthreads();
            if (j < NL) {
                // W_{j+1}[li] = A[li] P_j[li] for every sample of the chunk
                for (int li = 0; li <= Kp; ++li) {
                    stage<D, true>(sX, Ag + (int64_t)li * m);
                    stage<D, false>(sY, Pj + (int64_t)li * m);
                    __syncthreads();
                    float acc[TR][TR];
                    tile_mm<D>(acc, sX, sY, r0, c0);
                    tile_store<D, false>(Wb + (int64_t)li * m, acc, r0, c0);
                    __syncthreads();
                }
                F = Wb;
            }
        }

        if (MODE == MODE_VJP) {
            const double* rc = I.rho + (int64_t)c * nm;
            for (int64_t idx = tid; idx < Lm; idx += BNT) dAb[idx] = 0.f;
            for (int j = n; j >= 1; --j) {
                if (j < n) {
                    const float* Pj = tape + (int64_t)(j - 1) * Lm;
                    for (int li = 0; li <= Kp; ++li) {
                        // H_j = A^T G_{j+1}  (X = A^T, so stage A as is)
                        if (li >= first) {
                            stage<D, false>(sX, Ag + (int64_t)li * m);
                            stage<D, false>(sY, Gb + (int64_t)li * m);
                            __syncthreads();
                            float acc[TR][TR];
                            tile_mm<D>(acc, sX, sY, r0, c0);
                            tile_store<D, false>(Hb + (int64_t)li * m, acc, r0, c0);
                            __syncthreads();
                        }
                        // dA += G_{j+1} P_j^T  (X = G: stage G^T; Y = P^T: stage P^T)
                        stage<D, true>(sX, Gb + (int64_t)li * m);
                        stage<D, true>(sY, Pj + (int64_t)li * m);
                        __syncthreads();
                        float acc[TR][TR];
                        tile_mm<D>(acc, sX, sY, r0, c0);
                        tile_store<D, true>(dAb + (int64_t)li * m, acc, r0, c0);
                        __syncthreads();
                    }
                }
                for (int el = tid; el < m; el += BNT) {
                    const Carry<float> cy = split_carry<float>(rc[(int64_t)(j - 1) * m + el]);
                    RevState<float> s;
                    s.Rb = s.rlo = s.pend = s.R4l = s.R4 = s.H2 = s.H3 = 0.f;
                    for (int li = Kp; li >= first; --li) {
                        const float H = (j < n) ? Hb[(int64_t)li * m + el] : 0.f;
                        Gb[(int64_t)li * m + el] = rev_step<float, RULE>(s, H, li, kc, cy);
                    }
                    if (!riem0) Gb[el] = s.pend;
                }
                __syncthreads();
            }
            float* dAg = static_cast<float*>(I.dA) + b * m;
            for (int64_t idx = tid; idx < Lm; idx += BNT) {
                const int li = (int)(idx / m);
                if (RULE == R_RIEMANN && li == 0 && c > 0) continue;  // f_b unused by Riemann
                const float v = dAb[idx] + Gb[idx];
                const bool shared = (li == 0 && c > 0) || (li == Kp && c < I.C - 1);
                if (shared) atomicAdd(dAg + idx, v);
                else dAg[idx] = v;
            }
        }
        __syncthreads();
    }
}

template <int D, int RULE, int MODE>
cudaError_t set_big_attr() {
    static std::mutex mu;
    static std::vector<bool> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, false);
    if (done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(k_big<D, RULE, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(BigCfg<D>::SMEM * sizeof(float)));
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

template <int D, int RULE, int MODE>
cudaError_t launch_big_t(const LaunchArgs& a, int grid, bool prepare_only) {
    cudaError_t e = set_big_attr<D, RULE, MODE>();
    if (e != cudaSuccess || prepare_only) return e;
    k_big<D, RULE, MODE><<<grid, BNT, BigCfg<D>::SMEM * sizeof(float), a.stream>>>(
        a.insts, a.work, a.nwork, static_cast<float*>(a.scratch), a.slot_elems);
    return cudaGetLastError();
}

template <int D, int MODE>
cudaError_t launch_big_r(int rule, const LaunchArgs& a, int grid, bool prepare_only) {
    switch (rule) {
        case R_BOOLE: return launch_big_t<D, R_BOOLE, MODE>(a, grid, prepare_only);
        case R_SIMPSON: return launch_big_t<D, R_SIMPSON, MODE>(a, grid, prepare_only);
        case R_TRAP: return launch_big_t<D, R_TRAP, MODE>(a, grid, prepare_only);
        default: return launch_big_t<D, R_RIEMANN, MODE>(a, grid, prepare_only);
    }
}

}  // namespace

cudaError_t launch_big(int D, int rule, int mode, const LaunchArgs& a, int sms, bool prepare_only) {
    int grid = (int)std::min<int64_t>(a.grid, (int64_t)sms);
    if (grid < 1) grid = 1;
    if (D == 128)
        return mode == MODE_LOCAL ? launch_big_r<128, MODE_LOCAL>(rule, a, grid, prepare_only)
                                  : launch_big_r<128, MODE_VJP>(rule, a, grid, prepare_only);
    return mode == MODE_LOCAL ? launch_big_r<64, MODE_LOCAL>(rule, a, grid, prepare_only)
                              : launch_big_r<64, MODE_VJP>(rule, a, grid, prepare_only);
}

}  // namespace mgb
