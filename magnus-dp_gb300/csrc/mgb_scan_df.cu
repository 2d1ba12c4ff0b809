// Chunk scans of the mixed form at d = 16 and d = 32 in one launch, with the
// carries in double-FP32 arithmetic on the FP32 pipes.
//
//     pi^{c+1}_j = pi^c_j + Lambda^c_j + sum_{m<j} Lambda^c_{j-m} pi^c_m
//     rho^{c-1}_m = rho^c_m + sum_{j>m} (Lambda^c_{j-m})^T rho^c_j
//
// (Chen's identity and its adjoint.)  The FP64 form of these scans (one
// launch per chunk step, mgb_scan.cu) runs on GB300's 1/64-rate FP64 pipe:
// 38 ms per direction for 512 config4 instances.  Here one CTA owns one
// instance and walks all of its chunk steps; the state (pi or rho, n levels)
// and the step's transfers Lambda^c live in shared memory as unevaluated
// sums hi + lo of two floats (about 48 significant bits), and every
// product term is an error-free FP32 product plus the two cross terms:
//     a b = ah bh + (fma(ah, bh, -ah bh) + ah bl + al bh)
// accumulated with TwoSum into a (sum, correction) pair.  The carries stay
// far more accurate than the 1e-6 the mixed form promises (an FP32 scan cost
// ~1e-6 on high orders); the plain form keeps the FP64 scans.  Inputs and
// outputs remain the FP64 arrays pi, lam, rho of the instance descriptor.
// The level recursion runs in place: the forward scan updates levels n..1
// (level j reads only lower levels), the reverse one levels 1..n.
#include <cstdint>
#include <mutex>
#include <vector>

#include "mgb_kernels.h"

namespace mgb {
namespace {

constexpr int SNTD = 256;

__device__ __forceinline__ void df_split(double x, float& hi, float& lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}

// running sum of exact products: s (+ c)
struct DfAcc {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float ah, float al, float bh, float bl) {
        const float p = ah * bh;
        float e = fmaf(ah, bh, -p);
        e = fmaf(ah, bl, e);
        e = fmaf(al, bh, e);
        const float t = s + p;
        const float bb = t - s;
        const float err = (s - (t - bb)) + (p - bb);
        s = t;
        c += err + e;
    }
};

// x (hi, lo) += y (hi, lo) + acc, renormalised
__device__ __forceinline__ void df_update(float& xh, float& xl, float yh, float yl, const DfAcc& a) {
    float s = xh + yh;
    float bb = s - xh;
    float e = (xh - (s - bb)) + (yh - bb);
    e += xl + yl + a.c;
    const float s2 = s + a.s;
    bb = s2 - s;
    e += (s - (s2 - bb)) + (a.s - bb);
    xh = s2 + e;
    xl = e - (xh - s2);
}

// Per-thread RT x RT output tile of a D x D level: rows RT*(t/TPR).., cols RT*(t%TPR)..
template <int D>
struct DfTile {
    static constexpr int TPR = 16;      // threads per row of tiles
    static constexpr int RT = D / TPR;  // rows (and columns) per thread
    static_assert(RT >= 1 && TPR * TPR == SNTD, "tile mapping");
};

template <int D, bool REV>
__global__ void __launch_bounds__(SNTD) k_scan_df(const InstDev* __restrict__ insts, int f64io) {
    constexpr int m = D * D, RT = DfTile<D>::RT, TPR = DfTile<D>::TPR;
    extern __shared__ float shm[];
    const InstDev& I = insts[blockIdx.x];
    const int n = I.n, C = I.C;
    const int nm = n * m;
    float* const xh = shm;      // state (pi or rho), [n][D][D]
    float* const xl = xh + nm;
    float* const lh = xl + nm;  // Lambda^c
    float* const ll = lh + nm;
    const int tid = threadIdx.x, r0 = RT * (tid / TPR), c0 = RT * (tid % TPR);

    if (!REV) {
        for (int i = tid; i < nm; i += SNTD) {
            xh[i] = 0.f;
            xl[i] = 0.f;
            I.pi[i] = 0.0;  // pi^0
        }
    } else {
        // rho^{C-1} = tau; zero the dA rows shared by two chunks (the chunk
        // VJP kernels accumulate them with atomics)
        double* last = I.rho + (int64_t)(C - 1) * nm;
        for (int i = tid; i < nm; i += SNTD) {
            const double v = I.tau[i];
            last[i] = v;
            df_split(v, xh[i], xl[i]);
        }
        const bool f64 = f64io != 0;
        for (int64_t idx = tid; idx < (int64_t)(C - 1) * m; idx += SNTD) {
            const int c = 1 + (int)(idx / m), el = (int)(idx % m);
            store_out<double>(I.dA, (int64_t)c * I.K * m + el, 0.0, f64);
        }
    }
    __syncthreads();

    for (int step = 0; step < (REV ? C - 1 : C); ++step) {
        const int c = REV ? C - 1 - step : step;  // transfer Lambda^c
        if (I.lam_pair) {
            // the chunk kernel's FP32 pairs as they are (no FP64 work)
            const float2* lc = reinterpret_cast<const float2*>(I.lam) + (int64_t)c * nm;
            for (int i = tid; i < nm; i += SNTD) {
                const float2 v = lc[i];
                lh[i] = v.x;
                ll[i] = v.y;
            }
        } else {
            const double* lc = I.lam + (int64_t)c * nm;
            for (int i = tid; i < nm; i += SNTD) df_split(lc[i], lh[i], ll[i]);
        }
        __syncthreads();
        for (int it = 0; it < n; ++it) {
            const int j = REV ? 1 + it : n - it;  // level updated in place
            DfAcc acc[RT][RT];
            if (!REV) {
                // sum_{mm<j} Lambda_{j-mm} pi_mm
                for (int mm = 1; mm < j; ++mm) {
                    const float* ah = lh + (j - mm - 1) * m;
                    const float* al = ll + (j - mm - 1) * m;
                    const float* bh = xh + (mm - 1) * m;
                    const float* bl = xl + (mm - 1) * m;
#pragma unroll 4
                    for (int k = 0; k < D; ++k) {
                        float av[RT], alv[RT], bv[RT], blv[RT];
#pragma unroll
                        for (int a = 0; a < RT; ++a) {
                            av[a] = ah[(r0 + a) * D + k];
                            alv[a] = al[(r0 + a) * D + k];
                            bv[a] = bh[k * D + c0 + a];
                            blv[a] = bl[k * D + c0 + a];
                        }
#pragma unroll
                        for (int a = 0; a < RT; ++a)
#pragma unroll
                            for (int bq = 0; bq < RT; ++bq) acc[a][bq].add(av[a], alv[a], bv[bq], blv[bq]);
                    }
                }
            } else {
                // sum_{jj>j} (Lambda_{jj-j})^T rho_jj
                for (int jj = j + 1; jj <= n; ++jj) {
                    const float* ah = lh + (jj - j - 1) * m;
                    const float* al = ll + (jj - j - 1) * m;
                    const float* bh = xh + (jj - 1) * m;
                    const float* bl = xl + (jj - 1) * m;
#pragma unroll 4
                    for (int k = 0; k < D; ++k) {
                        float av[RT], alv[RT], bv[RT], blv[RT];
#pragma unroll
                        for (int a = 0; a < RT; ++a) {
                            av[a] = ah[k * D + r0 + a];
                            alv[a] = al[k * D + r0 + a];
                            bv[a] = bh[k * D + c0 + a];
                            blv[a] = bl[k * D + c0 + a];
                        }
#pragma unroll
                        for (int a = 0; a < RT; ++a)
#pragma unroll
                            for (int bq = 0; bq < RT; ++bq) acc[a][bq].add(av[a], alv[a], bv[bq], blv[bq]);
                    }
                }
            }
            // a level's update touches only that level, which no thread reads
            // in this pass; the barrier orders it before the next level's reads
            const int base = (j - 1) * m;
#pragma unroll
            for (int a = 0; a < RT; ++a)
#pragma unroll
                for (int bq = 0; bq < RT; ++bq) {
                    const int i = base + (r0 + a) * D + c0 + bq;
                    float h = xh[i], l = xl[i];
                    if (!REV) df_update(h, l, lh[i], ll[i], acc[a][bq]);
                    else df_update(h, l, 0.f, 0.f, acc[a][bq]);
                    xh[i] = h;
                    xl[i] = l;
                }
            __syncthreads();
        }
        // the new state to the FP64 arrays: pi^{c+1} / rho^{c-1}
        double* out = REV ? I.rho + (int64_t)(c - 1) * nm : I.pi + (int64_t)(c + 1) * nm;
        for (int i = tid; i < nm; i += SNTD) out[i] = (double)xh[i] + (double)xl[i];
        __syncthreads();
    }
}

// The shared-memory opt-in (the largest request, 200 KB) is made once per
// kernel and device, ahead of any stream capture (launch_scan_df with
// prepare_only, from the plan's set-up).
template <int D, bool REV>
cudaError_t scan_df_attr() {
    static std::mutex mu;
    static std::vector<bool> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, false);
    if (done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(k_scan_df<D, REV>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

template <int D, bool REV>
cudaError_t scan_df_go(const InstDev* insts, int count, size_t smem, int f64io, cudaStream_t st, bool prepare_only) {
    cudaError_t e = scan_df_attr<D, REV>();
    if (e != cudaSuccess || prepare_only) return e;
    k_scan_df<D, REV><<<(unsigned)count, SNTD, smem, st>>>(insts, f64io);
    return cudaGetLastError();
}

}  // namespace

size_t scan_df_smem(int d, int nmax) { return (size_t)4 * nmax * d * d * sizeof(float); }

bool scan_df_ok(int kind, int d, int nmax) {
    return kind == KIND_MATRIX && (d == 16 || d == 32) && scan_df_smem(d, nmax) <= 200 * 1024;
}

cudaError_t launch_scan_df(const InstDev* insts, int count, int d, int nmax, bool reverse, int f64io, cudaStream_t st,
                           bool prepare_only) {
    if (count <= 0 && !prepare_only) return cudaSuccess;
    const size_t smem = scan_df_smem(d, nmax);
    if (d == 16) return reverse ? scan_df_go<16, true>(insts, count, smem, f64io, st, prepare_only)
                                : scan_df_go<16, false>(insts, count, smem, f64io, st, prepare_only);
    return reverse ? scan_df_go<32, true>(insts, count, smem, f64io, st, prepare_only)
                   : scan_df_go<32, false>(insts, count, smem, f64io, st, prepare_only);
}

}  // namespace mgb
