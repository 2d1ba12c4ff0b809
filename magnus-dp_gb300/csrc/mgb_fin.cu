// The small FP64 algebra after the chunk scans (D^(q), E, Omega and the op
// output; their adjoint down to tau = dL/dT), spread over the GPU for matrix
// segments with d a multiple of 16.  The one-CTA-per-instance kernels of
// mgb_generic.cu (k_fin_fwd / k_fin_vjp) do the same sums; at d = 128 they
// held one SM each for tens of milliseconds per instance.  Here every
// d x d product sum is cut into T x T output tiles, one CTA per (instance,
// output matrix, tile) (mgb_tile64.cuh), with one launch per step of the
// recursions:
//   D^(q)_1 = 1,  D^(q)_k = s_q (T_{k-1} + sum_{j=1}^{k-2} T_j D^(q)_{k-j})   (k = 2..n, sequential)
//   E_m = sum_q w_q D^(q)_m,  Omega_1 = T_1,  Omega_k = sum_{j=1}^{k} T_j E_{k-j+1}
// and for the VJP, from Omega-bar:
//   Ebar_m = sum_{k>=m} T_{k-m+1}^T Obar_k (m >= 2),
//   tau_j = [j = 1] Obar_1 + sum_{k>=max(j,2)} Obar_k E_{k-j+1}^T,
//   per node q, k = n..2 (sequential): g = Dbar^(q)_k,
//     tau^(q)_j += s_q g D^(q)_{k-j}^T (j < k),  Dbar^(q)_{k-j} += s_q T_j^T g (k-j >= 2),
//   tau_j = sig^j (tau_j + sum_q tau^(q)_j).
// The per-node tau^(q) buffers keep concurrent CTAs from adding into the
// same output.
#include <cmath>
#include <vector>

#include "mgb_kernels.h"
#include "mgb_tile64.cuh"

namespace mgb {
namespace {

using namespace t64;

constexpr int ENT = 256;  // elementwise kernels

// totals T_j = sig^j pi[C]_j, D^(q)_1 = identity
__global__ void k_fin_tt(const InstDev* __restrict__ insts, int qmax) {
    const InstDev& I = insts[blockIdx.y];
    const int m = I.m, n = I.n, d = I.d;
    const int64_t nm = (int64_t)n * m;
    const double* Tk = I.pi + (int64_t)I.C * nm;
    for (int64_t idx = (int64_t)blockIdx.x * ENT + threadIdx.x; idx < nm; idx += (int64_t)gridDim.x * ENT) {
        const int j = 1 + (int)(idx / m);
        I.tt[idx] = Tk[idx] * pow(I.sig, (double)j);
    }
    for (int64_t idx = (int64_t)blockIdx.x * ENT + threadIdx.x; idx < (int64_t)I.Q * m; idx += (int64_t)gridDim.x * ENT) {
        const int q = (int)(idx / m), el = (int)(idx % m);
        I.dq[(int64_t)q * nm + el] = (el / d == el % d) ? 1.0 : 0.0;
    }
    (void)qmax;
}

// one step k of the D^(q) recursion: block -> (instance, q, tile)
template <int T>
__global__ void __launch_bounds__(SNT) k_fin_D(const InstDev* __restrict__ insts, int k, int qmax, int tpl) {
    constexpr int R = ScanTile<T>::R, P = ScanTile<T>::P;
    __shared__ double sX[T * P], sY[T * P];
    const int per = qmax * tpl;
    const InstDev& I = insts[blockIdx.x / per];
    const int rem = blockIdx.x % per, q = rem / tpl, tt = rem % tpl;
    if (q >= I.Q || k > I.n) return;
    const int d = I.d, m = I.m, tpr = d / T, r0 = (tt / tpr) * T, c0 = (tt % tpr) * T;
    const int64_t nm = (int64_t)I.n * m;
    double* Dq = I.dq + (int64_t)q * nm;
    double acc[R][R];
    tile_zero<T>(acc);
    for (int j = 1; j <= k - 2; ++j)
        tile_accumulate<T, false>(acc, I.tt + (int64_t)(j - 1) * m, Dq + (int64_t)(k - j - 1) * m, d, r0, c0, sX, sY);
    const double s = I.glx[q] - 1.0;
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) {
            const int64_t el = tile_el<T>(d, r0, c0, a, b);
            Dq[(int64_t)(k - 1) * m + el] = s * (I.tt[(int64_t)(k - 2) * m + el] + acc[a][b]);
        }
}

// E_m = sum_q w_q D^(q)_m
__global__ void k_fin_E(const InstDev* __restrict__ insts) {
    const InstDev& I = insts[blockIdx.y];
    const int64_t nm = (int64_t)I.n * I.m;
    for (int64_t idx = (int64_t)blockIdx.x * ENT + threadIdx.x; idx < nm; idx += (int64_t)gridDim.x * ENT) {
        double v = 0.0;
        for (int q = 0; q < I.Q; ++q) v += I.glw[q] * I.dq[(int64_t)q * nm + idx];
        I.ee[idx] = v;
    }
}

// Omega_k: block -> (instance, k, tile)
template <int T>
__global__ void __launch_bounds__(SNT) k_fin_omega(const InstDev* __restrict__ insts, int nmax, int tpl) {
    constexpr int R = ScanTile<T>::R, P = ScanTile<T>::P;
    __shared__ double sX[T * P], sY[T * P];
    const int per = nmax * tpl;
    const InstDev& I = insts[blockIdx.x / per];
    const int rem = blockIdx.x % per, k = 1 + rem / tpl, tt = rem % tpl;
    if (k > I.n) return;
    const int d = I.d, m = I.m, tpr = d / T, r0 = (tt / tpr) * T, c0 = (tt % tpr) * T;
    double acc[R][R];
    tile_zero<T>(acc);
    if (k > 1)
        for (int j = 1; j <= k; ++j)
            tile_accumulate<T, false>(acc, I.tt + (int64_t)(j - 1) * m, I.ee + (int64_t)(k - j) * m, d, r0, c0, sX, sY);
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) {
            const int64_t el = tile_el<T>(d, r0, c0, a, b);
            I.ob[(int64_t)(k - 1) * m + el] = k == 1 ? I.tt[el] : acc[a][b];
        }
}

// op output from Omega
__global__ void k_fin_out(const InstDev* __restrict__ insts, int f64io) {
    const InstDev& I = insts[blockIdx.y];
    const int m = I.m, n = I.n;
    const bool f64 = f64io != 0;
    const int64_t total = I.op == OP_MANY ? (int64_t)n * m : m;
    for (int64_t idx = (int64_t)blockIdx.x * ENT + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * ENT) {
        double v;
        if (I.op == OP_MANY) {
            v = I.ob[idx];
        } else if (I.op == OP_ONE) {
            v = I.ob[(int64_t)(n - 1) * m + idx];
        } else {
            v = 0.0;
            for (int k = 0; k < n; ++k) v += I.ob[(int64_t)k * m + idx];
        }
        store_out<double>(I.out, idx, v, f64);
    }
}

// Obar from the cotangent
__global__ void k_finv_obar(const InstDev* __restrict__ insts, int f64io) {
    const InstDev& I = insts[blockIdx.y];
    const int m = I.m, n = I.n;
    const bool f64 = f64io != 0;
    const int64_t nm = (int64_t)n * m;
    for (int64_t idx = (int64_t)blockIdx.x * ENT + threadIdx.x; idx < nm; idx += (int64_t)gridDim.x * ENT) {
        const int k = 1 + (int)(idx / m), el = (int)(idx % m);
        double v = 0.0;
        if (I.op == OP_MANY) v = load_in<double>(I.cot, (int64_t)(k - 1) * m + el, f64);
        else if (I.op == OP_SUM || k == n) v = load_in<double>(I.cot, el, f64);
        I.ob[idx] = v;
    }
}

// Ebar_m (which = 0) or tau_j from the Omega assembly (which = 1):
// block -> (instance, index, tile)
template <int T>
__global__ void __launch_bounds__(SNT) k_finv_bars(const InstDev* __restrict__ insts, int nmax, int tpl, int which) {
    constexpr int R = ScanTile<T>::R, P = ScanTile<T>::P;
    __shared__ double sX[T * P], sY[T * P];
    const int per = nmax * tpl;
    const InstDev& I = insts[blockIdx.x / per];
    const int rem = blockIdx.x % per, x = 1 + rem / tpl, tt = rem % tpl;
    const int n = I.n;
    if (x > n) return;
    const int d = I.d, m = I.m, tpr = d / T, r0 = (tt / tpr) * T, c0 = (tt % tpr) * T;
    double acc[R][R];
    tile_zero<T>(acc);
    if (which == 0) {
        if (x >= 2)  // Ebar_x = sum_{k>=x} T_{k-x+1}^T Obar_k
            for (int k = x; k <= n; ++k)
                tile_accumulate<T, true>(acc, I.tt + (int64_t)(k - x) * m, I.ob + (int64_t)(k - 1) * m, d, r0, c0, sX, sY);
    } else {  // tau_x = [x = 1] Obar_1 + sum_{k >= max(x, 2)} Obar_k E_{k-x+1}^T
        for (int k = (x > 2 ? x : 2); k <= n; ++k)
            tile_accumulate<T, false, true>(acc, I.ob + (int64_t)(k - 1) * m, I.ee + (int64_t)(k - x) * m, d, r0, c0,
                                            sX, sY);
    }
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) {
            const int64_t el = tile_el<T>(d, r0, c0, a, b);
            if (which == 0) I.eb[(int64_t)(x - 1) * m + el] = acc[a][b];
            else I.tau[(int64_t)(x - 1) * m + el] = acc[a][b] + (x == 1 ? I.ob[el] : 0.0);
        }
}

// Dbar^(q) = w_q Ebar, tau^(q) = 0
__global__ void k_finv_dbinit(const InstDev* __restrict__ insts) {
    const InstDev& I = insts[blockIdx.y];
    const int64_t nm = (int64_t)I.n * I.m;
    for (int64_t idx = (int64_t)blockIdx.x * ENT + threadIdx.x; idx < (int64_t)I.Q * nm;
         idx += (int64_t)gridDim.x * ENT) {
        const int q = (int)(idx / nm);
        I.dbq[idx] = I.glw[q] * I.eb[idx % nm];
        I.tauq[idx] = 0.0;
    }
}

// one step k of the D^(q) adjoint: block -> (instance, q, j in 1..k-1, tile)
template <int T>
__global__ void __launch_bounds__(SNT) k_finv_D(const InstDev* __restrict__ insts, int k, int qmax, int tpl) {
    constexpr int R = ScanTile<T>::R, P = ScanTile<T>::P;
    __shared__ double sX[T * P], sY[T * P];
    const int per = qmax * (k - 1) * tpl;
    const InstDev& I = insts[blockIdx.x / per];
    int rem = blockIdx.x % per;
    const int q = rem / ((k - 1) * tpl);
    rem %= (k - 1) * tpl;
    const int j = 1 + rem / tpl, tt = rem % tpl;
    if (q >= I.Q || k > I.n) return;
    const int d = I.d, m = I.m, tpr = d / T, r0 = (tt / tpr) * T, c0 = (tt % tpr) * T;
    const int64_t nm = (int64_t)I.n * m;
    const double s = I.glx[q] - 1.0;
    const double* g = I.dbq + (int64_t)q * nm + (int64_t)(k - 1) * m;
    const double* Dq = I.dq + (int64_t)q * nm;
    double acc[R][R];
    tile_zero<T>(acc);
    tile_accumulate<T, false, true>(acc, g, Dq + (int64_t)(k - j - 1) * m, d, r0, c0, sX, sY);  // g D_{k-j}^T
    double* tq = I.tauq + (int64_t)q * nm + (int64_t)(j - 1) * m;
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) tq[tile_el<T>(d, r0, c0, a, b)] += s * acc[a][b];
    if (k - j >= 2) {
        tile_zero<T>(acc);
        tile_accumulate<T, true>(acc, I.tt + (int64_t)(j - 1) * m, g, d, r0, c0, sX, sY);  // T_j^T g
        double* db = I.dbq + (int64_t)q * nm + (int64_t)(k - j - 1) * m;
#pragma unroll
        for (int a = 0; a < R; ++a)
#pragma unroll
            for (int b = 0; b < R; ++b) db[tile_el<T>(d, r0, c0, a, b)] += s * acc[a][b];
    }
}

// tau_j = sig^j (tau_j + sum_q tau^(q)_j)
__global__ void k_finv_final(const InstDev* __restrict__ insts) {
    const InstDev& I = insts[blockIdx.y];
    const int m = I.m;
    const int64_t nm = (int64_t)I.n * m;
    for (int64_t idx = (int64_t)blockIdx.x * ENT + threadIdx.x; idx < nm; idx += (int64_t)gridDim.x * ENT) {
        double v = I.tau[idx];
        for (int q = 0; q < I.Q; ++q) v += I.tauq[(int64_t)q * nm + idx];
        const int j = 1 + (int)(idx / m);
        I.tau[idx] = v * pow(I.sig, (double)j);
    }
}

// vjp = false: tt, D^(q), E, Omega (and the output if write_out);
// vjp = true: tau from the cotangent (needs the forward part's buffers).
template <int T>
cudaError_t fin_steps(const InstDev* insts, int count, int d, int nmax, bool vjp, int write_out, int f64io,
                      cudaStream_t st) {
    const int tpl = (d / T) * (d / T), qmax = nmax > 1 ? (nmax + 3) / 2 : 1;
    const dim3 eg(16, (unsigned)count);  // elementwise: 16 CTAs per instance
    if (!vjp) {
        k_fin_tt<<<eg, ENT, 0, st>>>(insts, qmax);
        for (int k = 2; k <= nmax; ++k)
            k_fin_D<T><<<(unsigned)(count * qmax * tpl), SNT, 0, st>>>(insts, k, qmax, tpl);
        k_fin_E<<<eg, ENT, 0, st>>>(insts);
        k_fin_omega<T><<<(unsigned)(count * nmax * tpl), SNT, 0, st>>>(insts, nmax, tpl);
        if (write_out) k_fin_out<<<eg, ENT, 0, st>>>(insts, f64io);
        return cudaGetLastError();
    }
    k_finv_obar<<<eg, ENT, 0, st>>>(insts, f64io);
    k_finv_bars<T><<<(unsigned)(count * nmax * tpl), SNT, 0, st>>>(insts, nmax, tpl, 0);
    k_finv_bars<T><<<(unsigned)(count * nmax * tpl), SNT, 0, st>>>(insts, nmax, tpl, 1);
    k_finv_dbinit<<<eg, ENT, 0, st>>>(insts);
    for (int k = nmax; k >= 2; --k)
        k_finv_D<T><<<(unsigned)(count * qmax * (k - 1) * tpl), SNT, 0, st>>>(insts, k, qmax, tpl);
    k_finv_final<<<eg, ENT, 0, st>>>(insts);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fin_tiled(const InstDev* insts, int count, int d, int nmax, bool vjp, int write_out, int f64io,
                             cudaStream_t st) {
    for (int i0 = 0; i0 < count; i0 += 65535) {  // instances ride gridDim.y in the elementwise kernels
        const int c = count - i0 < 65535 ? count - i0 : 65535;
        const cudaError_t e = (d % 32 == 0 && d >= 64) ? fin_steps<32>(insts + i0, c, d, nmax, vjp, write_out, f64io, st)
                                                       : fin_steps<16>(insts + i0, c, d, nmax, vjp, write_out, f64io, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace mgb
