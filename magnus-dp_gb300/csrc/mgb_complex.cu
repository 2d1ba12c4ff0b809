// Complex matrix problems through the real engine.  A complex d x d matrix
// Z = X + iY is carried as the real 2d x 2d matrix
//     R(Z) = [[X, -Y], [Y, X]],
// an algebra homomorphism (R(Z1 Z2) = R(Z1) R(Z2), R(a Z) = a R(Z) for real
// a), and the Magnus recursion uses only products, sums and real scalars, so
// the real problem of dimension 2d on R(A) has R(Omega) as its output (and
// R(P_k) in its carry record).  The reference's complex VJP is the bilinear
// one (sum dA * dZ = sum cot * dOut, tests/test_python_api.py:135); on the
// real problem it is obtained from the cotangent
//     R_c = [[Re C, Im C], [-Im C, Re C]] / 2        (= R(conj C) / 2)
// as  dA = (dR11 + dR22) + i (dR12 - dR21)  from the real gradient's blocks.
#include <cstdint>

#include "mgb_kernels.h"

namespace mgb {
namespace {

// count complex d x d matrices (interleaved re, im) -> real 2d x 2d blocks.
// cot: the cotangent form R(conj C) / 2 instead of R(Z).
template <class R>
__global__ void k_cplx_embed(const R* __restrict__ Z, R* __restrict__ out, int64_t count, int d, int cot) {
    const int64_t m = (int64_t)d * d, total = count * m;
    const int64_t d2 = 2 * (int64_t)d;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = idx / m;
        const int e = (int)(idx - t * m), i = e / d, j = e - i * d;
        R x = Z[2 * idx], y = Z[2 * idx + 1];
        R* o = out + t * d2 * d2;
        if (cot) {
            x *= R(0.5);
            y *= R(0.5);
            o[i * d2 + j] = x;
            o[i * d2 + j + d] = y;
            o[(i + d) * d2 + j] = -y;
            o[(i + d) * d2 + j + d] = x;
        } else {
            o[i * d2 + j] = x;
            o[i * d2 + j + d] = -y;
            o[(i + d) * d2 + j] = y;
            o[(i + d) * d2 + j + d] = x;
        }
    }
}

// real 2d x 2d blocks -> count complex d x d matrices.  grad = 0: values
// (X = top-left, Y = bottom-left); grad = 1: the bilinear gradient
// (dR11 + dR22) + i (dR12 - dR21).
template <class R>
__global__ void k_cplx_extract(const R* __restrict__ in, R* __restrict__ Z, int64_t count, int d, int grad) {
    const int64_t m = (int64_t)d * d, total = count * m;
    const int64_t d2 = 2 * (int64_t)d;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = idx / m;
        const int e = (int)(idx - t * m), i = e / d, j = e - i * d;
        const R* b = in + t * d2 * d2;
        if (grad) {
            Z[2 * idx] = b[i * d2 + j] + b[(i + d) * d2 + j + d];
            Z[2 * idx + 1] = b[i * d2 + j + d] - b[(i + d) * d2 + j];
        } else {
            Z[2 * idx] = b[i * d2 + j];
            Z[2 * idx + 1] = b[(i + d) * d2 + j];
        }
    }
}

// ---- complex SpaceCurve data
// The engine's SpaceCurve recursion is the associative quaternion product
// qmul(a, b) = b (x) a on a = (0, f), with the sign (-1)^(k-1) on order k
// (and (-1)^k on carry records).  Over complex f it runs as the matrix
// recursion on rho(a) = the right-multiplication map y -> y (x) a (rho is
// an algebra homomorphism for qmul), i.e. the real 8 x 8 problem on the
// embedding of the complex 4 x 4 rho(a); an element is the first column of
// its rho.  e_s (x) e_c = SGN[s][c] e_IDX[s][c] in the basis 1, i, j, k.
__device__ __constant__ int kIdx[4][4] = {{0, 1, 2, 3}, {1, 0, 3, 2}, {2, 3, 0, 1}, {3, 2, 1, 0}};
__device__ __constant__ int kSgn[4][4] = {{1, 1, 1, 1}, {1, -1, 1, -1}, {1, -1, -1, 1}, {1, 1, -1, -1}};

// one complex 4 x 4 matrix (re, im in registers) -> real 8 x 8 (cot form if cot)
template <class R>
__device__ __forceinline__ void put8(R* o, const R (&re)[4][4], const R (&im)[4][4], bool cot) {
    const R h = cot ? R(0.5) : R(1);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            const R x = re[r][c] * h, y = im[r][c] * h;
            o[r * 8 + c] = x;
            o[(r + 4) * 8 + c + 4] = x;
            o[r * 8 + c + 4] = cot ? y : -y;
            o[(r + 4) * 8 + c] = cot ? -y : y;
        }
}

template <class R>
__global__ void k_sc_embed(const R* __restrict__ F, R* __restrict__ out, int64_t S) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < S; i += (int64_t)gridDim.x * blockDim.x) {
        R are[4] = {R(0), F[6 * i], F[6 * i + 2], F[6 * i + 4]};
        R aim[4] = {R(0), F[6 * i + 1], F[6 * i + 3], F[6 * i + 5]};
        R re[4][4] = {}, im[4][4] = {};
        for (int s = 0; s < 4; ++s)
            for (int c = 0; c < 4; ++c) {
                re[kIdx[s][c]][s] += (R)kSgn[s][c] * are[c];
                im[kIdx[s][c]][s] += (R)kSgn[s][c] * aim[c];
            }
        put8(out + i * 64, re, im, false);
    }
}

// cotangent on the outputs (op one/many/sum over n orders) -> per-order 8 x 8
// cotangents of the op=many real problem
template <class R>
__global__ void k_sc_cot(const R* __restrict__ C, R* __restrict__ out, int n, int op) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;  // order k+1
    if (k >= n) return;
    R re[4][4] = {}, im[4][4] = {};
    const bool on = op == OP_MANY || op == OP_SUM || k == n - 1;
    const R sg = (k & 1) ? R(-1) : R(1);
    const R* c = C + (op == OP_MANY ? 6 * k : 0);
    if (on)
        for (int q = 0; q < 3; ++q) {
            re[q + 1][0] = sg * c[2 * q];
            im[q + 1][0] = sg * c[2 * q + 1];
        }
    put8(out + (int64_t)k * 64, re, im, true);
}

// per-order 8 x 8 results -> op(Omega) (n x 3 or 3 complex)
template <class R>
__global__ void k_sc_out(const R* __restrict__ in, R* __restrict__ Z, int n, int op) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;  // component q = t % 3 of output row t / 3
    const int rows = op == OP_MANY ? n : 1;
    if (t >= rows * 3) return;
    const int row = t / 3, q = t % 3;
    R xr = 0, xi = 0;
    for (int k = 0; k < n; ++k) {
        if (op == OP_MANY && k != row) continue;
        if (op == OP_ONE && k != n - 1) continue;
        const R sg = (k & 1) ? R(-1) : R(1);
        const R* b = in + (int64_t)k * 64;
        xr += sg * b[(q + 1) * 8];
        xi += sg * b[(q + 5) * 8];
    }
    Z[2 * t] = xr;
    Z[2 * t + 1] = xi;
}

// real gradients on rho(a_i) -> the bilinear gradient on f_i
template <class R>
__global__ void k_sc_grad(const R* __restrict__ dR, R* __restrict__ dF, int64_t S) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < S; i += (int64_t)gridDim.x * blockDim.x) {
        const R* b = dR + i * 64;
        for (int c = 1; c < 4; ++c) {
            R gr = 0, gi = 0;
            for (int s = 0; s < 4; ++s) {
                const int r = kIdx[s][c];
                const R sg = (R)kSgn[s][c];
                gr += sg * (b[r * 8 + s] + b[(r + 4) * 8 + s + 4]);
                gi += sg * (b[r * 8 + s + 4] - b[(r + 4) * 8 + s]);
            }
            dF[6 * i + 2 * (c - 1)] = gr;
            dF[6 * i + 2 * (c - 1) + 1] = gi;
        }
    }
}

// carry record of the real problem (Q, n-1, S) x 8 x 8 -> (Q, n-1, S, 2, 2)
// complex: the element P_k (first column), sign (-1)^k
template <class R>
__global__ void k_sc_carry(const R* __restrict__ in, R* __restrict__ Z, int64_t total, int64_t S, int n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int k = 2 + (int)((t / S) % (n - 1));
        const R sg = (k & 1) ? R(-1) : R(1);
        const R* b = in + t * 64;
        for (int q = 0; q < 4; ++q) {
            Z[8 * t + 2 * q] = sg * b[q * 8];
            Z[8 * t + 2 * q + 1] = sg * b[(q + 4) * 8];
        }
    }
}

unsigned grid_for(int64_t total) {
    const int64_t g = (total + 255) / 256;
    return (unsigned)(g < 1 ? 1 : (g > 65535 * 8 ? 65535 * 8 : g));
}

}  // namespace

cudaError_t launch_sc_complex(int what, bool f64, const void* src, void* dst, int64_t count, int n, int op,
                              cudaStream_t st) {
    const unsigned g = grid_for(count);
#define MGB_SC_LAUNCH(R)                                                                                      \
    switch (what) {                                                                                           \
        case SC_EMBED: k_sc_embed<R><<<g, 256, 0, st>>>(static_cast<const R*>(src), static_cast<R*>(dst), count); break; \
        case SC_COT: k_sc_cot<R><<<(n + 255) / 256, 256, 0, st>>>(static_cast<const R*>(src), static_cast<R*>(dst), n, op); break; \
        case SC_OUT: k_sc_out<R><<<(3 * n + 255) / 256, 256, 0, st>>>(static_cast<const R*>(src), static_cast<R*>(dst), n, op); break; \
        case SC_GRAD: k_sc_grad<R><<<g, 256, 0, st>>>(static_cast<const R*>(src), static_cast<R*>(dst), count); break; \
        default: k_sc_carry<R><<<g, 256, 0, st>>>(static_cast<const R*>(src), static_cast<R*>(dst), count * (n - 1) * ((n + 3) / 2), count, n); break; \
    }
    if (f64) {
        MGB_SC_LAUNCH(double)
    } else {
        MGB_SC_LAUNCH(float)
    }
#undef MGB_SC_LAUNCH
    return cudaGetLastError();
}

cudaError_t launch_cplx_embed(bool f64, const void* Z, void* out, int64_t count, int d, bool cot, cudaStream_t st) {
    const unsigned g = grid_for(count * d * d);
    if (f64) k_cplx_embed<double><<<g, 256, 0, st>>>(static_cast<const double*>(Z), static_cast<double*>(out), count, d, cot);
    else k_cplx_embed<float><<<g, 256, 0, st>>>(static_cast<const float*>(Z), static_cast<float*>(out), count, d, cot);
    return cudaGetLastError();
}

cudaError_t launch_cplx_extract(bool f64, const void* in, void* Z, int64_t count, int d, bool grad, cudaStream_t st) {
    const unsigned g = grid_for(count * d * d);
    if (f64) k_cplx_extract<double><<<g, 256, 0, st>>>(static_cast<const double*>(in), static_cast<double*>(Z), count, d, grad);
    else k_cplx_extract<float><<<g, 256, 0, st>>>(static_cast<const float*>(in), static_cast<float*>(Z), count, d, grad);
    return cudaGetLastError();
}

}  // namespace mgb
