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

unsigned grid_for(int64_t total) {
    const int64_t g = (total + 255) / 256;
    return (unsigned)(g < 1 ? 1 : (g > 65535 * 8 ? 65535 * 8 : g));
}

}  // namespace

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
