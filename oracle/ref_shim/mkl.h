// Naive CBLAS stand-in used only to compile the reference implementation as
// a test oracle in an environment without MKL/OpenBLAS.  It provides exactly
// the routines the reference's Blas matrix policy calls (sgemm/dgemm/cgemm/
// zgemm, ?axpy, ?scal, csscal/zdscal, ?copy) with row-major semantics.
// Rounding is that of a plain triple loop, not MKL's; the oracle therefore
// uses the Manual/Fixed2/SpaceCurve matrix policies for pinned comparisons.
#ifndef MAGNUS_ORACLE_CBLAS_SHIM_H
#define MAGNUS_ORACLE_CBLAS_SHIM_H

#include <complex>
#include <cstddef>
#include <vector>

enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

namespace magnus_oracle_shim {

template <class T>
inline void gemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb,
                 long m, long n, long k, T alpha, const T* a, long lda,
                 const T* b, long ldb, T beta, T* c, long ldc) {
    // Column-major callers are mapped onto the row-major loop by swapping
    // operands: C^T = B^T A^T.
    if (layout == CblasColMajor) {
        gemm<T>(CblasRowMajor, tb, ta, n, m, k, alpha, b, ldb, a, lda, beta, c, ldc);
        return;
    }
    std::vector<T> acc(static_cast<size_t>(m * n));
    for (long i = 0; i < m; ++i) {
        for (long j = 0; j < n; ++j) {
            T s = T(0);
            for (long p = 0; p < k; ++p) {
                T av = (ta == CblasNoTrans) ? a[i * lda + p] : a[p * lda + i];
                T bv = (tb == CblasNoTrans) ? b[p * ldb + j] : b[j * ldb + p];
                s += av * bv;
            }
            acc[static_cast<size_t>(i * n + j)] = s;
        }
    }
    for (long i = 0; i < m; ++i)
        for (long j = 0; j < n; ++j) {
            T prev = (beta == T(0)) ? T(0) : beta * c[i * ldc + j];
            c[i * ldc + j] = alpha * acc[static_cast<size_t>(i * n + j)] + prev;
        }
}

template <class T, class S>
inline void axpy(long n, S alpha, const T* x, long incx, T* y, long incy) {
    for (long i = 0; i < n; ++i) y[i * incy] += T(alpha) * x[i * incx];
}

template <class T, class S>
inline void scal(long n, S alpha, T* x, long incx) {
    for (long i = 0; i < n; ++i) x[i * incx] *= alpha;
}

template <class T>
inline void copy(long n, const T* x, long incx, T* y, long incy) {
    for (long i = 0; i < n; ++i) y[i * incy] = x[i * incx];
}

}  // namespace magnus_oracle_shim

using magnus_oracle_c32 = std::complex<float>;
using magnus_oracle_c64 = std::complex<double>;

inline void cblas_sgemm(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, long m, long n, long k,
                        float alpha, const float* a, long lda, const float* b, long ldb, float beta, float* c, long ldc) {
    magnus_oracle_shim::gemm<float>(l, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
inline void cblas_dgemm(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, long m, long n, long k,
                        double alpha, const double* a, long lda, const double* b, long ldb, double beta, double* c, long ldc) {
    magnus_oracle_shim::gemm<double>(l, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
inline void cblas_cgemm(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, long m, long n, long k,
                        const void* alpha, const void* a, long lda, const void* b, long ldb, const void* beta, void* c, long ldc) {
    magnus_oracle_shim::gemm<magnus_oracle_c32>(l, ta, tb, m, n, k, *static_cast<const magnus_oracle_c32*>(alpha),
        static_cast<const magnus_oracle_c32*>(a), lda, static_cast<const magnus_oracle_c32*>(b), ldb,
        *static_cast<const magnus_oracle_c32*>(beta), static_cast<magnus_oracle_c32*>(c), ldc);
}
inline void cblas_zgemm(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, long m, long n, long k,
                        const void* alpha, const void* a, long lda, const void* b, long ldb, const void* beta, void* c, long ldc) {
    magnus_oracle_shim::gemm<magnus_oracle_c64>(l, ta, tb, m, n, k, *static_cast<const magnus_oracle_c64*>(alpha),
        static_cast<const magnus_oracle_c64*>(a), lda, static_cast<const magnus_oracle_c64*>(b), ldb,
        *static_cast<const magnus_oracle_c64*>(beta), static_cast<magnus_oracle_c64*>(c), ldc);
}

inline void cblas_saxpy(long n, float alpha, const float* x, long incx, float* y, long incy) {
    magnus_oracle_shim::axpy(n, alpha, x, incx, y, incy);
}
inline void cblas_daxpy(long n, double alpha, const double* x, long incx, double* y, long incy) {
    magnus_oracle_shim::axpy(n, alpha, x, incx, y, incy);
}
inline void cblas_caxpy(long n, const void* alpha, const void* x, long incx, void* y, long incy) {
    magnus_oracle_shim::axpy(n, *static_cast<const magnus_oracle_c32*>(alpha), static_cast<const magnus_oracle_c32*>(x), incx,
                             static_cast<magnus_oracle_c32*>(y), incy);
}
inline void cblas_zaxpy(long n, const void* alpha, const void* x, long incx, void* y, long incy) {
    magnus_oracle_shim::axpy(n, *static_cast<const magnus_oracle_c64*>(alpha), static_cast<const magnus_oracle_c64*>(x), incx,
                             static_cast<magnus_oracle_c64*>(y), incy);
}

inline void cblas_sscal(long n, float alpha, float* x, long incx) { magnus_oracle_shim::scal(n, alpha, x, incx); }
inline void cblas_dscal(long n, double alpha, double* x, long incx) { magnus_oracle_shim::scal(n, alpha, x, incx); }
inline void cblas_csscal(long n, float alpha, void* x, long incx) {
    magnus_oracle_shim::scal(n, alpha, static_cast<magnus_oracle_c32*>(x), incx);
}
inline void cblas_zdscal(long n, double alpha, void* x, long incx) {
    magnus_oracle_shim::scal(n, alpha, static_cast<magnus_oracle_c64*>(x), incx);
}

inline void cblas_scopy(long n, const float* x, long incx, float* y, long incy) { magnus_oracle_shim::copy(n, x, incx, y, incy); }
inline void cblas_dcopy(long n, const double* x, long incx, double* y, long incy) { magnus_oracle_shim::copy(n, x, incx, y, incy); }
inline void cblas_ccopy(long n, const void* x, long incx, void* y, long incy) {
    magnus_oracle_shim::copy(n, static_cast<const magnus_oracle_c32*>(x), incx, static_cast<magnus_oracle_c32*>(y), incy);
}
inline void cblas_zcopy(long n, const void* x, long incx, void* y, long incy) {
    magnus_oracle_shim::copy(n, static_cast<const magnus_oracle_c64*>(x), incx, static_cast<magnus_oracle_c64*>(y), incy);
}

#endif
