/*
 * Stand-in for the two Intel MKL CBLAS symbols that the reference's CPU path
 * (simulation_cpu.h:301-325) calls.  TEST INFRASTRUCTURE ONLY: used solely to
 * compile the reference's own simulation_cpu.h into oracle/_ref, since MKL is
 * not installed.  Row-major gemv, y = alpha * op(A) x + beta * y, summed in
 * index order.
 */
#ifndef HJM_ORACLE_MKL_SHIM_H
#define HJM_ORACLE_MKL_SHIM_H

typedef int MKL_INT;
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;

#define HJM_SHIM_GEMV(NAME, T)                                                              \
    static inline void NAME(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE trans, MKL_INT m, MKL_INT n, \
                            T alpha, const T* a, MKL_INT lda, const T* x, MKL_INT incx,       \
                            T beta, T* y, MKL_INT incy)                                       \
    {                                                                                         \
        /* only the row-major layout is used by the reference */                              \
        (void)layout;                                                                         \
        if (trans == CblasNoTrans) {                                                          \
            for (MKL_INT i = 0; i < m; ++i) {                                                 \
                T s = 0;                                                                      \
                for (MKL_INT j = 0; j < n; ++j) s += a[(long)i * lda + j] * x[(long)j * incx]; \
                y[(long)i * incy] = alpha * s + beta * y[(long)i * incy];                     \
            }                                                                                 \
        } else {                                                                              \
            for (MKL_INT j = 0; j < n; ++j) {                                                 \
                T s = 0;                                                                      \
                for (MKL_INT i = 0; i < m; ++i) s += a[(long)i * lda + j] * x[(long)i * incx]; \
                y[(long)j * incy] = alpha * s + beta * y[(long)j * incy];                     \
            }                                                                                 \
        }                                                                                     \
    }

HJM_SHIM_GEMV(cblas_dgemv, double)
HJM_SHIM_GEMV(cblas_sgemv, float)

#endif
