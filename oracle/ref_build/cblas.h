/*
 * Minimal CBLAS declarations for building the reference Jet headers as a CPU
 * oracle. Test infrastructure only: nothing in the shipped library includes
 * this file.
 *
 * The reference calls cblas_{c,z}gemm / gemv / dotu_sub with the standard
 * CBLAS signature (TensorHelpers.hpp:47-111). numpy bundles an ILP64 OpenBLAS
 * whose CBLAS entry points carry a `scipy_` prefix and a `64_` suffix; these
 * inline forwarders map one onto the other. The integer arguments of the
 * ILP64 build are 64-bit.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
typedef enum CBLAS_ORDER CBLAS_LAYOUT;

typedef int64_t jetref_blasint;

void scipy_cblas_cgemm64_(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE,
                          jetref_blasint, jetref_blasint, jetref_blasint, const void *,
                          const void *, jetref_blasint, const void *, jetref_blasint,
                          const void *, void *, jetref_blasint);
void scipy_cblas_zgemm64_(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE,
                          jetref_blasint, jetref_blasint, jetref_blasint, const void *,
                          const void *, jetref_blasint, const void *, jetref_blasint,
                          const void *, void *, jetref_blasint);
void scipy_cblas_cgemv64_(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, jetref_blasint,
                          jetref_blasint, const void *, const void *, jetref_blasint,
                          const void *, jetref_blasint, const void *, void *,
                          jetref_blasint);
void scipy_cblas_zgemv64_(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, jetref_blasint,
                          jetref_blasint, const void *, const void *, jetref_blasint,
                          const void *, jetref_blasint, const void *, void *,
                          jetref_blasint);
void scipy_cblas_cdotu_sub64_(jetref_blasint, const void *, jetref_blasint, const void *,
                              jetref_blasint, void *);
void scipy_cblas_zdotu_sub64_(jetref_blasint, const void *, jetref_blasint, const void *,
                              jetref_blasint, void *);

static inline void cblas_cgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta,
                               enum CBLAS_TRANSPOSE tb, jetref_blasint m, jetref_blasint n,
                               jetref_blasint k, const void *alpha, const void *a,
                               jetref_blasint lda, const void *b, jetref_blasint ldb,
                               const void *beta, void *c, jetref_blasint ldc)
{
    scipy_cblas_cgemm64_(o, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
static inline void cblas_zgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta,
                               enum CBLAS_TRANSPOSE tb, jetref_blasint m, jetref_blasint n,
                               jetref_blasint k, const void *alpha, const void *a,
                               jetref_blasint lda, const void *b, jetref_blasint ldb,
                               const void *beta, void *c, jetref_blasint ldc)
{
    scipy_cblas_zgemm64_(o, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
static inline void cblas_cgemv(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE t, jetref_blasint m,
                               jetref_blasint n, const void *alpha, const void *a,
                               jetref_blasint lda, const void *x, jetref_blasint incx,
                               const void *beta, void *y, jetref_blasint incy)
{
    scipy_cblas_cgemv64_(o, t, m, n, alpha, a, lda, x, incx, beta, y, incy);
}
static inline void cblas_zgemv(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE t, jetref_blasint m,
                               jetref_blasint n, const void *alpha, const void *a,
                               jetref_blasint lda, const void *x, jetref_blasint incx,
                               const void *beta, void *y, jetref_blasint incy)
{
    scipy_cblas_zgemv64_(o, t, m, n, alpha, a, lda, x, incx, beta, y, incy);
}
static inline void cblas_cdotu_sub(jetref_blasint n, const void *x, jetref_blasint incx,
                                   const void *y, jetref_blasint incy, void *dotu)
{
    scipy_cblas_cdotu_sub64_(n, x, incx, y, incy, dotu);
}
static inline void cblas_zdotu_sub(jetref_blasint n, const void *x, jetref_blasint incx,
                                   const void *y, jetref_blasint incy, void *dotu)
{
    scipy_cblas_zdotu_sub64_(n, x, incx, y, incy, dotu);
}

#ifdef __cplusplus
}
#endif
