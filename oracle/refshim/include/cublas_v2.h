/*
 * Host stand-in for the four cuBLAS Level-1 routines the reference's FIRE
 * loops call (large_strain_relax.cu:642, :655-690, :743, :751;
 * network_mesh_relax.cu:917-970, :1030-1050, :1245), in host pointer mode,
 * on host memory.  Test infrastructure only.
 *
 * axpy uses a fused multiply-add per element, as a GPU BLAS does; dot, nrm2
 * and asum are sequential sums in index order.  cuBLAS's own summation order
 * is not specified, so results agree with a GPU run of the reference only to
 * rounding.
 */
#ifndef NR_REFSHIM_CUBLAS_V2_H
#define NR_REFSHIM_CUBLAS_V2_H

#include <cmath>

struct nr_refshim_cublas_ctx { int unused; };
typedef nr_refshim_cublas_ctx *cublasHandle_t;
typedef int cublasStatus_t;
enum { CUBLAS_STATUS_SUCCESS = 0 };

inline cublasStatus_t cublasCreate(cublasHandle_t *h) { *h = new nr_refshim_cublas_ctx(); return 0; }
inline cublasStatus_t cublasDestroy(cublasHandle_t h) { delete h; return 0; }

inline cublasStatus_t cublasDaxpy(cublasHandle_t, int n, const double *alpha, const double *x, int incx,
                                  double *y, int incy) {
    const double a = *alpha;
    for (int i = 0; i < n; ++i) y[i * incy] = std::fma(a, x[i * incx], y[i * incy]);
    return 0;
}
inline cublasStatus_t cublasDdot(cublasHandle_t, int n, const double *x, int incx, const double *y, int incy,
                                 double *result) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += x[i * incx] * y[i * incy];
    *result = s;
    return 0;
}
inline cublasStatus_t cublasDnrm2(cublasHandle_t, int n, const double *x, int incx, double *result) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += x[i * incx] * x[i * incx];
    *result = std::sqrt(s);
    return 0;
}
inline cublasStatus_t cublasDasum(cublasHandle_t, int n, const double *x, int incx, double *result) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += std::fabs(x[i * incx]);
    *result = s;
    return 0;
}

#endif
