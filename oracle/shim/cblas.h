/*
 * Minimal CBLAS stand-in, used ONLY to compile the reference library from its own
 * sources for the oracle (oracle/_ref).  The reference's trust-region code
 * (src/trust_region.c:56-269) calls four BLAS-1/2 routines; these are plain
 * loops with the standard CBLAS semantics (row-major, no-transpose dgemv only).
 *
 * Test infrastructure: never linked into the product library.
 */
#pragma once

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

static inline double cblas_ddot(const int n, const double* x, const int incx, const double* y, const int incy)
{
	double s = 0;
	for (int i = 0; i < n; i++) s += x[i * incx] * y[i * incy];
	return s;
}

static inline void cblas_dscal(const int n, const double a, double* x, const int incx)
{
	for (int i = 0; i < n; i++) x[i * incx] *= a;
}

static inline void cblas_daxpy(const int n, const double a, const double* x, const int incx, double* y, const int incy)
{
	for (int i = 0; i < n; i++) y[i * incy] += a * x[i * incx];
}

/* y = alpha * A x + beta * y with A row-major m x n (lda = row stride); NoTrans only. */
static inline void cblas_dgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE trans, const int m, const int n,
	const double alpha, const double* a, const int lda, const double* x, const int incx,
	const double beta, double* y, const int incy)
{
	(void)order; (void)trans;
	for (int i = 0; i < m; i++)
	{
		double s = 0;
		for (int j = 0; j < n; j++) s += a[(long)i * lda + j] * x[j * incx];
		y[i * incy] = alpha * s + (beta == 0 ? 0 : beta * y[i * incy]);
	}
}

/* Complex matrix-vector product, row-major, no-transpose only (dense-target test maps). */
static inline void cblas_zgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE trans, const int m, const int n,
	const void* alpha, const void* a, const int lda, const void* x, const int incx,
	const void* beta, void* y, const int incy)
{
	(void)order; (void)trans;
	const double* al = (const double*)alpha;
	const double* be = (const double*)beta;
	const double* A = (const double*)a;
	const double* X = (const double*)x;
	double* Y = (double*)y;
	for (int i = 0; i < m; i++)
	{
		double sr = 0, si = 0;
		for (int j = 0; j < n; j++)
		{
			const double ar = A[2 * ((long)i * lda + j)], ai = A[2 * ((long)i * lda + j) + 1];
			const double xr = X[2 * j * incx], xi = X[2 * j * incx + 1];
			sr += ar * xr - ai * xi;
			si += ar * xi + ai * xr;
		}
		const double yr = Y[2 * i * incy], yi = Y[2 * i * incy + 1];
		const double nr = al[0] * sr - al[1] * si + be[0] * yr - be[1] * yi;
		const double ni = al[0] * si + al[1] * sr + be[0] * yi + be[1] * yr;
		Y[2 * i * incy] = nr;
		Y[2 * i * incy + 1] = ni;
	}
}
