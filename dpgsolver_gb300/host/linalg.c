/* Small dense FP64 linear algebra used by the host setup.
 *
 * The reference inverts the mass matrix with LAPACKE_dsgesv (matrix_constructors_T.c:377-402) and multiplies with
 * cblas_dgemm (matrix_math_T.c:178-201).  Setup here only needs an LU factorisation with partial pivoting and a
 * plain triple loop; both run once per element group or per curved element. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "dpg_host.h"

int dpg_lu_factor(int n, double* a, int* piv)
{
	for (int k = 0; k < n; ++k) {
		int pr = k;
		double best = fabs(a[(size_t)k*n+k]);
		for (int i = k+1; i < n; ++i) {
			const double v = fabs(a[(size_t)i*n+k]);
			if (v > best) { best = v; pr = i; }
		}
		piv[k] = pr;
		if (best == 0.0) return -1;
		if (pr != k)
			for (int j = 0; j < n; ++j) {
				const double t = a[(size_t)k*n+j]; a[(size_t)k*n+j] = a[(size_t)pr*n+j]; a[(size_t)pr*n+j] = t;
			}
		const double inv = 1.0/a[(size_t)k*n+k];
		for (int i = k+1; i < n; ++i) {
			const double l = a[(size_t)i*n+k]*inv;
			a[(size_t)i*n+k] = l;
			if (l != 0.0)
				for (int j = k+1; j < n; ++j)
					a[(size_t)i*n+j] -= l*a[(size_t)k*n+j];
		}
	}
	return 0;
}

void dpg_lu_solve(int n, const double* lu, const int* piv, double* b)
{
	for (int k = 0; k < n; ++k) {
		const int pr = piv[k];
		if (pr != k) { const double t = b[k]; b[k] = b[pr]; b[pr] = t; }
	}
	for (int i = 0; i < n; ++i) {
		double s = b[i];
		for (int j = 0; j < i; ++j) s -= lu[(size_t)i*n+j]*b[j];
		b[i] = s;
	}
	for (int i = n-1; i >= 0; --i) {
		double s = b[i];
		for (int j = i+1; j < n; ++j) s -= lu[(size_t)i*n+j]*b[j];
		b[i] = s/lu[(size_t)i*n+i];
	}
}

int dpg_invert(int n, const double* a, double* a_inv)
{
	double* lu = (double*)malloc(sizeof(double)*(size_t)n*n);
	int* piv = (int*)malloc(sizeof(int)*(size_t)n);
	double* col = (double*)malloc(sizeof(double)*(size_t)n);
	memcpy(lu,a,sizeof(double)*(size_t)n*n);
	int rc = dpg_lu_factor(n,lu,piv);
	if (rc == 0) {
		for (int j = 0; j < n; ++j) {
			for (int i = 0; i < n; ++i) col[i] = (i == j);
			dpg_lu_solve(n,lu,piv,col);
			for (int i = 0; i < n; ++i) a_inv[(size_t)i*n+j] = col[i];
		}
	}
	free(lu); free(piv); free(col);
	return rc;
}

/* c = alpha*a*b + beta*c, all row-major; a [m x k], b [k x n]. */
void dpg_matmul(int m, int n, int k, double alpha, const double* a, const double* b, double beta, double* c)
{
	for (int i = 0; i < m; ++i)
	for (int j = 0; j < n; ++j) {
		double s = 0.0;
		for (int l = 0; l < k; ++l) s += a[(size_t)i*k+l]*b[(size_t)l*n+j];
		c[(size_t)i*n+j] = alpha*s + (beta == 0.0 ? 0.0 : beta*c[(size_t)i*n+j]);
	}
}
