/* Reference-element nodes, bases and dense operators for tensor-product elements (LINE, QUAD, HEX).
 *
 * Follows the reference's rules for the DG path:
 *   - solution basis: Lagrange on Gauss-Lobatto-Legendre nodes ("interp_tp GLL", "basis_sol lagrange";
 *     nodes.c:69-..., bases.c);
 *   - volume cubature: Gauss-Legendre of order p_c_x*p/2 = p, i.e. p+1 points per direction
 *     (nodes_operators.c:314-356 with p_c_x = 2 from simulation.c:494-495, CUB_C_DIV2 at :589-597);
 *   - face cubature: Gauss-Legendre with p+1 points per direction;
 *   - tensor-product node ordering with the first coordinate fastest (input/testing/unit/nodes/nodes_tp.data),
 *     and tensor-product operators as Kronecker products with the first factor fastest
 *     (input/testing/unit/operators/operators_tp.data, element_operators_tp.c);
 *   - tw operators are cv^T post-multiplied by the cubature weights (element_operators.h:26-27).
 * Local faces are ordered (r=-1, r=+1, s=-1, s=+1, t=-1, t=+1), matching the reference normals of
 * input/testing/integration/geom/TEST_straight_2d_quad_periodic.geom.data.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "dpg_host.h"

static void legendre_and_derivative(int n, double x, double* pn, double* dpn, double* pnm1)
{
	double p0 = 1.0, p1 = x;
	if (n == 0) { *pn = 1.0; *dpn = 0.0; *pnm1 = 0.0; return; }
	for (int k = 2; k <= n; ++k) {
		const double p2 = ((2.0*k-1.0)*x*p1 - (k-1.0)*p0)/k;
		p0 = p1; p1 = p2;
	}
	*pn = p1; *pnm1 = p0;
	/* P_n'(x) = n (x P_n - P_{n-1}) / (x^2 - 1), valid away from the end points where it is only used. */
	*dpn = n*(x*p1 - p0)/(x*x - 1.0);
}

/* Gauss-Legendre points and weights (n points), Newton iteration from Chebyshev guesses. */
void dpg_nodes_gl(int n, double* x, double* w)
{
	for (int i = 0; i < n; ++i) {
		double xi = -cos(M_PI*(i+0.75)/(n+0.5));
		for (int it = 0; it < 100; ++it) {
			double pn, dpn, pnm1;
			legendre_and_derivative(n,xi,&pn,&dpn,&pnm1);
			const double dx = pn/dpn;
			xi -= dx;
			if (fabs(dx) < 1e-16) break;
		}
		double pn, dpn, pnm1;
		legendre_and_derivative(n,xi,&pn,&dpn,&pnm1);
		x[i] = xi;
		w[i] = 2.0/((1.0-xi*xi)*dpn*dpn);
	}
	/* symmetrise */
	for (int i = 0; i < n/2; ++i) {
		const double a = 0.5*(x[n-1-i] - x[i]), b = 0.5*(w[i] + w[n-1-i]);
		x[i] = -a; x[n-1-i] = a; w[i] = w[n-1-i] = b;
	}
	if (n % 2 == 1) x[n/2] = 0.0;
}

/* Gauss-Jacobi points and weights of the weight (1 - x)^alpha on [-1, 1] (beta = 0): the roots of the Jacobi
 * polynomial P_n^(alpha,0) by Newton iteration with deflation, w_i = 2^(alpha+1) / ((1 - x_i^2) P_n'(x_i)^2); exact
 * for polynomials of degree 2n - 1 times the weight (the collapsed directions of simplex rules: alpha = 1 for the
 * triangle, 1 and 2 for the tetrahedron). */
static void jacobi_a0(int alpha, int n, double x, double* pn, double* dpn)
{
	const double al = alpha;
	double p0 = 1.0, p1 = 0.5*((al + 2.0)*x + al);
	if (n == 0) { *pn = 1.0; *dpn = 0.0; return; }
	for (int k = 1; k < n; ++k) {   /* three-term recurrence (beta = 0), a = 2k + alpha */
		const double a = 2.0*k + al;
		const double p2 = ((a + 1.0)*((a + 2.0)*a*x + al*al)*p1 - 2.0*(k + al)*k*(a + 2.0)*p0)
		                  /(2.0*(k + 1.0)*(k + al + 1.0)*a);
		p0 = p1; p1 = p2;
	}
	*pn = p1;
	/* (2n + alpha)(1 - x^2) P_n' = n (alpha - (2n + alpha) x) P_n + 2 (n + alpha) n P_{n-1} */
	*dpn = (n*(al - (2.0*n + al)*x)*p1 + 2.0*(n + al)*n*p0)/((2.0*n + al)*(1.0 - x*x));
}

void dpg_nodes_gj(int alpha, int n, double* x, double* w)
{
	for (int i = 0; i < n; ++i) {
		double xi = -cos(M_PI*(i + 0.75)/(n + 0.5));
		for (int it = 0; it < 200; ++it) {
			double pn, dpn;
			jacobi_a0(alpha,n,xi,&pn,&dpn);
			double defl = 0.0;
			for (int j = 0; j < i; ++j) defl += 1.0/(xi - x[j]);
			const double dx = pn/(dpn - pn*defl);
			xi -= dx;
			if (fabs(dx) < 1e-16) break;
		}
		x[i] = xi;
	}
	for (int i = 0; i < n; ++i)   /* ascending order */
		for (int j = i + 1; j < n; ++j)
			if (x[j] < x[i]) { const double t = x[i]; x[i] = x[j]; x[j] = t; }
	for (int i = 0; i < n; ++i) {
		double pn, dpn;
		jacobi_a0(alpha,n,x[i],&pn,&dpn);
		w[i] = ldexp(1.0,alpha + 1)/((1.0 - x[i]*x[i])*dpn*dpn);
	}
}

void dpg_nodes_gj10(int n, double* x, double* w) { dpg_nodes_gj(1,n,x,w); }

/* Gauss-Lobatto-Legendre points and weights (n >= 2 points): the end points plus the roots of P'_{n-1},
 * found by Newton iteration using the Legendre equation (1-x^2) P'' = 2x P' - N(N+1) P. */
void dpg_nodes_gll(int n, double* x, double* w)
{
	const int N = n-1;
	x[0] = -1.0; x[N] = 1.0;
	for (int i = 1; i < N; ++i) {
		double xi = -cos(M_PI*i/N);
		for (int it = 0; it < 100; ++it) {
			double pn, dpn, pnm1;
			legendre_and_derivative(N,xi,&pn,&dpn,&pnm1);
			const double d2 = (2.0*xi*dpn - N*(N+1.0)*pn)/(1.0-xi*xi);
			const double dx = dpn/d2;
			xi -= dx;
			if (fabs(dx) < 1e-16) break;
		}
		x[i] = xi;
	}
	for (int i = 0; i < n; ++i) {
		const double xi = x[i];
		double p0 = 1.0, p1 = xi;
		for (int k = 2; k <= N; ++k) {
			const double p2 = ((2.0*k-1.0)*xi*p1 - (k-1.0)*p0)/k;
			p0 = p1; p1 = p2;
		}
		w[i] = 2.0/(N*(N+1.0)*p1*p1);
	}
	for (int i = 0; i < n/2; ++i) {
		const double a = 0.5*(x[n-1-i] - x[i]), b = 0.5*(w[i] + w[n-1-i]);
		x[i] = -a; x[n-1-i] = a; w[i] = w[n-1-i] = b;
	}
	if (n % 2 == 1) x[n/2] = 0.0;
}

/* Values and derivatives of the n Lagrange polynomials on nodes xn at x. */
void dpg_lagrange_1d(int n, const double* xn, double x, double* val, double* der)
{
	for (int i = 0; i < n; ++i) {
		double v = 1.0;
		for (int j = 0; j < n; ++j)
			if (j != i) v *= (x - xn[j])/(xn[i] - xn[j]);
		val[i] = v;
		double dsum = 0.0;
		for (int k = 0; k < n; ++k) {
			if (k == i) continue;
			double t = 1.0/(xn[i] - xn[k]);
			for (int j = 0; j < n; ++j)
				if (j != i && j != k) t *= (x - xn[j])/(xn[i] - xn[j]);
			dsum += t;
		}
		der[i] = dsum;
	}
}

/* out = kron(b, a) in the reference's tensor-product ordering: the FIRST operator's indices run fastest.
 * out[(ia + ra*ib) , (ja + ca*jb)] = a[ia,ja] * b[ib,jb]; all row-major. */
void dpg_kron_rowmajor(int ra, int ca, const double* a, int rb, int cb, const double* b, double* out)
{
	const int rows = ra*rb, cols = ca*cb;
	for (int ib = 0; ib < rb; ++ib)
	for (int ia = 0; ia < ra; ++ia)
	for (int jb = 0; jb < cb; ++jb)
	for (int ja = 0; ja < ca; ++ja)
		out[(size_t)(ia+ra*ib)*cols + (ja+ca*jb)] = a[ia*ca+ja]*b[ib*cb+jb];
	(void)rows;
}

static double* dalloc(size_t n) { double* p = (double*)calloc(n ? n : 1, sizeof(double)); return p; }

/* Bernstein polynomial i of order p on [-1, 1]: binomial(p, i) ((1+r)/2)^i ((1-r)/2)^(p-i) (bases.c:1013-1019). */
static double bernstein(int p, int i, double r)
{
	double c = 1.0;
	for (int k = 1; k <= i; ++k) c = c*(double)(p - i + k)/(double)k;
	return c*pow(0.5*(1.0+r),i)*pow(0.5*(1.0-r),p-i);
}

/* Evaluate the tensor-product Lagrange basis (GLL nodes g, n1 per direction) and its gradient at point r. */
static void tp_basis_at(int d, int n1, const double* g, const double* r, double* val, double* grad /* [d][n_s] */);
void dpg_tp_basis_at(int d, int n1, const double* g, const double* r, double* val, double* grad)
{
	tp_basis_at(d,n1,g,r,val,grad);
}

static void tp_basis_at(int d, int n1, const double* g, const double* r, double* val, double* grad /* [d][n_s] */)
{
	double v1[DPG_DIM_MAX][16], d1[DPG_DIM_MAX][16];
	for (int a = 0; a < d; ++a)
		dpg_lagrange_1d(n1,g,r[a],v1[a],d1[a]);
	int n_s = 1;
	for (int a = 0; a < d; ++a) n_s *= n1;
	for (int s = 0; s < n_s; ++s) {
		int idx[DPG_DIM_MAX] = {0,0,0}, t = s;
		for (int a = 0; a < d; ++a) { idx[a] = t % n1; t /= n1; }
		double v = 1.0;
		for (int a = 0; a < d; ++a) v *= v1[a][idx[a]];
		val[s] = v;
		for (int dd = 0; dd < d; ++dd) {
			double gv = 1.0;
			for (int a = 0; a < d; ++a) gv *= (a == dd ? d1[a][idx[a]] : v1[a][idx[a]]);
			grad[(size_t)dd*n_s + s] = gv;
		}
	}
}

/* P1 (multilinear) geometry basis on the 2^d vertices (vertex k has coordinate bit a = (k>>a)&1). */
static void tp_p1_at(int d, const double* r, double* val, double* grad /* [d][n_ve] */)
{
	const int n_ve = 1 << d;
	for (int k = 0; k < n_ve; ++k) {
		double v = 1.0;
		double f[DPG_DIM_MAX], df[DPG_DIM_MAX];
		for (int a = 0; a < d; ++a) {
			const int b = (k >> a) & 1;
			f[a]  = b ? 0.5*(1.0+r[a]) : 0.5*(1.0-r[a]);
			df[a] = b ? 0.5 : -0.5;
			v *= f[a];
		}
		val[k] = v;
		for (int dd = 0; dd < d; ++dd) {
			double gv = 1.0;
			for (int a = 0; a < d; ++a) gv *= (a == dd ? df[a] : f[a]);
			grad[(size_t)dd*n_ve + k] = gv;
		}
	}
}

int dpg_element_ops_build(int e_type, int p, struct dpg_element_ops* ops)
{
	memset(ops,0,sizeof *ops);
	int d;
	switch (e_type) {
	case DPG_LINE: d = 1; break;
	case DPG_QUAD: d = 2; break;
	case DPG_HEX:  d = 3; break;
	case DPG_TRI:  return dpg_element_ops_build_tri(p,ops);
	case DPG_TET:  return dpg_element_ops_build_tet(p,ops);
	default: return -1;
	}
	if (p < 1 || p > 8) return -2;
	const int n1 = p+1;
	ops->e_type = e_type; ops->d = d; ops->p = p;
	int n_s = 1;
	for (int a = 0; a < d; ++a) n_s *= n1;
	const int n_c = n_s;                       /* GL, p+1 points per direction */
	int n_fc = 1;
	for (int a = 0; a < d-1; ++a) n_fc *= n1;  /* GL, p+1 points per face direction */
	ops->n_s = n_s; ops->n_c = n_c; ops->n_fl = 2*d; ops->n_fc = n_fc; ops->n_ve = 1 << d;
	const int n_fl = 2*d, n_ve = 1 << d;

	double gll[16], wgll[16], gl[16], wgl[16];
	dpg_nodes_gll(n1,gll,wgll);
	dpg_nodes_gl (n1,gl,wgl);

	ops->rst_vs = dalloc((size_t)n_s*d);
	ops->rst_vc = dalloc((size_t)n_c*d);
	ops->w_vc   = dalloc((size_t)n_c);
	for (int s = 0; s < n_s; ++s) {
		int t = s; double w = 1.0;
		for (int a = 0; a < d; ++a) {
			const int i = t % n1; t /= n1;
			ops->rst_vs[(size_t)s*d+a] = gll[i];
			ops->rst_vc[(size_t)s*d+a] = gl[i];
			w *= wgl[i];
		}
		ops->w_vc[s] = w;
	}

	/* face cubature: free coordinates of face (dir a fixed) in increasing dimension order, lowest fastest */
	ops->rst_fc = dalloc((size_t)n_fl*n_fc*d);
	ops->w_fc   = dalloc((size_t)n_fc);
	ops->normals_ref = dalloc((size_t)n_fl*d);
	for (int q = 0; q < n_fc; ++q) {
		int t = q; double w = 1.0;
		for (int a = 0; a < d-1; ++a) { w *= wgl[t % n1]; t /= n1; }
		ops->w_fc[q] = (d == 1 ? 1.0 : w);
	}
	for (int lf = 0; lf < n_fl; ++lf) {
		const int a_fix = lf/2;
		const double val = (lf % 2) ? 1.0 : -1.0;
		ops->normals_ref[(size_t)lf*d + a_fix] = val;
		for (int q = 0; q < n_fc; ++q) {
			int t = q;
			for (int a = 0; a < d; ++a) {
				double c;
				if (a == a_fix) c = val;
				else { c = gl[t % n1]; t /= n1; }
				ops->rst_fc[((size_t)lf*n_fc + q)*d + a] = c;
			}
		}
	}

	/* operators */
	ops->cv0_vs_vc = dalloc((size_t)n_c*n_s);
	ops->tw1_vt_vc = dalloc((size_t)d*n_s*n_c);
	ops->cv0_vs_fc = dalloc((size_t)n_fl*n_fc*n_s);
	ops->tw0_vt_fc = dalloc((size_t)n_fl*n_s*n_fc);
	ops->cv0_vv_vc = dalloc((size_t)n_c*n_ve);
	ops->cv1_vv_vc = dalloc((size_t)d*n_c*n_ve);
	ops->cv0_vv_fc = dalloc((size_t)n_fl*n_fc*n_ve);
	ops->cv1_vv_fc = dalloc((size_t)n_fl*d*n_fc*n_ve);
	double* val  = dalloc((size_t)n_s);
	double* grad = dalloc((size_t)d*n_s);
	double gval[8], ggrad[3*8];
	for (int c = 0; c < n_c; ++c) {
		const double* r = &ops->rst_vc[(size_t)c*d];
		tp_basis_at(d,n1,gll,r,val,grad);
		for (int s = 0; s < n_s; ++s) {
			ops->cv0_vs_vc[(size_t)c*n_s + s] = val[s];
			for (int dd = 0; dd < d; ++dd)
				ops->tw1_vt_vc[((size_t)dd*n_s + s)*n_c + c] = grad[(size_t)dd*n_s+s]*ops->w_vc[c];
		}
		tp_p1_at(d,r,gval,ggrad);
		for (int k = 0; k < n_ve; ++k) {
			ops->cv0_vv_vc[(size_t)c*n_ve + k] = gval[k];
			for (int dd = 0; dd < d; ++dd)
				ops->cv1_vv_vc[((size_t)dd*n_c + c)*n_ve + k] = ggrad[dd*n_ve+k];
		}
	}
	for (int lf = 0; lf < n_fl; ++lf)
	for (int q = 0; q < n_fc; ++q) {
		const double* r = &ops->rst_fc[((size_t)lf*n_fc + q)*d];
		tp_basis_at(d,n1,gll,r,val,grad);
		for (int s = 0; s < n_s; ++s) {
			ops->cv0_vs_fc[((size_t)lf*n_fc + q)*n_s + s] = val[s];
			ops->tw0_vt_fc[((size_t)lf*n_s + s)*n_fc + q] = val[s]*ops->w_fc[q];
		}
		tp_p1_at(d,r,gval,ggrad);
		for (int k = 0; k < n_ve; ++k) {
			ops->cv0_vv_fc[((size_t)lf*n_fc + q)*n_ve + k] = gval[k];
			for (int dd = 0; dd < d; ++dd)
				ops->cv1_vv_fc[(((size_t)lf*d + dd)*n_fc + q)*n_ve + k] = ggrad[dd*n_ve+k];
		}
	}
	free(val); free(grad);

	/* reference mass matrix M = cv0^T diag(w) cv0 and its inverse */
	double* m = dalloc((size_t)n_s*n_s);
	for (int i = 0; i < n_s; ++i)
	for (int j = 0; j < n_s; ++j) {
		double sum = 0.0;
		for (int c = 0; c < n_c; ++c)
			sum += ops->cv0_vs_vc[(size_t)c*n_s+i]*ops->w_vc[c]*ops->cv0_vs_vc[(size_t)c*n_s+j];
		m[(size_t)i*n_s+j] = sum;
	}
	ops->m_inv_ref = dalloc((size_t)n_s*n_s);
	int rc = dpg_invert(n_s,m,ops->m_inv_ref);
	free(m);
	if (rc) return rc;

	/* Bezier operators: ccBS0 = Bezier basis at the solution nodes (the Lagrange basis there is the identity),
	 * ccSB0 = its inverse, as the reference forms them by a solve with the full matrix */
	ops->bez1 = dalloc((size_t)n1*n1);
	ops->bez1_inv = dalloc((size_t)n1*n1);
	for (int n = 0; n < n1; ++n)
		for (int i = 0; i < n1; ++i) ops->bez1[(size_t)n*n1 + i] = bernstein(p,i,gll[n]);
	rc = dpg_invert(n1,ops->bez1,ops->bez1_inv);
	if (rc) return rc;
	ops->ccBS0_vs_vs = dalloc((size_t)n_s*n_s);
	ops->ccSB0_vs_vs = dalloc((size_t)n_s*n_s);
	for (int s = 0; s < n_s; ++s)
		for (int b = 0; b < n_s; ++b) {
			double v = 1.0;
			for (int a = 0, tb = b; a < d; ++a, tb /= n1) v *= bernstein(p,tb % n1,ops->rst_vs[(size_t)s*d+a]);
			ops->ccBS0_vs_vs[(size_t)s*n_s + b] = v;
		}
	return dpg_invert(n_s,ops->ccBS0_vs_vs,ops->ccSB0_vs_vs);
}

/* Bezier operators of a simplex (TRI: d = 2, TET: d = 3) of order p with the reference vertices V[d+1][d]: ccBS0 =
 * the Bernstein polynomials of degree p at the solution nodes, B_a(l) = p!/(a_0! ... a_d!) l_0^a_0 ... l_d^a_d in
 * the nodes' barycentric coordinates l (the basis of constructor_basis_si_bezier, bases.c:572-608, which builds the
 * same polynomials from collapsed coordinates), and ccSB0 = its inverse.  0 on success. */
int dpg_simplex_bezier_ops(struct dpg_element_ops* ops, const double (*V)[3])
{
	const int d = ops->d, p = ops->p, n_s = ops->n_s;
	double E[3][3] = {{0}}, Ei[9];
	for (int a = 0; a < d; ++a)
		for (int k = 0; k < d; ++k) E[a][k] = V[k+1][a] - V[0][a];
	double Ef[9];
	for (int a = 0; a < d; ++a) for (int k = 0; k < d; ++k) Ef[a*d + k] = E[a][k];
	int rc = dpg_invert(d,Ef,Ei);
	if (rc) return rc;
	double fact[DPG_P_MAX+1];
	fact[0] = 1.0;
	for (int i = 1; i <= DPG_P_MAX; ++i) fact[i] = fact[i-1]*i;
	ops->ccBS0_vs_vs = dalloc((size_t)n_s*n_s);
	ops->ccSB0_vs_vs = dalloc((size_t)n_s*n_s);
	for (int s = 0; s < n_s; ++s) {
		double l[4] = {1.0, 0.0, 0.0, 0.0};
		for (int k = 0; k < d; ++k) {
			double t = 0.0;
			for (int a = 0; a < d; ++a) t += Ei[k*d + a]*(ops->rst_vs[(size_t)s*d + a] - V[0][a]);
			l[k+1] = t;
			l[0] -= t;
		}
		int b = 0;   /* multi-indices (a_1, .., a_d) in lexicographic order, a_0 = p - their sum */
		for (int a1 = 0; a1 <= p; ++a1)
		for (int a2 = 0; a2 <= p - a1; ++a2)
		for (int a3 = 0; a3 <= (d == 3 ? p - a1 - a2 : 0); ++a3) {
			const int a0 = p - a1 - a2 - a3;
			ops->ccBS0_vs_vs[(size_t)s*n_s + b++] = fact[p]/(fact[a0]*fact[a1]*fact[a2]*fact[a3])*
			    pow(l[0],a0)*pow(l[1],a1)*pow(l[2],a2)*pow(l[3],a3);
		}
		if (b != n_s) return -1;
	}
	return dpg_invert(n_s,ops->ccBS0_vs_vs,ops->ccSB0_vs_vs);
}

/* Face operators of the order-p volume basis of ov at the face cubature of of, the operators of the same element type
 * and a higher order p_f (the reference's cv0_vs_fc[.][.][.][p_f][p], constructed like the equal-order ones from the
 * basis values at the face cubature nodes, element_operators.c): cv0 = phi(rst_fc(p_f)), tw0 = phi^T diag(w_fc(p_f)).
 * Stored in ov->cv0_vs_fcp[p_f] / tw0_vt_fcp[p_f]; 0 on success (or when already built). */
int dpg_element_face_ops_build(struct dpg_element_ops* ov, const struct dpg_element_ops* of)
{
	const int p_f = of->p, d = ov->d, n_s = ov->n_s, n_fl = ov->n_fl, n_fc = of->n_fc;
	if (of->e_type != ov->e_type || p_f <= ov->p || p_f > DPG_P_MAX) return -1;
	if (ov->cv0_vs_fcp[p_f]) return 0;
	const int n_pt = n_fl*n_fc;
	double* phi = dalloc((size_t)n_pt*n_s);
	double* cv0 = dalloc((size_t)n_pt*n_s);
	double* tw0 = dalloc((size_t)n_fl*n_s*n_fc);
	int rc = 0;
	if (ov->e_type == DPG_TRI) {
		rc = dpg_tri_lagrange_at(ov->p,ov->rst_vs,n_pt,of->rst_fc,phi);
	} else if (ov->e_type == DPG_TET) {
		rc = dpg_tet_lagrange_at(ov->p,ov->rst_vs,n_pt,of->rst_fc,phi);
	} else {
		const int n1 = ov->p + 1;
		double g1[16];
		for (int i = 0; i < n1; ++i) g1[i] = ov->rst_vs[(size_t)i*d];   /* the 1D GLL nodes: lowest index fastest */
		double* grad = dalloc((size_t)d*n_s);
		for (int k = 0; k < n_pt; ++k) tp_basis_at(d,n1,g1,&of->rst_fc[(size_t)k*d],&phi[(size_t)k*n_s],grad);
		free(grad);
	}
	if (rc) { free(phi); free(cv0); free(tw0); return rc; }
	for (int lf = 0; lf < n_fl; ++lf)
		for (int q = 0; q < n_fc; ++q)
			for (int s = 0; s < n_s; ++s) {
				const double v = phi[((size_t)lf*n_fc + q)*n_s + s];
				cv0[((size_t)lf*n_fc + q)*n_s + s] = v;
				tw0[((size_t)lf*n_s + s)*n_fc + q] = v*of->w_fc[q];
			}
	free(phi);
	ov->cv0_vs_fcp[p_f] = cv0;
	ov->tw0_vt_fcp[p_f] = tw0;
	return 0;
}

void dpg_element_ops_free(struct dpg_element_ops* ops)
{
	free(ops->rst_vs); free(ops->rst_vc); free(ops->w_vc); free(ops->rst_fc); free(ops->w_fc);
	free(ops->normals_ref); free(ops->cv0_vs_vc); free(ops->tw1_vt_vc); free(ops->cv0_vs_fc); free(ops->tw0_vt_fc);
	free(ops->cv0_vv_vc); free(ops->cv1_vv_vc); free(ops->cv0_vv_fc); free(ops->cv1_vv_fc); free(ops->m_inv_ref);
	free(ops->ccBS0_vs_vs); free(ops->ccSB0_vs_vs); free(ops->bez1); free(ops->bez1_inv);
	for (int k = 0; k <= DPG_P_MAX; ++k) { free(ops->cv0_vs_fcp[k]); free(ops->tw0_vt_fcp[k]); }
	memset(ops,0,sizeof *ops);
}
