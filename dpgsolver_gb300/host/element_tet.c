/* TET element operators (orders 1..4).
 *
 * Reference tetrahedron of the reference (nodes.c:508-515, element.c TET entry): the regular tetrahedron
 * v0 = (-1, -1/sqrt3, -1/sqrt6), v1 = (1, -1/sqrt3, -1/sqrt6), v2 = (0, 2/sqrt3, -1/sqrt6), v3 = (0, 0, 3/sqrt6),
 * edge length 2, centroid at the origin; local face f opposite vertex f with the face vertices of the reference's
 * f_ve = {2,3,1}, {2,3,0}, {0,1,3}, {0,1,2}.
 * Solution nodes: the equally spaced nodes of order p in barycentric coordinates, ordered by increasing l3, then
 * l2, then l1 (the reference reads alpha-optimised tetrahedron nodes from its node tables; the polynomial space is
 * the same, only the nodal coordinates of a state differ).
 * Basis: the Lagrange basis of the nodes through the inverse Vandermonde matrix of the monomials x^i y^j z^k
 * (i + j + k <= p) in the reference coordinates (centred at the origin).
 * Volume cubature: orders 1..3 the fully symmetric rules of gen_tet_rules.py (strength 2p: 4, 14, 24 points, as
 * the reference's Witherden-Vincent volume rules); order 4 the collapsed (Duffy) rule, (a, b, c) in [-1,1]^3 ->
 * xi3 = (1+c)/2, xi2 = (1+b)(1-c)/4, xi1 = (1+a)(1-b)(1-c)/8, Gauss-Legendre in a, Gauss-Jacobi of the weights
 * (1-b) and (1-c)^2 in b and c, 5 points each: 125 points exact to degree 9.
 * Face cubature: the fully symmetric triangle rules of gen_tri_rules.py (strength 2p, as the reference's
 * Witherden-Vincent face rules), invariant under the face's vertex permutations so that both sides of a face see
 * the same points; weights of the reference face's area (sqrt3).
 * Geometry basis: the barycentric (P1) functions.  Bezier operators of the positivity limiter: the Bernstein
 * polynomials of degree p at the nodes and their inverse (dpg_simplex_bezier_ops; no 1D factors). */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "dpg_host.h"
#include "tet_sym_rules.inc"
#include "tri_sym_rules.inc"

#define SQ3 1.7320508075688772
#define SQ6 2.4494897427831779

static const double TV[4][3] = {{-1.0, -1.0/SQ3, -1.0/SQ6}, {1.0, -1.0/SQ3, -1.0/SQ6},
                                {0.0, 2.0/SQ3, -1.0/SQ6}, {0.0, 0.0, 3.0/SQ6}};
static const int TFVE[4][3] = {{2,3,1}, {2,3,0}, {0,1,3}, {0,1,2}};

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* barycentric coordinates l[4] of x and their constant gradients g[4][3] */
static void bary(const double* x, double* l, double (*g)[3])
{
	/* columns of M: v_k - v0 (k = 1..3); (l1, l2, l3) = M^-1 (x - v0) */
	double M[3][3], Mi[3][3];
	for (int k = 0; k < 3; ++k)
		for (int a = 0; a < 3; ++a) M[a][k] = TV[k+1][a] - TV[0][a];
	const double det = M[0][0]*(M[1][1]*M[2][2] - M[1][2]*M[2][1]) - M[0][1]*(M[1][0]*M[2][2] - M[1][2]*M[2][0])
	                 + M[0][2]*(M[1][0]*M[2][1] - M[1][1]*M[2][0]);
	Mi[0][0] =  (M[1][1]*M[2][2] - M[1][2]*M[2][1])/det; Mi[0][1] = -(M[0][1]*M[2][2] - M[0][2]*M[2][1])/det;
	Mi[0][2] =  (M[0][1]*M[1][2] - M[0][2]*M[1][1])/det; Mi[1][0] = -(M[1][0]*M[2][2] - M[1][2]*M[2][0])/det;
	Mi[1][1] =  (M[0][0]*M[2][2] - M[0][2]*M[2][0])/det; Mi[1][2] = -(M[0][0]*M[1][2] - M[0][2]*M[1][0])/det;
	Mi[2][0] =  (M[1][0]*M[2][1] - M[1][1]*M[2][0])/det; Mi[2][1] = -(M[0][0]*M[2][1] - M[0][1]*M[2][0])/det;
	Mi[2][2] =  (M[0][0]*M[1][1] - M[0][1]*M[1][0])/det;
	const double dx[3] = {x[0] - TV[0][0], x[1] - TV[0][1], x[2] - TV[0][2]};
	l[0] = 1.0;
	for (int k = 0; k < 3; ++k) {
		l[k+1] = Mi[k][0]*dx[0] + Mi[k][1]*dx[1] + Mi[k][2]*dx[2];
		l[0] -= l[k+1];
		if (g) for (int a = 0; a < 3; ++a) g[k+1][a] = Mi[k][a];
	}
	if (g) for (int a = 0; a < 3; ++a) g[0][a] = -(g[1][a] + g[2][a] + g[3][a]);
}

void dpg_tet_p1_at(const double* r, double* val, double* grad)
{
	double g[4][3];
	bary(r,val,g);
	if (grad)   /* [d][n_ve] */
		for (int a = 0; a < 3; ++a)
			for (int k = 0; k < 4; ++k) grad[a*4 + k] = g[k][a];
}

/* monomials x^i y^j z^k (i + j + k <= p; i outer, then j, then k) and their gradients */
static void monomials(int p, const double* x, double* m, double* mx, double* my, double* mz)
{
	int n = 0;
	for (int i = 0; i <= p; ++i)
		for (int j = 0; i + j <= p; ++j)
			for (int k = 0; i + j + k <= p; ++k, ++n) {
				const double xi = pow(x[0],i), yj = pow(x[1],j), zk = pow(x[2],k);
				m[n] = xi*yj*zk;
				if (mx) {
					mx[n] = i ? i*pow(x[0],i-1)*yj*zk : 0.0;
					my[n] = j ? j*xi*pow(x[1],j-1)*zk : 0.0;
					mz[n] = k ? k*xi*yj*pow(x[2],k-1) : 0.0;
				}
			}
}

static int nodes(int p, double* rst)
{
	int n = 0;
	for (int c = 0; c <= p; ++c)
		for (int b = 0; b + c <= p; ++b)
			for (int a = 0; a + b + c <= p; ++a, ++n) {
				const double l[4] = {(double)(p - a - b - c)/p, (double)a/p, (double)b/p, (double)c/p};
				for (int d = 0; d < 3; ++d) {
					double s = 0.0;
					for (int k = 0; k < 4; ++k) s += l[k]*TV[k][d];
					rst[3*n + d] = s;
				}
			}
	return n;
}

/* Lagrange basis of the nodes rst_vs (order p) and its gradient at n_pt points: out[n_pt][n_s], gout[3][n_pt][n_s] */
static int lagrange(int p, const double* rst_vs, int n_pt, const double* pts, double* out, double* gout)
{
	const int n_s = (p+1)*(p+2)*(p+3)/6;
	double* V = zalloc((size_t)n_s*n_s);
	double* Vi = zalloc((size_t)n_s*n_s);
	double m[35], mx[35], my[35], mz[35];
	for (int i = 0; i < n_s; ++i) {
		monomials(p,&rst_vs[3*i],m,NULL,NULL,NULL);
		for (int k = 0; k < n_s; ++k) V[(size_t)i*n_s + k] = m[k];
	}
	const int rc = dpg_invert(n_s,V,Vi);
	if (!rc)
		for (int t = 0; t < n_pt; ++t) {
			monomials(p,&pts[3*t],m,mx,my,mz);
			for (int j = 0; j < n_s; ++j) {
				double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
				for (int k = 0; k < n_s; ++k) {
					const double v = Vi[(size_t)k*n_s + j];
					a0 += m[k]*v; a1 += mx[k]*v; a2 += my[k]*v; a3 += mz[k]*v;
				}
				out[(size_t)t*n_s + j] = a0;
				if (gout) {
					gout[((size_t)0*n_pt + t)*n_s + j] = a1;
					gout[((size_t)1*n_pt + t)*n_s + j] = a2;
					gout[((size_t)2*n_pt + t)*n_s + j] = a3;
				}
			}
		}
	free(V); free(Vi);
	return rc;
}

int dpg_tet_lagrange_at(int p, const double* rst_vs, int n_pt, const double* pts, double* out)
{
	return lagrange(p,rst_vs,n_pt,pts,out,NULL);
}

int dpg_element_ops_build_tet(int p, struct dpg_element_ops* ops)
{
	memset(ops,0,sizeof *ops);
	if (p < 1 || p > 4) return -2;   /* face rules up to strength 8 */
	static const int* const n_rule[5] = {NULL, &tri_sym_n2, &tri_sym_n4, &tri_sym_n6, &tri_sym_n8};
	static const double (*const rule[5])[4] = {NULL, tri_sym_rule2, tri_sym_rule4, tri_sym_rule6, tri_sym_rule8};
	static const int* const n_vrule[4] = {NULL, &tet_sym_n2, &tet_sym_n4, &tet_sym_n6};
	static const double (*const vrule[4])[5] = {NULL, tet_sym_rule2, tet_sym_rule4, tet_sym_rule6};
	const int q = p + 1;
	const int d = 3, n_s = (p+1)*(p+2)*(p+3)/6, n_c = (p <= 3 ? *n_vrule[p] : q*q*q), n_fc = *n_rule[p], n_fl = 4, n_ve = 4;
	ops->e_type = DPG_TET; ops->d = d; ops->p = p;
	ops->n_s = n_s; ops->n_c = n_c; ops->n_fl = n_fl; ops->n_fc = n_fc; ops->n_ve = n_ve;

	ops->rst_vs = zalloc((size_t)n_s*d);
	nodes(p,ops->rst_vs);

	/* volume cubature */
	double ga[16], wa[16], gb[16], wb[16], gc[16], wc[16];
	dpg_nodes_gl(q,ga,wa);
	dpg_nodes_gj(1,q,gb,wb);
	dpg_nodes_gj(2,q,gc,wc);
	double E[3][3];
	for (int k = 0; k < 3; ++k)
		for (int a = 0; a < 3; ++a) E[k][a] = TV[k+1][a] - TV[0][a];
	const double vol6 = fabs(E[0][0]*(E[1][1]*E[2][2] - E[1][2]*E[2][1]) - E[0][1]*(E[1][0]*E[2][2] - E[1][2]*E[2][0])
	                       + E[0][2]*(E[1][0]*E[2][1] - E[1][1]*E[2][0]));
	ops->rst_vc = zalloc((size_t)n_c*d);
	ops->w_vc = zalloc((size_t)n_c);
	if (p <= 3) {   /* symmetric rule: barycentric points, weights of the reference tetrahedron's volume |det|/6 */
		for (int cc = 0; cc < n_c; ++cc) {
			for (int dd = 0; dd < 3; ++dd) {
				double x = 0.0;
				for (int k = 0; k < 4; ++k) x += vrule[p][cc][k]*TV[k][dd];
				ops->rst_vc[3*cc + dd] = x;
			}
			ops->w_vc[cc] = vrule[p][cc][4]*vol6/6.0;
		}
	} else
	for (int ic = 0; ic < q; ++ic)
		for (int ib = 0; ib < q; ++ib)
			for (int ia = 0; ia < q; ++ia) {
				const int cc = (ic*q + ib)*q + ia;
				const double a = ga[ia], b = gb[ib], c = gc[ic];
				const double x3 = 0.5*(1.0 + c), x2 = 0.25*(1.0 + b)*(1.0 - c), x1 = 0.125*(1.0 + a)*(1.0 - b)*(1.0 - c);
				for (int dd = 0; dd < 3; ++dd)
					ops->rst_vc[3*cc + dd] = TV[0][dd] + x1*E[0][dd] + x2*E[1][dd] + x3*E[2][dd];
				ops->w_vc[cc] = wa[ia]*wb[ib]*wc[ic]/64.0*vol6;
			}

	/* face cubature and outward reference normals */
	ops->rst_fc = zalloc((size_t)n_fl*n_fc*d);
	ops->w_fc = zalloc((size_t)n_fc);
	ops->normals_ref = zalloc((size_t)n_fl*d);
	for (int k = 0; k < n_fc; ++k) ops->w_fc[k] = rule[p][k][3]*SQ3;
	double l0[4], g0[4][3];
	bary(TV[0],l0,g0);
	for (int f = 0; f < n_fl; ++f) {
		for (int k = 0; k < n_fc; ++k)
			for (int dd = 0; dd < 3; ++dd) {
				double s = 0.0;
				for (int j = 0; j < 3; ++j) s += rule[p][k][j]*TV[TFVE[f][j]][dd];
				ops->rst_fc[((size_t)f*n_fc + k)*d + dd] = s;
			}
		const double len = sqrt(g0[f][0]*g0[f][0] + g0[f][1]*g0[f][1] + g0[f][2]*g0[f][2]);
		for (int dd = 0; dd < 3; ++dd) ops->normals_ref[f*d + dd] = -g0[f][dd]/len;
	}

	/* operators */
	ops->cv0_vs_vc = zalloc((size_t)n_c*n_s);
	ops->tw1_vt_vc = zalloc((size_t)d*n_s*n_c);
	ops->cv0_vs_fc = zalloc((size_t)n_fl*n_fc*n_s);
	ops->tw0_vt_fc = zalloc((size_t)n_fl*n_s*n_fc);
	ops->cv0_vv_vc = zalloc((size_t)n_c*n_ve);
	ops->cv1_vv_vc = zalloc((size_t)d*n_c*n_ve);
	ops->cv0_vv_fc = zalloc((size_t)n_fl*n_fc*n_ve);
	ops->cv1_vv_fc = zalloc((size_t)n_fl*d*n_fc*n_ve);
	double* g = zalloc((size_t)d*n_c*n_s);
	int rc = lagrange(p,ops->rst_vs,n_c,ops->rst_vc,ops->cv0_vs_vc,g);
	if (!rc) rc = lagrange(p,ops->rst_vs,n_fl*n_fc,ops->rst_fc,ops->cv0_vs_fc,NULL);
	if (rc) { free(g); return rc; }
	for (int dd = 0; dd < d; ++dd)
		for (int s = 0; s < n_s; ++s)
			for (int cc = 0; cc < n_c; ++cc)
				ops->tw1_vt_vc[((size_t)dd*n_s + s)*n_c + cc] = g[((size_t)dd*n_c + cc)*n_s + s]*ops->w_vc[cc];
	free(g);
	for (int f = 0; f < n_fl; ++f)
		for (int s = 0; s < n_s; ++s)
			for (int k = 0; k < n_fc; ++k)
				ops->tw0_vt_fc[((size_t)f*n_s + s)*n_fc + k] = ops->cv0_vs_fc[((size_t)f*n_fc + k)*n_s + s]*ops->w_fc[k];
	double lv[4], gv[4][3];
	for (int cc = 0; cc < n_c; ++cc) {
		bary(&ops->rst_vc[3*cc],lv,gv);
		for (int k = 0; k < n_ve; ++k) {
			ops->cv0_vv_vc[(size_t)cc*n_ve + k] = lv[k];
			for (int dd = 0; dd < d; ++dd) ops->cv1_vv_vc[((size_t)dd*n_c + cc)*n_ve + k] = gv[k][dd];
		}
	}
	for (int f = 0; f < n_fl; ++f)
		for (int k = 0; k < n_fc; ++k) {
			bary(&ops->rst_fc[((size_t)f*n_fc + k)*d],lv,gv);
			for (int v = 0; v < n_ve; ++v) {
				ops->cv0_vv_fc[((size_t)f*n_fc + k)*n_ve + v] = lv[v];
				for (int dd = 0; dd < d; ++dd) ops->cv1_vv_fc[(((size_t)f*d + dd)*n_fc + k)*n_ve + v] = gv[v][dd];
			}
		}

	/* reference mass matrix and its inverse */
	double* mm = zalloc((size_t)n_s*n_s);
	for (int i = 0; i < n_s; ++i)
		for (int j = 0; j < n_s; ++j) {
			double sum = 0.0;
			for (int cc = 0; cc < n_c; ++cc)
				sum += ops->cv0_vs_vc[(size_t)cc*n_s+i]*ops->w_vc[cc]*ops->cv0_vs_vc[(size_t)cc*n_s+j];
			mm[(size_t)i*n_s+j] = sum;
		}
	ops->m_inv_ref = zalloc((size_t)n_s*n_s);
	rc = dpg_invert(n_s,mm,ops->m_inv_ref);
	free(mm);
	if (!rc) rc = dpg_simplex_bezier_ops(ops,TV);
	return rc;
}
