/* Set-up of the CPU oracle (TEST INFRASTRUCTURE ONLY; see oracle_dg.h): mesh, reference-element operators,
 * geometry, face connectivity, initial solution and L2 errors, computed here from the problem parameters alone.
 * Nothing in this file calls or links the library under test; the data model it fills is the plain layout of
 * include/dpg_simulation.h, which the residual restatement in oracle_dg.c reads.
 *
 * Algorithms (chosen to differ from the library's own set-up where the mathematics allows, so that the two
 * check each other):
 *   - 1D nodes (constructor_const_Nodes_tp, element/nodes.c:69; GL and GLL of the jacobi-0.9.2 library): the
 *     Gauss-Legendre points are the eigenvalues of the Legendre Jacobi matrix, the interior Gauss-Lobatto points
 *     those of the Jacobi(1,1) matrix (Golub-Welsch), each isolated by bisection on the Sturm sequence of the
 *     tridiagonal matrix; weights from the classical closed forms;
 *   - basis operators: the reference forms the operators of its Lagrange solution basis from the orthonormal
 *     tensor-product Legendre basis (constructor_basis_tp_orthonormal / constructor_grad_basis_tp_orthonormal,
 *     element/bases.c) and the inverse of its Vandermonde matrix at the solution nodes (element_operators.c);
 *     here cv0_vs_vc = Phi(r_vc) V^-1, d/dr_a: dPhi_a(r_vc) V^-1, faces alike, with V = Phi(r_vs) inverted by
 *     Gauss-Jordan elimination;
 *   - cubature: volume GL with p+1 points per direction (p_c = 2p, CUB_C_DIV2, nodes_operators.c:342-345,589-597),
 *     face GL with p+1 points per face direction, tensor-product order with the first coordinate fastest;
 *     tw1_vt_vc[a] = (d/dr_a cv0)^T diag(w_vc), tw0_vt_fc = cv0_vs_fc^T diag(w_fc) (element_operators.h:26-27);
 *   - geometry (set_up_solver_geometry_T, geometry/geometry_T.c:165-185): the P1 (multilinear) geometry basis is
 *     the order-1 Lagrange basis on the 2^d vertices, formed the same modal way; J = dx/dr at each cubature node,
 *     metrics m_ij = detJ (J^-1)_ji from a Gauss-Jordan inverse (the cofactors of compute_cofactors_T,
 *     geometry_T.c:89-120), jacobian_det_vc = detJ (compute_detJV_T); face normals metrics . n_ref and their
 *     length (compute_normals_T / compute_unit_normals_and_det_T, geometry_T.c:56-140) from side 0 of the face;
 *     the mass matrix per volume is formed in oracle_dg.c (constructor_mass_T);
 *   - connectivity: faces are found by matching the centroids of the volumes' local faces modulo the periodic
 *     box, the two sides ordered by (volume, local face); the right-side face-node order nc_fc by matching
 *     physical face cubature nodes (the role of the reference's nc_fc / permute_Multiarray_T_fc,
 *     compute_face_rlhs_T.c:312-318);
 *   - mesh: the structured periodic box (volume i + nx (j + ny k), vertices in tensor-product order) with the
 *     seeded splitmix64 vertex jitter of the benchmark meshes, or a gmsh 2.2 ASCII file (mesh_readers.c: $Nodes,
 *     $Elements; quadrilateral vertices counter-clockwise, hexahedra bottom then top face), converted to
 *     tensor-product vertex order and mirrored in the last reference direction where the map comes out
 *     left-handed;
 *   - initial and exact solutions: Shu's isentropic vortex (3D: axis along z), the advected sine, the free stream;
 *     L2 errors as SUMMATION_L2_VOL (compute_error.c:545-555) of rho, u, v, (w), p or of u.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_dg.h"

#define OR_GM1 0.4
#define OR_GAMMA 1.4

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* ---- 1D nodes ------------------------------------------------------------------------------------------- */

/* Number of eigenvalues below x of the symmetric tridiagonal matrix with zero diagonal and off-diagonal b[0..n-2]
 * (Sturm sequence of the leading principal minors). */
static int sturm_count(int n, const double* b, double x)
{
	int cnt = 0;
	double q = -x;                       /* d_1 = a_1 - x */
	if (q < 0.0) ++cnt;
	for (int i = 1; i < n; ++i) {
		if (q == 0.0) q = 1e-300;
		q = -x - b[i-1]*b[i-1]/q;
		if (q < 0.0) ++cnt;
	}
	return cnt;
}

/* Eigenvalues (ascending) of that matrix in [-1, 1], each isolated by bisection to the last bit. */
static void tridiag_eigs(int n, const double* b, double* ev)
{
	for (int k = 0; k < n; ++k) {
		double lo = -1.0, hi = 1.0;
		for (int it = 0; it < 200; ++it) {
			const double mid = 0.5*(lo + hi);
			if (mid <= lo || mid >= hi) break;
			if (sturm_count(n,b,mid) > k) hi = mid; else lo = mid;
		}
		ev[k] = 0.5*(lo + hi);
	}
}

/* Legendre P_n(x) and P_n'(x) by the three-term recurrence. */
static void legendre(int n, double x, double* p, double* dp)
{
	double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
	if (n == 0) { *p = 1.0; *dp = 0.0; return; }
	for (int k = 2; k <= n; ++k) {
		const double p2 = ((2.0*k - 1.0)*x*p1 - (k - 1.0)*p0)/k;
		const double d2 = d0 + (2.0*k - 1.0)*p1;       /* P_k' = P_{k-2}' + (2k-1) P_{k-1} */
		p0 = p1; p1 = p2; d0 = d1; d1 = d2;
	}
	*p = p1; *dp = d1;
}

void oracle_nodes_gl(int n, double* x, double* w)
{
	double b[32] = {0};
	for (int k = 1; k < n; ++k) b[k-1] = k/sqrt(4.0*k*k - 1.0);
	tridiag_eigs(n,b,x);
	for (int i = 0; i < n; ++i) {
		double p, dp;
		legendre(n,x[i],&p,&dp);
		w[i] = 2.0/((1.0 - x[i]*x[i])*dp*dp);
	}
}

void oracle_nodes_gll(int n, double* x, double* w)
{
	x[0] = -1.0; x[n-1] = 1.0;
	if (n > 2) {
		double b[32] = {0};
		for (int k = 1; k < n-2; ++k) b[k-1] = sqrt(k*(k + 2.0)/((2.0*k + 1.0)*(2.0*k + 3.0)));
		tridiag_eigs(n-2,b,x+1);
	}
	for (int i = 0; i < n; ++i) {
		double p, dp;
		legendre(n-1,x[i],&p,&dp);
		w[i] = 2.0/(n*(n - 1.0)*p*p);
	}
}

/* ---- modal basis, Vandermonde ------------------------------------------------------------------------------ */

/* orthonormal Legendre phi_k = sqrt(k + 1/2) P_k and its derivative */
static void ortho1(int k, double x, double* v, double* dv)
{
	double p, dp;
	legendre(k,x,&p,&dp);
	const double s = sqrt(k + 0.5);
	*v = s*p; *dv = s*dp;
}

/* Tensor-product orthonormal basis (n1 modes per direction) at point r: val[n_b], grad[d][n_b]. */
static void ortho_tp(int d, int n1, const double* r, double* val, double* grad)
{
	int n_b = 1;
	for (int a = 0; a < d; ++a) n_b *= n1;
	for (int j = 0; j < n_b; ++j) {
		double f[3], df[3];
		for (int a = 0, t = j; a < d; ++a, t /= n1) ortho1(t % n1,r[a],&f[a],&df[a]);
		double v = 1.0;
		for (int a = 0; a < d; ++a) v *= f[a];
		val[j] = v;
		for (int g = 0; g < d; ++g) {
			double gv = 1.0;
			for (int a = 0; a < d; ++a) gv *= (a == g ? df[a] : f[a]);
			grad[(size_t)g*n_b + j] = gv;
		}
	}
}

/* Gauss-Jordan inverse with partial pivoting; returns 0, or -1 for a singular matrix. */
int oracle_gj_invert(int n, const double* a, double* inv)
{
	double* m = zalloc((size_t)n*2*n);
	for (int i = 0; i < n; ++i) {
		for (int j = 0; j < n; ++j) m[(size_t)i*2*n + j] = a[(size_t)i*n + j];
		m[(size_t)i*2*n + n + i] = 1.0;
	}
	for (int c = 0; c < n; ++c) {
		int pr = c;
		for (int i = c+1; i < n; ++i) if (fabs(m[(size_t)i*2*n + c]) > fabs(m[(size_t)pr*2*n + c])) pr = i;
		if (m[(size_t)pr*2*n + c] == 0.0) { free(m); return -1; }
		if (pr != c)
			for (int j = 0; j < 2*n; ++j) { double t = m[(size_t)c*2*n+j]; m[(size_t)c*2*n+j] = m[(size_t)pr*2*n+j]; m[(size_t)pr*2*n+j] = t; }
		const double piv = m[(size_t)c*2*n + c];
		for (int j = 0; j < 2*n; ++j) m[(size_t)c*2*n + j] /= piv;
		for (int i = 0; i < n; ++i) {
			if (i == c) continue;
			const double f = m[(size_t)i*2*n + c];
			if (f == 0.0) continue;
			for (int j = 0; j < 2*n; ++j) m[(size_t)i*2*n + j] -= f*m[(size_t)c*2*n + j];
		}
	}
	for (int i = 0; i < n; ++i)
		for (int j = 0; j < n; ++j) inv[(size_t)i*n + j] = m[(size_t)i*2*n + n + j];
	free(m);
	return 0;
}

/* Lagrange-basis values (and gradients) at n_pt points: out = Phi(r) V^-1, gout[a] = dPhi_a(r) V^-1. */
static void lagrange_at(int d, int n1, const double* vinv, int n_pt, const double* r, double* out, double* gout)
{
	int n_b = 1;
	for (int a = 0; a < d; ++a) n_b *= n1;
	double* val = zalloc((size_t)n_b);
	double* grad = zalloc((size_t)d*n_b);
	for (int q = 0; q < n_pt; ++q) {
		ortho_tp(d,n1,&r[(size_t)q*d],val,grad);
		for (int s = 0; s < n_b; ++s) {
			double acc = 0.0;
			for (int j = 0; j < n_b; ++j) acc += val[j]*vinv[(size_t)j*n_b + s];
			if (out) out[(size_t)q*n_b + s] = acc;
			if (gout)
				for (int a = 0; a < d; ++a) {
					double g = 0.0;
					for (int j = 0; j < n_b; ++j) g += grad[(size_t)a*n_b + j]*vinv[(size_t)j*n_b + s];
					gout[((size_t)a*n_pt + q)*n_b + s] = g;
				}
		}
	}
	free(val); free(grad);
}

/* Inverse Vandermonde matrix of the tensor-product Lagrange basis on the 1D nodes x1 (n1 per direction). */
static double* vandermonde_inverse(int d, int n1, const double* x1)
{
	int n_b = 1;
	for (int a = 0; a < d; ++a) n_b *= n1;
	double* V = zalloc((size_t)n_b*n_b);
	double* vinv = zalloc((size_t)n_b*n_b);
	double* grad = zalloc((size_t)d*n_b);
	for (int s = 0; s < n_b; ++s) {
		double r[3];
		for (int a = 0, t = s; a < d; ++a, t /= n1) r[a] = x1[t % n1];
		ortho_tp(d,n1,r,&V[(size_t)s*n_b],grad);
	}
	oracle_gj_invert(n_b,V,vinv);
	free(V); free(grad);
	return vinv;
}

/* d/dr_a of the order-p tensor-product Lagrange basis on the GLL nodes at n_pt points r: out[a][q][s]. */
void oracle_grad_operator(int d, int p, int n_pt, const double* r, double* out)
{
	double gll[16], w[16];
	oracle_nodes_gll(p + 1,gll,w);
	double* vinv = vandermonde_inverse(d,p + 1,gll);
	lagrange_at(d,p + 1,vinv,n_pt,r,NULL,out);
	free(vinv);
}

/* ---- element operators ------------------------------------------------------------------------------------- */

static int build_ops(int d, int p, struct dpg_element_ops* ops)
{
	memset(ops,0,sizeof *ops);
	const int n1 = p+1;
	int n_s = 1, n_fc = 1;
	for (int a = 0; a < d; ++a) n_s *= n1;
	for (int a = 0; a < d-1; ++a) n_fc *= n1;
	const int n_c = n_s, n_fl = 2*d, n_ve = 1 << d;
	ops->e_type = (d == 2 ? DPG_QUAD : DPG_HEX); ops->d = d; ops->p = p;
	ops->n_s = n_s; ops->n_c = n_c; ops->n_fl = n_fl; ops->n_fc = n_fc; ops->n_ve = n_ve;

	double gll[16], wgll[16], gl[16], wgl[16], vtx[2] = {-1.0, 1.0};
	oracle_nodes_gll(n1,gll,wgll);
	oracle_nodes_gl(n1,gl,wgl);

	ops->rst_vs = zalloc((size_t)n_s*d);
	ops->rst_vc = zalloc((size_t)n_c*d);
	ops->w_vc = zalloc((size_t)n_c);
	for (int s = 0; s < n_s; ++s) {
		double w = 1.0;
		for (int a = 0, t = s; a < d; ++a, t /= n1) {
			ops->rst_vs[(size_t)s*d + a] = gll[t % n1];
			ops->rst_vc[(size_t)s*d + a] = gl[t % n1];
			w *= wgl[t % n1];
		}
		ops->w_vc[s] = w;
	}
	ops->w_fc = zalloc((size_t)n_fc);
	ops->rst_fc = zalloc((size_t)n_fl*n_fc*d);
	ops->normals_ref = zalloc((size_t)n_fl*d);
	for (int q = 0; q < n_fc; ++q) {
		double w = 1.0;
		for (int a = 0, t = q; a < d-1; ++a, t /= n1) w *= wgl[t % n1];
		ops->w_fc[q] = w;
	}
	for (int lf = 0; lf < n_fl; ++lf) {
		const int af = lf/2;
		const double side = (lf & 1) ? 1.0 : -1.0;
		ops->normals_ref[(size_t)lf*d + af] = side;
		for (int q = 0; q < n_fc; ++q)
			for (int a = 0, t = q; a < d; ++a) {
				double c;
				if (a == af) c = side;
				else { c = gl[t % n1]; t /= n1; }
				ops->rst_fc[((size_t)lf*n_fc + q)*d + a] = c;
			}
	}

	double* vinv = vandermonde_inverse(d,n1,gll);
	ops->cv0_vs_vc = zalloc((size_t)n_c*n_s);
	double* dv = zalloc((size_t)d*n_c*n_s);
	lagrange_at(d,n1,vinv,n_c,ops->rst_vc,ops->cv0_vs_vc,dv);
	ops->tw1_vt_vc = zalloc((size_t)d*n_s*n_c);
	for (int a = 0; a < d; ++a)
		for (int s = 0; s < n_s; ++s)
			for (int c = 0; c < n_c; ++c)
				ops->tw1_vt_vc[((size_t)a*n_s + s)*n_c + c] = dv[((size_t)a*n_c + c)*n_s + s]*ops->w_vc[c];
	free(dv);
	ops->cv0_vs_fc = zalloc((size_t)n_fl*n_fc*n_s);
	lagrange_at(d,n1,vinv,n_fl*n_fc,ops->rst_fc,ops->cv0_vs_fc,NULL);
	ops->tw0_vt_fc = zalloc((size_t)n_fl*n_s*n_fc);
	for (int lf = 0; lf < n_fl; ++lf)
		for (int s = 0; s < n_s; ++s)
			for (int q = 0; q < n_fc; ++q)
				ops->tw0_vt_fc[((size_t)lf*n_s + s)*n_fc + q] = ops->cv0_vs_fc[((size_t)lf*n_fc + q)*n_s + s]*ops->w_fc[q];
	free(vinv);

	/* P1 geometry basis: order-1 Lagrange on the vertices */
	double* ginv = vandermonde_inverse(d,2,vtx);
	ops->cv0_vv_vc = zalloc((size_t)n_c*n_ve);
	ops->cv1_vv_vc = zalloc((size_t)d*n_c*n_ve);
	lagrange_at(d,2,ginv,n_c,ops->rst_vc,ops->cv0_vv_vc,ops->cv1_vv_vc);
	ops->cv0_vv_fc = zalloc((size_t)n_fl*n_fc*n_ve);
	ops->cv1_vv_fc = zalloc((size_t)n_fl*d*n_fc*n_ve);
	for (int lf = 0; lf < n_fl; ++lf)
		lagrange_at(d,2,ginv,n_fc,&ops->rst_fc[(size_t)lf*n_fc*d],&ops->cv0_vv_fc[(size_t)lf*n_fc*n_ve],
		            &ops->cv1_vv_fc[(size_t)lf*d*n_fc*n_ve]);
	free(ginv);
	return 0;
}

/* ---- TRI (the reference triangle v0 = (-1, -1/sqrt3), v1 = (1, -1/sqrt3), v2 = (0, 2/sqrt3); face f opposite
 * vertex f, f_ve = {1,2}, {0,2}, {0,1}: element.c:453-466 of the reference) --------------------------------------- */
#define OR_S3 1.7320508075688772
static const double TRI_VX[3] = {-1.0, 1.0, 0.0}, TRI_VY[3] = {-1.0/OR_S3, -1.0/OR_S3, 2.0/OR_S3};
static const int TRI_FVE[3][2] = {{1,2}, {0,2}, {0,1}};

/* barycentric coordinates of (x, y) and their gradients gl[k][a] */
static void tri_bary(double x, double y, double* l, double (*gl)[2])
{
	/* solve [v1 - v0, v2 - v0] (l1, l2) = (x, y) - v0 */
	const double a = TRI_VX[1] - TRI_VX[0], b = TRI_VX[2] - TRI_VX[0];
	const double c = TRI_VY[1] - TRI_VY[0], e = TRI_VY[2] - TRI_VY[0];
	const double det = a*e - b*c, px = x - TRI_VX[0], py = y - TRI_VY[0];
	l[1] = (e*px - b*py)/det;
	l[2] = (-c*px + a*py)/det;
	l[0] = 1.0 - l[1] - l[2];
	if (gl) {
		gl[1][0] = e/det;  gl[1][1] = -b/det;
		gl[2][0] = -c/det; gl[2][1] = a/det;
		gl[0][0] = -gl[1][0] - gl[2][0]; gl[0][1] = -gl[1][1] - gl[2][1];
	}
}

/* warp of the equidistant nodes onto the GLL nodes at r (the interpolant of gll_i - eq_i through the equidistant
 * nodes, formed here through a Legendre Vandermonde solve), divided by 1 - r^2 inside (-1, 1) */
static double tri_warp(int p, double r)
{
	const int n = p + 1;
	double gll[16], w[16], V[256], Vinv[256], eq[16];
	oracle_nodes_gll(n,gll,w);
	for (int i = 0; i < n; ++i) eq[i] = -1.0 + 2.0*i/p;
	for (int i = 0; i < n; ++i)
		for (int k = 0; k < n; ++k) { double pk, dpk; legendre(k,eq[i],&pk,&dpk); V[i*n + k] = pk; }
	oracle_gj_invert(n,V,Vinv);
	/* interpolant coefficients c = Vinv (gll - eq), evaluated at r */
	double out = 0.0;
	for (int k = 0; k < n; ++k) {
		double ck = 0.0;
		for (int i = 0; i < n; ++i) ck += Vinv[k*n + i]*(gll[i] - eq[i]);
		double pk, dpk;
		legendre(k,r,&pk,&dpk);
		out += ck*pk;
	}
	if (fabs(r) >= 1.0 - 1e-10) return 0.0;
	return out/(1.0 - r*r);
}

/* alpha-optimised warp-and-blend nodes (Warburton 2006), rows of increasing barycentric coordinate of v2 */
static void tri_nodes(int p, double* xy)
{
	static const double alpha_opt[15] = {0.0, 0.0, 1.4152, 0.1001, 0.2751, 0.9800, 1.0999, 1.2832, 1.3648, 1.4773,
	                                     1.4959, 1.5743, 1.5770, 1.6223, 1.6258};
	const double al = p <= 15 ? alpha_opt[p-1] : 5.0/3.0;
	int k = 0;
	for (int n = 0; n <= p; ++n)
		for (int m = 0; m + n <= p; ++m, ++k) {
			const double la = (double)n/p, lc = (double)m/p, lb = 1.0 - la - lc;   /* weights of v2, v1, v0 */
			double x = lb*TRI_VX[0] + lc*TRI_VX[1] + la*TRI_VX[2];
			double y = lb*TRI_VY[0] + lc*TRI_VY[1] + la*TRI_VY[2];
			const double d1 = 4.0*lb*lc*tri_warp(p,lc - lb)*(1.0 + al*al*la*la);
			const double d2 = 4.0*la*lc*tri_warp(p,la - lc)*(1.0 + al*al*lb*lb);
			const double d3 = 4.0*la*lb*tri_warp(p,lb - la)*(1.0 + al*al*lc*lc);
			/* the three warps along the edge directions v0->v1, v1->v2, v2->v0 (unit vectors at 0, 120, 240 deg) */
			x += d1 - 0.5*d2 - 0.5*d3;
			y += 0.5*OR_S3*d2 - 0.5*OR_S3*d3;
			xy[2*k] = x; xy[2*k+1] = y;
		}
}

/* monomials x^i y^j (i + j <= p) and their gradients at (x, y) */
static void tri_monomials(int p, double x, double y, double* m, double* mx, double* my)
{
	int k = 0;
	for (int i = 0; i <= p; ++i)
		for (int j = 0; i + j <= p; ++j, ++k) {
			m[k] = pow(x,i)*pow(y,j);
			mx[k] = i ? i*pow(x,i-1)*pow(y,j) : 0.0;
			my[k] = j ? j*pow(x,i)*pow(y,j-1) : 0.0;
		}
}

static int build_ops_tri(int p, struct dpg_element_ops* ops, int n_rule, const double* rule)
{
	memset(ops,0,sizeof *ops);
	const int d = 2, n_s = (p+1)*(p+2)/2, nq = p + 2, n_c = (n_rule > 0 ? n_rule : nq*nq), n_fc = p + 1, n_fl = 3, n_ve = 3;
	ops->e_type = DPG_TRI; ops->d = d; ops->p = p;
	ops->n_s = n_s; ops->n_c = n_c; ops->n_fl = n_fl; ops->n_fc = n_fc; ops->n_ve = n_ve;
	ops->rst_vs = zalloc((size_t)n_s*d);
	tri_nodes(p,ops->rst_vs);
	/* Stroud's collapsed Gauss rule: the square [-1,1]^2 onto the triangle v0, v1, v2 by
	 * x = v0 + (1+a)(1-b)/4 (v1 - v0) + (1+b)/2 (v2 - v0), Jacobian |v1-v0 x v2-v0| (1-b)/8 */
	double g[16], wg[16];
	oracle_nodes_gl(nq,g,wg);
	const double area2 = (TRI_VX[1]-TRI_VX[0])*(TRI_VY[2]-TRI_VY[0]) - (TRI_VX[2]-TRI_VX[0])*(TRI_VY[1]-TRI_VY[0]);
	ops->rst_vc = zalloc((size_t)n_c*d);
	ops->w_vc = zalloc((size_t)n_c);
	for (int c = 0; c < n_rule; ++c) {   /* a given rule: x = sum_k l_k v_k, weight w |triangle| */
		const double* l = &rule[(size_t)c*4];
		ops->rst_vc[2*c]   = l[0]*TRI_VX[0] + l[1]*TRI_VX[1] + l[2]*TRI_VX[2];
		ops->rst_vc[2*c+1] = l[0]*TRI_VY[0] + l[1]*TRI_VY[1] + l[2]*TRI_VY[2];
		ops->w_vc[c] = l[3]*0.5*fabs(area2);
	}
	for (int ib = 0; ib < (n_rule > 0 ? 0 : nq); ++ib)
		for (int ia = 0; ia < nq; ++ia) {
			const int c = ib*nq + ia;
			const double s1 = 0.25*(1.0 + g[ia])*(1.0 - g[ib]), s2 = 0.5*(1.0 + g[ib]);
			ops->rst_vc[2*c]   = TRI_VX[0] + s1*(TRI_VX[1]-TRI_VX[0]) + s2*(TRI_VX[2]-TRI_VX[0]);
			ops->rst_vc[2*c+1] = TRI_VY[0] + s1*(TRI_VY[1]-TRI_VY[0]) + s2*(TRI_VY[2]-TRI_VY[0]);
			ops->w_vc[c] = wg[ia]*wg[ib]*area2*(1.0 - g[ib])/8.0;
		}
	double gf[16], wf[16];
	oracle_nodes_gl(n_fc,gf,wf);
	ops->w_fc = zalloc((size_t)n_fc);
	for (int q = 0; q < n_fc; ++q) ops->w_fc[q] = wf[q];
	ops->rst_fc = zalloc((size_t)n_fl*n_fc*d);
	ops->normals_ref = zalloc((size_t)n_fl*d);
	for (int f = 0; f < n_fl; ++f) {
		const int a = TRI_FVE[f][0], b = TRI_FVE[f][1];
		for (int q = 0; q < n_fc; ++q) {
			ops->rst_fc[((size_t)f*n_fc + q)*d]     = 0.5*(1.0 - gf[q])*TRI_VX[a] + 0.5*(1.0 + gf[q])*TRI_VX[b];
			ops->rst_fc[((size_t)f*n_fc + q)*d + 1] = 0.5*(1.0 - gf[q])*TRI_VY[a] + 0.5*(1.0 + gf[q])*TRI_VY[b];
		}
		/* the outward normal of the edge opposite vertex f is -grad l_f / |grad l_f| */
		double l[3], gl[3][2];
		tri_bary(0.0,0.0,l,gl);
		const double len = sqrt(gl[f][0]*gl[f][0] + gl[f][1]*gl[f][1]);
		ops->normals_ref[f*d] = -gl[f][0]/len; ops->normals_ref[f*d+1] = -gl[f][1]/len;
	}
	/* Lagrange basis of the nodes from the monomial Vandermonde matrix */
	double* V = zalloc((size_t)n_s*n_s);
	double* Vi = zalloc((size_t)n_s*n_s);
	double m[64], mx[64], my[64];
	for (int i = 0; i < n_s; ++i) {
		tri_monomials(p,ops->rst_vs[2*i],ops->rst_vs[2*i+1],m,mx,my);
		for (int k = 0; k < n_s; ++k) V[(size_t)i*n_s + k] = m[k];
	}
	if (oracle_gj_invert(n_s,V,Vi)) { free(V); free(Vi); return -1; }
	ops->cv0_vs_vc = zalloc((size_t)n_c*n_s);
	ops->tw1_vt_vc = zalloc((size_t)d*n_s*n_c);
	ops->cv0_vs_fc = zalloc((size_t)n_fl*n_fc*n_s);
	ops->tw0_vt_fc = zalloc((size_t)n_fl*n_s*n_fc);
	ops->cv0_vv_vc = zalloc((size_t)n_c*n_ve);
	ops->cv1_vv_vc = zalloc((size_t)d*n_c*n_ve);
	ops->cv0_vv_fc = zalloc((size_t)n_fl*n_fc*n_ve);
	ops->cv1_vv_fc = zalloc((size_t)n_fl*d*n_fc*n_ve);
	for (int c = 0; c < n_c; ++c) {
		tri_monomials(p,ops->rst_vc[2*c],ops->rst_vc[2*c+1],m,mx,my);
		for (int s2 = 0; s2 < n_s; ++s2) {
			double v = 0.0, vx = 0.0, vy = 0.0;
			for (int k = 0; k < n_s; ++k) { v += m[k]*Vi[(size_t)k*n_s + s2]; vx += mx[k]*Vi[(size_t)k*n_s + s2]; vy += my[k]*Vi[(size_t)k*n_s + s2]; }
			ops->cv0_vs_vc[(size_t)c*n_s + s2] = v;
			ops->tw1_vt_vc[((size_t)0*n_s + s2)*n_c + c] = vx*ops->w_vc[c];
			ops->tw1_vt_vc[((size_t)1*n_s + s2)*n_c + c] = vy*ops->w_vc[c];
		}
		double l[3], gl[3][2];
		tri_bary(ops->rst_vc[2*c],ops->rst_vc[2*c+1],l,gl);
		for (int k = 0; k < 3; ++k) {
			ops->cv0_vv_vc[(size_t)c*n_ve + k] = l[k];
			for (int a = 0; a < d; ++a) ops->cv1_vv_vc[((size_t)a*n_c + c)*n_ve + k] = gl[k][a];
		}
	}
	for (int f = 0; f < n_fl; ++f)
		for (int q = 0; q < n_fc; ++q) {
			const double* r = &ops->rst_fc[((size_t)f*n_fc + q)*d];
			tri_monomials(p,r[0],r[1],m,mx,my);
			for (int s2 = 0; s2 < n_s; ++s2) {
				double v = 0.0;
				for (int k = 0; k < n_s; ++k) v += m[k]*Vi[(size_t)k*n_s + s2];
				ops->cv0_vs_fc[((size_t)f*n_fc + q)*n_s + s2] = v;
				ops->tw0_vt_fc[((size_t)f*n_s + s2)*n_fc + q] = v*ops->w_fc[q];
			}
			double l[3], gl[3][2];
			tri_bary(r[0],r[1],l,gl);
			for (int k = 0; k < 3; ++k) {
				ops->cv0_vv_fc[((size_t)f*n_fc + q)*n_ve + k] = l[k];
				for (int a = 0; a < d; ++a) ops->cv1_vv_fc[(((size_t)f*d + a)*n_fc + q)*n_ve + k] = gl[k][a];
			}
		}
	free(V); free(Vi);
	return 0;
}

/* ---- TET (the reference tetrahedron v0 = (-1, -1/sqrt3, -1/sqrt6), v1 = (1, -1/sqrt3, -1/sqrt6),
 * v2 = (0, 2/sqrt3, -1/sqrt6), v3 = (0, 0, 3/sqrt6) of nodes.c:508-515; face f opposite vertex f with the face
 * vertices f_ve = {2,3,1}, {2,3,0}, {0,1,3}, {0,1,2} of element.c) ---------------------------------------------- */
#define OR_S6 2.4494897427831779
static const double TET_V[4][3] = {{-1.0, -1.0/OR_S3, -1.0/OR_S6}, {1.0, -1.0/OR_S3, -1.0/OR_S6},
                                   {0.0, 2.0/OR_S3, -1.0/OR_S6}, {0.0, 0.0, 3.0/OR_S6}};
static const int TET_FVE[4][3] = {{2,3,1}, {2,3,0}, {0,1,3}, {0,1,2}};

/* barycentric coordinates of x (Cramer's rule on [v1 - v0, v2 - v0, v3 - v0]) and their gradients */
static void tet_bary(const double* x, double* l, double (*gl)[3])
{
	double A[9], Ai[9];
	for (int a = 0; a < 3; ++a)
		for (int k = 0; k < 3; ++k) A[a*3 + k] = TET_V[k+1][a] - TET_V[0][a];
	oracle_gj_invert(3,A,Ai);
	l[0] = 1.0;
	for (int k = 0; k < 3; ++k) {
		double s = 0.0;
		for (int a = 0; a < 3; ++a) s += Ai[k*3 + a]*(x[a] - TET_V[0][a]);
		l[k+1] = s;
		l[0] -= s;
		if (gl) for (int a = 0; a < 3; ++a) gl[k+1][a] = Ai[k*3 + a];
	}
	if (gl) for (int a = 0; a < 3; ++a) gl[0][a] = -(gl[1][a] + gl[2][a] + gl[3][a]);
}

/* equally spaced nodes of order p: barycentric (p-a-b-c, a, b, c)/p, c outer, then b, then a */
static void tet_nodes(int p, double* xyz)
{
	int n = 0;
	for (int c = 0; c <= p; ++c)
		for (int b = 0; b + c <= p; ++b)
			for (int a = 0; a + b + c <= p; ++a, ++n) {
				const double l[4] = {(double)(p - a - b - c)/p, (double)a/p, (double)b/p, (double)c/p};
				for (int d = 0; d < 3; ++d) xyz[3*n + d] = l[0]*TET_V[0][d] + l[1]*TET_V[1][d] + l[2]*TET_V[2][d] + l[3]*TET_V[3][d];
			}
}

/* monomials l1^a l2^b l3^c (a + b + c <= p) in the barycentric coordinates and their x gradients */
static void tet_monomials(int p, const double* x, double* m, double (*gm)[3])
{
	double l[4], gl[4][3];
	tet_bary(x,l,gl);
	int k = 0;
	for (int a = 0; a <= p; ++a)
		for (int b = 0; a + b <= p; ++b)
			for (int c = 0; a + b + c <= p; ++c, ++k) {
				const double pa = pow(l[1],a), pb = pow(l[2],b), pc = pow(l[3],c);
				m[k] = pa*pb*pc;
				if (gm) {
					const double da = a ? a*pow(l[1],a-1)*pb*pc : 0.0;
					const double db = b ? b*pa*pow(l[2],b-1)*pc : 0.0;
					const double dc = c ? c*pa*pb*pow(l[3],c-1) : 0.0;
					for (int d = 0; d < 3; ++d) gm[k][d] = da*gl[1][d] + db*gl[2][d] + dc*gl[3][d];
				}
			}
}

/* Lagrange basis (values, gradients [3][n_pt][n_s]) of the order-p nodes at n_pt points */
static int tet_lagrange(int p, const double* nodes, int n_pt, const double* x, double* out, double* gout)
{
	const int n_s = (p+1)*(p+2)*(p+3)/6;
	double* V = zalloc((size_t)n_s*n_s);
	double* Vi = zalloc((size_t)n_s*n_s);
	double m[35], gm[35][3];
	for (int i = 0; i < n_s; ++i) {
		tet_monomials(p,&nodes[3*i],m,NULL);
		for (int k = 0; k < n_s; ++k) V[(size_t)i*n_s + k] = m[k];
	}
	if (oracle_gj_invert(n_s,V,Vi)) { free(V); free(Vi); return -1; }
	for (int t = 0; t < n_pt; ++t) {
		tet_monomials(p,&x[3*t],m,gm);
		for (int j = 0; j < n_s; ++j) {
			double v = 0.0, g[3] = {0.0, 0.0, 0.0};
			for (int k = 0; k < n_s; ++k) {
				const double c = Vi[(size_t)k*n_s + j];
				v += m[k]*c;
				for (int d = 0; d < 3; ++d) g[d] += gm[k][d]*c;
			}
			if (out) out[(size_t)t*n_s + j] = v;
			if (gout) for (int d = 0; d < 3; ++d) gout[((size_t)d*n_pt + t)*n_s + j] = g[d];
		}
	}
	free(V); free(Vi);
	return 0;
}

/* A symmetric triangle rule (weights summing to 1, barycentric points): Stroud's collapsed Gauss rule with p + 2
 * points per direction (exact to 2p + 1) averaged over the six permutations of the barycentric coordinates, points
 * that coincide merged; pts[n][3], w[n]; returns n */
static int tri_rule_symmetric(int p, double (*pts)[3], double* w)
{
	const int nq = p + 2;
	double g[16], wg[16];
	oracle_nodes_gl(nq,g,wg);
	static const int perm[6][3] = {{0,1,2}, {0,2,1}, {1,0,2}, {1,2,0}, {2,0,1}, {2,1,0}};
	int n = 0;
	for (int ib = 0; ib < nq; ++ib)
		for (int ia = 0; ia < nq; ++ia) {
			const double l1 = 0.25*(1.0 + g[ia])*(1.0 - g[ib]), l2 = 0.5*(1.0 + g[ib]);
			const double bl[3] = {1.0 - l1 - l2, l1, l2};
			const double wt = wg[ia]*wg[ib]*(1.0 - g[ib])/8.0*2.0/6.0;   /* unit-area weights / 6 */
			for (int q = 0; q < 6; ++q) {
				const double c[3] = {bl[perm[q][0]], bl[perm[q][1]], bl[perm[q][2]]};
				int found = -1;
				for (int k = 0; k < n && found < 0; ++k)
					if (fabs(pts[k][0] - c[0]) < 1e-14 && fabs(pts[k][1] - c[1]) < 1e-14) found = k;
				if (found >= 0) { w[found] += wt; continue; }
				pts[n][0] = c[0]; pts[n][1] = c[1]; pts[n][2] = c[2]; w[n] = wt; ++n;
			}
		}
	return n;
}

static int build_ops_tet(int p, struct dpg_element_ops* ops, int n_rule, const double* rule, int n_frule,
                         const double* frule)
{
	memset(ops,0,sizeof *ops);
	if (p < 1 || p > 4) return -1;
	const int d = 3, n_s = (p+1)*(p+2)*(p+3)/6, nq = p + 2, n_c = (n_rule > 0 ? n_rule : nq*nq*nq), n_fl = 4, n_ve = 4;
	const int n_fmax = (n_frule > 6*nq*nq ? n_frule : 6*nq*nq);
	double (*fp)[3] = malloc(sizeof *fp*n_fmax);
	double* fw = zalloc((size_t)n_fmax);
	int n_fc = 0;
	if (n_frule > 0) {
		for (int q = 0; q < n_frule; ++q) {
			for (int k = 0; k < 3; ++k) fp[q][k] = frule[(size_t)q*4 + k];
			fw[q] = frule[(size_t)q*4 + 3];
		}
		n_fc = n_frule;
	} else {
		n_fc = tri_rule_symmetric(p,fp,fw);
	}
	ops->e_type = DPG_TET; ops->d = d; ops->p = p;
	ops->n_s = n_s; ops->n_c = n_c; ops->n_fl = n_fl; ops->n_fc = n_fc; ops->n_ve = n_ve;
	ops->rst_vs = zalloc((size_t)n_s*d);
	tet_nodes(p,ops->rst_vs);
	/* Stroud's conical product rule: x = v0 + s1 (v1 - v0) + s2 (v2 - v0) + s3 (v3 - v0) with
	 * s3 = (1+c)/2, s2 = (1+b)(1-c)/4, s1 = (1+a)(1-b)(1-c)/8 on Gauss points; Jacobian (1-b)(1-c)^2/64 |det| */
	double g[16], wg[16], A[9];
	oracle_nodes_gl(nq,g,wg);
	for (int a = 0; a < 3; ++a)
		for (int k = 0; k < 3; ++k) A[a*3 + k] = TET_V[k+1][a] - TET_V[0][a];
	const double det = fabs(A[0]*(A[4]*A[8] - A[5]*A[7]) - A[1]*(A[3]*A[8] - A[5]*A[6]) + A[2]*(A[3]*A[7] - A[4]*A[6]));
	ops->rst_vc = zalloc((size_t)n_c*d);
	ops->w_vc = zalloc((size_t)n_c);
	for (int cc = 0; cc < n_rule; ++cc) {   /* a given rule: x = sum_k l_k v_k, weight w |tetrahedron| */
		const double* l = &rule[(size_t)cc*5];
		for (int dd = 0; dd < 3; ++dd)
			ops->rst_vc[3*cc + dd] = l[0]*TET_V[0][dd] + l[1]*TET_V[1][dd] + l[2]*TET_V[2][dd] + l[3]*TET_V[3][dd];
		ops->w_vc[cc] = l[4]*det/6.0;
	}
	for (int ic = 0; ic < (n_rule > 0 ? 0 : nq); ++ic)
		for (int ib = 0; ib < nq; ++ib)
			for (int ia = 0; ia < nq; ++ia) {
				const int cc = (ic*nq + ib)*nq + ia;
				const double s3 = 0.5*(1.0 + g[ic]), s2 = 0.25*(1.0 + g[ib])*(1.0 - g[ic]);
				const double s1 = 0.125*(1.0 + g[ia])*(1.0 - g[ib])*(1.0 - g[ic]);
				for (int dd = 0; dd < 3; ++dd)
					ops->rst_vc[3*cc + dd] = TET_V[0][dd] + s1*A[dd*3] + s2*A[dd*3 + 1] + s3*A[dd*3 + 2];
				ops->w_vc[cc] = wg[ia]*wg[ib]*wg[ic]*(1.0 - g[ib])*(1.0 - g[ic])*(1.0 - g[ic])/64.0*det;
			}
	/* faces: the symmetric rule on each face, weights of the face's area (equilateral, side 2: sqrt3) */
	ops->w_fc = zalloc((size_t)n_fc);
	ops->rst_fc = zalloc((size_t)n_fl*n_fc*d);
	ops->normals_ref = zalloc((size_t)n_fl*d);
	for (int q = 0; q < n_fc; ++q) ops->w_fc[q] = fw[q]*OR_S3;
	double l0[4], gl0[4][3];
	tet_bary(TET_V[0],l0,gl0);
	for (int f = 0; f < n_fl; ++f) {
		for (int q = 0; q < n_fc; ++q)
			for (int dd = 0; dd < 3; ++dd)
				ops->rst_fc[((size_t)f*n_fc + q)*d + dd] = fp[q][0]*TET_V[TET_FVE[f][0]][dd] + fp[q][1]*TET_V[TET_FVE[f][1]][dd]
				                                          + fp[q][2]*TET_V[TET_FVE[f][2]][dd];
		const double len = sqrt(gl0[f][0]*gl0[f][0] + gl0[f][1]*gl0[f][1] + gl0[f][2]*gl0[f][2]);
		for (int dd = 0; dd < 3; ++dd) ops->normals_ref[f*d + dd] = -gl0[f][dd]/len;
	}
	free(fp); free(fw);
	ops->cv0_vs_vc = zalloc((size_t)n_c*n_s);
	ops->tw1_vt_vc = zalloc((size_t)d*n_s*n_c);
	ops->cv0_vs_fc = zalloc((size_t)n_fl*n_fc*n_s);
	ops->tw0_vt_fc = zalloc((size_t)n_fl*n_s*n_fc);
	double* gv = zalloc((size_t)d*n_c*n_s);
	if (tet_lagrange(p,ops->rst_vs,n_c,ops->rst_vc,ops->cv0_vs_vc,gv) ||
	    tet_lagrange(p,ops->rst_vs,n_fl*n_fc,ops->rst_fc,ops->cv0_vs_fc,NULL)) { free(gv); return -1; }
	for (int dd = 0; dd < d; ++dd)
		for (int s2 = 0; s2 < n_s; ++s2)
			for (int cc = 0; cc < n_c; ++cc)
				ops->tw1_vt_vc[((size_t)dd*n_s + s2)*n_c + cc] = gv[((size_t)dd*n_c + cc)*n_s + s2]*ops->w_vc[cc];
	free(gv);
	for (int f = 0; f < n_fl; ++f)
		for (int s2 = 0; s2 < n_s; ++s2)
			for (int q = 0; q < n_fc; ++q)
				ops->tw0_vt_fc[((size_t)f*n_s + s2)*n_fc + q] = ops->cv0_vs_fc[((size_t)f*n_fc + q)*n_s + s2]*ops->w_fc[q];
	ops->cv0_vv_vc = zalloc((size_t)n_c*n_ve);
	ops->cv1_vv_vc = zalloc((size_t)d*n_c*n_ve);
	ops->cv0_vv_fc = zalloc((size_t)n_fl*n_fc*n_ve);
	ops->cv1_vv_fc = zalloc((size_t)n_fl*d*n_fc*n_ve);
	double l[4], gl[4][3];
	for (int cc = 0; cc < n_c; ++cc) {
		tet_bary(&ops->rst_vc[3*cc],l,gl);
		for (int k = 0; k < 4; ++k) {
			ops->cv0_vv_vc[(size_t)cc*n_ve + k] = l[k];
			for (int dd = 0; dd < d; ++dd) ops->cv1_vv_vc[((size_t)dd*n_c + cc)*n_ve + k] = gl[k][dd];
		}
	}
	for (int f = 0; f < n_fl; ++f)
		for (int q = 0; q < n_fc; ++q) {
			tet_bary(&ops->rst_fc[((size_t)f*n_fc + q)*d],l,gl);
			for (int k = 0; k < 4; ++k) {
				ops->cv0_vv_fc[((size_t)f*n_fc + q)*n_ve + k] = l[k];
				for (int dd = 0; dd < d; ++dd) ops->cv1_vv_fc[(((size_t)f*d + dd)*n_fc + q)*n_ve + k] = gl[k][dd];
			}
		}
	return 0;
}

static void free_ops(struct dpg_element_ops* o)
{
	free(o->rst_vs); free(o->rst_vc); free(o->w_vc); free(o->rst_fc); free(o->w_fc); free(o->normals_ref);
	free(o->cv0_vs_vc); free(o->tw1_vt_vc); free(o->cv0_vs_fc); free(o->tw0_vt_fc); free(o->cv0_vv_vc);
	free(o->cv1_vv_vc); free(o->cv0_vv_fc); free(o->cv1_vv_fc); free(o->m_inv_ref); free(o->ccBS0_vs_vs);
	free(o->ccSB0_vs_vs); free(o->bez1); free(o->bez1_inv);
	for (int k = 0; k <= DPG_P_MAX; ++k) { free(o->cv0_vs_fcp[k]); free(o->tw0_vt_fcp[k]); }
	memset(o,0,sizeof *o);
}

/* Mixed orders: the order-p basis of ov at the face cubature nodes of of (order p_f > p), its own Lagrange basis
 * (TRI: monomial Vandermonde; QUAD/HEX: orthonormal tensor-product Vandermonde on the GLL nodes) evaluated there, as
 * the reference's cv0_vs_fc[.][.][.][p_f][p] (compute_face_rlhs_T.c:67-80); tw0 = phi^T diag(w_fc(p_f)). */
static int face_ops_higher(struct dpg_element_ops* ov, const struct dpg_element_ops* of)
{
	const int p = ov->p, p_f = of->p, d = ov->d, n_s = ov->n_s, n_fl = ov->n_fl, n_fc = of->n_fc, n_pt = n_fl*n_fc;
	if (p_f <= p || p_f > DPG_P_MAX) return -1;
	if (ov->cv0_vs_fcp[p_f]) return 0;
	double* phi = zalloc((size_t)n_pt*n_s);
	if (ov->e_type == DPG_TET) {
		if (tet_lagrange(p,ov->rst_vs,n_pt,of->rst_fc,phi,NULL)) { free(phi); return -1; }
	} else if (ov->e_type == DPG_TRI) {
		double* V = zalloc((size_t)n_s*n_s);
		double* Vi = zalloc((size_t)n_s*n_s);
		double m[64], mx[64], my[64];
		for (int i = 0; i < n_s; ++i) {
			tri_monomials(p,ov->rst_vs[2*i],ov->rst_vs[2*i+1],m,mx,my);
			for (int k = 0; k < n_s; ++k) V[(size_t)i*n_s + k] = m[k];
		}
		if (oracle_gj_invert(n_s,V,Vi)) { free(V); free(Vi); free(phi); return -1; }
		for (int t = 0; t < n_pt; ++t) {
			tri_monomials(p,of->rst_fc[2*t],of->rst_fc[2*t+1],m,mx,my);
			for (int s2 = 0; s2 < n_s; ++s2) {
				double v = 0.0;
				for (int k = 0; k < n_s; ++k) v += m[k]*Vi[(size_t)k*n_s + s2];
				phi[(size_t)t*n_s + s2] = v;
			}
		}
		free(V); free(Vi);
	} else {
		double gll[16], w[16];
		oracle_nodes_gll(p + 1,gll,w);
		double* vinv = vandermonde_inverse(d,p + 1,gll);
		lagrange_at(d,p + 1,vinv,n_pt,of->rst_fc,phi,NULL);
		free(vinv);
	}
	double* tw0 = zalloc((size_t)n_fl*n_s*n_fc);
	for (int lf = 0; lf < n_fl; ++lf)
		for (int s2 = 0; s2 < n_s; ++s2)
			for (int q = 0; q < n_fc; ++q)
				tw0[((size_t)lf*n_s + s2)*n_fc + q] = phi[((size_t)lf*n_fc + q)*n_s + s2]*of->w_fc[q];
	ov->cv0_vs_fcp[p_f] = phi;
	ov->tw0_vt_fcp[p_f] = tw0;
	return 0;
}

/* ---- meshes ------------------------------------------------------------------------------------------------ */

struct or_mesh { int d, n_vol; double* xyz_ve; double lo[3], hi[3]; int geom; };

static uint64_t splitmix(uint64_t* s)
{
	uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30))*0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27))*0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

static int mesh_box(const struct oracle_params* prm, struct or_mesh* m)
{
	const int d = prm->d;
	const int nx = prm->n_elem[0], ny = prm->n_elem[1], nz = (d == 3 ? prm->n_elem[2] : 1);
	m->d = d; m->n_vol = nx*ny*nz;
	int wall[3] = {0,0,0};   /* a direction with boundary conditions: no periodic image, vertices stay on the walls */
	for (int a = 0; a < d; ++a) wall[a] = (prm->bc_side[2*a] != 0);
	for (int a = 0; a < 3; ++a) { m->lo[a] = prm->lo[a]; m->hi[a] = (a < d && wall[a]) ? prm->lo[a] : prm->hi[a]; }
	m->xyz_ve = zalloc((size_t)m->n_vol*DPG_NVE_MAX*3);
	double* jit = zalloc((size_t)nx*ny*nz*3);
	double h[3] = {0,0,0};
	for (int a = 0; a < d; ++a) h[a] = (prm->hi[a] - prm->lo[a])/prm->n_elem[a];
	if (prm->jitter > 0.0) {
		/* one draw per (grid vertex, direction); vertex (i, j, k) of the periodic grid, i fastest */
		uint64_t st = prm->seed*0x2545F4914F6CDD1Dull + 1;
		for (size_t q = 0; q < (size_t)nx*ny*nz; ++q)
			for (int a = 0; a < d; ++a) {
				const double u = (double)(splitmix(&st) >> 11)*(1.0/9007199254740992.0);
				jit[q*3 + a] = prm->jitter*h[a]*(2.0*u - 1.0);
			}
	}
	const int n[3] = {nx, ny, nz};
	for (int k = 0; k < nz; ++k)
	for (int j = 0; j < ny; ++j)
	for (int i = 0; i < nx; ++i) {
		const int v = i + nx*(j + ny*k);
		for (int kv = 0; kv < (1 << d); ++kv) {
			const int g[3] = {i + (kv & 1), j + ((kv >> 1) & 1), k + ((kv >> 2) & 1)};
			const size_t q = (size_t)(g[0] % nx) + (size_t)nx*((g[1] % ny) + (size_t)ny*(d == 3 ? g[2] % nz : 0));
			double* x = &m->xyz_ve[((size_t)v*DPG_NVE_MAX + kv)*3];
			for (int a = 0; a < 3; ++a) {
				if (a >= d) { x[a] = 0.0; continue; }
				const int on_wall = wall[a] && (g[a] == 0 || g[a] == n[a]);
				x[a] = prm->lo[a] + g[a]*h[a] + (on_wall ? 0.0 : jit[q*3 + a]);
			}
		}
	}
	free(jit);
	return 0;
}

/* TRI box: the jittered periodic vertex grid of mesh_box (same draws), each cell (i, j) split into the triangles
 * [(i,j), (i+1,j), (i+1,j+1)] and [(i,j), (i+1,j+1), (i,j+1)], volume 2 (i + nx j) + t */
static int mesh_tri(const struct oracle_params* prm, struct or_mesh* m)
{
	const int nx = prm->n_elem[0], ny = prm->n_elem[1];
	if (prm->d != 2 || nx < 1 || ny < 1) return -1;
	m->d = 2; m->n_vol = 2*nx*ny;
	for (int a = 0; a < 3; ++a) { m->lo[a] = prm->lo[a]; m->hi[a] = a < 2 ? prm->hi[a] : prm->lo[a]; }
	m->xyz_ve = zalloc((size_t)m->n_vol*DPG_NVE_MAX*3);
	double* jit = zalloc((size_t)nx*ny*2);
	const double h[2] = {(prm->hi[0] - prm->lo[0])/nx, (prm->hi[1] - prm->lo[1])/ny};
	if (prm->jitter > 0.0) {
		uint64_t st = prm->seed*0x2545F4914F6CDD1Dull + 1;
		for (size_t q = 0; q < (size_t)nx*ny; ++q)
			for (int a = 0; a < 2; ++a) {
				const double u = (double)(splitmix(&st) >> 11)*(1.0/9007199254740992.0);
				jit[q*2 + a] = prm->jitter*h[a]*(2.0*u - 1.0);
			}
	}
	static const int cn[2][3][2] = {{{0,0}, {1,0}, {1,1}}, {{0,0}, {1,1}, {0,1}}};
	for (int j = 0; j < ny; ++j)
		for (int i = 0; i < nx; ++i)
			for (int t = 0; t < 2; ++t)
				for (int k = 0; k < 3; ++k) {
					const int gi = i + cn[t][k][0], gj = j + cn[t][k][1];
					const size_t q = (size_t)(gi % nx) + (size_t)nx*(gj % ny);
					double* x = &m->xyz_ve[((size_t)(2*(i + nx*j) + t)*DPG_NVE_MAX + k)*3];
					x[0] = prm->lo[0] + gi*h[0] + jit[q*2];
					x[1] = prm->lo[1] + gj*h[1] + jit[q*2 + 1];
				}
	free(jit);
	return 0;
}

/* Periodic box of cells split into six tetrahedra each along the diagonal (0,0,0)-(1,1,1): for the axis
 * permutations (0,1,2), (0,2,1), (1,0,2), (1,2,0), (2,0,1), (2,1,0) the cell vertices (0,0,0), e_pi0,
 * e_pi0 + e_pi1, (1,1,1), the first two exchanged for the odd permutations (positive orientation); volume
 * 6 (i + nx (j + ny k)) + t; jitter as the box's (seeded, 3 draws per periodic grid point). */
static int mesh_tet(const struct oracle_params* prm, struct or_mesh* m)
{
	const int nx = prm->n_elem[0], ny = prm->n_elem[1], nz = prm->n_elem[2];
	if (prm->d != 3 || nx < 1 || ny < 1 || nz < 1) return -1;
	m->d = 3; m->n_vol = 6*nx*ny*nz;
	for (int a = 0; a < 3; ++a) { m->lo[a] = prm->lo[a]; m->hi[a] = prm->hi[a]; }
	m->xyz_ve = zalloc((size_t)m->n_vol*DPG_NVE_MAX*3);
	double* jit = zalloc((size_t)nx*ny*nz*3);
	const double h[3] = {(prm->hi[0] - prm->lo[0])/nx, (prm->hi[1] - prm->lo[1])/ny, (prm->hi[2] - prm->lo[2])/nz};
	if (prm->jitter > 0.0) {
		uint64_t st = prm->seed*0x2545F4914F6CDD1Dull + 1;
		for (size_t q = 0; q < (size_t)nx*ny*nz; ++q)
			for (int a = 0; a < 3; ++a) {
				const double u = (double)(splitmix(&st) >> 11)*(1.0/9007199254740992.0);
				jit[q*3 + a] = prm->jitter*h[a]*(2.0*u - 1.0);
			}
	}
	static const int pm[6][3] = {{0,1,2}, {0,2,1}, {1,0,2}, {1,2,0}, {2,0,1}, {2,1,0}};
	for (int k = 0; k < nz; ++k)
		for (int j = 0; j < ny; ++j)
			for (int i = 0; i < nx; ++i)
				for (int t = 0; t < 6; ++t) {
					int c[4][3] = {{0,0,0}, {0,0,0}, {0,0,0}, {1,1,1}};
					c[1][pm[t][0]] = 1;
					c[2][pm[t][0]] = 1; c[2][pm[t][1]] = 1;
					/* the sign of the permutation: the orientation of (e_pi0, e_pi0 + e_pi1, (1,1,1)) */
					const int par = (pm[t][0] > pm[t][1]) + (pm[t][0] > pm[t][2]) + (pm[t][1] > pm[t][2]);
					const int order[4] = {par & 1 ? 1 : 0, par & 1 ? 0 : 1, 2, 3};
					for (int kv = 0; kv < 4; ++kv) {
						const int* cv = c[order[kv]];
						const int gi = i + cv[0], gj = j + cv[1], gk = k + cv[2];
						const size_t q = (size_t)(gi % nx) + (size_t)nx*((gj % ny) + (size_t)ny*(gk % nz));
						double* x = &m->xyz_ve[((size_t)(6*(i + nx*(j + ny*k)) + t)*DPG_NVE_MAX + kv)*3];
						x[0] = prm->lo[0] + gi*h[0] + jit[q*3];
						x[1] = prm->lo[1] + gj*h[1] + jit[q*3 + 1];
						x[2] = prm->lo[2] + gk*h[2] + jit[q*3 + 2];
					}
				}
	free(jit);
	return 0;
}

/* The annulus: volume i + nr j spans [r_i, r_{i+1}] x [theta_j, theta_{j+1}] uniformly; vertices stored as (r, theta). */
static int mesh_annulus(const struct oracle_params* prm, struct or_mesh* m)
{
	const int nr = prm->n_elem[0], nt = prm->n_elem[1];
	if (prm->d != 2 || nr < 1 || nt < 3) return -1;
	m->d = 2; m->n_vol = nr*nt; m->geom = DPG_GEOM_CYLINDER;
	for (int a = 0; a < 3; ++a) m->lo[a] = m->hi[a] = 0.0;
	m->xyz_ve = zalloc((size_t)m->n_vol*DPG_NVE_MAX*3);
	const double dr = (prm->hi[0] - prm->lo[0])/nr, dth = 2.0*M_PI/nt;
	for (int j = 0; j < nt; ++j)
		for (int i = 0; i < nr; ++i)
			for (int kv = 0; kv < 4; ++kv) {
				double* x = &m->xyz_ve[((size_t)(i + nr*j)*DPG_NVE_MAX + kv)*3];
				x[0] = prm->lo[0] + (i + (kv & 1))*dr;
				x[1] = (j + ((kv >> 1) & 1))*dth;
			}
	return 0;
}

static int next_section(FILE* fp, const char* name, char* line, size_t n)
{
	while (fgets(line,(int)n,fp))
		if (!strncmp(line,name,strlen(name))) return 1;
	return 0;
}

/* gmsh 2.2 ASCII: 4-node quadrilaterals (type 3, d = 2) or 8-node hexahedra (type 5, d = 3) as volumes. */
static int mesh_gmsh(const char* path, int d, int e_type, struct or_mesh* m)
{
	const int tri = (e_type == DPG_TRI), tet = (e_type == DPG_TET);
	FILE* fp = fopen(path,"r");
	if (!fp) return -1;
	char line[1024];
	if (!next_section(fp,"$Nodes",line,sizeof line)) { fclose(fp); return -1; }
	long n_node = 0;
	if (!fgets(line,sizeof line,fp) || sscanf(line,"%ld",&n_node) != 1 || n_node <= 0) { fclose(fp); return -1; }
	long* tag = malloc(sizeof(long)*(size_t)n_node);
	double* xyz = zalloc((size_t)n_node*3);
	long max_tag = 0;
	for (long i = 0; i < n_node; ++i) {
		if (!fgets(line,sizeof line,fp) || sscanf(line,"%ld %lf %lf %lf",&tag[i],&xyz[3*i],&xyz[3*i+1],&xyz[3*i+2]) != 4) {
			free(tag); free(xyz); fclose(fp); return -1;
		}
		if (tag[i] > max_tag) max_tag = tag[i];
	}
	long* idx = malloc(sizeof(long)*(size_t)(max_tag + 1));
	for (long i = 0; i <= max_tag; ++i) idx[i] = -1;
	for (long i = 0; i < n_node; ++i) idx[tag[i]] = i;
	if (!next_section(fp,"$Elements",line,sizeof line)) { free(tag); free(xyz); free(idx); fclose(fp); return -1; }
	long n_el = 0;
	if (!fgets(line,sizeof line,fp) || sscanf(line,"%ld",&n_el) != 1) { free(tag); free(xyz); free(idx); fclose(fp); return -1; }
	/* gmsh 2: triangle, 3: quadrangle, 4: tetrahedron, 5: hexahedron */
	const int want = tri ? 2 : tet ? 4 : (d == 2 ? 3 : 5), nv = tri ? 3 : tet ? 4 : 1 << d;
	m->d = d; m->n_vol = 0;
	m->xyz_ve = zalloc((size_t)n_el*DPG_NVE_MAX*3);
	for (int a = 0; a < 3; ++a) { m->lo[a] = 1e300; m->hi[a] = -1e300; }
	for (long i = 0; i < n_node; ++i)
		for (int a = 0; a < d; ++a) {
			if (xyz[3*i+a] < m->lo[a]) m->lo[a] = xyz[3*i+a];
			if (xyz[3*i+a] > m->hi[a]) m->hi[a] = xyz[3*i+a];
		}
	/* gmsh vertex k -> tensor-product position */
	static const int tp_of_gmsh[8] = {0, 1, 3, 2, 4, 5, 7, 6};
	for (long e = 0; e < n_el; ++e) {
		if (!fgets(line,sizeof line,fp)) break;
		char* cur = line;
		long vals[64];
		int nvals = 0;
		while (nvals < 64) {
			char* end;
			const long x = strtol(cur,&end,10);
			if (end == cur) break;
			vals[nvals++] = x;
			cur = end;
		}
		if (nvals < 3 || vals[1] != want) continue;
		const int ntag = (int)vals[2];
		if (nvals < 3 + ntag + nv) continue;
		double* x = &m->xyz_ve[(size_t)m->n_vol*DPG_NVE_MAX*3];
		if (tri) {   /* counter-clockwise, as the reference triangle's v0, v1, v2 */
			for (int k = 0; k < 3; ++k) {
				const long nd = idx[vals[3 + ntag + k]];
				for (int a = 0; a < 3; ++a) x[k*3 + a] = xyz[3*nd + a];
			}
			const double cr = (x[3] - x[0])*(x[7] - x[1]) - (x[4] - x[1])*(x[6] - x[0]);
			if (cr < 0.0) for (int a = 0; a < 3; ++a) { const double t = x[3 + a]; x[3 + a] = x[6 + a]; x[6 + a] = t; }
			++m->n_vol;
			continue;
		}
		if (tet) {   /* positively oriented, as the reference tetrahedron's v0..v3; else v0 and v1 exchanged */
			for (int k = 0; k < 4; ++k) {
				const long nd = idx[vals[3 + ntag + k]];
				for (int a = 0; a < 3; ++a) x[k*3 + a] = xyz[3*nd + a];
			}
			double e[3][3];
			for (int k = 0; k < 3; ++k)
				for (int a = 0; a < 3; ++a) e[k][a] = x[(k + 1)*3 + a] - x[a];
			const double det = e[0][0]*(e[1][1]*e[2][2] - e[1][2]*e[2][1]) - e[0][1]*(e[1][0]*e[2][2] - e[1][2]*e[2][0])
			                 + e[0][2]*(e[1][0]*e[2][1] - e[1][1]*e[2][0]);
			if (det < 0.0) for (int a = 0; a < 3; ++a) { const double t = x[a]; x[a] = x[3 + a]; x[3 + a] = t; }
			++m->n_vol;
			continue;
		}
		for (int k = 0; k < nv; ++k) {
			const long nd = idx[vals[3 + ntag + k]];
			for (int a = 0; a < 3; ++a) x[tp_of_gmsh[k]*3 + a] = xyz[3*nd + a];
		}
		/* orientation: sign of det(dx/dr) at the centre; mirror in the last reference direction if negative */
		double J[3][3] = {{0}};
		for (int k = 0; k < nv; ++k)
			for (int a = 0; a < d; ++a) {
				double g = 1.0;
				for (int b = 0; b < d; ++b) g *= (b == a ? (((k >> b) & 1) ? 0.5 : -0.5) : 0.5);
				for (int i = 0; i < d; ++i) J[i][a] += g*x[k*3 + i];
			}
		const double det = (d == 2 ? J[0][0]*J[1][1] - J[0][1]*J[1][0]
		                    : J[0][0]*(J[1][1]*J[2][2] - J[1][2]*J[2][1]) - J[0][1]*(J[1][0]*J[2][2] - J[1][2]*J[2][0])
		                      + J[0][2]*(J[1][0]*J[2][1] - J[1][1]*J[2][0]));
		if (det < 0.0) {
			const int half = nv/2;
			for (int k = 0; k < half; ++k)
				for (int a = 0; a < 3; ++a) { double t = x[k*3+a]; x[k*3+a] = x[(k+half)*3+a]; x[(k+half)*3+a] = t; }
		}
		++m->n_vol;
	}
	free(tag); free(xyz); free(idx); fclose(fp);
	return m->n_vol > 0 ? 0 : -1;
}

/* ---- geometry ------------------------------------------------------------------------------------------------ */

static void p1_map(int d, int n_ve, const double* phi, const double* xv, double* x)
{
	for (int i = 0; i < 3; ++i) x[i] = 0.0;
	for (int i = 0; i < d; ++i)
		for (int k = 0; k < n_ve; ++k) x[i] += phi[k]*xv[k*3 + i];
}

struct face_key { double c[3]; int vol, lf; };

static int cmp_fk(const void* a, const void* b)
{
	const struct face_key* x = a;
	const struct face_key* y = b;
	return (x->c[0] > y->c[0]) - (x->c[0] < y->c[0]);
}

static void wrap_point(int d, const double* lo, const double* L, double tol, double* c)
{
	for (int a = 0; a < d; ++a) {
		if (!(L[a] > 0.0)) continue;
		double t = (c[a] - lo[a])/L[a];
		t -= floor(t);
		if (t > 1.0 - tol) t -= 1.0;
		c[a] = lo[a] + t*L[a];
	}
}

static double wrapped_dist2(int d, const double* L, const double* x, const double* y)
{
	double s = 0.0;
	for (int a = 0; a < d; ++a) {
		double dx = x[a] - y[a];
		if (L[a] > 0.0) dx -= L[a]*nearbyint(dx/L[a]);
		s += dx*dx;
	}
	return s;
}

/* Geometry of one volume: straight volumes the P1 map of their vertices; curved (annulus) volumes the order-p
 * interpolant through the parametric map of their (r, theta) cell at the GLL solution nodes (the geometry nodes of a
 * curved volume, p_g = p, geometry_T.c:225-229; geometry_parametric_T.c:128-171). */
struct geo_ctx {
	int d, n_ve, n_s, curved, tri, tet;
	const struct dpg_element_ops* ops;
	double* vinv;      /* inverse Vandermonde matrix of the order-p Lagrange basis (curved)       */
	double* ginv;      /* inverse Vandermonde matrix of the order-1 (vertex) basis                */
	double X[125][3];  /* geometry nodes of the current volume (curved)                           */
	const double* xv;  /* vertices of the current volume                                         */
};

static void geo_volume(struct geo_ctx* g, const double* xv)
{
	g->xv = xv;
	if (!g->curved) return;
	for (int s = 0; s < g->n_s; ++s) {
		const double* r = &g->ops->rst_vs[(size_t)s*g->d];
		double rr = 0.0, th = 0.0;
		for (int k = 0; k < 4; ++k) {
			const double w = (((k & 1) ? 0.5*(1.0 + r[0]) : 0.5*(1.0 - r[0]))*(((k >> 1) & 1) ? 0.5*(1.0 + r[1]) : 0.5*(1.0 - r[1])));
			rr += w*xv[k*3]; th += w*xv[k*3 + 1];
		}
		g->X[s][0] = rr*cos(th); g->X[s][1] = rr*sin(th); g->X[s][2] = 0.0;
	}
}

/* x and J = dx/dr at the reference point r; returns detJ and the cofactors m[i][j] = detJ (J^-1)_ji. */
static double geo_at(const struct geo_ctx* g, const double* r, double* x, double m[3][3])
{
	const int d = g->d;
	const int n = g->curved ? g->n_s : g->n_ve;
	double val[125], grad[3*125], J[9] = {0}, Ji[9];
	if (g->tri) {
		double gl[3][2];
		tri_bary(r[0],r[1],val,gl);
		for (int k = 0; k < 3; ++k) { grad[k] = gl[k][0]; grad[n + k] = gl[k][1]; }
	} else if (g->tet) {
		double gl[4][3];
		tet_bary(r,val,gl);
		for (int k = 0; k < 4; ++k)
			for (int a = 0; a < 3; ++a) grad[(size_t)a*n + k] = gl[k][a];
	} else {
		lagrange_at(d,g->curved ? g->ops->p + 1 : 2,g->curved ? g->vinv : g->ginv,1,r,val,grad);
	}
	for (int i = 0; i < 3; ++i) x[i] = 0.0;
	for (int k = 0; k < n; ++k) {
		const double* xk = g->curved ? g->X[k] : &g->xv[k*3];
		for (int i = 0; i < d; ++i) {
			x[i] += val[k]*xk[i];
			for (int a = 0; a < d; ++a) J[i*d + a] += grad[(size_t)a*n + k]*xk[i];
		}
	}
	double lu[9];
	memcpy(lu,J,sizeof lu);
	double det = 1.0;
	for (int c = 0; c < d; ++c) {
		int pr = c;
		for (int rr = c+1; rr < d; ++rr) if (fabs(lu[rr*d+c]) > fabs(lu[pr*d+c])) pr = rr;
		if (pr != c) { for (int j = 0; j < d; ++j) { double t = lu[c*d+j]; lu[c*d+j] = lu[pr*d+j]; lu[pr*d+j] = t; } det = -det; }
		det *= lu[c*d+c];
		for (int rr = c+1; rr < d; ++rr) {
			const double f = lu[rr*d+c]/lu[c*d+c];
			for (int j = c; j < d; ++j) lu[rr*d+j] -= f*lu[c*d+j];
		}
	}
	oracle_gj_invert(d,J,Ji);
	for (int i = 0; i < d; ++i)
		for (int j = 0; j < d; ++j) m[i][j] = det*Ji[j*d + i];
	return det;
}

static int build_sim(const struct oracle_params* prm, const struct or_mesh* mesh, struct dpg_sim** out)
{
	const int d = prm->d;
	const int ns_pde = (prm->pde_index == DPG_PDE_NAVIER_STOKES);
	struct dpg_sim* sim = calloc(1,sizeof *sim);
	sim->d = d;
	sim->pde_index = prm->pde_index;
	sim->n_var = sim->n_eq = ((prm->pde_index == DPG_PDE_EULER || ns_pde) ? d + 2 : 1);
	sim->ind_num_flux[0] = prm->num_flux;
	sim->ind_num_flux[1] = ns_pde ? DPG_NUM_FLUX_BR2_STABLE : DPG_NUM_FLUX_INVALID;
	sim->test_case = prm->test_case;
	memcpy(sim->b_adv,prm->b_adv,sizeof sim->b_adv);
	memcpy(sim->vortex,prm->vortex,sizeof sim->vortex);
	for (int a = 0; a < 3; ++a) { sim->domain_lo[a] = mesh->lo[a]; sim->domain_hi[a] = mesh->hi[a]; }
	sim->geom = mesh->geom;
	sim->mu = prm->mu; sim->Pr = prm->Pr; sim->r_s = 1.0;
	sim->bc_omega = prm->omega;
	sim->bc_rho = prm->wall_p/(sim->r_s*prm->wall_T);
	sim->bc_E = prm->wall_p/OR_GM1 + 0.5*sim->bc_rho*(prm->omega*prm->lo[0])*(prm->omega*prm->lo[0]);
	memcpy(sim->bc_state,prm->bc_state,sizeof sim->bc_state);
	sim->tc_data[0] = prm->lo[0]; sim->tc_data[1] = prm->hi[0]; sim->tc_data[2] = prm->wall_p; sim->tc_data[3] = prm->wall_T;
	/* one operator set per order; mixed orders: volume v has order p + (splitmix64 draw v) mod (p_max - p + 1),
	 * the draws in volume order from the state p_seed */
	const int p_lo = prm->p, p_hi = prm->p_max > prm->p ? prm->p_max : prm->p;
	sim->n_ops = p_hi - p_lo + 1;
	sim->ops = calloc((size_t)sim->n_ops,sizeof *sim->ops);
	const int tri = (prm->e_type == DPG_TRI), tet = (prm->e_type == DPG_TET);
	for (int k = 0; k < sim->n_ops; ++k) {
		const int pk = p_lo + k, nr = (pk <= 8 && prm->vrule[pk] ? prm->vrule_n[pk] : 0);
		if (tri) { if (d != 2 || build_ops_tri(pk,&sim->ops[k],nr,prm->vrule[pk])) { oracle_sim_free(sim); return -1; } }
		else if (tet) {
			const int nf = (pk <= 8 && prm->frule[pk] ? prm->frule_n[pk] : 0);
			if (d != 3 || build_ops_tet(pk,&sim->ops[k],nr,prm->vrule[pk],nf,prm->frule[pk])) { oracle_sim_free(sim); return -1; }
		}
		else build_ops(d,p_lo + k,&sim->ops[k]);
	}
	const struct dpg_element_ops* ops = &sim->ops[0];
	const int n_fl = ops->n_fl, n_ve = ops->n_ve, n_var = sim->n_var;
	const int n_vol = mesh->n_vol;
	sim->n_vol = n_vol;
	sim->vol_ops = calloc((size_t)n_vol,sizeof(int));
	sim->vol_p = calloc((size_t)n_vol,sizeof(int));
	sim->vol_affine = calloc((size_t)n_vol,sizeof(int));
	sim->vol_dof_off = calloc((size_t)n_vol + 1,sizeof(int64_t));
	sim->vol_geo_off = calloc((size_t)n_vol + 1,sizeof(int64_t));
	sim->vol_minv_off = calloc((size_t)n_vol + 1,sizeof(int64_t));
	{
		uint64_t st = prm->p_seed;
		for (int v = 0; v < n_vol; ++v) {
			const int pv = p_lo + (p_hi > p_lo ? (int)(splitmix(&st) % (uint64_t)(p_hi - p_lo + 1)) : 0);
			sim->vol_p[v] = pv; sim->vol_ops[v] = pv - p_lo;
			sim->vol_dof_off[v+1] = sim->vol_dof_off[v] + (int64_t)sim->ops[pv - p_lo].n_s*n_var;
			sim->vol_geo_off[v+1] = sim->vol_geo_off[v] + sim->ops[pv - p_lo].n_c;
		}
	}
	const int64_t n_geo = sim->vol_geo_off[n_vol];
	sim->xyz_ve = zalloc((size_t)n_vol*DPG_NVE_MAX*3);
	memcpy(sim->xyz_ve,mesh->xyz_ve,sizeof(double)*(size_t)n_vol*DPG_NVE_MAX*3);
	sim->sol_coef = zalloc((size_t)sim->vol_dof_off[n_vol]);
	sim->sol_coef_p = zalloc((size_t)sim->vol_dof_off[n_vol]);
	sim->rhs = zalloc((size_t)sim->vol_dof_off[n_vol]);
	sim->metrics_vc = zalloc((size_t)n_geo*d*d);
	sim->jacobian_det_vc = zalloc((size_t)n_geo);
	sim->xyz_vc = zalloc((size_t)n_geo*d);

	struct geo_ctx* g = calloc(1,sizeof *g);
	g->d = d; g->n_ve = n_ve; g->n_s = ops->n_s; g->ops = ops; g->curved = (mesh->geom == DPG_GEOM_CYLINDER);
	g->tri = tri; g->tet = tet;
	{
		double gll[16], w[16], vtx[2] = {-1.0, 1.0};
		oracle_nodes_gll(prm->p + 1,gll,w);
		g->vinv = vandermonde_inverse(d,prm->p + 1,gll);
		g->ginv = vandermonde_inverse(d,2,vtx);
	}
#define FAIL(code) do { free(g->vinv); free(g->ginv); free(g); oracle_sim_free(sim); return (code); } while (0)

	/* volume geometry, at every cubature node of the volume's order */
	for (int v = 0; v < n_vol; ++v) {
		const struct dpg_element_ops* ov = &sim->ops[sim->vol_ops[v]];
		const int n_c = ov->n_c;
		const int64_t go = sim->vol_geo_off[v];
		geo_volume(g,&sim->xyz_ve[(size_t)v*DPG_NVE_MAX*3]);
		for (int c = 0; c < n_c; ++c) {
			double m[3][3], x[3];
			const double det = geo_at(g,&ov->rst_vc[(size_t)c*d],x,m);
			if (!(det > 0.0)) FAIL(-2);
			sim->jacobian_det_vc[go + c] = det;
			for (int i = 0; i < d; ++i)
				for (int j = 0; j < d; ++j) sim->metrics_vc[(size_t)go*d*d + c + (size_t)n_c*(i + d*j)] = m[i][j];
			for (int i = 0; i < d; ++i) sim->xyz_vc[(size_t)go*d + c + (size_t)n_c*i] = x[i];
		}
	}

	/* faces: centroid of every local face (in physical coordinates), wrapped into the periodic box, matched within a
	 * tolerance; a local face without a match is a boundary face */
	double L[3] = {0,0,0}, hmin = 1e300;
	for (int a = 0; a < d; ++a) L[a] = mesh->hi[a] - mesh->lo[a];
	/* a straight mesh with walls across direction a is not periodic in a (a mesh file's bounding box says nothing
	 * about it) */
	if (!g->curved)
		for (int a = 0; a < d; ++a) if (prm->bc_side[2*a] != 0) L[a] = 0.0;
	const size_t n_ent = (size_t)n_vol*n_fl;
	struct face_key* ent = malloc(sizeof *ent*n_ent);
	for (int v = 0; v < n_vol; ++v) {
		const double* xv0 = &sim->xyz_ve[(size_t)v*DPG_NVE_MAX*3];
		double xv[8*3];
		for (int k = 0; k < n_ve; ++k)
			for (int i = 0; i < 3; ++i) xv[k*3 + i] = xv0[k*3 + i];
		if (g->curved)
			for (int k = 0; k < n_ve; ++k) { const double rr = xv0[k*3], th = xv0[k*3 + 1]; xv[k*3] = rr*cos(th); xv[k*3 + 1] = rr*sin(th); }
		for (int a = 0; a < d; ++a) {
			const int o = (tri || tet) ? a + 1 : (1 << a);   /* simplices: the edges from v0 */
			double l = 0.0;
			for (int i = 0; i < d; ++i) l += (xv[o*3 + i] - xv[i])*(xv[o*3 + i] - xv[i]);
			if (sqrt(l) < hmin) hmin = sqrt(l);
		}
		for (int lf = 0; lf < n_fl; ++lf) {
			struct face_key* e = &ent[(size_t)v*n_fl + lf];
			e->vol = v; e->lf = lf;
			e->c[0] = e->c[1] = e->c[2] = 0.0;
			if (tri) {
				for (int k = 0; k < 2; ++k)
					for (int i = 0; i < d; ++i) e->c[i] += 0.5*xv[TRI_FVE[lf][k]*3 + i];
			} else if (tet) {
				for (int k = 0; k < 3; ++k)
					for (int i = 0; i < d; ++i) e->c[i] += xv[TET_FVE[lf][k]*3 + i]/3.0;
			} else {
				const int af = lf/2, sd = lf & 1;
				for (int k = 0; k < n_ve; ++k)
					if (((k >> af) & 1) == sd)
						for (int i = 0; i < d; ++i) e->c[i] += xv[k*3 + i]/(double)(n_ve/2);
			}
			wrap_point(d,mesh->lo,L,1e-9,e->c);
		}
	}
	const double tol = 1e-6*hmin;
	qsort(ent,n_ent,sizeof *ent,cmp_fk);
	int* partner = malloc(sizeof(int)*n_ent);
	for (size_t i = 0; i < n_ent; ++i) partner[i] = -1;
	for (size_t i = 0; i < n_ent; ++i) {
		if (partner[i] >= 0) continue;
		for (size_t j = i + 1; j < n_ent && ent[j].c[0] - ent[i].c[0] < tol; ++j) {
			if (partner[j] >= 0) continue;
			if (wrapped_dist2(d,L,ent[i].c,ent[j].c) < tol*tol) { partner[i] = (int)j; partner[j] = (int)i; break; }
		}
		/* a centroid on the periodic seam may have been wrapped to the other end of the box */
		if (partner[i] < 0)
			for (size_t j = 0; j < n_ent; ++j)
				if (j != i && partner[j] < 0 && wrapped_dist2(d,L,ent[i].c,ent[j].c) < tol*tol) {
					partner[i] = (int)j; partner[j] = (int)i; break;
				}
	}
	/* faces in the order of their side-0 (volume, local face); boundary faces: side 1 = -1 */
	int* first = malloc(sizeof(int)*n_ent);       /* entry (v n_fl + lf) -> sorted index */
	for (size_t i = 0; i < n_ent; ++i) first[(size_t)ent[i].vol*n_fl + ent[i].lf] = (int)i;
	int n_face = 0;
	for (size_t key = 0; key < n_ent; ++key) {
		const int i = first[key], j = partner[i];
		if (j < 0 || (size_t)ent[j].vol*n_fl + ent[j].lf > key) ++n_face;
	}
	sim->n_face = n_face;
	sim->face_vol = calloc((size_t)2*n_face,sizeof(int));
	sim->face_lf = calloc((size_t)2*n_face,sizeof(int));
	sim->face_nfc = calloc((size_t)n_face,sizeof(int));
	sim->face_bc = calloc((size_t)n_face,sizeof(int));
	sim->face_geo_off = calloc((size_t)n_face + 1,sizeof(int64_t));
	sim->face_p = calloc((size_t)n_face,sizeof(int));
	sim->vol_face = calloc((size_t)n_vol*DPG_NFL_MAX,sizeof(int));
	sim->vol_face_side = calloc((size_t)n_vol*DPG_NFL_MAX,sizeof(int));
	int f = 0, bad = 0;
	for (size_t key = 0; key < n_ent; ++key) {
		const int i = first[key], j = partner[i];
		if (j >= 0 && (size_t)ent[j].vol*n_fl + ent[j].lf < key) continue;
		sim->face_vol[2*f] = ent[i].vol; sim->face_lf[2*f] = ent[i].lf;
		sim->vol_face[ent[i].vol*DPG_NFL_MAX + ent[i].lf] = f; sim->vol_face_side[ent[i].vol*DPG_NFL_MAX + ent[i].lf] = 0;
		if (j >= 0) {
			sim->face_vol[2*f + 1] = ent[j].vol; sim->face_lf[2*f + 1] = ent[j].lf;
			sim->vol_face[ent[j].vol*DPG_NFL_MAX + ent[j].lf] = f; sim->vol_face_side[ent[j].vol*DPG_NFL_MAX + ent[j].lf] = 1;
		} else {
			/* boundary: the box side (x-, x+, y-, ...) the face centroid lies on, or the annulus wall (local face 0
			 * inner, 1 outer) */
			sim->face_vol[2*f + 1] = -1; sim->face_lf[2*f + 1] = -1;
			int side = ent[i].lf;
			if (!g->curved) {
				side = -1;
				for (int a = 0; a < d; ++a) {
					if (fabs(ent[i].c[a] - prm->lo[a]) < tol) side = 2*a;
					else if (fabs(ent[i].c[a] - prm->hi[a]) < tol) side = 2*a + 1;
				}
			}
			sim->face_bc[f] = side >= 0 ? prm->bc_side[side] : 0;
			if (sim->face_bc[f] == 0) bad = 1;   /* an unmatched face where the problem is periodic */
		}
		/* the face's order and cubature: the larger order of its volumes (face_solver.c:123-132) */
		int pf = sim->vol_p[ent[i].vol];
		if (j >= 0 && sim->vol_p[ent[j].vol] > pf) pf = sim->vol_p[ent[j].vol];
		sim->face_p[f] = pf;
		sim->face_nfc[f] = sim->ops[pf - p_lo].n_fc;
		for (int sd = 0; sd < 2; ++sd) {
			const int v = sim->face_vol[2*f + sd];
			if (v >= 0 && sim->vol_p[v] < pf && face_ops_higher(&sim->ops[sim->vol_ops[v]],&sim->ops[pf - p_lo])) bad = 1;
		}
		++f;
	}
	free(ent); free(partner); free(first);
	if (bad) FAIL(-3);
	sim->face_geo_off[0] = 0;
	for (int q = 0; q < n_face; ++q) sim->face_geo_off[q+1] = sim->face_geo_off[q] + sim->face_nfc[q];
	const int64_t n_fnode = sim->face_geo_off[n_face];
	sim->nc_fc = calloc((size_t)n_fnode,sizeof(int));
	sim->normals_fc = zalloc((size_t)n_fnode*d);
	sim->jacobian_det_fc = zalloc((size_t)n_fnode);
	sim->xyz_fc = zalloc((size_t)n_fnode*d);
	int nfc_max = 0;
	for (int k = 0; k < sim->n_ops; ++k) if (sim->ops[k].n_fc > nfc_max) nfc_max = sim->ops[k].n_fc;
	double (*pl)[3] = malloc(sizeof *pl*(size_t)nfc_max), (*pr)[3] = malloc(sizeof *pr*(size_t)nfc_max);
	for (int q0 = 0; q0 < n_face; ++q0) {
		const int vl = sim->face_vol[2*q0], lfl = sim->face_lf[2*q0];
		const int vr = sim->face_vol[2*q0 + 1], lfr = sim->face_lf[2*q0 + 1];
		const struct dpg_element_ops* fo = &sim->ops[sim->face_p[q0] - p_lo];   /* the face's cubature */
		const int n_fc = fo->n_fc;
		const int64_t fgo = sim->face_geo_off[q0];
		const double* nref = &fo->normals_ref[(size_t)lfl*d];
		geo_volume(g,&sim->xyz_ve[(size_t)vl*DPG_NVE_MAX*3]);
		for (int q = 0; q < n_fc; ++q) {
			double m[3][3];
			geo_at(g,&fo->rst_fc[((size_t)lfl*n_fc + q)*d],pl[q],m);
			double n[3] = {0,0,0}, len = 0.0;
			for (int i = 0; i < d; ++i) {
				for (int r = 0; r < d; ++r) n[i] += m[i][r]*nref[r];
				len += n[i]*n[i];
			}
			len = sqrt(len);
			sim->jacobian_det_fc[fgo + q] = len;
			for (int i = 0; i < d; ++i) sim->normals_fc[(size_t)(fgo + q)*d + i] = n[i]/len;
			for (int i = 0; i < d; ++i) sim->xyz_fc[(size_t)fgo*d + q + (size_t)n_fc*i] = pl[q][i];
		}
		if (vr < 0) {
			for (int q = 0; q < n_fc; ++q) sim->nc_fc[fgo + q] = q;
			continue;
		}
		geo_volume(g,&sim->xyz_ve[(size_t)vr*DPG_NVE_MAX*3]);
		for (int q = 0; q < n_fc; ++q) {
			double m[3][3];
			geo_at(g,&fo->rst_fc[((size_t)lfr*n_fc + q)*d],pr[q],m);
		}
		for (int q = 0; q < n_fc; ++q) {
			int best = -1;
			double bd = 1e300;
			for (int qq = 0; qq < n_fc; ++qq) {
				const double dd = wrapped_dist2(d,L,pl[q],pr[qq]);
				if (dd < bd) { bd = dd; best = qq; }
			}
			if (!(bd < tol*tol)) { free(pl); free(pr); FAIL(-4); }
			sim->nc_fc[fgo + q] = best;
		}
	}
	free(pl); free(pr);
	free(g->vinv); free(g->ginv); free(g);
#undef FAIL
	oracle_initial_solution(sim,sim->sol_coef);
	*out = sim;
	return 0;
}

int oracle_sim_structured(const struct oracle_params* prm, struct dpg_sim** out)
{
	*out = NULL;
	if (prm->d < 2 || prm->d > 3 || prm->p < 1 || prm->p > 8) return -1;
	struct or_mesh m;
	memset(&m,0,sizeof m);
	if (prm->mesh_kind == 1) { if (mesh_annulus(prm,&m)) { free(m.xyz_ve); return -1; } }
	else if (prm->e_type == DPG_TRI) { if (mesh_tri(prm,&m)) { free(m.xyz_ve); return -1; } }
	else if (prm->e_type == DPG_TET) { if (mesh_tet(prm,&m)) { free(m.xyz_ve); return -1; } }
	else mesh_box(prm,&m);
	const int rc = build_sim(prm,&m,out);
	free(m.xyz_ve);
	return rc;
}

int oracle_sim_gmsh(const struct oracle_params* prm, const char* path, struct dpg_sim** out)
{
	*out = NULL;
	if (prm->d < 2 || prm->d > 3 || prm->p < 1 || prm->p > 8) return -1;
	struct or_mesh m;
	memset(&m,0,sizeof m);
	if (mesh_gmsh(path,prm->d,prm->e_type,&m)) { free(m.xyz_ve); return -1; }
	const int rc = build_sim(prm,&m,out);
	free(m.xyz_ve);
	return rc;
}

void oracle_sim_free(struct dpg_sim* sim)
{
	if (!sim) return;
	for (int i = 0; i < sim->n_ops; ++i) free_ops(&sim->ops[i]);
	free(sim->ops);
	free(sim->vol_ops); free(sim->vol_p); free(sim->vol_affine); free(sim->vol_dof_off); free(sim->vol_geo_off);
	free(sim->vol_minv_off); free(sim->xyz_ve); free(sim->sol_coef); free(sim->sol_coef_p); free(sim->rhs);
	free(sim->metrics_vc); free(sim->jacobian_det_vc); free(sim->xyz_vc); free(sim->m_inv);
	free(sim->vol_face); free(sim->vol_face_side);
	free(sim->face_vol); free(sim->face_lf); free(sim->face_nfc); free(sim->face_bc); free(sim->face_geo_off);
	free(sim->nc_fc); free(sim->normals_fc); free(sim->jacobian_det_fc); free(sim->xyz_fc); free(sim->face_p);
	free(sim);
}

/* ---- solutions and errors ------------------------------------------------------------------------------------ */

static double wrap1(double x, double lo, double hi)
{
	const double L = hi - lo;
	double y = fmod(x - lo,L);
	if (y < 0.0) y += L;
	return lo + y;
}

void oracle_exact_solution(const struct dpg_sim* sim, double t, const double* x, double* u)
{
	const int d = sim->d;
	if (sim->test_case == DPG_TC_ADVECTION_SINE) {
		const double xs = x[0] - sim->b_adv[0]*t, ys = x[1] - sim->b_adv[1]*t;
		u[0] = sin(2.0*M_PI*xs)*sin(2.0*M_PI*ys);
		return;
	}
	if (sim->test_case == DPG_TC_PERIODIC_VORTEX) {
		/* constructor_sol_periodic_vortex_T with set_xy_c / set_data_periodic_vortex (solution_periodic_vortex_T.c) */
		const double* q = sim->vortex;   /* r_v, theta, V_inf, p_inf, t_inf, Rg */
		const double rho_inf = q[3]/(q[5]*q[4]), con = 0.1*q[2];
		const double period = (fmod(q[1],M_PI/2.0) < 1e-15) ? 2.0 : 2.0*sqrt(2.0);
		double u_inf = q[2]*cos(q[1]), v_inf = q[2]*sin(q[1]);
		if (fabs(u_inf) < 1e-16) u_inf = 1e-16;
		if (fabs(v_inf) < 1e-16) v_inf = 1e-16;
		const double f = fmod(t*q[2] + 0.5*period,period)/period;
		const double xc = (f - 0.5)*period*cos(q[1]), yc = (f - 0.5)*period*sin(q[1]);
		const double rv2 = q[0]*q[0];
		const double r2 = (pow(x[0] - xc,2.0) + pow(x[1] - yc,2.0))/rv2;
		const double uu = u_inf - con*(x[1] - yc)/rv2*exp(-0.5*r2);
		const double vv = v_inf + con*(x[0] - xc)/rv2*exp(-0.5*r2);
		const double pp = q[3] - rho_inf*(con*con)/(2.0*rv2)*exp(-r2);
		u[0] = rho_inf; u[1] = rho_inf*uu; u[2] = rho_inf*vv;
		if (d == 3) u[3] = 0.0;
		u[d + 1] = pp/OR_GM1 + 0.5*rho_inf*(uu*uu + vv*vv);
		return;
	}
	if (sim->test_case == DPG_TC_TAYLOR_COUETTE) {
		/* constructor_sol_taylor_couette (solution_taylor_couette_T.c), zero temperature gradient at r_o */
		const double ri = sim->tc_data[0], ro = sim->tc_data[1], p_i = sim->tc_data[2], t_i = sim->tc_data[3];
		const double kappa = sim->mu*(OR_GAMMA*sim->r_s/OR_GM1)/sim->Pr;
		const double c = sim->bc_omega/(1.0/(ri*ri) - 1.0/(ro*ro));
		const double r = sqrt(x[0]*x[0] + x[1]*x[1]), th = atan2(x[1],x[0]);
		const double vt = c*(1.0/r - r/(ro*ro));
		const double t = t_i - 2.0*c*c/(ro*ro)*sim->mu/kappa*log(r/ri) - c*c*sim->mu/kappa*(1.0/(r*r) - 1.0/(ri*ri));
		const double rho = p_i/(sim->r_s*t), uu = -sin(th)*vt, vv = cos(th)*vt;
		u[0] = rho; u[1] = rho*uu; u[2] = rho*vv;
		u[3] = p_i/OR_GM1 + 0.5*rho*(uu*uu + vv*vv);
		return;
	}
	const double* vx = sim->vortex;   /* beta, xc, yc, rho, u, v, w, p */
	double rho = vx[3], uu = vx[4], vv = vx[5], ww = vx[6], p = vx[7];
	if (sim->test_case == DPG_TC_ISENTROPIC_VORTEX) {
		const double Lx = sim->domain_hi[0] - sim->domain_lo[0], Ly = sim->domain_hi[1] - sim->domain_lo[1];
		/* the advected centre and the nearest periodic image, in periodic directions (zero extent: a wall) */
		double dx = x[0] - (Lx > 0.0 ? wrap1(vx[1] + vx[4]*t,sim->domain_lo[0],sim->domain_hi[0]) : vx[1] + vx[4]*t);
		double dy = x[1] - (Ly > 0.0 ? wrap1(vx[2] + vx[5]*t,sim->domain_lo[1],sim->domain_hi[1]) : vx[2] + vx[5]*t);
		if (Lx > 0.0) dx -= Lx*nearbyint(dx/Lx);
		if (Ly > 0.0) dy -= Ly*nearbyint(dy/Ly);
		const double g = exp(0.5*(1.0 - dx*dx - dy*dy));
		const double T0 = vx[7]/vx[3];
		const double T = T0 - OR_GM1*vx[0]*vx[0]/(8.0*OR_GAMMA*M_PI*M_PI)*g*g;
		rho = vx[3]*pow(T/T0,1.0/OR_GM1);
		p = rho*T;
		uu = vx[4] - vx[0]/(2.0*M_PI)*dy*g;
		vv = vx[5] + vx[0]/(2.0*M_PI)*dx*g;
	}
	u[0] = rho;
	u[1] = rho*uu;
	u[2] = rho*vv;
	if (d == 3) u[3] = rho*ww;
	const double ke = 0.5*rho*(uu*uu + vv*vv + (d == 3 ? ww*ww : 0.0));
	u[d + 1] = p/OR_GM1 + ke;
}

/* Multilinear shape functions at r in closed form, exact at the vertices (a solution node on the periodic seam must
 * land exactly on it: the nearest periodic image of the vortex centre is ambiguous there). */
static void p1_shape(int d, const double* r, double* phi)
{
	for (int k = 0; k < (1 << d); ++k) {
		double t = 1.0;
		for (int a = 0; a < d; ++a) t *= ((k >> a) & 1) ? 0.5*(1.0 + r[a]) : 0.5*(1.0 - r[a]);
		phi[k] = t;
	}
}

void oracle_initial_solution(const struct dpg_sim* sim, double* sol)
{
	const int d = sim->d, n_var = sim->n_var;
	for (int v = 0; v < sim->n_vol; ++v) {
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
		const int n_s = ops->n_s, n_ve = ops->n_ve;
		const double* xv = &sim->xyz_ve[(size_t)v*DPG_NVE_MAX*3];
		double* sc = &sol[sim->vol_dof_off[v]];
		for (int s = 0; s < n_s; ++s) {
			double x[3], u[5], phi[8];
			if (ops->e_type == DPG_TRI) tri_bary(ops->rst_vs[(size_t)s*d],ops->rst_vs[(size_t)s*d + 1],phi,NULL);
			else if (ops->e_type == DPG_TET) tet_bary(&ops->rst_vs[(size_t)s*d],phi,NULL);
			else p1_shape(d,&ops->rst_vs[(size_t)s*d],phi);
			p1_map(d,n_ve,phi,xv,x);
			if (sim->geom == DPG_GEOM_CYLINDER) { const double rr = x[0], th = x[1]; x[0] = rr*cos(th); x[1] = rr*sin(th); }
			oracle_exact_solution(sim,0.0,x,u);
			for (int var = 0; var < n_var; ++var) sc[s + (size_t)n_s*var] = u[var];
		}
	}
}

static void error_vars(const struct dpg_sim* sim, const double* u, double* e)
{
	const int d = sim->d;
	if (sim->n_var != d + 2) { e[0] = u[0]; return; }
	double ke = 0.0;
	e[0] = u[0];
	for (int a = 0; a < d; ++a) { e[1 + a] = u[1 + a]/u[0]; ke += u[1 + a]*e[1 + a]; }
	e[d + 1] = OR_GM1*(u[d + 1] - 0.5*ke);
}

int oracle_l2_error(const struct dpg_sim* sim, const double* sol, double t, double* err)
{
	const int d = sim->d, n_var = sim->n_var;
	double acc[5] = {0,0,0,0,0}, vol = 0.0;
	for (int v = 0; v < sim->n_vol; ++v) {
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
		const int n_s = ops->n_s, n_c = ops->n_c;
		const int64_t go = sim->vol_geo_off[v];
		const double* sc = &sol[sim->vol_dof_off[v]];
		for (int c = 0; c < n_c; ++c) {
			double uh[5], ue[5], eh[5], ee[5], x[3] = {0,0,0};
			for (int var = 0; var < n_var; ++var) {
				double s = 0.0;
				for (int i = 0; i < n_s; ++i) s += ops->cv0_vs_vc[(size_t)c*n_s + i]*sc[i + (size_t)n_s*var];
				uh[var] = s;
			}
			for (int a = 0; a < d; ++a) x[a] = sim->xyz_vc[(size_t)go*d + c + (size_t)n_c*a];
			oracle_exact_solution(sim,t,x,ue);
			error_vars(sim,uh,eh);
			error_vars(sim,ue,ee);
			const double wj = ops->w_vc[c]*sim->jacobian_det_vc[go + c];
			for (int var = 0; var < n_var; ++var) acc[var] += wj*(eh[var] - ee[var])*(eh[var] - ee[var]);
			vol += wj;
		}
	}
	for (int var = 0; var < n_var; ++var) err[var] = sqrt(acc[var]/vol);
	return 0;
}
