/* Triangle (TRI) element operators for DG of order p on the reference's equilateral triangle.
 *
 * Reference element (element.c:453-466 of the reference): vertices v0 = (-1, -1/sqrt3), v1 = (1, -1/sqrt3),
 * v2 = (0, 2/sqrt3); local face f is the edge opposite vertex f (f_ve = {1,2}, {0,2}, {0,1}), parametrised from its
 * first to its second vertex by t in [-1, 1] (unit speed: every edge has length 2).
 *
 * Solution nodes: the alpha-optimised ("AO") warp-and-blend nodes of Warburton (2006; Hesthaven & Warburton,
 * Nodal Discontinuous Galerkin Methods, 2008, section 6.1): equidistant barycentric nodes displaced along the three
 * edge directions by the 1D warp from equidistant to Gauss-Lobatto-Legendre nodes, blended by 4 L_i L_j and the
 * optimised (1 + (alpha L)^2) factor, alpha from the published table for p <= 15.  Ordered by rows of increasing L1
 * (the barycentric coordinate of v2), then increasing L3 within a row.
 * Basis: the orthonormal polynomials of Proriol, Koornwinder and Dubiner in collapsed coordinates, turned into the
 * Lagrange basis of the nodes with the inverse Vandermonde matrix.
 * Volume cubature: orders 1..4 the fully symmetric rules of strength 2p derived by gen_tri_rules.py, which are the
 * reference's Witherden-Vincent rules (input/nodes/tri/WV<2p>.txt); higher orders a collapsed-coordinate (Duffy)
 * rule, Gauss-Legendre in a and Gauss-Jacobi of the weight (1 - b) in b, p + 1 points each (exact to 2p + 1).
 * Face cubature: Gauss-Legendre with p + 1 points on each edge (exact to degree 2p + 1).
 * Bezier operators of the positivity limiter: the Bernstein polynomials of degree p at the nodes and their inverse
 * (dpg_simplex_bezier_ops; no 1D factors). */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "dpg_host.h"
#include "tri_sym_rules.inc"

#define SQ3 1.7320508075688772

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* orthonormal Jacobi polynomial P_n^(a,b)(x) on [-1, 1] (weight (1-x)^a (1+x)^b) and its derivative */
static void jacobi_p(int n, double a, double b, double x, double* val, double* der)
{
	/* three-term recurrence of the normalised polynomials */
	const double g0 = pow(2.0,a+b+1.0)/(a+b+1.0)*tgamma(a+1.0)*tgamma(b+1.0)/tgamma(a+b+1.0);
	double pm1 = 1.0/sqrt(g0), p = 0.0;
	if (n == 0) { *val = pm1; if (der) *der = 0.0; return; }
	const double g1 = (a+1.0)*(b+1.0)/(a+b+3.0)*g0;
	double p0 = ((a+b+2.0)*x/2.0 + (a-b)/2.0)/sqrt(g1);
	double aold = 2.0/(2.0+a+b)*sqrt((a+1.0)*(b+1.0)/(a+b+3.0));
	for (int i = 1; i < n; ++i) {
		const double h1 = 2.0*i + a + b;
		const double anew = 2.0/(h1+2.0)*sqrt((i+1.0)*(i+1.0+a+b)*(i+1.0+a)*(i+1.0+b)/(h1+1.0)/(h1+3.0));
		const double bnew = -(a*a - b*b)/h1/(h1+2.0);
		p = (-aold*pm1 + (x - bnew)*p0)/anew;
		pm1 = p0; p0 = p;
		aold = anew;
	}
	*val = p0;
	if (der) {
		double v = 0.0;
		if (n > 0) jacobi_p(n-1,a+1.0,b+1.0,x,&v,NULL);
		*der = sqrt(n*(n+a+b+1.0))*v;
	}
}

/* equilateral (x, y) -> standard triangle (r, s) with vertices (-1,-1), (1,-1), (-1,1) */
static void xy_to_rs(double x, double y, double* r, double* s)
{
	*s = 2.0*(y + 1.0/SQ3)/SQ3 - 1.0;
	*r = x - (*s + 1.0)/2.0;
}

/* the orthonormal basis (ordered i + j <= p, j fastest within i) and its gradient in (x, y) at one point */
static void pkd_basis(int p, double x, double y, double* val, double* gx, double* gy)
{
	double r, s;
	xy_to_rs(x,y,&r,&s);
	const double a = (fabs(s - 1.0) > 1e-14) ? 2.0*(1.0 + r)/(1.0 - s) - 1.0 : -1.0;
	const double b = s;
	int k = 0;
	for (int i = 0; i <= p; ++i)
		for (int j = 0; j <= p - i; ++j, ++k) {
			double fa, dfa, gb, dgb;
			jacobi_p(i,0.0,0.0,a,&fa,&dfa);
			jacobi_p(j,2.0*i+1.0,0.0,b,&gb,&dgb);
			const double om = 1.0 - b;
			const double c = pow(0.5*om,(double)i);
			val[k] = sqrt(2.0)*fa*gb*c;
			/* d/dr and d/ds of fa(a) gb(b) ((1-b)/2)^i with a = 2(1+r)/(1-s) - 1, b = s */
			double dr = dfa*gb;
			if (i > 0) dr *= pow(0.5*om,(double)(i-1));
			double ds = dfa*gb*(0.5*(1.0 + a));
			if (i > 0) ds *= pow(0.5*om,(double)(i-1));
			double t = dgb*c;
			if (i > 0) t -= 0.5*i*gb*pow(0.5*om,(double)(i-1));
			ds += fa*t;
			dr *= sqrt(2.0); ds *= sqrt(2.0);
			/* (x, y) = (r + (s+1)/2, -1/sqrt3 + (s+1) sqrt3/2): dr/dx = 1, dr/dy = -1/sqrt3, ds/dy = 2/sqrt3 */
			gx[k] = dr;
			gy[k] = -dr/SQ3 + ds*2.0/SQ3;
		}
}

/* 1D warp from equidistant to GLL nodes, evaluated at rout (Hesthaven & Warburton, Warpfactor) */
static double warp_factor(int p, double rout)
{
	double gll[16], wgll[16];
	dpg_nodes_gll(p+1,gll,wgll);
	double warp = 0.0;
	for (int i = 0; i <= p; ++i) {
		/* Lagrange polynomial of the equidistant node i at rout */
		const double ri = -1.0 + 2.0*i/p;
		double l = 1.0;
		for (int j = 0; j <= p; ++j) if (j != i) l *= (rout - (-1.0 + 2.0*j/p))/(ri - (-1.0 + 2.0*j/p));
		warp += l*(gll[i] - ri);
	}
	const int zerof = fabs(rout) < 1.0 - 1e-10;
	const double sf = 1.0 - (zerof ? rout*rout : 0.0);
	return zerof ? warp/sf : 0.0*warp;
}

static void ao_nodes(int p, double* xy)
{
	static const double alpopt[15] = {0.0000, 0.0000, 1.4152, 0.1001, 0.2751, 0.9800, 1.0999, 1.2832, 1.3648, 1.4773,
	                                  1.4959, 1.5743, 1.5770, 1.6223, 1.6258};
	const double alpha = (p < 16) ? alpopt[p-1] : 5.0/3.0;
	int k = 0;
	for (int n = 0; n <= p; ++n)
		for (int m = 0; m <= p - n; ++m, ++k) {
			const double L1 = (double)n/p, L3 = (double)m/p, L2 = 1.0 - L1 - L3;
			double x = -L2 + L3, y = (-L2 - L3 + 2.0*L1)/SQ3;
			const double b1 = 4.0*L2*L3, b2 = 4.0*L1*L3, b3 = 4.0*L1*L2;
			const double w1 = b1*warp_factor(p,L3 - L2)*(1.0 + (alpha*L1)*(alpha*L1));
			const double w2 = b2*warp_factor(p,L1 - L3)*(1.0 + (alpha*L2)*(alpha*L2));
			const double w3 = b3*warp_factor(p,L2 - L1)*(1.0 + (alpha*L3)*(alpha*L3));
			x += w1 + cos(2.0*M_PI/3.0)*w2 + cos(4.0*M_PI/3.0)*w3;
			y += sin(2.0*M_PI/3.0)*w2 + sin(4.0*M_PI/3.0)*w3;
			xy[2*k] = x; xy[2*k+1] = y;
		}
}

/* barycentric P1 basis of v0, v1, v2 at (x, y) and its (constant) gradient [d][3] */
static void p1_tri(double x, double y, double* val, double* grad)
{
	const double l2 = (SQ3*y + 1.0)/3.0;                /* v2 = (0, 2/sqrt3) */
	const double l1 = (x + 1.0 - l2)/2.0;               /* v1 = (1, -1/sqrt3) */
	const double l0 = 1.0 - l1 - l2;
	val[0] = l0; val[1] = l1; val[2] = l2;
	if (grad) {
		const double dl2x = 0.0, dl2y = SQ3/3.0;
		const double dl1x = 0.5, dl1y = -dl2y/2.0;
		grad[0] = -dl1x - dl2x; grad[1] = dl1x; grad[2] = dl2x;          /* d/dx */
		grad[3] = -dl1y - dl2y; grad[4] = dl1y; grad[5] = dl2y;          /* d/dy */
	}
}

void dpg_tri_p1_at(const double* r, double* val, double* grad)
{
	p1_tri(r[0],r[1],val,grad);
}

int dpg_tri_lagrange_at(int p, const double* rst_vs, int n_pt, const double* pts, double* out)
{
	const int n_s = (p+1)*(p+2)/2;
	double* V = zalloc((size_t)n_s*n_s);
	double* Vinv = zalloc((size_t)n_s*n_s);
	double* pv = zalloc((size_t)n_s);
	double* px = zalloc((size_t)n_s);
	double* py = zalloc((size_t)n_s);
	for (int i = 0; i < n_s; ++i) {
		pkd_basis(p,rst_vs[2*i],rst_vs[2*i+1],pv,px,py);
		for (int k = 0; k < n_s; ++k) V[(size_t)i*n_s + k] = pv[k];
	}
	const int rc = dpg_invert(n_s,V,Vinv);
	if (!rc)
		for (int t = 0; t < n_pt; ++t) {
			pkd_basis(p,pts[2*t],pts[2*t+1],pv,px,py);
			for (int j = 0; j < n_s; ++j) {
				double a = 0.0;
				for (int k = 0; k < n_s; ++k) a += pv[k]*Vinv[(size_t)k*n_s + j];
				out[(size_t)t*n_s + j] = a;
			}
		}
	free(V); free(Vinv); free(pv); free(px); free(py);
	return rc;
}

int dpg_element_ops_build_tri(int p, struct dpg_element_ops* ops)
{
	memset(ops,0,sizeof *ops);
	if (p < 1 || p > 8) return -2;
	static const int* const n_vrule[5] = {NULL, &tri_sym_n2, &tri_sym_n4, &tri_sym_n6, &tri_sym_n8};
	static const double (*const vrule[5])[4] = {NULL, tri_sym_rule2, tri_sym_rule4, tri_sym_rule6, tri_sym_rule8};
	const int q = p + 1;
	const int d = 2, n_s = (p+1)*(p+2)/2, n_c = (p <= 4 ? *n_vrule[p] : q*q), n_fc = p + 1, n_fl = 3, n_ve = 3;
	ops->e_type = DPG_TRI; ops->d = d; ops->p = p;
	ops->n_s = n_s; ops->n_c = n_c; ops->n_fl = n_fl; ops->n_fc = n_fc; ops->n_ve = n_ve;
	static const double VX[3] = {-1.0, 1.0, 0.0}, VY[3] = {-1.0/SQ3, -1.0/SQ3, 2.0/SQ3};
	static const int FVE[3][2] = {{1,2}, {0,2}, {0,1}};

	ops->rst_vs = zalloc((size_t)n_s*d);
	ao_nodes(p,ops->rst_vs);

	/* volume cubature: orders 1..4 the fully symmetric rules of strength 2p (gen_tri_rules.py: the reference's
	 * Witherden-Vincent rules, 3 / 6 / 12 / 16 points), weights of the triangle's area sqrt3; higher orders the
	 * collapsed (Duffy) rule, (a, b) in [-1,1]^2 with r = (1+a)(1-b)/2 - 1, s = b: Gauss-Legendre in a and
	 * Gauss-Jacobi of the weight (1 - b) in b, p + 1 points each, exact to degree 2p + 1; weight w_a w_b / 2, mapped to
	 * the equilateral triangle (Jacobian sqrt3/2) */
	double ga[16], wa[16], gb[16], wb[16];
	dpg_nodes_gl(q,ga,wa);
	dpg_nodes_gj10(q,gb,wb);
	ops->rst_vc = zalloc((size_t)n_c*d);
	ops->w_vc = zalloc((size_t)n_c);
	if (p <= 4) {
		for (int c = 0; c < n_c; ++c) {
			const double* l = vrule[p][c];
			ops->rst_vc[2*c]   = l[0]*VX[0] + l[1]*VX[1] + l[2]*VX[2];
			ops->rst_vc[2*c+1] = l[0]*VY[0] + l[1]*VY[1] + l[2]*VY[2];
			ops->w_vc[c] = l[3]*SQ3;
		}
	} else
	for (int ib = 0; ib < q; ++ib)
		for (int ia = 0; ia < q; ++ia) {
			const int c = ib*q + ia;
			const double a = ga[ia], b = gb[ib];
			const double r = 0.5*(1.0 + a)*(1.0 - b) - 1.0, s = b;
			ops->rst_vc[2*c] = r + (s + 1.0)/2.0;
			ops->rst_vc[2*c+1] = -1.0/SQ3 + (s + 1.0)*SQ3/2.0;
			ops->w_vc[c] = wa[ia]*wb[ib]*0.5*SQ3/2.0;
		}

	/* face cubature and outward reference normals */
	double gf[16], wf[16];
	dpg_nodes_gl(n_fc,gf,wf);
	ops->rst_fc = zalloc((size_t)n_fl*n_fc*d);
	ops->w_fc = zalloc((size_t)n_fc);
	ops->normals_ref = zalloc((size_t)n_fl*d);
	for (int k = 0; k < n_fc; ++k) ops->w_fc[k] = wf[k];
	for (int f = 0; f < n_fl; ++f) {
		const int va = FVE[f][0], vb = FVE[f][1], vo = f;
		for (int k = 0; k < n_fc; ++k) {
			const double t = gf[k];
			ops->rst_fc[((size_t)f*n_fc + k)*d]     = 0.5*(1.0 - t)*VX[va] + 0.5*(1.0 + t)*VX[vb];
			ops->rst_fc[((size_t)f*n_fc + k)*d + 1] = 0.5*(1.0 - t)*VY[va] + 0.5*(1.0 + t)*VY[vb];
		}
		double nx = VY[vb] - VY[va], ny = -(VX[vb] - VX[va]);
		const double mx = 0.5*(VX[va] + VX[vb]) - VX[vo], my = 0.5*(VY[va] + VY[vb]) - VY[vo];
		if (nx*mx + ny*my < 0.0) { nx = -nx; ny = -ny; }
		const double len = sqrt(nx*nx + ny*ny);
		ops->normals_ref[f*d] = nx/len; ops->normals_ref[f*d+1] = ny/len;
	}

	/* Lagrange basis of the nodes: phi = psi V^-1, V[i][k] = psi_k(node i) */
	double* V = zalloc((size_t)n_s*n_s);
	double* Vinv = zalloc((size_t)n_s*n_s);
	double* pv = zalloc((size_t)n_s);
	double* px = zalloc((size_t)n_s);
	double* py = zalloc((size_t)n_s);
	for (int i = 0; i < n_s; ++i) {
		pkd_basis(p,ops->rst_vs[2*i],ops->rst_vs[2*i+1],pv,px,py);
		for (int k = 0; k < n_s; ++k) V[(size_t)i*n_s + k] = pv[k];
	}
	int rc = dpg_invert(n_s,V,Vinv);
	if (rc) { free(V); free(Vinv); free(pv); free(px); free(py); return rc; }
	/* phi_j(x) = sum_k psi_k(x) Vinv[k][j] */
	double* phi = zalloc((size_t)n_s);
	double* phx = zalloc((size_t)n_s);
	double* phy = zalloc((size_t)n_s);
#define LAGRANGE_AT(X, Y) do { \
		pkd_basis(p,(X),(Y),pv,px,py); \
		for (int j = 0; j < n_s; ++j) { \
			double a0 = 0.0, a1 = 0.0, a2 = 0.0; \
			for (int k = 0; k < n_s; ++k) { \
				const double vk = Vinv[(size_t)k*n_s + j]; \
				a0 += pv[k]*vk; a1 += px[k]*vk; a2 += py[k]*vk; \
			} \
			phi[j] = a0; phx[j] = a1; phy[j] = a2; \
		} } while (0)

	ops->cv0_vs_vc = zalloc((size_t)n_c*n_s);
	ops->tw1_vt_vc = zalloc((size_t)d*n_s*n_c);
	ops->cv0_vs_fc = zalloc((size_t)n_fl*n_fc*n_s);
	ops->tw0_vt_fc = zalloc((size_t)n_fl*n_s*n_fc);
	ops->cv0_vv_vc = zalloc((size_t)n_c*n_ve);
	ops->cv1_vv_vc = zalloc((size_t)d*n_c*n_ve);
	ops->cv0_vv_fc = zalloc((size_t)n_fl*n_fc*n_ve);
	ops->cv1_vv_fc = zalloc((size_t)n_fl*d*n_fc*n_ve);
	double gval[3], ggrad[6];
	for (int c = 0; c < n_c; ++c) {
		const double x = ops->rst_vc[2*c], y = ops->rst_vc[2*c+1];
		LAGRANGE_AT(x,y);
		for (int s = 0; s < n_s; ++s) {
			ops->cv0_vs_vc[(size_t)c*n_s + s] = phi[s];
			ops->tw1_vt_vc[((size_t)0*n_s + s)*n_c + c] = phx[s]*ops->w_vc[c];
			ops->tw1_vt_vc[((size_t)1*n_s + s)*n_c + c] = phy[s]*ops->w_vc[c];
		}
		p1_tri(x,y,gval,ggrad);
		for (int k = 0; k < n_ve; ++k) {
			ops->cv0_vv_vc[(size_t)c*n_ve + k] = gval[k];
			for (int dd = 0; dd < d; ++dd) ops->cv1_vv_vc[((size_t)dd*n_c + c)*n_ve + k] = ggrad[dd*3 + k];
		}
	}
	for (int f = 0; f < n_fl; ++f)
		for (int k = 0; k < n_fc; ++k) {
			const double x = ops->rst_fc[((size_t)f*n_fc + k)*d], y = ops->rst_fc[((size_t)f*n_fc + k)*d + 1];
			LAGRANGE_AT(x,y);
			for (int s = 0; s < n_s; ++s) {
				ops->cv0_vs_fc[((size_t)f*n_fc + k)*n_s + s] = phi[s];
				ops->tw0_vt_fc[((size_t)f*n_s + s)*n_fc + k] = phi[s]*ops->w_fc[k];
			}
			p1_tri(x,y,gval,ggrad);
			for (int v = 0; v < n_ve; ++v) {
				ops->cv0_vv_fc[((size_t)f*n_fc + k)*n_ve + v] = gval[v];
				for (int dd = 0; dd < d; ++dd)
					ops->cv1_vv_fc[(((size_t)f*d + dd)*n_fc + k)*n_ve + v] = ggrad[dd*3 + v];
			}
		}
#undef LAGRANGE_AT
	free(V); free(Vinv); free(pv); free(px); free(py); free(phi); free(phx); free(phy);

	/* reference mass matrix and its inverse */
	double* m = zalloc((size_t)n_s*n_s);
	for (int i = 0; i < n_s; ++i)
		for (int j = 0; j < n_s; ++j) {
			double sum = 0.0;
			for (int c = 0; c < n_c; ++c)
				sum += ops->cv0_vs_vc[(size_t)c*n_s+i]*ops->w_vc[c]*ops->cv0_vs_vc[(size_t)c*n_s+j];
			m[(size_t)i*n_s+j] = sum;
		}
	ops->m_inv_ref = zalloc((size_t)n_s*n_s);
	rc = dpg_invert(n_s,m,ops->m_inv_ref);
	free(m);
	if (!rc) {
		static const double V[3][3] = {{-1.0, -1.0/SQ3, 0.0}, {1.0, -1.0/SQ3, 0.0}, {0.0, 2.0/SQ3, 0.0}};
		rc = dpg_simplex_bezier_ops(ops,V);
	}
	return rc;
}
