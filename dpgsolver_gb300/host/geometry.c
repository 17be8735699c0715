/* Geometry of straight-sided (P1 geometry basis) volumes and faces: metric terms, Jacobian determinants, unit
 * normals, surface Jacobians, face node correspondence and mass-matrix inverses.
 *
 * Follows set_up_solver_geometry_T (geometry_T.c:165-185):
 *   - metrics_vc are the cofactors of the Jacobian dx/dr, stored [n_c, d, d] column-major with
 *     m_ij = detJ * dr_j/dx_i at column (i + d*j) (compute_cofactors_T, geometry_T.c:562-583; the reference only
 *     implements d <= 2 there and stops with EXIT_ADD_SUPPORT for d = 3, so the 3D cofactors follow the same
 *     definition);
 *   - jacobian_det_vc = det(dx/dr) (compute_detJV_T, geometry_T.c:484-544);
 *   - normals_fc = normalise(sum_r n_ref[r] * m[:, r]) with jacobian_det_fc = |.| (compute_normals_T,
 *     geometry_T.c:412-445 and compute_unit_normals_and_det_T), evaluated from side 0 of the face;
 *   - m_inv = (cv0^T diag(w_vc * detJ) cv0)^-1 (constructor_mass_T, volume_solver_T.c:115-131), stored only for
 *     volumes whose map is not affine.
 * For a P1 map the reference's interpolation of metric terms from metric nodes to cubature nodes is exact, so the
 * metric terms are evaluated at the cubature nodes directly.
 *
 * Curved volumes (DPG_GEOM_CYLINDER, the parametric annulus): the geometry is of the solution order p (p_g = p for
 * curved volumes, compute_geometry_volume_T, geometry_T.c:225-229) on the GLL solution nodes: the geometry nodes are
 * the parametric map x = r cos(theta), y = r sin(theta) of the volume's (r, theta) bilinear map
 * (constructor_xyz_cylinder_parametric_T, geometry_parametric_T.c:128-171), and the metric terms, Jacobians and
 * normals come from the derivatives of that order-p interpolant (in 2D the cofactors are entries of J, so the
 * reference's interpolation of them from the metric nodes is exact here too).
 * Boundary faces (face_vol[2f+1] = -1) take their geometry from side 0 and keep the identity node order.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "dpg_host.h"

static double det_and_cof(int d, const double J[3][3], double m[3][3])
{
	if (d == 1) { m[0][0] = 1.0; return J[0][0]; }
	if (d == 2) {
		m[0][0] =  J[1][1]; m[0][1] = -J[1][0];
		m[1][0] = -J[0][1]; m[1][1] =  J[0][0];
		return J[0][0]*J[1][1] - J[0][1]*J[1][0];
	}
	for (int i = 0; i < 3; ++i)
	for (int j = 0; j < 3; ++j) {
		const int i1 = (i+1)%3, i2 = (i+2)%3, j1 = (j+1)%3, j2 = (j+2)%3;
		m[i][j] = J[i1][j1]*J[i2][j2] - J[i1][j2]*J[i2][j1];
	}
	return J[0][0]*m[0][0] + J[0][1]*m[0][1] + J[0][2]*m[0][2];
}

/* Jacobian J[i][a] = dx_i/dr_a from P1 basis derivatives grad[a][k] (stride n_ve) and vertex coordinates. */
static void jacobian_at(int d, int n_ve, const double* grad, size_t stride_a, const double* xyz_ve, double J[3][3])
{
	for (int i = 0; i < d; ++i)
	for (int a = 0; a < d; ++a) {
		double s = 0.0;
		for (int k = 0; k < n_ve; ++k) s += grad[a*stride_a + k]*xyz_ve[k*3 + i];
		J[i][a] = s;
	}
}

/* Geometry nodes of a curved volume: X[s][i] at the solution (GLL) nodes rst_vs of its (r, theta) cell. */
static void cylinder_nodes(const struct dpg_element_ops* ops, const double* rt_ve, double (*X)[3])
{
	const int d = ops->d;
	for (int s = 0; s < ops->n_s; ++s) {
		const double* r = &ops->rst_vs[(size_t)s*d];
		double rr = 0.0, th = 0.0;
		for (int k = 0; k < 4; ++k) {
			double w = 1.0;
			for (int a = 0; a < 2; ++a) w *= ((k >> a) & 1) ? 0.5*(1.0 + r[a]) : 0.5*(1.0 - r[a]);
			rr += w*rt_ve[k*3]; th += w*rt_ve[k*3 + 1];
		}
		X[s][0] = rr*cos(th); X[s][1] = rr*sin(th); X[s][2] = 0.0;
	}
}

/* J = dx/dr and x at reference point r of the order-p interpolant through the geometry nodes X. */
static void curved_at(const struct dpg_element_ops* ops, const double (*X)[3], const double* r, double J[3][3], double* x)
{
	const int d = ops->d, n1 = ops->p + 1, n_s = ops->n_s;
	double g1[16], val[125], grad[3*125];
	for (int i = 0; i < n1; ++i) g1[i] = ops->rst_vs[(size_t)i*d];   /* the 1D GLL nodes: first n1 solution nodes */
	dpg_tp_basis_at(d,n1,g1,r,val,grad);
	for (int i = 0; i < d; ++i) {
		x[i] = 0.0;
		for (int s = 0; s < n_s; ++s) x[i] += val[s]*X[s][i];
		for (int a = 0; a < d; ++a) {
			double t = 0.0;
			for (int s = 0; s < n_s; ++s) t += grad[(size_t)a*n_s + s]*X[s][i];
			J[i][a] = t;
		}
	}
}

int dpg_setup_geometry(struct dpg_sim* sim)
{
	const int d = sim->d;
	const int curved = (sim->geom == DPG_GEOM_CYLINDER);
	double (*X)[3] = NULL, (*Xr)[3] = NULL;
	if (curved) {
		X = malloc(sizeof *X*125);
		Xr = malloc(sizeof *Xr*125);
		if (!X || !Xr) { free(X); free(Xr); return -13; }
	}
	/* ---- volumes ---- */
	for (int v = 0; v < sim->n_vol; ++v) {
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
		const int n_c = ops->n_c, n_ve = ops->n_ve;
		const double* xyz_ve = &sim->xyz_ve[(size_t)v*DPG_NVE_MAX*3];
		double* met = &sim->metrics_vc[(size_t)sim->vol_geo_off[v]*d*d];
		double* jdet = &sim->jacobian_det_vc[sim->vol_geo_off[v]];
		double* xyz = &sim->xyz_vc[(size_t)sim->vol_geo_off[v]*d];
		if (curved) cylinder_nodes(ops,xyz_ve,X);
		for (int c = 0; c < n_c; ++c) {
			double J[3][3] = {{0}}, m[3][3], xc[3] = {0,0,0};
			if (curved) curved_at(ops,(const double (*)[3])X,&ops->rst_vc[(size_t)c*d],J,xc);
			else jacobian_at(d,n_ve,&ops->cv1_vv_vc[(size_t)c*n_ve],(size_t)n_c*n_ve,xyz_ve,J);
			const double det = det_and_cof(d,J,m);
			if (!(det > 0.0)) { free(X); free(Xr); return -10; }
			jdet[c] = det;
			for (int i = 0; i < d; ++i)
			for (int j = 0; j < d; ++j)
				met[c + (size_t)n_c*(i + d*j)] = m[i][j];
			for (int i = 0; i < d; ++i) {
				double s = 0.0;
				if (curved) s = xc[i];
				else for (int k = 0; k < n_ve; ++k) s += ops->cv0_vv_vc[(size_t)c*n_ve+k]*xyz_ve[k*3+i];
				xyz[c + (size_t)n_c*i] = s;
			}
		}
		/* affine test: all metric terms equal to those of node 0 */
		double scale = 0.0;
		for (int k = 0; k < d*d; ++k) scale = fmax(scale,fabs(met[(size_t)n_c*k]));
		int affine = !curved;
		for (int c = 1; c < n_c && affine; ++c)
			for (int k = 0; k < d*d; ++k)
				if (fabs(met[c + (size_t)n_c*k] - met[(size_t)n_c*k]) > 1e-13*scale) { affine = 0; break; }
		sim->vol_affine[v] = affine;
	}

	/* ---- faces ---- */
	double per_len[DPG_DIM_MAX];
	for (int a = 0; a < d; ++a) per_len[a] = sim->domain_hi[a] - sim->domain_lo[a];
	for (int f = 0; f < sim->n_face; ++f) {
		const int vl = sim->face_vol[2*f], lfl = sim->face_lf[2*f];
		/* the face's cubature: that of its order (mixed orders: the larger of its volumes'); the local face
		 * geometry (nodes, P1 basis, reference normals) is the element type's, the same at every order */
		const struct dpg_element_ops* ops = &sim->ops[dpg_face_order(sim,f) - sim->ops[0].p];
		const int n_fc = ops->n_fc, n_ve = ops->n_ve;
		const double* xyz_ve = &sim->xyz_ve[(size_t)vl*DPG_NVE_MAX*3];
		const int64_t off = sim->face_geo_off[f];
		double* nrm = &sim->normals_fc[(size_t)off*d];
		double* jf  = &sim->jacobian_det_fc[off];
		double* xf  = &sim->xyz_fc[(size_t)off*d];
		const double* nref = &ops->normals_ref[(size_t)lfl*d];
		if (curved) cylinder_nodes(ops,xyz_ve,X);
		for (int q = 0; q < n_fc; ++q) {
			double J[3][3] = {{0}}, m[3][3], xq[3] = {0,0,0};
			if (curved) curved_at(ops,(const double (*)[3])X,&ops->rst_fc[((size_t)lfl*n_fc + q)*d],J,xq);
			else jacobian_at(d,n_ve,&ops->cv1_vv_fc[((size_t)lfl*d*n_fc + q)*n_ve],(size_t)n_fc*n_ve,xyz_ve,J);
			det_and_cof(d,J,m);
			double n[3] = {0,0,0}, len = 0.0;
			for (int i = 0; i < d; ++i) {
				for (int r = 0; r < d; ++r) n[i] += nref[r]*m[i][r];
				len += n[i]*n[i];
			}
			len = sqrt(len);
			jf[q] = len;
			for (int i = 0; i < d; ++i) nrm[(size_t)q*d+i] = n[i]/len;
			for (int i = 0; i < d; ++i) {
				double s = 0.0;
				if (curved) s = xq[i];
				else
					for (int k = 0; k < n_ve; ++k)
						s += ops->cv0_vv_fc[((size_t)lfl*n_fc + q)*n_ve+k]*xyz_ve[k*3+i];
				xf[q + (size_t)n_fc*i] = s;
			}
		}
		/* node correspondence with side 1: match physical coordinates (modulo the periodic box). */
		int* nc = &sim->nc_fc[off];
		const int vr = sim->face_vol[2*f+1];
		if (vr < 0) { for (int q = 0; q < n_fc; ++q) nc[q] = q; continue; }
		const int lfr = sim->face_lf[2*f+1];
		const struct dpg_element_ops* opr = ops;
		const double* xyz_ver = &sim->xyz_ve[(size_t)vr*DPG_NVE_MAX*3];
		double xr[64*3];
		if (curved) cylinder_nodes(opr,xyz_ver,Xr);
		for (int q = 0; q < n_fc; ++q) {
			double J[3][3], xq[3] = {0,0,0};
			if (curved) curved_at(opr,(const double (*)[3])Xr,&opr->rst_fc[((size_t)lfr*n_fc + q)*d],J,xq);
			for (int i = 0; i < d; ++i) {
				double s = 0.0;
				if (curved) s = xq[i];
				else
					for (int k = 0; k < n_ve; ++k)
						s += opr->cv0_vv_fc[((size_t)lfr*n_fc + q)*opr->n_ve+k]*xyz_ver[k*3+i];
				xr[q*3+i] = s;
			}
		}
		double hscale = 0.0;
		for (int i = 0; i < d; ++i) hscale = fmax(hscale,fabs(xf[(size_t)n_fc*i] - xf[(size_t)n_fc*i + n_fc-1]));
		for (int q = 0; q < n_fc; ++q) {
			int best = -1; double bd = 1e300;
			for (int qq = 0; qq < n_fc; ++qq) {
				double dist = 0.0;
				for (int i = 0; i < d; ++i) {
					double dx = xf[q + (size_t)n_fc*i] - xr[qq*3+i];
					if (per_len[i] > 0.0) dx -= per_len[i]*nearbyint(dx/per_len[i]);
					dist += dx*dx;
				}
				if (dist < bd) { bd = dist; best = qq; }
			}
			if (sqrt(bd) > 1e-8*(hscale > 0 ? hscale : 1.0)) { free(X); free(Xr); return -12; }
			nc[q] = best;
		}
	}
	free(X); free(Xr);
	return 0;
}

/* Mass-matrix inverses of the non-affine volumes (affine volumes use m_inv_ref / detJ, which is the same matrix).
 * vol_minv_off must already give the storage of each volume (0 doubles for affine volumes). */
int dpg_setup_mass_inverse(struct dpg_sim* sim)
{
	for (int v = 0; v < sim->n_vol; ++v) {
		if (sim->vol_minv_off[v+1] == sim->vol_minv_off[v]) continue;
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
		const int n_c = ops->n_c, n_s = ops->n_s;
		const double* jdet = &sim->jacobian_det_vc[sim->vol_geo_off[v]];
		double* mass = (double*)malloc(sizeof(double)*(size_t)n_s*n_s);
		for (int i = 0; i < n_s; ++i)
		for (int j = 0; j < n_s; ++j) {
			double s = 0.0;
			for (int c = 0; c < n_c; ++c)
				s += ops->cv0_vs_vc[(size_t)c*n_s+i]*ops->w_vc[c]*jdet[c]*ops->cv0_vs_vc[(size_t)c*n_s+j];
			mass[(size_t)i*n_s+j] = s;
		}
		const int rc = dpg_invert(n_s,mass,&sim->m_inv[sim->vol_minv_off[v]]);
		free(mass);
		if (rc) return -11;
	}
	return 0;
}
