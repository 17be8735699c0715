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

int dpg_setup_geometry(struct dpg_sim* sim)
{
	const int d = sim->d;
	/* ---- volumes ---- */
	for (int v = 0; v < sim->n_vol; ++v) {
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
		const int n_c = ops->n_c, n_ve = ops->n_ve;
		const double* xyz_ve = &sim->xyz_ve[(size_t)v*DPG_NVE_MAX*3];
		double* met = &sim->metrics_vc[(size_t)sim->vol_geo_off[v]*d*d];
		double* jdet = &sim->jacobian_det_vc[sim->vol_geo_off[v]];
		double* xyz = &sim->xyz_vc[(size_t)sim->vol_geo_off[v]*d];
		for (int c = 0; c < n_c; ++c) {
			double J[3][3] = {{0}}, m[3][3];
			jacobian_at(d,n_ve,&ops->cv1_vv_vc[(size_t)c*n_ve],(size_t)n_c*n_ve,xyz_ve,J);
			const double det = det_and_cof(d,J,m);
			if (!(det > 0.0)) return -10;
			jdet[c] = det;
			for (int i = 0; i < d; ++i)
			for (int j = 0; j < d; ++j)
				met[c + (size_t)n_c*(i + d*j)] = m[i][j];
			for (int i = 0; i < d; ++i) {
				double s = 0.0;
				for (int k = 0; k < n_ve; ++k) s += ops->cv0_vv_vc[(size_t)c*n_ve+k]*xyz_ve[k*3+i];
				xyz[c + (size_t)n_c*i] = s;
			}
		}
		/* affine test: all metric terms equal to those of node 0 */
		double scale = 0.0;
		for (int k = 0; k < d*d; ++k) scale = fmax(scale,fabs(met[(size_t)n_c*k]));
		int affine = 1;
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
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[vl]];
		const int n_fc = ops->n_fc, n_ve = ops->n_ve;
		const double* xyz_ve = &sim->xyz_ve[(size_t)vl*DPG_NVE_MAX*3];
		const int64_t off = sim->face_geo_off[f];
		double* nrm = &sim->normals_fc[(size_t)off*d];
		double* jf  = &sim->jacobian_det_fc[off];
		double* xf  = &sim->xyz_fc[(size_t)off*d];
		const double* nref = &ops->normals_ref[(size_t)lfl*d];
		for (int q = 0; q < n_fc; ++q) {
			double J[3][3] = {{0}}, m[3][3];
			jacobian_at(d,n_ve,&ops->cv1_vv_fc[((size_t)lfl*d*n_fc + q)*n_ve],(size_t)n_fc*n_ve,xyz_ve,J);
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
		const struct dpg_element_ops* opr = &sim->ops[sim->vol_ops[vr]];
		const double* xyz_ver = &sim->xyz_ve[(size_t)vr*DPG_NVE_MAX*3];
		double xr[64*3];
		for (int q = 0; q < n_fc; ++q)
			for (int i = 0; i < d; ++i) {
				double s = 0.0;
				for (int k = 0; k < n_ve; ++k)
					s += opr->cv0_vv_fc[((size_t)lfr*n_fc + q)*opr->n_ve+k]*xyz_ver[k*3+i];
				xr[q*3+i] = s;
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
			if (sqrt(bd) > 1e-8*(hscale > 0 ? hscale : 1.0)) return -12;
			nc[q] = best;
		}
	}
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
