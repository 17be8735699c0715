/* Simulation set-up: structured periodic meshes of QUAD/HEX elements, volumes, faces, element operators, geometry
 * and the initial solution; control-file parsing; L2 errors.
 *
 * Mirrors the reference's set-up sequence for the DG residual path:
 *   constructor_Simulation (simulation.c:128-144; control-file keys of set_simulation_core, :371-431, and the
 *   test-case keys of read_test_case_parameters, test_case_T.c:258-302), the volume/face lists with neigh_info
 *   (face.h:47-97), set_up_solver_geometry_T (geometry_T.c:165-185) and set_initial_solution.
 * Structured meshes: element e = i + nx*(j + ny*k); face f = d*e + a joins the +a face of e (ind_lf = 2a+1) with the
 * -a face of its periodic neighbour (ind_lf = 2a), side 0 being the smaller (volume, local face) as in the
 * reference's constructor_Faces.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dpg_host.h"
#include "dpg_gb300.h"

const char* dpg_status_string(int status)
{
	switch (status) {
	case DPG_OK:                return "ok";
	case DPG_ERR_INVALID:       return "invalid argument";
	case DPG_ERR_UNSUPPORTED:   return "unsupported";
	case DPG_ERR_CUDA:          return "cuda error";
	case DPG_ERR_NONFINITE:     return "non-finite residual";
	case DPG_ERR_TIMEOUT:       return "device wait timed out";
	case DPG_ERR_NOT_CONVERGED: return "not converged";
	case DPG_ERR_NO_DEVICE:     return "no cuda device";
	case DPG_ERR_IO:            return "i/o error";
	case DPG_ERR_TOO_LARGE:     return "problem exceeds the fixed scratch of the allocation-free entry point";
	default:                    return "unknown status";
	}
}

void dpg_sim_params_default(struct dpg_sim_params* prm)
{
	memset(prm,0,sizeof *prm);
	prm->d = 2; prm->e_type = DPG_QUAD; prm->p = 2;
	prm->n_elem[0] = prm->n_elem[1] = prm->n_elem[2] = 16;
	prm->lo[0] = prm->lo[1] = -5.0; prm->hi[0] = prm->hi[1] = 5.0;
	prm->lo[2] = 0.0; prm->hi[2] = 2.5;
	prm->pde_index = DPG_PDE_EULER;
	prm->num_flux = DPG_NUM_FLUX_ROE_PIKE;
	prm->test_case = DPG_TC_ISENTROPIC_VORTEX;
	const double vx[8] = {5.0, 0.0, 0.0, 1.0, 1.0, 1.0, 0.0, 1.0};
	memcpy(prm->vortex,vx,sizeof vx);
	prm->b_adv[0] = 1.0; prm->b_adv[1] = 0.5;
	prm->solver_proc = DPG_SOLVER_E; prm->solver_type_e = DPG_SOLVER_E_SSP_RK_33;
	prm->dt = 0.0; prm->time_final = 10.0;
	prm->seed = 0;
	prm->mesh_kind = DPG_MESH_BOX;
	prm->num_flux_2nd = DPG_NUM_FLUX_INVALID;
	prm->mu = 0.0; prm->Pr = 0.72; prm->omega = 0.0;
	const double fs[5] = {1.0, 1.0, 0.0, 0.0, 1.0};
	memcpy(prm->bc_state,fs,sizeof fs);
	prm->wall_p = 1.0; prm->wall_T = 1.0;
}

#define ALLOC(ptr,n) do { const size_t n_alloc_ = (size_t)(n); (ptr) = calloc(n_alloc_ > 0 ? n_alloc_ : 1, sizeof *(ptr)); if (!(ptr)) goto fail; } while (0)

static int euler_like(int pde) { return pde == DPG_PDE_EULER || pde == DPG_PDE_NAVIER_STOKES; }

static int check_params(const struct dpg_sim_params* prm)
{
	const int d = prm->d;
	if (d < 2 || d > 3) return DPG_ERR_UNSUPPORTED;
	if ((d == 2 && prm->e_type != DPG_QUAD && prm->e_type != DPG_TRI) ||
	    (d == 3 && prm->e_type != DPG_HEX && prm->e_type != DPG_TET))
		return DPG_ERR_UNSUPPORTED;
	/* TRI, TET: periodic structured meshes of linear advection or the Euler equations; TET of orders 1..4 */
	if (prm->e_type == DPG_TRI || prm->e_type == DPG_TET) {
		if ((prm->pde_index != DPG_PDE_ADVECTION && prm->pde_index != DPG_PDE_EULER) || prm->mesh_kind != DPG_MESH_BOX)
			return DPG_ERR_UNSUPPORTED;
		for (int k = 0; k < 2*d; ++k) if (prm->bc_side[k] != 0) return DPG_ERR_UNSUPPORTED;
		if (prm->e_type == DPG_TET && (prm->p > 4 || prm->p_max > 4)) return DPG_ERR_UNSUPPORTED;
	}
	if (prm->pde_index != DPG_PDE_EULER && prm->pde_index != DPG_PDE_ADVECTION &&
	    prm->pde_index != DPG_PDE_NAVIER_STOKES) return DPG_ERR_UNSUPPORTED;
	if (prm->p < 1 || prm->p > DPG_P_MAX) return DPG_ERR_INVALID;
	/* mixed orders: linear advection and the Euler equations on periodic straight-sided meshes */
	if (prm->p_max > prm->p) {
		if (prm->p_max > DPG_P_MAX) return DPG_ERR_INVALID;
		if ((prm->pde_index != DPG_PDE_ADVECTION && prm->pde_index != DPG_PDE_EULER) || prm->mesh_kind != DPG_MESH_BOX)
			return DPG_ERR_UNSUPPORTED;
		for (int k = 0; k < 2*d; ++k) if (prm->bc_side[k] != 0) return DPG_ERR_UNSUPPORTED;
	}
	if (euler_like(prm->pde_index) &&
	    prm->num_flux != DPG_NUM_FLUX_ROE_PIKE && prm->num_flux != DPG_NUM_FLUX_LAX_FRIEDRICHS) return DPG_ERR_UNSUPPORTED;
	if (prm->pde_index == DPG_PDE_ADVECTION && prm->num_flux != DPG_NUM_FLUX_UPWIND) return DPG_ERR_UNSUPPORTED;
	/* Navier-Stokes: BR2 viscous flux with a positive constant viscosity (num_flux_2nd, test_case_T.h:116) */
	if (prm->pde_index == DPG_PDE_NAVIER_STOKES &&
	    (prm->num_flux_2nd != DPG_NUM_FLUX_BR2_STABLE || !(prm->mu > 0.0) || !(prm->Pr > 0.0))) return DPG_ERR_UNSUPPORTED;
	if (prm->mesh_kind == DPG_MESH_ANNULUS && d != 2) return DPG_ERR_UNSUPPORTED;
	/* boundary conditions: the Euler ones for the Euler and Navier-Stokes equations, the no-slip walls for
	 * Navier-Stokes only; none for advection (its meshes are periodic) */
	const int n_sides = (prm->mesh_kind == DPG_MESH_ANNULUS ? 2 : 2*d);
	for (int k = 0; k < n_sides; ++k) {
		const int bc = prm->bc_side[k];
		if (bc == 0) continue;
		if (prm->pde_index == DPG_PDE_ADVECTION) return DPG_ERR_UNSUPPORTED;
		if (bc == DPG_BC_RIEMANN || bc == DPG_BC_SLIPWALL) continue;
		if ((bc == DPG_BC_NOSLIP_ADIABATIC || bc == DPG_BC_NOSLIP_ALL_ROTATING) &&
		    prm->pde_index == DPG_PDE_NAVIER_STOKES) continue;
		return DPG_ERR_UNSUPPORTED;
	}
	if (prm->mesh_kind == DPG_MESH_ANNULUS && (prm->bc_side[0] == 0 || prm->bc_side[1] == 0)) return DPG_ERR_INVALID;
	if (prm->mesh_kind == DPG_MESH_BOX)
		for (int a = 0; a < d; ++a)
			if ((prm->bc_side[2*a] == 0) != (prm->bc_side[2*a+1] == 0)) return DPG_ERR_INVALID;   /* periodic pairs */
	return DPG_OK;
}

/* Everything after the mesh: operators, volume and face storage, geometry, mass inverses, initial solution. */
static int sim_build(const struct dpg_sim_params* prm, const struct dpg_mesh* mesh, struct dpg_sim** sim_out)
{
	const int d = prm->d;
	struct dpg_sim* sim = calloc(1,sizeof *sim);
	if (!sim) return DPG_ERR_INVALID;
	sim->d = d;
	sim->pde_index = prm->pde_index;
	sim->n_var = sim->n_eq = (euler_like(prm->pde_index) ? d+2 : 1);
	sim->ind_num_flux[0] = prm->num_flux;
	sim->ind_num_flux[1] = (prm->pde_index == DPG_PDE_NAVIER_STOKES ? prm->num_flux_2nd : DPG_NUM_FLUX_INVALID);
	sim->geom = mesh->geom;
	sim->mu = prm->mu; sim->Pr = prm->Pr; sim->r_s = 1.0;
	sim->bc_omega = prm->omega;
	sim->bc_rho = prm->wall_p/(sim->r_s*prm->wall_T);
	memcpy(sim->bc_state,prm->bc_state,sizeof sim->bc_state);
	sim->tc_data[0] = prm->lo[0]; sim->tc_data[1] = prm->hi[0]; sim->tc_data[2] = prm->wall_p; sim->tc_data[3] = prm->wall_T;
	sim->solver_proc = prm->solver_proc; sim->solver_type_e = prm->solver_type_e;
	sim->test_case = prm->test_case;
	sim->dt = prm->dt; sim->time = 0.0; sim->time_final = prm->time_final;
	memcpy(sim->b_adv,prm->b_adv,sizeof sim->b_adv);
	memcpy(sim->vortex,prm->vortex,sizeof sim->vortex);
	for (int a = 0; a < DPG_DIM_MAX; ++a) { sim->domain_lo[a] = mesh->lo[a]; sim->domain_hi[a] = mesh->hi[a]; }

	/* element operators of every order present: ops[k] has order p_lo + k */
	int p_lo = prm->p, p_hi = (prm->p_max > prm->p ? prm->p_max : prm->p);
	if (mesh->vol_p) {   /* given orders (the reference's per-volume p_ref) */
		p_lo = DPG_P_MAX; p_hi = 1;
		for (int v = 0; v < mesh->n_vol; ++v) {
			if (mesh->vol_p[v] < p_lo) p_lo = mesh->vol_p[v];
			if (mesh->vol_p[v] > p_hi) p_hi = mesh->vol_p[v];
		}
	}
	sim->n_ops = p_hi - p_lo + 1;
	ALLOC(sim->ops,sim->n_ops);
	for (int k = 0; k < sim->n_ops; ++k)
		if (dpg_element_ops_build(prm->e_type,p_lo + k,&sim->ops[k]) != 0) { dpg_sim_destroy(sim); return DPG_ERR_INVALID; }
	const int n_fl = sim->ops[0].n_fl, n_var = sim->n_var;

	const int n_vol = mesh->n_vol;
	sim->n_vol = n_vol;
	ALLOC(sim->vol_ops,n_vol); ALLOC(sim->vol_p,n_vol); ALLOC(sim->vol_affine,n_vol);
	ALLOC(sim->vol_dof_off,n_vol+1); ALLOC(sim->vol_geo_off,n_vol+1); ALLOC(sim->vol_minv_off,n_vol+1);
	ALLOC(sim->xyz_ve,(size_t)n_vol*DPG_NVE_MAX*3);
	ALLOC(sim->vol_face,(size_t)n_vol*DPG_NFL_MAX); ALLOC(sim->vol_face_side,(size_t)n_vol*DPG_NFL_MAX);
	/* each volume's order: given, or uniform draws from p_lo .. p_hi in volume order (splitmix64 from p_seed) */
	{
		uint64_t st = prm->p_seed;
		for (int v = 0; v < n_vol; ++v) {
			int pv = p_lo;
			if (mesh->vol_p) pv = mesh->vol_p[v];
			else if (p_hi > p_lo) pv += (int)(dpg_splitmix64(&st) % (uint64_t)(p_hi - p_lo + 1));
			sim->vol_p[v] = pv; sim->vol_ops[v] = pv - p_lo;
		}
	}
	sim->vol_dof_off[0] = sim->vol_geo_off[0] = 0;
	for (int v = 0; v < n_vol; ++v) {
		const struct dpg_element_ops* ov = &sim->ops[sim->vol_ops[v]];
		sim->vol_dof_off[v+1] = sim->vol_dof_off[v] + (int64_t)ov->n_s*n_var;
		sim->vol_geo_off[v+1] = sim->vol_geo_off[v] + ov->n_c;
	}
	const int64_t n_geo = sim->vol_geo_off[n_vol];
	memcpy(sim->xyz_ve,mesh->xyz_ve,sizeof(double)*(size_t)n_vol*DPG_NVE_MAX*3);
	ALLOC(sim->sol_coef,sim->vol_dof_off[n_vol]); ALLOC(sim->sol_coef_p,sim->vol_dof_off[n_vol]);
	ALLOC(sim->rhs,sim->vol_dof_off[n_vol]);
	ALLOC(sim->metrics_vc,(size_t)n_geo*d*d); ALLOC(sim->jacobian_det_vc,(size_t)n_geo);
	ALLOC(sim->xyz_vc,(size_t)n_geo*d);

	/* faces: the mesh's two sides of each face; every local face of every volume on exactly one face */
	const int n_face = mesh->n_face;
	sim->n_face = n_face;
	ALLOC(sim->face_vol,2*n_face); ALLOC(sim->face_lf,2*n_face); ALLOC(sim->face_nfc,n_face);
	ALLOC(sim->face_bc,n_face); ALLOC(sim->face_geo_off,n_face+1); ALLOC(sim->face_p,n_face);
	for (size_t q = 0; q < (size_t)n_vol*DPG_NFL_MAX; ++q) sim->vol_face[q] = -1;
	for (int f = 0; f < n_face; ++f) {
		sim->face_bc[f] = (mesh->face_bc ? mesh->face_bc[f] : 0);
		for (int sd = 0; sd < 2; ++sd) {
			const int v = mesh->face_vol[2*f+sd], lf = mesh->face_lf[2*f+sd];
			if (sd == 1 && v < 0 && sim->face_bc[f] != 0) {   /* a boundary face: one side */
				sim->face_vol[2*f+1] = -1; sim->face_lf[2*f+1] = -1;
				continue;
			}
			if (v < 0 || v >= n_vol || lf < 0 || lf >= n_fl || sim->vol_face[v*DPG_NFL_MAX + lf] != -1) {
				dpg_sim_destroy(sim);
				return DPG_ERR_INVALID;
			}
			sim->face_vol[2*f+sd] = v; sim->face_lf[2*f+sd] = lf;
			sim->vol_face[v*DPG_NFL_MAX + lf] = f; sim->vol_face_side[v*DPG_NFL_MAX + lf] = sd;
		}
		/* the face's order: the larger of its volumes' (compute_face_reference_order, face_solver.c:123-132) */
		const int vr = sim->face_vol[2*f+1];
		int pf = sim->vol_p[sim->face_vol[2*f]];
		if (vr >= 0 && sim->vol_p[vr] > pf) pf = sim->vol_p[vr];
		sim->face_p[f] = pf;
		sim->face_nfc[f] = sim->ops[pf - p_lo].n_fc;
		for (int sd = 0; sd < 2; ++sd) {
			const int v = sim->face_vol[2*f+sd];
			if (v >= 0 && sim->vol_p[v] < pf &&
			    dpg_element_face_ops_build(&sim->ops[sim->vol_ops[v]],&sim->ops[pf - p_lo]) != 0) {
				dpg_sim_destroy(sim);
				return DPG_ERR_INVALID;
			}
		}
	}
	for (int v = 0; v < n_vol; ++v)
		for (int lf = 0; lf < n_fl; ++lf)
			if (sim->vol_face[v*DPG_NFL_MAX + lf] < 0) { dpg_sim_destroy(sim); return DPG_ERR_INVALID; }
	sim->face_geo_off[0] = 0;
	for (int f = 0; f < n_face; ++f) sim->face_geo_off[f+1] = sim->face_geo_off[f] + sim->face_nfc[f];
	const int64_t n_fnode = sim->face_geo_off[n_face];
	ALLOC(sim->nc_fc,(size_t)n_fnode); ALLOC(sim->normals_fc,(size_t)n_fnode*d);
	ALLOC(sim->jacobian_det_fc,(size_t)n_fnode); ALLOC(sim->xyz_fc,(size_t)n_fnode*d);

	if (dpg_setup_geometry(sim) != 0) { dpg_sim_destroy(sim); return DPG_ERR_INVALID; }
	sim->vol_minv_off[0] = 0;
	for (int v = 0; v < n_vol; ++v) {
		const int n_s = sim->ops[sim->vol_ops[v]].n_s;
		sim->vol_minv_off[v+1] = sim->vol_minv_off[v] + (sim->vol_affine[v] ? 0 : (int64_t)n_s*n_s);
	}
	ALLOC(sim->m_inv,sim->vol_minv_off[n_vol]);
	if (dpg_setup_mass_inverse(sim) != 0) { dpg_sim_destroy(sim); return DPG_ERR_INVALID; }

	/* the rotating wall's imposed total energy: p / (gamma - 1) + rho |V|^2 / 2 at the inner radius */
	{
		const double vt = sim->bc_omega*sim->tc_data[0];
		sim->bc_E = prm->wall_p/DPG_GM1 + 0.5*sim->bc_rho*vt*vt;
	}
	dpg_set_initial_solution(sim);
	*sim_out = sim;
	return DPG_OK;
fail:
	dpg_sim_destroy(sim);
	return DPG_ERR_INVALID;
}

int dpg_sim_create(const struct dpg_sim_params* prm, struct dpg_sim** sim_out)
{
	if (!prm || !sim_out) return DPG_ERR_INVALID;
	*sim_out = NULL;
	int rc = check_params(prm);
	if (rc) return rc;
	struct dpg_mesh mesh;
	if (prm->mesh_kind == DPG_MESH_ANNULUS) {
		if ((rc = dpg_mesh_annulus(prm,&mesh))) return rc;
	} else if (prm->e_type == DPG_TRI) {
		for (int a = 0; a < 2; ++a)
			if (prm->n_elem[a] < 1 || !(prm->hi[a] > prm->lo[a])) return DPG_ERR_INVALID;
		if ((rc = dpg_mesh_tri_structured(prm,&mesh))) return rc;
	} else if (prm->e_type == DPG_TET) {
		for (int a = 0; a < 3; ++a)
			if (prm->n_elem[a] < 1 || !(prm->hi[a] > prm->lo[a])) return DPG_ERR_INVALID;
		if ((rc = dpg_mesh_tet_structured(prm,&mesh))) return rc;
	} else {
		for (int a = 0; a < prm->d; ++a)
			if (prm->n_elem[a] < 1 || !(prm->hi[a] > prm->lo[a])) return DPG_ERR_INVALID;
		if ((rc = dpg_mesh_structured(prm,&mesh))) return rc;
	}
	rc = sim_build(prm,&mesh,sim_out);
	dpg_mesh_free(&mesh);
	return rc;
}

int dpg_sim_create_from_gmsh(const struct dpg_sim_params* prm, const char* msh_path, struct dpg_sim** sim_out)
{
	if (!prm || !msh_path || !sim_out) return DPG_ERR_INVALID;
	*sim_out = NULL;
	int rc = check_params(prm);
	if (rc) return rc;
	struct dpg_mesh mesh;
	if ((rc = dpg_mesh_read_gmsh(msh_path,prm->d,prm->e_type,&mesh))) return rc;
	rc = sim_build(prm,&mesh,sim_out);
	dpg_mesh_free(&mesh);
	return rc;
}

/* The reference's own volume and face lists (struct Volume, volume.h:36-57; struct Face with neigh_info[2],
 * face.h:40-97; Solver_Volume_T::sol_coef) -> the data model: the vertices and the two sides of every face are taken
 * as given (side 0 = neigh_info[0], the volume whose outward normal is the face's), the operators, geometry and node
 * correspondences are formed here as for any other mesh.  Straight-sided QUAD / HEX volumes. */
int dpg_sim_create_from_lists(const struct dpg_sim_params* prm, int n_vol, const struct dpg_ref_volume* vols,
                              int n_face, const struct dpg_ref_face* faces, struct dpg_sim** sim_out)
{
	if (!prm || !vols || !faces || !sim_out || n_vol < 1 || n_face < 1) return DPG_ERR_INVALID;
	*sim_out = NULL;
	int rc = check_params(prm);
	if (rc) return rc;
	if (prm->mesh_kind != DPG_MESH_BOX) return DPG_ERR_UNSUPPORTED;
	/* per-volume orders (an adapted mesh): within 1 .. DPG_P_MAX, mixed ones for linear advection only */
	int given_p = 0, mixed = 0;
	for (int v = 0; v < n_vol; ++v) {
		const int pv = vols[v].p_ref > 0 ? vols[v].p_ref : prm->p;
		if (vols[v].p_ref < 0 || pv > DPG_P_MAX) return DPG_ERR_INVALID;
		given_p |= (vols[v].p_ref > 0);
		mixed |= (pv != (vols[0].p_ref > 0 ? vols[0].p_ref : prm->p));
	}
	if (mixed && prm->pde_index != DPG_PDE_ADVECTION && prm->pde_index != DPG_PDE_EULER) return DPG_ERR_UNSUPPORTED;
	const int d = prm->d, n_ve = 1 << d;
	struct dpg_mesh mesh;
	memset(&mesh,0,sizeof mesh);
	mesh.d = d; mesh.n_vol = n_vol; mesh.n_face = n_face; mesh.geom = DPG_GEOM_STRAIGHT;
	mesh.xyz_ve = calloc((size_t)n_vol*DPG_NVE_MAX*3,sizeof(double));
	mesh.face_vol = malloc(sizeof(int)*2*(size_t)n_face);
	mesh.face_lf = malloc(sizeof(int)*2*(size_t)n_face);
	mesh.face_bc = malloc(sizeof(int)*(size_t)n_face);
	if (!mesh.xyz_ve || !mesh.face_vol || !mesh.face_lf || !mesh.face_bc) { dpg_mesh_free(&mesh); return DPG_ERR_INVALID; }
	for (int a = 0; a < 3; ++a) { mesh.lo[a] = (a < d ? 1e300 : 0.0); mesh.hi[a] = (a < d ? -1e300 : 0.0); }
	if (given_p) {
		mesh.vol_p = malloc(sizeof(int)*(size_t)n_vol);
		if (!mesh.vol_p) { dpg_mesh_free(&mesh); return DPG_ERR_INVALID; }
		for (int v = 0; v < n_vol; ++v) mesh.vol_p[v] = vols[v].p_ref > 0 ? vols[v].p_ref : prm->p;
	}
	for (int v = 0; v < n_vol; ++v) {
		if (!vols[v].xyz_ve) { dpg_mesh_free(&mesh); return DPG_ERR_INVALID; }
		for (int k = 0; k < n_ve; ++k)
			for (int a = 0; a < d; ++a) {
				const double x = vols[v].xyz_ve[(size_t)k*d + a];
				if (!isfinite(x)) { dpg_mesh_free(&mesh); return DPG_ERR_INVALID; }
				mesh.xyz_ve[((size_t)v*DPG_NVE_MAX + k)*3 + a] = x;
				if (x < mesh.lo[a]) mesh.lo[a] = x;
				if (x > mesh.hi[a]) mesh.hi[a] = x;
			}
	}
	for (int f = 0; f < n_face; ++f) {
		const struct dpg_ref_face* fc = &faces[f];
		const int boundary = (fc->volume[1] < 0);
		const int bc = boundary ? fc->bc % 10000 : 0;   /* BC_STEP_SC: straight and curved boundaries alike */
		if (fc->volume[0] < 0 || fc->volume[0] >= n_vol || fc->volume[1] >= n_vol) { dpg_mesh_free(&mesh); return DPG_ERR_INVALID; }
		if (boundary && bc != DPG_BC_RIEMANN && bc != DPG_BC_SLIPWALL && bc != DPG_BC_NOSLIP_ADIABATIC &&
		    bc != DPG_BC_NOSLIP_ALL_ROTATING) { dpg_mesh_free(&mesh); return DPG_ERR_UNSUPPORTED; }
		mesh.face_vol[2*f] = fc->volume[0]; mesh.face_vol[2*f+1] = fc->volume[1];
		mesh.face_lf[2*f] = fc->ind_lf[0];  mesh.face_lf[2*f+1] = boundary ? -1 : fc->ind_lf[1];
		mesh.face_bc[f] = bc;
	}
	/* the periodic lengths: the parameters' box where it is given (a jittered periodic mesh moves its boundary
	 * vertices with their images, past the box), else the vertices' bounding box */
	for (int a = 0; a < d; ++a)
		if (prm->hi[a] > prm->lo[a]) { mesh.lo[a] = prm->lo[a]; mesh.hi[a] = prm->hi[a]; }
	rc = sim_build(prm,&mesh,sim_out);
	dpg_mesh_free(&mesh);
	if (rc) return rc;
	struct dpg_sim* sim = *sim_out;
	for (int v = 0; v < n_vol; ++v)
		if (vols[v].sol_coef)
			memcpy(&sim->sol_coef[sim->vol_dof_off[v]],vols[v].sol_coef,
			       sizeof(double)*(size_t)(sim->vol_dof_off[v+1] - sim->vol_dof_off[v]));
	return DPG_OK;
}

void dpg_sim_destroy(struct dpg_sim* sim)
{
	if (!sim) return;
	for (int i = 0; i < sim->n_ops && sim->ops; ++i) dpg_element_ops_free(&sim->ops[i]);
	free(sim->ops);
	free(sim->vol_ops); free(sim->vol_p); free(sim->vol_affine); free(sim->vol_dof_off); free(sim->vol_geo_off);
	free(sim->vol_minv_off); free(sim->xyz_ve); free(sim->sol_coef); free(sim->sol_coef_p); free(sim->rhs);
	free(sim->metrics_vc); free(sim->jacobian_det_vc); free(sim->xyz_vc); free(sim->m_inv);
	free(sim->vol_face); free(sim->vol_face_side);
	free(sim->face_vol); free(sim->face_lf); free(sim->face_nfc); free(sim->face_bc); free(sim->face_geo_off);
	free(sim->nc_fc); free(sim->normals_fc); free(sim->jacobian_det_fc); free(sim->xyz_fc); free(sim->face_p);
	free(sim);
}

/* ---- control files ---------------------------------------------------------------------------------------- */

static int key_is(const char* line, const char* key)
{
	const size_t n = strlen(key);
	while (*line == ' ' || *line == '\t') ++line;
	return strncmp(line,key,n) == 0 && (line[n] == ' ' || line[n] == '\t');
}

/* ---- the reference's own control files ----------------------------------------------------------------------
 * A control file with pde_spec is read as the reference reads it: set_simulation_core (simulation.c:371-431) for the
 * mesh and order keys, the mesh name of mesh_name_assemble (simulation.c:624-640) --
 *   mesh_path + geom_name/pde_name/pde_spec/[geom_spec/] + mesh_domain__<mesh_generator name>__<mesh_type>_ml<ml>.msh
 * for a mesh_path containing "../meshes/", mesh_path itself otherwise -- and the test case's parameter files
 * input_files/<pde_name>/<pde_spec>/test_case[_<ext>].data and solution[_<ext>].data (read_test_case_parameters,
 * test_case_T.c:258-302; set_up_input_name, file_processing.c:640-675).  The reference finds those under its
 * compiled-in PROJECT_INPUT_DIR; here the input directory is $DPG_INPUT_DIR, else the nearest ancestor of the control
 * file's directory holding input_files/<pde_name>/<pde_spec>/.  Relative mesh paths resolve against the control file's
 * directory, then the working directory.  Provided: DG (fe_method 1) on GLL / Lagrange, QUAD / HEX, the test cases
 * euler/periodic/periodic_vortex and the Euler / advection keys of this path; anything else DPG_ERR_UNSUPPORTED. */
struct ref_ctrl {
	char pde_name[64], pde_spec[128], geom_name[64], geom_spec[64], mesh_gen[128], mesh_format[32], mesh_domain[32];
	char mesh_type[32], mesh_path[400], interp_tp[16], basis_sol[32], tc_ext[64], sol_ext[64];
	int d, ml, p, method;
};

static void read_word(const char* line, char* out, size_t n)
{
	char buf[512];
	if (sscanf(line,"%*s %511s",buf) == 1) { strncpy(out,buf,n-1); out[n-1] = 0; }
}

static int file_exists(const char* path)
{
	FILE* t = fopen(path,"r");
	if (!t) return 0;
	fclose(t);
	return 1;
}

/* the directory holding input_files/<pde>/<spec>/test_case.data */
static int find_input_dir(const char* ctrl_path, const struct ref_ctrl* rc, char* dir, size_t n)
{
	char probe[1400];
	const char* env = getenv("DPG_INPUT_DIR");
	if (env && env[0]) {
		snprintf(probe,sizeof probe,"%s/input_files/%s/%s/",env,rc->pde_name,rc->pde_spec);
		snprintf(dir,n,"%s",env);
		return 0;
	}
	char base[1024];
	snprintf(base,sizeof base,"%s",ctrl_path);
	char* slash = strrchr(base,'/');
	if (slash) *slash = 0; else snprintf(base,sizeof base,".");
	for (int up = 0; up < 8; ++up) {
		snprintf(probe,sizeof probe,"%s/input_files/%s/%s/test_case%s%s.data",base,rc->pde_name,rc->pde_spec,
		         rc->tc_ext[0] ? "_" : "",rc->tc_ext);
		if (file_exists(probe)) { snprintf(dir,n,"%s",base); return 0; }
		const size_t len = strlen(base);
		if (len + 4 >= sizeof base) break;
		strcat(base,"/..");
	}
	return -1;
}

static int create_from_reference_ctrl(const char* ctrl_path, FILE* fp, struct dpg_sim** sim_out)
{
	struct ref_ctrl rc;
	memset(&rc,0,sizeof rc);
	rc.method = 1;
	snprintf(rc.geom_spec,sizeof rc.geom_spec,"NONE");
	char line[512];
	while (fgets(line,sizeof line,fp)) {
		if (line[0] == '#' || line[0] == '/') continue;
		if (key_is(line,"pde_name"))  read_word(line,rc.pde_name,sizeof rc.pde_name);
		if (key_is(line,"pde_spec"))  read_word(line,rc.pde_spec,sizeof rc.pde_spec);
		if (key_is(line,"geom_name")) read_word(line,rc.geom_name,sizeof rc.geom_name);
		if (key_is(line,"geom_spec")) read_word(line,rc.geom_spec,sizeof rc.geom_spec);
		if (key_is(line,"dimension")) sscanf(line,"%*s %d",&rc.d);
		if (key_is(line,"mesh_generator")) read_word(line,rc.mesh_gen,sizeof rc.mesh_gen);
		if (key_is(line,"mesh_format"))    read_word(line,rc.mesh_format,sizeof rc.mesh_format);
		if (key_is(line,"mesh_domain"))    read_word(line,rc.mesh_domain,sizeof rc.mesh_domain);
		if (key_is(line,"mesh_type"))      read_word(line,rc.mesh_type,sizeof rc.mesh_type);
		if (key_is(line,"mesh_level"))     sscanf(line,"%*s %d",&rc.ml);
		if (key_is(line,"mesh_path"))      read_word(line,rc.mesh_path,sizeof rc.mesh_path);
		if (key_is(line,"interp_tp"))      read_word(line,rc.interp_tp,sizeof rc.interp_tp);
		if (key_is(line,"basis_sol"))      read_word(line,rc.basis_sol,sizeof rc.basis_sol);
		if (key_is(line,"p_ref"))          sscanf(line,"%*s %d",&rc.p);
		if (key_is(line,"fe_method"))      sscanf(line,"%*s %d",&rc.method);
		if (key_is(line,"test_case_extension")) read_word(line,rc.tc_ext,sizeof rc.tc_ext);
		if (key_is(line,"solution_extension"))  read_word(line,rc.sol_ext,sizeof rc.sol_ext);
	}
	fclose(fp);
	if (rc.method != 1) return DPG_ERR_UNSUPPORTED;   /* DG only */
	if ((rc.interp_tp[0] && strcmp(rc.interp_tp,"GLL")) || (rc.basis_sol[0] && strcmp(rc.basis_sol,"lagrange")))
		return DPG_ERR_UNSUPPORTED;
	if (rc.mesh_format[0] && strcmp(rc.mesh_format,"gmsh")) return DPG_ERR_UNSUPPORTED;

	struct dpg_sim_params prm;
	dpg_sim_params_default(&prm);
	prm.d = rc.d;
	prm.p = rc.p;
	if (!strcmp(rc.mesh_type,"quad")) prm.e_type = DPG_QUAD;
	else if (!strcmp(rc.mesh_type,"hex")) prm.e_type = DPG_HEX;
	else if (!strcmp(rc.mesh_type,"tri")) prm.e_type = DPG_TRI;
	else return DPG_ERR_UNSUPPORTED;
	if (!strcmp(rc.pde_name,"euler")) prm.pde_index = DPG_PDE_EULER;
	else if (!strcmp(rc.pde_name,"advection")) prm.pde_index = DPG_PDE_ADVECTION;
	else return DPG_ERR_UNSUPPORTED;

	/* test_case.data and solution.data */
	char indir[1024], path[1600];
	if (find_input_dir(ctrl_path,&rc,indir,sizeof indir)) return DPG_ERR_IO;
	snprintf(path,sizeof path,"%s/input_files/%s/%s/test_case%s%s.data",indir,rc.pde_name,rc.pde_spec,
	         rc.tc_ext[0] ? "_" : "",rc.tc_ext);
	FILE* tf = fopen(path,"r");
	if (!tf) return DPG_ERR_IO;
	char s1[128];
	while (fgets(line,sizeof line,tf)) {
		if (key_is(line,"solver_proc") && sscanf(line,"%*s %127s",s1) == 1) {
			if (!strcmp(s1,"explicit")) prm.solver_proc = DPG_SOLVER_E;
			else if (!strcmp(s1,"implicit")) prm.solver_proc = DPG_SOLVER_I;
			else prm.solver_proc = DPG_SOLVER_EI;
		}
		if (key_is(line,"solver_type_e") && sscanf(line,"%*s %127s",s1) == 1) {
			if (!strcmp(s1,"ssp_rk_33")) prm.solver_type_e = DPG_SOLVER_E_SSP_RK_33;
			else if (!strcmp(s1,"forward_euler")) prm.solver_type_e = DPG_SOLVER_E_EULER;
		}
		if (key_is(line,"num_flux_1st") && sscanf(line,"%*s %127s",s1) == 1) {
			if (!strcmp(s1,"Roe-Pike")) prm.num_flux = DPG_NUM_FLUX_ROE_PIKE;
			else if (!strcmp(s1,"Lax-Friedrichs")) prm.num_flux = DPG_NUM_FLUX_LAX_FRIEDRICHS;
			else if (!strcmp(s1,"upwind")) prm.num_flux = DPG_NUM_FLUX_UPWIND;
			else { fclose(tf); return DPG_ERR_UNSUPPORTED; }
		}
		if (key_is(line,"time_step"))  sscanf(line,"%*s %lf",&prm.dt);
		if (key_is(line,"time_final")) sscanf(line,"%*s %lf",&prm.time_final);
	}
	fclose(tf);
	if (!strcmp(rc.pde_name,"euler") && !strcmp(rc.pde_spec,"periodic/periodic_vortex")) {
		snprintf(path,sizeof path,"%s/input_files/%s/%s/solution%s%s.data",indir,rc.pde_name,rc.pde_spec,
		         rc.sol_ext[0] ? "_" : "",rc.sol_ext);
		FILE* sf = fopen(path,"r");
		if (!sf) return DPG_ERR_IO;
		static const char* keys[6] = {"r_v", "theta", "V_inf", "p_inf", "t_inf", "Rg"};
		int found = 0;
		while (fgets(line,sizeof line,sf))
			for (int k = 0; k < 6; ++k)
				if (key_is(line,keys[k]) && sscanf(line,"%*s %lf",&prm.vortex[k]) == 1) ++found;
		fclose(sf);
		if (found != 6) return DPG_ERR_IO;   /* the reference stops: "Did not find the required number of variables" */
		prm.test_case = DPG_TC_PERIODIC_VORTEX;
	} else {
		return DPG_ERR_UNSUPPORTED;
	}

	{   /* a method outside this path is refused before any mesh file is looked for */
		const int rcp = check_params(&prm);
		if (rcp) return rcp;
	}
	/* the mesh name (mesh_name_assemble) */
	char mesh[1200];
	if (strstr(rc.mesh_path,"../meshes/")) {
		char gen[128];
		const char* b = strrchr(rc.mesh_gen,'/');
		snprintf(gen,sizeof gen,"%s",b ? b + 1 : rc.mesh_gen);
		char* dot = strrchr(gen,'.');
		if (dot) *dot = 0;
		char spec[80] = "";
		if (strcmp(rc.geom_spec,"NONE")) snprintf(spec,sizeof spec,"%s/",rc.geom_spec);
		snprintf(mesh,sizeof mesh,"%s%s/%s/%s/%s%s__%s__%s_ml%d.msh",rc.mesh_path,rc.geom_name,rc.pde_name,rc.pde_spec,
		         spec,rc.mesh_domain,gen,rc.mesh_type,rc.ml);
	} else {
		snprintf(mesh,sizeof mesh,"%s",rc.mesh_path);
	}
	const char* slash = strrchr(ctrl_path,'/');
	if (mesh[0] != '/' && slash) {
		snprintf(path,sizeof path,"%.*s/%s",(int)(slash - ctrl_path),ctrl_path,mesh);
		if (file_exists(path)) return dpg_sim_create_from_gmsh(&prm,path,sim_out);
	}
	if (!file_exists(mesh)) return DPG_ERR_IO;
	return dpg_sim_create_from_gmsh(&prm,mesh,sim_out);
}

int dpg_sim_create_from_ctrl(const char* ctrl_path, struct dpg_sim** sim_out)
{
	if (!ctrl_path || !sim_out) return DPG_ERR_INVALID;
	*sim_out = NULL;
	FILE* fp = fopen(ctrl_path,"r");
	if (!fp) return DPG_ERR_IO;
	{   /* the reference's format: pde_spec names the test case */
		char line[512];
		int ref = 0;
		while (fgets(line,sizeof line,fp)) if (key_is(line,"pde_spec")) { ref = 1; break; }
		rewind(fp);
		if (ref) return create_from_reference_ctrl(ctrl_path,fp,sim_out);
	}
	struct dpg_sim_params prm;
	dpg_sim_params_default(&prm);
	char line[512], s1[128], mesh_path[400] = "";
	while (fgets(line,sizeof line,fp)) {
		if (line[0] == '#' || line[0] == '/') continue;
		if (key_is(line,"pde_name") && sscanf(line,"%*s %127s",s1) == 1) {
			if (!strcmp(s1,"euler")) prm.pde_index = DPG_PDE_EULER;
			else if (!strcmp(s1,"advection")) prm.pde_index = DPG_PDE_ADVECTION;
			else { fclose(fp); return DPG_ERR_UNSUPPORTED; }
		}
		if (key_is(line,"dimension")) sscanf(line,"%*s %d",&prm.d);
		if (key_is(line,"mesh_type") && sscanf(line,"%*s %127s",s1) == 1) {
			if (!strcmp(s1,"quad")) prm.e_type = DPG_QUAD;
			else if (!strcmp(s1,"hex")) prm.e_type = DPG_HEX;
			else if (!strcmp(s1,"tri")) prm.e_type = DPG_TRI;
			else if (!strcmp(s1,"tet")) prm.e_type = DPG_TET;
			else { fclose(fp); return DPG_ERR_UNSUPPORTED; }
		}
		if (key_is(line,"mesh_elements")) sscanf(line,"%*s %d %d %d",&prm.n_elem[0],&prm.n_elem[1],&prm.n_elem[2]);
		if (key_is(line,"mesh_path"))     sscanf(line,"%*s %399s",mesh_path);
		if (key_is(line,"mesh_format") && sscanf(line,"%*s %127s",s1) == 1 && strcmp(s1,"gmsh")) {
			fclose(fp);
			return DPG_ERR_UNSUPPORTED;
		}
		if (key_is(line,"domain_lo"))     sscanf(line,"%*s %lf %lf %lf",&prm.lo[0],&prm.lo[1],&prm.lo[2]);
		if (key_is(line,"domain_hi"))     sscanf(line,"%*s %lf %lf %lf",&prm.hi[0],&prm.hi[1],&prm.hi[2]);
		if (key_is(line,"mesh_jitter"))   sscanf(line,"%*s %lf",&prm.jitter);
		if (key_is(line,"mesh_seed"))     { unsigned long long sd = 0; sscanf(line,"%*s %llu",&sd); prm.seed = sd; }
		/* p_ref p [p_max]: with a range, each volume's order is drawn from it (seeded by p_seed) */
		if (key_is(line,"p_ref"))         sscanf(line,"%*s %d %d",&prm.p,&prm.p_max);
		if (key_is(line,"p_seed"))        { unsigned long long sd = 0; sscanf(line,"%*s %llu",&sd); prm.p_seed = sd; }
		if (key_is(line,"num_flux_1st") && sscanf(line,"%*s %127s",s1) == 1) {
			if (!strcmp(s1,"Roe-Pike")) prm.num_flux = DPG_NUM_FLUX_ROE_PIKE;
			else if (!strcmp(s1,"Lax-Friedrichs")) prm.num_flux = DPG_NUM_FLUX_LAX_FRIEDRICHS;
			else if (!strcmp(s1,"upwind")) prm.num_flux = DPG_NUM_FLUX_UPWIND;
			else { fclose(fp); return DPG_ERR_UNSUPPORTED; }
		}
		if (key_is(line,"solver_type_e") && sscanf(line,"%*s %127s",s1) == 1) {
			if (!strcmp(s1,"ssp_rk_33")) prm.solver_type_e = DPG_SOLVER_E_SSP_RK_33;
			else if (!strcmp(s1,"forward_euler")) prm.solver_type_e = DPG_SOLVER_E_EULER;
			else { fclose(fp); return DPG_ERR_UNSUPPORTED; }
		}
		if (key_is(line,"time_step"))  sscanf(line,"%*s %lf",&prm.dt);
		if (key_is(line,"time_final")) sscanf(line,"%*s %lf",&prm.time_final);
		if (key_is(line,"test_case") && sscanf(line,"%*s %127s",s1) == 1) {
			if (!strcmp(s1,"isentropic_vortex")) prm.test_case = DPG_TC_ISENTROPIC_VORTEX;
			else if (!strcmp(s1,"advection_sine")) prm.test_case = DPG_TC_ADVECTION_SINE;
			else if (!strcmp(s1,"free_stream")) prm.test_case = DPG_TC_FREE_STREAM;
			else { fclose(fp); return DPG_ERR_UNSUPPORTED; }
		}
		if (key_is(line,"vortex_strength")) sscanf(line,"%*s %lf",&prm.vortex[0]);
		if (key_is(line,"vortex_centre"))   sscanf(line,"%*s %lf %lf",&prm.vortex[1],&prm.vortex[2]);
		if (key_is(line,"free_stream"))     sscanf(line,"%*s %lf %lf %lf %lf %lf",&prm.vortex[3],&prm.vortex[4],
		                                           &prm.vortex[5],&prm.vortex[6],&prm.vortex[7]);
		if (key_is(line,"b_adv"))           sscanf(line,"%*s %lf %lf %lf",&prm.b_adv[0],&prm.b_adv[1],&prm.b_adv[2]);
	}
	fclose(fp);
	if (!mesh_path[0]) return dpg_sim_create(&prm,sim_out);
	/* a gmsh mesh (mesh_path): relative to the control file's directory, else to the working directory */
	char full[1024];
	const char* slash = strrchr(ctrl_path,'/');
	if (mesh_path[0] != '/' && slash) {
		snprintf(full,sizeof full,"%.*s/%s",(int)(slash - ctrl_path),ctrl_path,mesh_path);
		FILE* t = fopen(full,"r");
		if (t) { fclose(t); return dpg_sim_create_from_gmsh(&prm,full,sim_out); }
	}
	return dpg_sim_create_from_gmsh(&prm,mesh_path,sim_out);
}

/* ---- accessors ---------------------------------------------------------------------------------------------- */

int dpg_sim_info(const struct dpg_sim* sim, int64_t* info)
{
	if (!sim || !info) return DPG_ERR_INVALID;
	info[0] = sim->d; info[1] = sim->n_var; info[2] = sim->n_vol; info[3] = sim->n_face;
	info[4] = sim->vol_dof_off[sim->n_vol];
	info[5] = sim->ops[0].n_s; info[6] = sim->ops[0].n_c; info[7] = sim->ops[0].n_fc;
	info[8] = sim->ops[0].p; info[9] = sim->ops[0].e_type;
	return DPG_OK;
}

int dpg_sim_get_sol_coef(const struct dpg_sim* sim, double* out)
{
	if (!sim || !out) return DPG_ERR_INVALID;
	memcpy(out,sim->sol_coef,sizeof(double)*(size_t)sim->vol_dof_off[sim->n_vol]);
	return DPG_OK;
}

int dpg_sim_set_sol_coef(struct dpg_sim* sim, const double* in)
{
	if (!sim || !in) return DPG_ERR_INVALID;
	memcpy(sim->sol_coef,in,sizeof(double)*(size_t)sim->vol_dof_off[sim->n_vol]);
	return DPG_OK;
}

int dpg_sim_get_rhs(const struct dpg_sim* sim, double* out)
{
	if (!sim || !out) return DPG_ERR_INVALID;
	memcpy(out,sim->rhs,sizeof(double)*(size_t)sim->vol_dof_off[sim->n_vol]);
	return DPG_OK;
}

int dpg_sim_set_time(struct dpg_sim* sim, double t)
{
	if (!sim) return DPG_ERR_INVALID;
	sim->time = t;
	return DPG_OK;
}

const struct dpg_sim* dpg_sim_view(const struct dpg_sim* sim) { return sim; }

/* Primitive variables used in the error of the Euler equations (compute_error_euler.c): rho, u, v, (w), p. */
static void to_error_vars(const struct dpg_sim* sim, const double* u, double* e)
{
	const int d = sim->d;
	if (sim->n_var != d + 2) { e[0] = u[0]; return; }
	const double rho = u[0];
	double V2 = 0.0;
	for (int a = 0; a < d; ++a) { e[1+a] = u[1+a]/rho; V2 += e[1+a]*e[1+a]; }
	e[0] = rho;
	e[d+1] = DPG_GM1*(u[d+1] - 0.5*rho*V2);
}

int dpg_sim_l2_error(const struct dpg_sim* sim, double t, double* err_out, int n_err_max)
{
	if (!sim || !err_out) return DPG_ERR_INVALID;
	const int d = sim->d, n_var = sim->n_var;
	if (n_err_max < n_var) return DPG_ERR_INVALID;
	double acc[DPG_NVAR_MAX] = {0}, vol = 0.0;
	for (int v = 0; v < sim->n_vol; ++v) {
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
		const int n_s = ops->n_s, n_c = ops->n_c;
		const double* sc = &sim->sol_coef[sim->vol_dof_off[v]];
		const double* jd = &sim->jacobian_det_vc[sim->vol_geo_off[v]];
		const double* xyz = &sim->xyz_vc[(size_t)sim->vol_geo_off[v]*d];
		for (int c = 0; c < n_c; ++c) {
			double uh[DPG_NVAR_MAX], ue[DPG_NVAR_MAX], x[3] = {0,0,0}, eh[DPG_NVAR_MAX], ee[DPG_NVAR_MAX];
			for (int var = 0; var < n_var; ++var) {
				double s = 0.0;
				for (int i = 0; i < n_s; ++i) s += ops->cv0_vs_vc[(size_t)c*n_s+i]*sc[i + (size_t)n_s*var];
				uh[var] = s;
			}
			for (int a = 0; a < d; ++a) x[a] = xyz[c + (size_t)n_c*a];
			dpg_exact_solution(sim,t,x,ue);
			to_error_vars(sim,uh,eh);
			to_error_vars(sim,ue,ee);
			const double wj = ops->w_vc[c]*jd[c];
			for (int var = 0; var < n_var; ++var) acc[var] += wj*(eh[var]-ee[var])*(eh[var]-ee[var]);
			vol += wj;
		}
	}
	for (int var = 0; var < n_var; ++var) err_out[var] = sqrt(acc[var]/vol);
	return DPG_OK;
}

double dpg_sim_max_wave_speed(const struct dpg_sim* sim)
{
	if (!sim) return 0.0;
	const int d = sim->d;
	if (sim->n_var != d + 2) {
		double b2 = 0.0;
		for (int a = 0; a < d; ++a) b2 += sim->b_adv[a]*sim->b_adv[a];
		return sqrt(b2);
	}
	double smax = 0.0;
	for (int v = 0; v < sim->n_vol; ++v) {
		const int n_s = sim->ops[sim->vol_ops[v]].n_s;
		const double* sc = &sim->sol_coef[sim->vol_dof_off[v]];
		for (int i = 0; i < n_s; ++i) {
			const double rho = sc[i];
			double V2 = 0.0;
			for (int a = 0; a < d; ++a) { const double u = sc[i + (size_t)n_s*(1+a)]/rho; V2 += u*u; }
			const double p = DPG_GM1*(sc[i + (size_t)n_s*(d+1)] - 0.5*rho*V2);
			const double s = sqrt(V2) + sqrt(DPG_GAMMA*p/rho);
			if (s > smax) smax = s;
		}
	}
	return smax;
}
