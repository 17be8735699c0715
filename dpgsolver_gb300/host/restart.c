/* Restart files in the reference's format (a gmsh 2.2 mesh followed by the solution's Bezier coefficients):
 *   dpg_sim_write_restart   output_restart_gmsh (restart_writers.c:126-145): $Nodes (the volumes' distinct vertices),
 *                           $Elements (the volumes, gmsh vertex order, two zero tags; a periodic mesh has no boundary
 *                           faces to list), $SolutionCoefficients ("volume p n_coef n_var" and the Bezier
 *                           coefficients of fprintf_solution_bezier_gmsh, column-major [n_coef, n_var], 15 decimals);
 *   dpg_sim_read_restart    set_sol_restart_T (restart_T.c:62-87, constructor_sol_restart :140-166): the solution of
 *                           the simulation's mesh at its solution nodes, evaluated from the restart file's Bezier
 *                           expansion in the restart volume that contains each node (found through a bucket grid of
 *                           the restart volumes' boxes -- the reference searches an approximate-nearest-neighbour
 *                           tree -- and the inverse of the volume's multilinear map by Newton iterations, as its
 *                           inverse_mapping.c).  The meshes need not match: coarser, finer or of another order.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dpg_host.h"
#include "dpg_gb300.h"

/* Bernstein polynomial i of order p on [-1, 1] (bases.c:1013-1019) */
static double bernstein(int p, int i, double r)
{
	double c = 1.0;
	for (int k = 1; k <= i; ++k) c = c*(double)(p - i + k)/(double)k;
	return c*pow(0.5*(1.0+r),i)*pow(0.5*(1.0-r),p-i);
}

static int cmp_xyz(const void* a, const void* b)
{
	const double* x = a;
	const double* y = b;
	for (int i = 0; i < 3; ++i)
		if (x[i] != y[i]) return x[i] < y[i] ? -1 : 1;
	return 0;
}

int dpg_sim_write_restart(const struct dpg_sim* sim, const char* path)
{
	if (!sim || !path) return DPG_ERR_INVALID;
	if (sim->pde_index != DPG_PDE_EULER && sim->pde_index != DPG_PDE_ADVECTION) return DPG_ERR_UNSUPPORTED;
	/* tensor-product volumes of one order */
	if (sim->ops[0].e_type == DPG_TRI || sim->ops[0].e_type == DPG_TET || sim->n_ops != 1) return DPG_ERR_UNSUPPORTED;
	const int d = sim->d, n_ve = 1 << d, n_vol = sim->n_vol;
	const struct dpg_element_ops* ops = &sim->ops[0];
	const int n_s = ops->n_s, n_var = sim->n_var;
	/* distinct vertices: sorted copies of all volume vertices, duplicates (bitwise equal) merged */
	const size_t n_all = (size_t)n_vol*n_ve;
	double* xs = malloc(sizeof(double)*3*n_all);
	double* b = malloc(sizeof(double)*(size_t)n_s*n_var);
	if (!xs || !b) { free(xs); free(b); return DPG_ERR_INVALID; }
	for (int v = 0; v < n_vol; ++v)
		for (int k = 0; k < n_ve; ++k)
			memcpy(&xs[3*((size_t)v*n_ve + k)],&sim->xyz_ve[((size_t)v*DPG_NVE_MAX + k)*3],3*sizeof(double));
	qsort(xs,n_all,3*sizeof(double),cmp_xyz);
	size_t n_u = 0;
	for (size_t i = 0; i < n_all; ++i)
		if (n_u == 0 || cmp_xyz(&xs[3*i],&xs[3*(n_u-1)]) != 0) memmove(&xs[3*n_u++],&xs[3*i],3*sizeof(double));
	FILE* fp = fopen(path,"w");
	if (!fp) { free(xs); free(b); return DPG_ERR_IO; }
	fprintf(fp,"$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%zu\n",n_u);
	for (size_t i = 0; i < n_u; ++i) fprintf(fp,"%zu %.17g %.17g %.17g\n",i+1,xs[3*i],xs[3*i+1],xs[3*i+2]);
	fprintf(fp,"$EndNodes\n$Elements\n%d\n",n_vol);
	static const int gmsh_of_tp_quad[4] = {0,1,3,2}, gmsh_of_tp_hex[8] = {0,1,3,2,4,5,7,6};
	const int* perm = (d == 2 ? gmsh_of_tp_quad : gmsh_of_tp_hex);
	for (int v = 0; v < n_vol; ++v) {
		fprintf(fp,"%d %d 2 0 0",v+1,d == 2 ? 3 : 5);
		for (int k = 0; k < n_ve; ++k) {
			const double* x = &sim->xyz_ve[((size_t)v*DPG_NVE_MAX + perm[k])*3];
			const double* hit = bsearch(x,xs,n_u,3*sizeof(double),cmp_xyz);
			fprintf(fp," %zu",(size_t)((hit - xs)/3) + 1);
		}
		fprintf(fp,"\n");
	}
	fprintf(fp,"$EndElements\n$SolutionCoefficients\n%d\n",n_vol);
	for (int v = 0; v < n_vol; ++v) {
		const double* u = &sim->sol_coef[sim->vol_dof_off[v]];
		for (int var = 0; var < n_var; ++var)   /* Bezier coefficients: ccSB0 u (constructor_s_coef_bezier) */
			for (int i = 0; i < n_s; ++i) {
				double s = 0.0;
				for (int j = 0; j < n_s; ++j) s += ops->ccSB0_vs_vs[(size_t)i*n_s + j]*u[j + (size_t)n_s*var];
				b[i + (size_t)n_s*var] = s;
			}
		fprintf(fp,"%d %d %d %d",v+1,sim->vol_p[v],n_s,n_var);
		for (int i = 0; i < n_s*n_var; ++i) fprintf(fp," % .*e",15,b[i]);
		fprintf(fp,"\n");
	}
	fprintf(fp,"$EndSolutionCoefficients\n");
	const int bad = ferror(fp);
	fclose(fp);
	free(xs); free(b);
	return bad ? DPG_ERR_IO : DPG_OK;
}

/* ---- reading --------------------------------------------------------------------------------------------- */

struct restart_vol {
	double x[8][3];   /* vertices, tensor-product order */
	double lo[3], hi[3];
	int p, n_coef;
	double* coef;     /* [n_coef, n_var] column-major Bezier coefficients */
};

/* multilinear map of a tensor-product volume and its Jacobian at reference point r */
static void p1_map(int d, const double (*x)[3], const double* r, double* out, double (*J)[3])
{
	for (int i = 0; i < 3; ++i) { out[i] = 0.0; for (int a = 0; a < 3; ++a) J[i][a] = 0.0; }
	for (int k = 0; k < (1 << d); ++k) {
		double phi = 1.0, dphi[3];
		for (int a = 0; a < d; ++a) {
			const double s = ((k >> a) & 1) ? 1.0 : -1.0;
			phi *= 0.5*(1.0 + s*r[a]);
		}
		for (int a = 0; a < d; ++a) {
			const double s = ((k >> a) & 1) ? 1.0 : -1.0;
			double g = 0.5*s;
			for (int c = 0; c < d; ++c)
				if (c != a) g *= 0.5*(1.0 + (((k >> c) & 1) ? 1.0 : -1.0)*r[c]);
			dphi[a] = g;
		}
		for (int i = 0; i < d; ++i) {
			out[i] += phi*x[k][i];
			for (int a = 0; a < d; ++a) J[i][a] += dphi[a]*x[k][i];
		}
	}
}

/* Reference coordinates r in [-1, 1]^d of point y in the tensor-product volume with vertices x (Newton on the
 * multilinear map, as the reference's constructor_inverse_mapping, inverse_mapping.c); 1 if y lies inside (within
 * tolerance), 0 otherwise. */
int dpg_p1_inverse_map(int d, const double (*x)[3], const double* y, double* r)
{
	for (int a = 0; a < 3; ++a) r[a] = 0.0;
	for (int it = 0; it < 30; ++it) {
		double f[3], J[3][3];
		p1_map(d,x,r,f,J);
		double res[3] = {f[0]-y[0], f[1]-y[1], f[2]-y[2]}, dr[3] = {0,0,0};
		if (d == 2) {
			const double det = J[0][0]*J[1][1] - J[0][1]*J[1][0];
			if (det == 0.0) return 0;
			dr[0] = ( J[1][1]*res[0] - J[0][1]*res[1])/det;
			dr[1] = (-J[1][0]*res[0] + J[0][0]*res[1])/det;
		} else {
			double A[3][3];
			memcpy(A,J,sizeof A);
			const double det = A[0][0]*(A[1][1]*A[2][2]-A[1][2]*A[2][1]) - A[0][1]*(A[1][0]*A[2][2]-A[1][2]*A[2][0])
			                 + A[0][2]*(A[1][0]*A[2][1]-A[1][1]*A[2][0]);
			if (det == 0.0) return 0;
			for (int c = 0; c < 3; ++c) {   /* Cramer's rule */
				double M[3][3];
				memcpy(M,A,sizeof M);
				for (int i = 0; i < 3; ++i) M[i][c] = res[i];
				dr[c] = (M[0][0]*(M[1][1]*M[2][2]-M[1][2]*M[2][1]) - M[0][1]*(M[1][0]*M[2][2]-M[1][2]*M[2][0])
				       + M[0][2]*(M[1][0]*M[2][1]-M[1][1]*M[2][0]))/det;
			}
		}
		double step = 0.0;
		for (int a = 0; a < d; ++a) { r[a] -= dr[a]; step = fmax(step,fabs(dr[a])); }
		if (step < 1e-14) break;
		if (fabs(r[0]) > 3.0 || fabs(r[1]) > 3.0 || fabs(r[2]) > 3.0) return 0;   /* far outside: not this volume */
	}
	for (int a = 0; a < d; ++a)
		if (fabs(r[a]) > 1.0 + 1e-9) return 0;
	return 1;
}

int dpg_sim_read_restart(struct dpg_sim* sim, const char* path)
{
	if (!sim || !path) return DPG_ERR_INVALID;
	/* tensor-product volumes of one order */
	if (sim->ops[0].e_type == DPG_TRI || sim->ops[0].e_type == DPG_TET || sim->n_ops != 1) return DPG_ERR_UNSUPPORTED;
	const int d = sim->d, n_ve = 1 << d, n_var = sim->n_var;
	FILE* fp = fopen(path,"r");
	if (!fp) return DPG_ERR_IO;
	int rc = DPG_OK, n_nodes = 0, n_rv = 0, max_id = 0;
	double* node_x = NULL;
	int* node_id = NULL;
	int* index = NULL;
	struct restart_vol* rv = NULL;
	int* bucket_start = NULL;
	int* bucket_list = NULL;
	char* line = malloc(1 << 20);
	if (!line) { fclose(fp); return DPG_ERR_INVALID; }
	const int line_len = 1 << 20;
	while (fgets(line,line_len,fp)) {
		if (!strncmp(line,"$Nodes",6)) {
			if (!fgets(line,line_len,fp) || sscanf(line,"%d",&n_nodes) != 1 || n_nodes < 1) { rc = DPG_ERR_IO; goto done; }
			node_x = malloc(sizeof(double)*3*(size_t)n_nodes);
			node_id = malloc(sizeof(int)*(size_t)n_nodes);
			if (!node_x || !node_id) { rc = DPG_ERR_INVALID; goto done; }
			for (int i = 0; i < n_nodes; ++i) {
				if (!fgets(line,line_len,fp) ||
				    sscanf(line,"%d %lf %lf %lf",&node_id[i],&node_x[3*i],&node_x[3*i+1],&node_x[3*i+2]) != 4 ||
				    node_id[i] < 1) { rc = DPG_ERR_IO; goto done; }
				if (node_id[i] > max_id) max_id = node_id[i];
			}
			index = malloc(sizeof(int)*((size_t)max_id + 1));
			if (!index) { rc = DPG_ERR_INVALID; goto done; }
			for (int i = 0; i <= max_id; ++i) index[i] = -1;
			for (int i = 0; i < n_nodes; ++i) index[node_id[i]] = i;
		} else if (!strncmp(line,"$Elements",9)) {
			int n_el = 0;
			if (!index || !fgets(line,line_len,fp) || sscanf(line,"%d",&n_el) != 1 || n_el < 0) { rc = DPG_ERR_IO; goto done; }
			rv = calloc((size_t)(n_el > 0 ? n_el : 1),sizeof *rv);
			if (!rv) { rc = DPG_ERR_INVALID; goto done; }
			static const int tp_of_gmsh_quad[4] = {0,1,3,2}, tp_of_gmsh_hex[8] = {0,1,3,2,4,5,7,6};
			const int* perm = (d == 2 ? tp_of_gmsh_quad : tp_of_gmsh_hex);
			for (int e = 0; e < n_el; ++e) {
				if (!fgets(line,line_len,fp)) { rc = DPG_ERR_IO; goto done; }
				long val[40];
				int nv = 0;
				char* s = line;
				char* end = NULL;
				while (nv < 40) { const long x = strtol(s,&end,10); if (end == s) break; val[nv++] = x; s = end; }
				if (nv < 3 || nv < 3 + val[2]) { rc = DPG_ERR_IO; goto done; }
				const int type = (int)val[1];
				if (type != (d == 2 ? 3 : 5)) continue;   /* boundary faces of a restart file: not needed here */
				if (nv - 3 - val[2] != n_ve) { rc = DPG_ERR_IO; goto done; }
				struct restart_vol* r = &rv[n_rv++];
				for (int k = 0; k < n_ve; ++k) {
					const long id = val[3 + val[2] + perm[k]];
					if (id < 1 || id > max_id || index[id] < 0) { rc = DPG_ERR_IO; goto done; }
					for (int i = 0; i < 3; ++i) r->x[k][i] = node_x[3*index[id] + i];
				}
				for (int i = 0; i < 3; ++i) { r->lo[i] = 1e300; r->hi[i] = -1e300; }
				for (int k = 0; k < n_ve; ++k)
					for (int i = 0; i < d; ++i) { r->lo[i] = fmin(r->lo[i],r->x[k][i]); r->hi[i] = fmax(r->hi[i],r->x[k][i]); }
			}
		} else if (!strncmp(line,"$SolutionCoefficients",21)) {
			int n_sol = 0;
			if (!rv || !fgets(line,line_len,fp) || sscanf(line,"%d",&n_sol) != 1 || n_sol != n_rv) { rc = DPG_ERR_IO; goto done; }
			for (int e = 0; e < n_sol; ++e) {
				if (!fgets(line,line_len,fp)) { rc = DPG_ERR_IO; goto done; }
				char* s = line;
				char* end = NULL;
				const long iv = strtol(s,&end,10); s = end;
				const long p = strtol(s,&end,10); s = end;
				const long nc = strtol(s,&end,10); s = end;
				const long nvr = strtol(s,&end,10); s = end;
				long n1 = p + 1, ns = 1;
				for (int a = 0; a < d; ++a) ns *= n1;
				if (iv != e + 1 || p < 0 || p > 8 || nc != ns || nvr != n_var) { rc = DPG_ERR_IO; goto done; }
				rv[e].p = (int)p; rv[e].n_coef = (int)nc;
				rv[e].coef = malloc(sizeof(double)*(size_t)(nc*nvr));
				if (!rv[e].coef) { rc = DPG_ERR_INVALID; goto done; }
				for (long i = 0; i < nc*nvr; ++i) {
					rv[e].coef[i] = strtod(s,&end);
					if (end == s) { rc = DPG_ERR_IO; goto done; }
					s = end;
				}
			}
		}
	}
	if (!rv || n_rv < 1 || !rv[n_rv-1].coef) { rc = DPG_ERR_IO; goto done; }

	/* bucket grid over the restart volumes' boxes (cell ~ the largest box) */
	double glo[3] = {1e300,1e300,1e300}, ghi[3] = {-1e300,-1e300,-1e300}, hmax = 0.0;
	for (int e = 0; e < n_rv; ++e)
		for (int i = 0; i < d; ++i) {
			glo[i] = fmin(glo[i],rv[e].lo[i]); ghi[i] = fmax(ghi[i],rv[e].hi[i]);
			hmax = fmax(hmax,rv[e].hi[i] - rv[e].lo[i]);
		}
	int nb[3] = {1,1,1};
	for (int i = 0; i < d; ++i) {
		nb[i] = (int)((ghi[i] - glo[i])/hmax) + 1;
		if (nb[i] > 4096) nb[i] = 4096;
	}
	const size_t n_cells = (size_t)nb[0]*nb[1]*nb[2];
	bucket_start = calloc(n_cells + 1,sizeof(int));
	if (!bucket_start) { rc = DPG_ERR_INVALID; goto done; }
	#define CELL(i,x) (int)fmin((double)(nb[i]-1),fmax(0.0,floor(((x) - glo[i])/(ghi[i] - glo[i] + 1e-300)*nb[i])))
	for (int pass = 0; pass < 2; ++pass) {   /* count, then fill: each volume in every cell its box touches */
		int* fill = NULL;
		if (pass == 1) {
			for (size_t c = 0; c < n_cells; ++c) bucket_start[c+1] += bucket_start[c];
			bucket_list = malloc(sizeof(int)*(size_t)(bucket_start[n_cells] > 0 ? bucket_start[n_cells] : 1));
			fill = calloc(n_cells,sizeof(int));
			if (!bucket_list || !fill) { free(fill); rc = DPG_ERR_INVALID; goto done; }
		}
		for (int e = 0; e < n_rv; ++e) {
			int c0[3] = {0,0,0}, c1[3] = {0,0,0};
			for (int i = 0; i < d; ++i) { c0[i] = CELL(i,rv[e].lo[i]); c1[i] = CELL(i,rv[e].hi[i]); }
			for (int k = c0[2]; k <= c1[2]; ++k)
			for (int j = c0[1]; j <= c1[1]; ++j)
			for (int i = c0[0]; i <= c1[0]; ++i) {
				const size_t c = (size_t)i + (size_t)nb[0]*(j + (size_t)nb[1]*k);
				if (pass == 0) ++bucket_start[c+1];
				else bucket_list[bucket_start[c] + fill[c]++] = e;
			}
		}
		free(fill);
	}

	/* the solution nodes of the simulation's volumes: evaluate the restart expansion there */
	const struct dpg_element_ops* ops = &sim->ops[0];
	const int n_s = ops->n_s;
	for (int v = 0; v < sim->n_vol && rc == DPG_OK; ++v) {
		const double (*xv)[3] = (const double (*)[3])&sim->xyz_ve[(size_t)v*DPG_NVE_MAX*3];
		double* u = &sim->sol_coef[sim->vol_dof_off[v]];
		double cv[3] = {0,0,0};
		for (int k = 0; k < n_ve; ++k)
			for (int i = 0; i < d; ++i) cv[i] += xv[k][i]/n_ve;
		for (int s = 0; s < n_s; ++s) {
			double y0[3], J[3][3], r[3], rb[3] = {0,0,0};
			p1_map(d,xv,&ops->rst_vs[(size_t)s*d],y0,J);
			/* a node on a face of the restart mesh lies in several restart volumes, whose (discontinuous) expansions
			 * differ there: take the one nearest the simulation volume (centroid distance), so that a restart on the
			 * same mesh gives back each volume's own values.  A node outside the restart mesh's volumes (jittered
			 * periodic boundaries) is looked up at its periodic images. */
			int found = -1;
			double best = 1e300;
			const int n_shift = (d == 2 ? 9 : 27);
			for (int sh = 0; sh < n_shift && found < 0; ++sh) {
				const int order[3] = {0, 1, -1};   /* the node itself first */
				double y[3] = {y0[0], y0[1], y0[2]}, yc[3] = {cv[0], cv[1], cv[2]};
				for (int i = 0, t = sh; i < d; ++i, t /= 3) {
					const double shift = order[t % 3]*(sim->domain_hi[i] - sim->domain_lo[i]);
					y[i] += shift;
					yc[i] += shift;
				}
				int c[3] = {0,0,0};
				for (int i = 0; i < d; ++i) c[i] = CELL(i,y[i]);
				const size_t cell = (size_t)c[0] + (size_t)nb[0]*(c[1] + (size_t)nb[1]*c[2]);
				for (int q = bucket_start[cell]; q < bucket_start[cell+1]; ++q) {
					const int e = bucket_list[q];
					int inside_box = 1;
					for (int i = 0; i < d; ++i)
						if (y[i] < rv[e].lo[i] - 1e-9*hmax || y[i] > rv[e].hi[i] + 1e-9*hmax) inside_box = 0;
					if (!inside_box || !dpg_p1_inverse_map(d,(const double (*)[3])rv[e].x,y,r)) continue;
					double dist = 0.0;
					for (int i = 0; i < d; ++i) {
						double ce = 0.0;
						for (int k = 0; k < n_ve; ++k) ce += rv[e].x[k][i]/n_ve;
						dist += (ce - yc[i])*(ce - yc[i]);
					}
					if (dist < best) { best = dist; found = e; memcpy(rb,r,sizeof rb); }
				}
			}
			if (found < 0) { rc = DPG_ERR_UNSUPPORTED; break; }   /* a node outside the restart mesh */
			memcpy(r,rb,sizeof r);
			const struct restart_vol* re = &rv[found];
			const int n1 = re->p + 1;
			for (int var = 0; var < n_var; ++var) {
				double val = 0.0;
				for (int bidx = 0; bidx < re->n_coef; ++bidx) {
					double phi = 1.0;
					for (int a = 0, t = bidx; a < d; ++a, t /= n1) phi *= bernstein(re->p,t % n1,r[a]);
					val += phi*re->coef[bidx + (size_t)re->n_coef*var];
				}
				u[s + (size_t)n_s*var] = val;   /* Lagrange basis: the coefficient is the value at the node */
			}
		}
	}
	#undef CELL
done:
	fclose(fp);
	free(line); free(node_x); free(node_id); free(index); free(bucket_start); free(bucket_list);
	if (rv) { for (int e = 0; e < n_rv; ++e) free(rv[e].coef); free(rv); }
	return rc;
}
