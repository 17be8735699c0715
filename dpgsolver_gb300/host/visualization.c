/* Solution output for visualisation: the reference's serial VTK XML unstructured-grid file of the volume solution
 * (output_visualization_vtk_sol, visualization.c:302-350; pieces per volume, fprint_vtk_piece_sol_grad :675-860).
 *
 * One <Piece> per volume, in volume order.  Its points are the equally spaced nodes of the volume's order p on the
 * reference element mapped by the volume's geometry (P1 map of the vertices; the parametric map for the curved
 * annulus), and its cells split the element into p^d linear sub-cells (VTK_QUAD / VTK_HEXAHEDRON) or p^2 triangles
 * (VTK_TRIANGLE), as the reference's plotting nodes and connectivity do.  Point data: "index" and "p_ref" of the
 * volume (Int32), then the solution interpolated to the points by the volume's basis -- "u" for advection; the
 * primitive variables "$\rho$", "$\mathbf{v}$" (3 components), "$\mathit{p}$" for the Euler and Navier-Stokes
 * equations (convert_variables 'c' -> 'p') -- and, for the Euler test cases (all have an exact solution), the
 * absolute errors "$|\rho-\rho_e|$", "$|\mathbf{v}-\mathbf{v}_e|$" (per component), "$|p-p_e|$" in primitive
 * variables of the exact solution at the solution nodes interpolated to the points (vv0_vs_vp, :500-511).  The gradient
 * output of Navier-Stokes volumes (grad_coef) is not written.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dpg_gb300.h"
#include "dpg_host.h"

enum { VTK_TRIANGLE = 5, VTK_QUAD = 9, VTK_HEXAHEDRON = 12 };

/* equally spaced reference points of order p: TP (p+1)^d, first coordinate fastest; TRI (p+1)(p+2)/2 with the
 * barycentric index (i along v0->v1, j along v0->v2), rows of increasing j */
static int plot_points(const struct dpg_element_ops* o, double* r)
{
	const int p = o->p, d = o->d;
	if (o->e_type == DPG_TRI) {
		static const double VX[3] = {-1.0, 1.0, 0.0}, VY[3] = {-0.5773502691896258, -0.5773502691896258, 1.1547005383792515};
		int k = 0;
		for (int j = 0; j <= p; ++j)
			for (int i = 0; i + j <= p; ++i, ++k) {
				const double a = (double)i/p, b = (double)j/p, c = 1.0 - a - b;
				r[2*k]   = c*VX[0] + a*VX[1] + b*VX[2];
				r[2*k+1] = c*VY[0] + a*VY[1] + b*VY[2];
			}
		return k;
	}
	int n = 1;
	for (int a = 0; a < d; ++a) n *= p + 1;
	for (int s = 0; s < n; ++s)
		for (int a = 0, t = s; a < d; ++a, t /= (p + 1)) r[(size_t)s*d + a] = -1.0 + 2.0*(t % (p + 1))/p;
	return n;
}

/* linear sub-cells of the plot points: connectivity (local point numbers) into conn, returns the number of cells */
static int plot_cells(const struct dpg_element_ops* o, int* conn, int* n_per_cell)
{
	const int p = o->p, d = o->d, n1 = p + 1;
	int c = 0;
	if (o->e_type == DPG_TRI) {
		*n_per_cell = 3;
		int row0 = 0;   /* first point of row j */
		for (int j = 0; j < p; ++j) {
			const int len = p + 1 - j, row1 = row0 + len;
			for (int i = 0; i + j < p; ++i) {
				conn[3*c] = row0 + i; conn[3*c+1] = row0 + i + 1; conn[3*c+2] = row1 + i; ++c;
				if (i + j + 1 < p) { conn[3*c] = row0 + i + 1; conn[3*c+1] = row1 + i + 1; conn[3*c+2] = row1 + i; ++c; }
			}
			row0 = row1;
		}
		return c;
	}
	if (d == 2) {
		*n_per_cell = 4;
		for (int j = 0; j < p; ++j)
			for (int i = 0; i < p; ++i, ++c) {
				const int b = i + n1*j;
				conn[4*c] = b; conn[4*c+1] = b + 1; conn[4*c+2] = b + 1 + n1; conn[4*c+3] = b + n1;
			}
		return c;
	}
	*n_per_cell = 8;
	for (int k = 0; k < p; ++k)
		for (int j = 0; j < p; ++j)
			for (int i = 0; i < p; ++i, ++c) {
				const int b = i + n1*(j + n1*k), s = n1*n1;
				const int q[8] = {b, b + 1, b + 1 + n1, b + n1, b + s, b + 1 + s, b + 1 + n1 + s, b + n1 + s};
				memcpy(&conn[8*c],q,sizeof q);
			}
	return c;
}

/* the nodal basis of o at n_pt reference points: phi[n_pt][n_s] */
static int basis_at(const struct dpg_element_ops* o, int n_pt, const double* r, double* phi)
{
	if (o->e_type == DPG_TRI) return dpg_tri_lagrange_at(o->p,o->rst_vs,n_pt,r,phi);
	const int d = o->d, n1 = o->p + 1;
	double g1[16], grad[3*729];
	for (int i = 0; i < n1; ++i) g1[i] = o->rst_vs[(size_t)i*d];
	for (int k = 0; k < n_pt; ++k) dpg_tp_basis_at(d,n1,g1,&r[(size_t)k*d],&phi[(size_t)k*o->n_s],grad);
	return 0;
}

/* physical coordinates of a reference point of volume v (P1 map; the annulus: (r, theta) bilinear then polar) */
static void map_point(const struct dpg_sim* sim, const struct dpg_element_ops* o, int v, const double* r, double* x)
{
	const int d = sim->d, n_ve = o->n_ve;
	const double* xv = &sim->xyz_ve[(size_t)v*DPG_NVE_MAX*3];
	double w[DPG_NVE_MAX];
	if (o->e_type == DPG_TRI) {
		dpg_tri_p1_at(r,w,NULL);
	} else {
		for (int k = 0; k < n_ve; ++k) {
			double t = 1.0;
			for (int a = 0; a < d; ++a) t *= ((k >> a) & 1) ? 0.5*(1.0 + r[a]) : 0.5*(1.0 - r[a]);
			w[k] = t;
		}
	}
	x[0] = x[1] = x[2] = 0.0;
	for (int k = 0; k < n_ve; ++k)
		for (int a = 0; a < d; ++a) x[a] += w[k]*xv[k*3 + a];
	if (sim->geom == DPG_GEOM_CYLINDER) { const double rr = x[0], th = x[1]; x[0] = rr*cos(th); x[1] = rr*sin(th); }
}

static void to_primitive(int d, const double* u, double* w)
{
	double ke = 0.0;
	w[0] = u[0];
	for (int a = 0; a < d; ++a) { w[1 + a] = u[1 + a]/u[0]; ke += u[1 + a]*w[1 + a]; }
	w[d + 1] = DPG_GM1*(u[d + 1] - 0.5*ke);
}

static void write_scalar(FILE* fp, const char* name, int n, const double* vals, int stride)
{
	fprintf(fp,"\t\t<DataArray type=\"Float64\" Name=\"%s\" format=\"ascii\">\n\t\t\t",name);
	for (int k = 0; k < n; ++k) fprintf(fp,"% .15e ",vals[(size_t)k*stride]);
	fprintf(fp,"\n\t\t</DataArray>\n");
}

static void write_vector(FILE* fp, const char* name, int n, int d, const double* vals, int stride, int first)
{
	fprintf(fp,"\t\t<DataArray type=\"Float64\" Name=\"%s\" NumberOfComponents=\"3\" format=\"ascii\">\n\t\t\t",name);
	for (int k = 0; k < n; ++k)
		for (int a = 0; a < 3; ++a) fprintf(fp,"% .15e ",a < d ? vals[(size_t)k*stride + first + a] : 0.0);
	fprintf(fp,"\n\t\t</DataArray>\n");
}

int dpg_sim_write_vtk(const struct dpg_sim* sim, const char* path)
{
	if (!sim || !path) return DPG_ERR_INVALID;
	if (sim->ops[0].e_type == DPG_TET) return DPG_ERR_UNSUPPORTED;   /* plotting sub-cells: QUAD, HEX, TRI */
	FILE* fp = fopen(path,"w");
	if (!fp) return DPG_ERR_IO;
	const int d = sim->d, n_var = sim->n_var;
	const int euler = (n_var == d + 2);
	const int with_error = (sim->pde_index == DPG_PDE_EULER);
	int max_pts = 0, max_s = 0;
	for (int k = 0; k < sim->n_ops; ++k) {
		int n = 1;
		for (int a = 0; a < d; ++a) n *= sim->ops[k].p + 1;
		if (n > max_pts) max_pts = n;
		if (sim->ops[k].n_s > max_s) max_s = sim->ops[k].n_s;
	}
	double* r = malloc(sizeof(double)*(size_t)max_pts*d);
	double* phi = malloc(sizeof(double)*(size_t)max_pts*max_s);
	double* x = malloc(sizeof(double)*(size_t)max_pts*3);
	double* w = malloc(sizeof(double)*(size_t)max_pts*DPG_NVAR_MAX);   /* plotted variables */
	double* e = malloc(sizeof(double)*(size_t)max_pts*DPG_NVAR_MAX);   /* their errors      */
	double* ex = malloc(sizeof(double)*(size_t)max_s*DPG_NVAR_MAX);    /* exact solution at the solution nodes */
	int* conn = malloc(sizeof(int)*(size_t)8*max_pts);
	int rc = DPG_OK;
	if (!r || !phi || !x || !w || !e || !ex || !conn) { rc = DPG_ERR_INVALID; goto done; }
	fprintf(fp,"<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
	           "<UnstructuredGrid>\n");
	for (int v = 0; v < sim->n_vol; ++v) {
		const struct dpg_element_ops* o = &sim->ops[sim->vol_ops[v]];
		const int n_pt = plot_points(o,r);
		int npc = 0;
		const int n_cell = plot_cells(o,conn,&npc);
		if (basis_at(o,n_pt,r,phi)) { rc = DPG_ERR_INVALID; goto done; }
		const double* sc = &sim->sol_coef[sim->vol_dof_off[v]];
		if (with_error)   /* the exact solution at the solution nodes, interpolated like the solution (vv0_vs_vp) */
			for (int i = 0; i < o->n_s; ++i) {
				double xs[3];
				map_point(sim,o,v,&o->rst_vs[(size_t)i*d],xs);
				dpg_exact_solution(sim,sim->time,xs,&ex[(size_t)i*DPG_NVAR_MAX]);
			}
		for (int k = 0; k < n_pt; ++k) {
			map_point(sim,o,v,&r[(size_t)k*d],&x[(size_t)k*3]);
			double u[DPG_NVAR_MAX], ue[DPG_NVAR_MAX];
			for (int var = 0; var < n_var; ++var) {
				double s = 0.0;
				for (int i = 0; i < o->n_s; ++i) s += phi[(size_t)k*o->n_s + i]*sc[i + (size_t)o->n_s*var];
				u[var] = s;
			}
			if (euler) to_primitive(d,u,&w[(size_t)k*DPG_NVAR_MAX]);
			else w[(size_t)k*DPG_NVAR_MAX] = u[0];
			if (with_error) {
				double pe[DPG_NVAR_MAX];
				for (int var = 0; var < n_var; ++var) {
					double s = 0.0;
					for (int i = 0; i < o->n_s; ++i) s += phi[(size_t)k*o->n_s + i]*ex[(size_t)i*DPG_NVAR_MAX + var];
					ue[var] = s;
				}
				to_primitive(d,ue,pe);
				for (int var = 0; var < n_var; ++var)
					e[(size_t)k*DPG_NVAR_MAX + var] = fabs(pe[var] - w[(size_t)k*DPG_NVAR_MAX + var]);
			}
		}
		fprintf(fp,"\n<Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n",n_pt,n_cell);
		fprintf(fp,"\t<Points>\n\t\t<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n\t\t\t");
		for (int k = 0; k < n_pt; ++k) fprintf(fp,"% .15e % .15e % .15e ",x[3*k],x[3*k+1],x[3*k+2]);
		fprintf(fp,"\n\t\t</DataArray>\n\t</Points>\n\t<Cells>\n");
		fprintf(fp,"\t\t<DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n\t\t\t");
		for (int c = 0; c < n_cell*npc; ++c) fprintf(fp,"%d ",conn[c]);
		fprintf(fp,"\n\t\t</DataArray>\n\t\t<DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n\t\t\t");
		for (int c = 1; c <= n_cell; ++c) fprintf(fp,"%d ",c*npc);
		fprintf(fp,"\n\t\t</DataArray>\n\t\t<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n\t\t\t");
		const int type = (o->e_type == DPG_TRI ? VTK_TRIANGLE : d == 2 ? VTK_QUAD : VTK_HEXAHEDRON);
		for (int c = 0; c < n_cell; ++c) fprintf(fp,"%d ",type);
		fprintf(fp,"\n\t\t</DataArray>\n\t</Cells>\n\t<PointData Scalars=\"Scalars\" Vectors=\"Vectors\">\n");
		fprintf(fp,"\t\t<DataArray type=\"Int32\" Name=\"index\" format=\"ascii\">\n\t\t\t");
		for (int k = 0; k < n_pt; ++k) fprintf(fp,"%d ",v);
		fprintf(fp,"\n\t\t</DataArray>\n\t\t<DataArray type=\"Int32\" Name=\"p_ref\" format=\"ascii\">\n\t\t\t");
		for (int k = 0; k < n_pt; ++k) fprintf(fp,"%d ",o->p);
		fprintf(fp,"\n\t\t</DataArray>\n");
		if (euler) {
			write_scalar(fp,"$\\rho$",n_pt,w,DPG_NVAR_MAX);
			write_vector(fp,"$\\mathbf{v}$",n_pt,d,w,DPG_NVAR_MAX,1);
			write_scalar(fp,"$\\mathit{p}$",n_pt,w + d + 1,DPG_NVAR_MAX);
			if (with_error) {
				write_scalar(fp,"$|\\rho-\\rho_e|$",n_pt,e,DPG_NVAR_MAX);
				write_vector(fp,"$|\\mathbf{v}-\\mathbf{v}_e|$",n_pt,d,e,DPG_NVAR_MAX,1);
				write_scalar(fp,"$|p-p_e|$",n_pt,e + d + 1,DPG_NVAR_MAX);
			}
		} else {
			write_scalar(fp,"u",n_pt,w,DPG_NVAR_MAX);
		}
		fprintf(fp,"\t</PointData>\n</Piece>\n");
	}
	fprintf(fp,"</UnstructuredGrid>\n</VTKFile>\n");
done:
	if (fclose(fp) != 0 && rc == DPG_OK) rc = DPG_ERR_IO;
	free(r); free(phi); free(x); free(w); free(e); free(ex); free(conn);
	return rc;
}
