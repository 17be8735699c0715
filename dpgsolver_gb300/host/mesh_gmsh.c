/* Mesh sources of the host set-up: the structured periodic box and the reader of gmsh 2.2 ASCII meshes.
 *
 * Both produce the volume / face tables of struct dpg_mesh (dpg_host.h): vertices of each volume in tensor-product
 * order (vertex k has coordinate bit a = (k >> a) & 1 along reference direction a, the order of the reference's
 * P1 geometry basis) and, per face, its two (volume, local face) sides, local face lf = 2 a + (0 | 1) on the -a / +a
 * side.  Geometry (normals, face-node correspondence nc_fc by coordinate matching modulo the periodic lengths) is
 * computed afterwards from these tables.
 *
 * gmsh reader: follows the reference's mesh reader (mesh_readers.c: $Nodes, $Elements with their tags, $Periodic
 * node correspondences at :225-378) for the element types of this path -- 4-node quadrilaterals in 2D, 8-node
 * hexahedra in 3D; boundary lines (2D) and quadrilaterals (3D) carry the boundary conditions in their physical tags
 * (bc_base + BC_*, definitions_bc.h; taken modulo BC_STEP_SC = 10000); points are read past.  Interior faces are
 * paired by the vertex sets of the volumes' local faces.  A face with no partner is a boundary face when a boundary
 * element with its vertices carries a condition of this path (Riemann, slip wall, adiabatic or rotating no-slip
 * wall); otherwise it must consist of $Periodic nodes and is paired with its periodic image across the box (the
 * periodic lengths: the extents of the vertices' bounding box).  Other conditions are refused
 * (DPG_ERR_UNSUPPORTED), as are other element types (mixed or curved meshes).
 * The gmsh vertex order of a quadrilateral is counter-clockwise, of a hexahedron bottom then top face
 * counter-clockwise; volumes whose tensor-product map comes out left-handed are mirrored in the last reference
 * direction.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dpg_host.h"
#include "dpg_gb300.h"

void dpg_mesh_free(struct dpg_mesh* m)
{
	if (!m) return;
	free(m->xyz_ve); free(m->face_vol); free(m->face_lf); free(m->face_bc); free(m->vol_p);
	memset(m,0,sizeof *m);
}

/* ---- structured periodic box ---------------------------------------------------------------------------- */

/* splitmix64: seeded uniform numbers for the vertex jitter and the orders of mixed-order meshes */
uint64_t dpg_splitmix64(uint64_t* s)
{
	uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}
static double urand(uint64_t* s) { return (double)(dpg_splitmix64(s) >> 11) * (1.0/9007199254740992.0); }

/* Faces in the order of the reference's constructor_Faces (computational_elements/face.c:108-148): volumes in order,
 * their local faces in order, a face created by the first volume that reaches it -- that volume is side 0
 * (neigh_info[0]) -- and joined to the neighbour's opposite local face; a local face without a neighbour is a
 * boundary face (side 1 = -1) with the code bc_of[v n_fl + lf].  nb[v n_fl + lf]: neighbour volume or -1. */
static int faces_in_reference_order(int n_vol, int n_fl, const int* nb, const int* bc_of, struct dpg_mesh* m)
{
	int* seen = calloc((size_t)n_vol*n_fl,sizeof(int));
	m->face_vol = calloc((size_t)2*n_vol*n_fl,sizeof(int));
	m->face_lf = calloc((size_t)2*n_vol*n_fl,sizeof(int));
	m->face_bc = calloc((size_t)n_vol*n_fl,sizeof(int));
	if (!seen || !m->face_vol || !m->face_lf || !m->face_bc) { free(seen); return DPG_ERR_INVALID; }
	int f = 0;
	for (int v = 0; v < n_vol; ++v)
		for (int lf = 0; lf < n_fl; ++lf) {
			if (seen[v*n_fl + lf]) continue;
			seen[v*n_fl + lf] = 1;
			const int w = nb[v*n_fl + lf], lw = lf ^ 1;
			m->face_vol[2*f] = v;  m->face_lf[2*f] = lf;
			m->face_vol[2*f+1] = w; m->face_lf[2*f+1] = (w < 0 ? -1 : lw);
			m->face_bc[f] = (w < 0 ? bc_of[v*n_fl + lf] : 0);
			if (w >= 0) seen[w*n_fl + lw] = 1;
			++f;
		}
	m->n_face = f;
	free(seen);
	return DPG_OK;
}

int dpg_mesh_structured(const struct dpg_sim_params* prm, struct dpg_mesh* m)
{
	memset(m,0,sizeof *m);
	const int d = prm->d, n_fl = 2*d;
	const int nx = prm->n_elem[0], ny = prm->n_elem[1], nz = (d == 3 ? prm->n_elem[2] : 1);
	const int n_vol = nx*ny*nz;
	m->d = d; m->n_vol = n_vol;
	/* a direction is periodic when neither of its sides carries a boundary condition */
	int periodic[3] = {1,1,1};
	for (int a = 0; a < d; ++a) periodic[a] = (prm->bc_side[2*a] == 0 && prm->bc_side[2*a+1] == 0);
	for (int a = 0; a < 3; ++a) {
		m->lo[a] = prm->lo[a]; m->hi[a] = prm->hi[a];
		if (a < d && !periodic[a]) m->hi[a] = m->lo[a];   /* zero extent: no periodic image in this direction */
	}
	m->xyz_ve = calloc((size_t)n_vol*DPG_NVE_MAX*3,sizeof(double));
	int* nb = calloc((size_t)n_vol*n_fl,sizeof(int));
	int* bc_of = calloc((size_t)n_vol*n_fl,sizeof(int));
	/* vertex grid with periodic-consistent jitter: vertex (i,j,k), i in [0,nx], is the image of (i mod nx, ...) */
	const int nvx = nx, nvy = ny, nvz = nz;
	double* jit = calloc((size_t)nvx*nvy*nvz*3,sizeof(double));
	if (!m->xyz_ve || !nb || !bc_of || !jit) { free(jit); free(nb); free(bc_of); dpg_mesh_free(m); return DPG_ERR_INVALID; }
	double h[3];
	for (int a = 0; a < 3; ++a) h[a] = (a < d ? (prm->hi[a]-prm->lo[a])/prm->n_elem[a] : 0.0);
	if (prm->jitter > 0.0) {
		uint64_t st = prm->seed*0x2545F4914F6CDD1Dull + 1;
		for (size_t q = 0; q < (size_t)nvx*nvy*nvz; ++q)
			for (int a = 0; a < d; ++a)
				jit[q*3+a] = prm->jitter*h[a]*(2.0*urand(&st) - 1.0);
	}
	const int ne[3] = {nx, ny, nz};
	for (int k = 0; k < nz; ++k)
	for (int j = 0; j < ny; ++j)
	for (int i = 0; i < nx; ++i) {
		const int v = i + nx*(j + ny*k);
		const int ijk[3] = {i, j, k};
		for (int kv = 0; kv < (1 << d); ++kv) {
			const int bi = kv & 1, bj = (kv >> 1) & 1, bk = (kv >> 2) & 1;
			const int gi = i+bi, gj = j+bj, gk = k+bk;
			/* jitter of a wall vertex keeps it on its wall: only periodic directions share images */
			const size_t q = (size_t)(gi % nvx) + (size_t)nvx*((gj % nvy) + (size_t)nvy*(d == 3 ? gk % nvz : 0));
			const int on_wall[3] = {!periodic[0] && (gi == 0 || gi == nx), !periodic[1] && (gj == 0 || gj == ny),
			                        d == 3 && !periodic[2] && (gk == 0 || gk == nz)};
			double* x = &m->xyz_ve[((size_t)v*DPG_NVE_MAX + kv)*3];
			x[0] = prm->lo[0] + gi*h[0] + (on_wall[0] ? 0.0 : jit[q*3+0]);
			x[1] = prm->lo[1] + gj*h[1] + (on_wall[1] ? 0.0 : jit[q*3+1]);
			x[2] = (d == 3 ? prm->lo[2] + gk*h[2] + (on_wall[2] ? 0.0 : jit[q*3+2]) : 0.0);
		}
		for (int a = 0; a < d; ++a)
			for (int sd = 0; sd < 2; ++sd) {
				int t[3] = {ijk[0], ijk[1], ijk[2]};
				t[a] += (sd ? 1 : -1);
				int w;
				if (t[a] < 0 || t[a] >= ne[a]) {
					if (periodic[a]) { t[a] = (t[a] + ne[a]) % ne[a]; w = t[0] + nx*(t[1] + ny*t[2]); }
					else w = -1;
				} else w = t[0] + nx*(t[1] + ny*t[2]);
				nb[v*n_fl + 2*a + sd] = w;
				bc_of[v*n_fl + 2*a + sd] = (w < 0 ? prm->bc_side[2*a + sd] : 0);
			}
	}
	free(jit);
	const int rc = faces_in_reference_order(n_vol,n_fl,nb,bc_of,m);
	free(nb); free(bc_of);
	if (rc) dpg_mesh_free(m);
	return rc;
}

/* The annulus lo[0] <= r <= hi[0] of nr = n_elem[0] radial x nt = n_elem[1] azimuthal curved QUADs, periodic in theta:
 * volume i + nr j spans [r_i, r_i+1] x [theta_j, theta_j+1] (uniform), reference direction 0 radial, 1 azimuthal
 * (a right-handed map).  The vertices are stored as (r, theta); the geometry is the parametric map
 * x = r cos(theta), y = r sin(theta) of geometry_parametric_T.c:128-171 (whose square-annulus input mesh it maps to
 * this uniform polar grid), interpolated at the geometry nodes (order p) by the geometry set-up.  Local face 0 of the
 * innermost volumes carries bc_side[0], local face 1 of the outermost bc_side[1]. */
int dpg_mesh_annulus(const struct dpg_sim_params* prm, struct dpg_mesh* m)
{
	memset(m,0,sizeof *m);
	const int nr = prm->n_elem[0], nt = prm->n_elem[1], n_fl = 4;
	if (prm->d != 2 || nr < 1 || nt < 3 || !(prm->hi[0] > prm->lo[0]) || !(prm->lo[0] > 0.0)) return DPG_ERR_INVALID;
	const int n_vol = nr*nt;
	m->d = 2; m->n_vol = n_vol;
	m->xyz_ve = calloc((size_t)n_vol*DPG_NVE_MAX*3,sizeof(double));
	int* nb = calloc((size_t)n_vol*n_fl,sizeof(int));
	int* bc_of = calloc((size_t)n_vol*n_fl,sizeof(int));
	if (!m->xyz_ve || !nb || !bc_of) { free(nb); free(bc_of); dpg_mesh_free(m); return DPG_ERR_INVALID; }
	const double dr = (prm->hi[0] - prm->lo[0])/nr, dth = 2.0*M_PI/nt;
	for (int j = 0; j < nt; ++j)
	for (int i = 0; i < nr; ++i) {
		const int v = i + nr*j;
		for (int kv = 0; kv < 4; ++kv) {
			double* x = &m->xyz_ve[((size_t)v*DPG_NVE_MAX + kv)*3];
			x[0] = prm->lo[0] + (i + (kv & 1))*dr;
			x[1] = (j + ((kv >> 1) & 1))*dth;
		}
		nb[v*n_fl + 0] = (i > 0 ? v - 1 : -1);
		nb[v*n_fl + 1] = (i < nr-1 ? v + 1 : -1);
		nb[v*n_fl + 2] = i + nr*((j + nt - 1) % nt);
		nb[v*n_fl + 3] = i + nr*((j + 1) % nt);
		bc_of[v*n_fl + 0] = (i == 0 ? prm->bc_side[0] : 0);
		bc_of[v*n_fl + 1] = (i == nr-1 ? prm->bc_side[1] : 0);
	}
	/* no periodic box: faces are matched in physical coordinates (theta = 2 pi and 0 give the same points) */
	for (int a = 0; a < 3; ++a) m->lo[a] = m->hi[a] = 0.0;
	m->geom = DPG_GEOM_CYLINDER;
	const int rc = faces_in_reference_order(n_vol,n_fl,nb,bc_of,m);
	free(nb); free(bc_of);
	if (rc) dpg_mesh_free(m);
	return rc;
}

/* ---- gmsh 2.2 ASCII ---------------------------------------------------------------------------------------- */

struct face_entry { int key[4]; int vol, lf; };

static int cmp_key(const struct face_entry* x, const struct face_entry* y)
{
	for (int i = 0; i < 4; ++i)
		if (x->key[i] != y->key[i]) return x->key[i] < y->key[i] ? -1 : 1;
	return 0;
}

/* total order: vertex set, then volume, then local face (side 0 of a face: its smaller (volume, local face)) */
static int cmp_face(const void* a, const void* b)
{
	const struct face_entry* x = a;
	const struct face_entry* y = b;
	const int c = cmp_key(x,y);
	if (c) return c;
	if (x->vol != y->vol) return x->vol < y->vol ? -1 : 1;
	return (x->lf > y->lf) - (x->lf < y->lf);
}

static int cmp_int(const void* a, const void* b)
{
	const int x = *(const int*)a, y = *(const int*)b;
	return (x > y) - (x < y);
}

static int starts(const char* line, const char* tag) { return strncmp(line,tag,strlen(tag)) == 0; }

int dpg_mesh_read_gmsh(const char* path, int d, int e_type, struct dpg_mesh* m)
{
	memset(m,0,sizeof *m);
	if (d != 2 && d != 3) return DPG_ERR_INVALID;
	const int tri = (e_type == DPG_TRI), tet = (e_type == DPG_TET), simplex = tri || tet;
	if ((tri && d != 2) || (tet && d != 3)) return DPG_ERR_INVALID;
	if (e_type != DPG_TRI && e_type != DPG_QUAD && e_type != DPG_HEX && e_type != DPG_TET) return DPG_ERR_UNSUPPORTED;
	FILE* fp = fopen(path,"r");
	if (!fp) return DPG_ERR_IO;
	/* gmsh: 2 = 3-node triangle, 3 = 4-node quadrilateral, 4 = 4-node tetrahedron, 5 = 8-node hexahedron */
	const int vol_type = tri ? 2 : tet ? 4 : (d == 2 ? 3 : 5), n_ve = tri ? 3 : tet ? 4 : 1 << d;
	const int nvf = tri ? 2 : tet ? 3 : 1 << (d-1);   /* vertices of a face */
	int rc = DPG_OK;
	int n_nodes = 0, max_id = 0, n_vol = 0, vol_cap = 0, n_pairs = 0, pair_cap = 0;
	int* node_id = NULL;          /* [n_nodes] gmsh node numbers                  */
	double* node_x = NULL;        /* [n_nodes][3]                                 */
	int* vol_nodes = NULL;        /* [n_vol][n_ve] gmsh node numbers, gmsh order  */
	int* pairs = NULL;            /* [n_pairs][2] (slave, master) gmsh numbers    */
	int n_bel = 0, bel_cap = 0;
	int* bel = NULL;              /* boundary elements [n_bel][5]: physical tag, then 2^(d-1) gmsh numbers */
	int* index = NULL;            /* gmsh number -> node index                     */
	struct face_entry* fe = NULL;
	int seen_format = 0;
	char line[1024];
	while (fgets(line,sizeof line,fp)) {
		if (starts(line,"$MeshFormat")) {
			double ver = 0.0; int ftype = -1;
			if (!fgets(line,sizeof line,fp) || sscanf(line,"%lf %d",&ver,&ftype) != 2) { rc = DPG_ERR_IO; goto done; }
			if (ver < 2.0 || ver >= 3.0 || ftype != 0) { rc = DPG_ERR_UNSUPPORTED; goto done; }   /* 2.x ASCII only */
			seen_format = 1;
		} else if (starts(line,"$Nodes")) {
			if (!fgets(line,sizeof line,fp) || sscanf(line,"%d",&n_nodes) != 1 || n_nodes < 1) { rc = DPG_ERR_IO; goto done; }
			node_id = malloc(sizeof(int)*(size_t)n_nodes);
			node_x = malloc(sizeof(double)*3*(size_t)n_nodes);
			if (!node_id || !node_x) { rc = DPG_ERR_INVALID; goto done; }
			for (int i = 0; i < n_nodes; ++i) {
				if (!fgets(line,sizeof line,fp) ||
				    sscanf(line,"%d %lf %lf %lf",&node_id[i],&node_x[3*i],&node_x[3*i+1],&node_x[3*i+2]) != 4 ||
				    node_id[i] < 1) { rc = DPG_ERR_IO; goto done; }
				if (node_id[i] > max_id) max_id = node_id[i];
			}
		} else if (starts(line,"$Elements")) {
			int n_el = 0;
			if (!fgets(line,sizeof line,fp) || sscanf(line,"%d",&n_el) != 1 || n_el < 0) { rc = DPG_ERR_IO; goto done; }
			for (int i = 0; i < n_el; ++i) {
				if (!fgets(line,sizeof line,fp)) { rc = DPG_ERR_IO; goto done; }
				char* s = line;
				char* end = NULL;
				long val[64];
				int nv = 0;
				for (;;) {   /* id type n_tags tags... nodes... */
					const long x = strtol(s,&end,10);
					if (end == s) break;
					if (nv == 64) { rc = DPG_ERR_UNSUPPORTED; goto done; }
					val[nv++] = x;
					s = end;
				}
				if (nv < 3 || nv < 3 + val[2]) { rc = DPG_ERR_IO; goto done; }
				const int type = (int)val[1], n_tags = (int)val[2], n_el_nodes = nv - 3 - n_tags;
				if (type == vol_type) {
					if (n_el_nodes != n_ve) { rc = DPG_ERR_IO; goto done; }
					if (n_vol == vol_cap) {
						vol_cap = vol_cap ? 2*vol_cap : 256;
						int* t = realloc(vol_nodes,sizeof(int)*(size_t)vol_cap*n_ve);
						if (!t) { rc = DPG_ERR_INVALID; goto done; }
						vol_nodes = t;
					}
					for (int k = 0; k < n_ve; ++k) vol_nodes[(size_t)n_vol*n_ve + k] = (int)val[3 + n_tags + k];
					++n_vol;
				} else if ((d == 2 && type == 1) || (d == 3 && type == (tet ? 2 : 3))) {
					/* boundary lines (2D), quadrilaterals or triangles (3D): their physical tag is the boundary
					 * condition of the volume face with the same vertices (bc_base + BC_*, definitions_bc.h) */
					if (n_el_nodes != nvf) { rc = DPG_ERR_IO; goto done; }
					if (n_bel == bel_cap) {
						bel_cap = bel_cap ? 2*bel_cap : 256;
						int* t = realloc(bel,sizeof(int)*5*(size_t)bel_cap);
						if (!t) { rc = DPG_ERR_INVALID; goto done; }
						bel = t;
					}
					bel[5*n_bel] = n_tags > 0 ? (int)val[3] : 0;
					for (int k = 0; k < 4; ++k) bel[5*n_bel + 1 + k] = (k < nvf ? (int)val[3 + n_tags + k] : -1);
					++n_bel;
				} else if (type == 15 || type == 1) {
					/* points; lines of a 3D mesh */
				} else {
					rc = DPG_ERR_UNSUPPORTED;   /* triangles, tetrahedra, prisms, pyramids, curved elements */
					goto done;
				}
			}
		} else if (starts(line,"$Periodic")) {
			int n_ent = 0;
			if (!fgets(line,sizeof line,fp) || sscanf(line,"%d",&n_ent) != 1) { rc = DPG_ERR_IO; goto done; }
			for (int en = 0; en < n_ent; ++en) {
				int dim, t1, t2, n_corr = 0;
				if (!fgets(line,sizeof line,fp) || sscanf(line,"%d %d %d",&dim,&t1,&t2) != 3) { rc = DPG_ERR_IO; goto done; }
				if (!fgets(line,sizeof line,fp)) { rc = DPG_ERR_IO; goto done; }
				if (starts(line,"Affine") && !fgets(line,sizeof line,fp)) { rc = DPG_ERR_IO; goto done; }
				if (sscanf(line,"%d",&n_corr) != 1 || n_corr < 0) { rc = DPG_ERR_IO; goto done; }
				for (int c = 0; c < n_corr; ++c) {
					int a, b;
					if (!fgets(line,sizeof line,fp) || sscanf(line,"%d %d",&a,&b) != 2) { rc = DPG_ERR_IO; goto done; }
					if (n_pairs == pair_cap) {
						pair_cap = pair_cap ? 2*pair_cap : 256;
						int* t = realloc(pairs,sizeof(int)*2*(size_t)pair_cap);
						if (!t) { rc = DPG_ERR_INVALID; goto done; }
						pairs = t;
					}
					pairs[2*n_pairs] = a; pairs[2*n_pairs+1] = b;
					++n_pairs;
				}
			}
		}
	}
	if (!seen_format || n_nodes < 1 || n_vol < 1) { rc = DPG_ERR_IO; goto done; }

	/* node numbers -> indices; the periodic correspondences must name existing nodes */
	index = malloc(sizeof(int)*((size_t)max_id + 1));
	if (!index) { rc = DPG_ERR_INVALID; goto done; }
	for (int i = 0; i <= max_id; ++i) index[i] = -1;
	for (int i = 0; i < n_nodes; ++i) index[node_id[i]] = i;
	for (int p = 0; p < n_pairs; ++p) {
		const int a = pairs[2*p], b = pairs[2*p+1];
		if (a < 1 || b < 1 || a > max_id || b > max_id || index[a] < 0 || index[b] < 0) { rc = DPG_ERR_IO; goto done; }
	}

	/* boundary elements: vertex sets as sorted node indices, for the lookup of unmatched faces */
	for (int b = 0; b < n_bel; ++b) {
		int* k = &bel[5*b + 1];
		for (int q = 0; q < nvf; ++q) {
			if (k[q] < 1 || k[q] > max_id || index[k[q]] < 0) { rc = DPG_ERR_IO; goto done; }
			k[q] = index[k[q]];
		}
		qsort(k,(size_t)nvf,sizeof(int),cmp_int);
	}

	m->d = d; m->n_vol = n_vol;
	m->xyz_ve = calloc((size_t)n_vol*DPG_NVE_MAX*3,sizeof(double));
	int* vidx = malloc(sizeof(int)*(size_t)n_vol*n_ve);   /* node indices in tensor-product order */
	if (!m->xyz_ve || !vidx) { free(vidx); rc = DPG_ERR_INVALID; goto done; }
	static const int tp_of_gmsh_quad[4] = {0,1,3,2}, tp_of_gmsh_hex[8] = {0,1,3,2,4,5,7,6}, simplex_id[4] = {0,1,2,3};
	const int* perm = simplex ? simplex_id : (d == 2 ? tp_of_gmsh_quad : tp_of_gmsh_hex);
	for (int v = 0; v < n_vol; ++v) {
		int* vi = &vidx[(size_t)v*n_ve];
		for (int k = 0; k < n_ve; ++k) {
			const int id = vol_nodes[(size_t)v*n_ve + perm[k]];
			if (id < 1 || id > max_id || index[id] < 0) { free(vidx); rc = DPG_ERR_IO; goto done; }
			vi[k] = index[id];
		}
		/* right-handed tensor-product map: det[x_1 - x_0, x_2 - x_0 (, x_4 - x_0)] > 0, else mirror the last direction;
		 * a triangle: counter-clockwise v0, v1, v2 (the reference triangle's order), else v1 and v2 exchanged; a
		 * tetrahedron: det[x_1 - x_0, x_2 - x_0, x_3 - x_0] > 0 (the reference tetrahedron's), else v0 and v1 exchanged */
		const double* x0 = &node_x[3*vi[0]];
		double e[3][3];
		for (int a = 0; a < d; ++a)
			for (int i = 0; i < 3; ++i) e[a][i] = node_x[3*vi[simplex ? a + 1 : 1 << a] + i] - x0[i];
		const double det = (d == 2 ? e[0][0]*e[1][1] - e[0][1]*e[1][0]
		                           : e[0][0]*(e[1][1]*e[2][2] - e[1][2]*e[2][1]) - e[0][1]*(e[1][0]*e[2][2] - e[1][2]*e[2][0])
		                             + e[0][2]*(e[1][0]*e[2][1] - e[1][1]*e[2][0]));
		if (!(det != 0.0)) { free(vidx); rc = DPG_ERR_INVALID; goto done; }
		if (det < 0.0 && tri) {
			const int t = vi[1]; vi[1] = vi[2]; vi[2] = t;
		} else if (det < 0.0 && tet) {
			const int t = vi[0]; vi[0] = vi[1]; vi[1] = t;
		} else if (det < 0.0) {
			const int bit = 1 << (d-1);
			for (int k = 0; k < n_ve; ++k)
				if (!(k & bit)) { const int t = vi[k]; vi[k] = vi[k | bit]; vi[k | bit] = t; }
		}
		for (int k = 0; k < n_ve; ++k)
			for (int i = 0; i < 3; ++i) m->xyz_ve[((size_t)v*DPG_NVE_MAX + k)*3 + i] = node_x[3*vi[k] + i];
	}
	/* bounding box: the periodic lengths */
	for (int i = 0; i < 3; ++i) { m->lo[i] = 1e300; m->hi[i] = -1e300; }
	for (size_t q = 0; q < (size_t)n_vol*n_ve; ++q)
		for (int i = 0; i < 3; ++i) {
			const double x = node_x[3*vidx[q] + i];
			if (x < m->lo[i]) m->lo[i] = x;
			if (x > m->hi[i]) m->hi[i] = x;
		}
	if (d == 2) { m->lo[2] = 0.0; m->hi[2] = 0.0; }

	/* faces.  Interior faces: the local faces' vertex sets, sorted; equal sets pair up.  Boundary faces (the rest):
	 * every vertex a node of the $Periodic correspondences; paired with their periodic image, found by the face
	 * centroid reduced modulo the box's extents (a vertex-set test through the correspondences is ambiguous on
	 * meshes one or two elements wide, where distinct faces share their periodic images' vertices). */
	static const int tri_fve[3][2] = {{1,2}, {0,2}, {0,1}};
	static const int tet_fve[4][3] = {{2,3,1}, {2,3,0}, {0,1,3}, {0,1,2}};
	const int n_fl = tri ? 3 : tet ? 4 : 2*d;
	const size_t n_ent = (size_t)n_vol*n_fl;
	fe = malloc(sizeof *fe*n_ent);
	unsigned char* periodic_node = calloc((size_t)n_nodes,1);
	if (!fe || !periodic_node) { free(vidx); free(periodic_node); rc = DPG_ERR_INVALID; goto done; }
	for (int p = 0; p < n_pairs; ++p) { periodic_node[index[pairs[2*p]]] = 1; periodic_node[index[pairs[2*p+1]]] = 1; }
	double per[3];
	for (int i = 0; i < 3; ++i) per[i] = m->hi[i] - m->lo[i];
	for (int v = 0; v < n_vol; ++v)
		for (int lf = 0; lf < n_fl; ++lf) {
			struct face_entry* f = &fe[(size_t)v*n_fl + lf];
			const int a = lf/2, side = lf % 2;
			int c = 0;
			if (tri) { f->key[c++] = vidx[(size_t)v*n_ve + tri_fve[lf][0]]; f->key[c++] = vidx[(size_t)v*n_ve + tri_fve[lf][1]]; }
			else if (tet) for (int k = 0; k < 3; ++k) f->key[c++] = vidx[(size_t)v*n_ve + tet_fve[lf][k]];
			else
				for (int k = 0; k < n_ve; ++k)
					if (((k >> a) & 1) == side) f->key[c++] = vidx[(size_t)v*n_ve + k];
			for (; c < 4; ++c) f->key[c] = -1;
			qsort(f->key,(size_t)nvf,sizeof(int),cmp_int);
			f->vol = v; f->lf = lf;
		}
	qsort(fe,n_ent,sizeof *fe,cmp_face);
	m->face_vol = malloc(sizeof(int)*2*n_ent);   /* two slots per face; a boundary face uses one local face */
	m->face_lf = malloc(sizeof(int)*2*n_ent);
	m->face_bc = calloc(n_ent,sizeof(int));
	struct face_entry* bf = malloc(sizeof *bf*n_ent);
	struct face_entry* wf = malloc(sizeof *wf*n_ent);   /* faces with a boundary condition, and their codes */
	int* wbc = malloc(sizeof(int)*n_ent);
	if (!m->face_vol || !m->face_lf || !m->face_bc || !bf || !wf || !wbc) {
		free(vidx); free(periodic_node); free(bf); free(wf); free(wbc); rc = DPG_ERR_INVALID; goto done;
	}
	int nf = 0;
	size_t nb = 0, nw = 0;
	for (size_t i = 0; i < n_ent;) {
		size_t j = i + 1;
		while (j < n_ent && cmp_key(&fe[i],&fe[j]) == 0) ++j;
		if (j - i == 2) {
			m->face_vol[2*nf] = fe[i].vol;   m->face_lf[2*nf] = fe[i].lf;
			m->face_vol[2*nf+1] = fe[i+1].vol; m->face_lf[2*nf+1] = fe[i+1].lf;
			++nf;
		} else if (j - i == 1) {
			/* a boundary element with the face's vertices and a wall / far-field code: a boundary face */
			int code = 0;
			for (int b = 0; b < n_bel && !code; ++b) {
				int same = 1;
				for (int c = 0; c < nvf; ++c) same &= (bel[5*b + 1 + c] == fe[i].key[c]);
				if (!same) continue;
				const int bc = bel[5*b] % 10000;   /* BC_STEP_SC: straight and curved numbering alike */
				if (bc == DPG_BC_RIEMANN || bc == DPG_BC_SLIPWALL || bc == DPG_BC_NOSLIP_ADIABATIC ||
				    bc == DPG_BC_NOSLIP_ALL_ROTATING)
					code = bc;
				else if (bc < 51 || bc > 56) {   /* neither periodic (PERIODIC_XL .. ZR) nor a condition of this path */
					free(vidx); free(periodic_node); free(bf); free(wf); free(wbc); rc = DPG_ERR_UNSUPPORTED; goto done;
				}
			}
			if (code) { wf[nw] = fe[i]; wbc[nw++] = code; i = j; continue; }
			for (int c = 0; c < nvf; ++c)
				if (!periodic_node[fe[i].key[c]]) {
					free(vidx); free(periodic_node); free(bf); free(wf); free(wbc); rc = DPG_ERR_UNSUPPORTED; goto done;
				}
			bf[nb] = fe[i];
			/* key: centroid cell, each coordinate reduced modulo the extent and quantised to 2^-20 of it */
			for (int c = 0; c < 3; ++c) {
				double x = 0.0;
				if (c < d) {
					for (int q = 0; q < nvf; ++q) x += node_x[3*fe[i].key[q] + c];
					x = (x/nvf - m->lo[c])/per[c];
				}
				long long cell = (long long)floor(x*1048576.0 + 0.5) % 1048576;
				if (cell < 0) cell += 1048576;
				bf[nb].key[c] = (int)cell;
			}
			bf[nb].key[3] = 0;
			++nb;
		} else {
			free(vidx); free(periodic_node); free(bf); free(wf); free(wbc); rc = DPG_ERR_INVALID; goto done;   /* > 2 volumes on a face */
		}
		i = j;
	}
	free(periodic_node);
	free(vidx);
	qsort(bf,nb,sizeof *bf,cmp_face);
	for (size_t i = 0; i < nb; i += 2) {
		if (i + 1 >= nb || cmp_key(&bf[i],&bf[i+1]) != 0 || (i + 2 < nb && cmp_key(&bf[i+1],&bf[i+2]) == 0)) {
			free(bf); free(wf); free(wbc); rc = DPG_ERR_UNSUPPORTED; goto done;   /* a boundary face without a periodic image */
		}
		m->face_vol[2*nf] = bf[i].vol;   m->face_lf[2*nf] = bf[i].lf;
		m->face_vol[2*nf+1] = bf[i+1].vol; m->face_lf[2*nf+1] = bf[i+1].lf;
		++nf;
	}
	for (size_t i = 0; i < nw; ++i) {   /* boundary faces: one side */
		m->face_vol[2*nf] = wf[i].vol; m->face_lf[2*nf] = wf[i].lf;
		m->face_vol[2*nf+1] = -1;      m->face_lf[2*nf+1] = -1;
		m->face_bc[nf] = wbc[i];
		++nf;
	}
	free(bf); free(wf); free(wbc);
	m->n_face = nf;
done:
	fclose(fp);
	free(node_id); free(node_x); free(vol_nodes); free(pairs); free(index); free(fe); free(bel);
	if (rc != DPG_OK) dpg_mesh_free(m);
	return rc;
}

/* A periodic 2D box of nx x ny cells, each split along its diagonal from (i, j) to (i+1, j+1) into the TRIs
 * [(i,j), (i+1,j), (i+1,j+1)] and [(i,j), (i+1,j+1), (i,j+1)] (counter-clockwise, the order of the reference
 * triangle's vertices v0, v1, v2), numbered cell by cell (i fastest).  Vertex (i, j) is the image of
 * (i mod nx, j mod ny); the jitter (uniform in +-jitter h per coordinate, seeded) is the same for a vertex and its
 * images.  Local face f of a TRI is the edge opposite vertex f; faces pair by their two vertices' images and are
 * listed in the order of their side-0 (volume, local face), side 0 the smaller. */
int dpg_mesh_tri_structured(const struct dpg_sim_params* prm, struct dpg_mesh* m)
{
	memset(m,0,sizeof *m);
	if (prm->d != 2) return DPG_ERR_UNSUPPORTED;
	const int nx = prm->n_elem[0], ny = prm->n_elem[1], n_vol = 2*nx*ny, n_fl = 3;
	if (nx < 1 || ny < 1) return DPG_ERR_INVALID;
	m->d = 2; m->n_vol = n_vol;
	for (int a = 0; a < 3; ++a) { m->lo[a] = prm->lo[a]; m->hi[a] = (a < 2 ? prm->hi[a] : prm->lo[a]); }
	m->xyz_ve = calloc((size_t)n_vol*DPG_NVE_MAX*3,sizeof(double));
	double* jit = calloc((size_t)nx*ny*2,sizeof(double));
	int* vid = malloc(sizeof(int)*(size_t)n_vol*3*2);        /* grid coordinates (unwrapped) of each volume's vertices */
	if (!m->xyz_ve || !jit || !vid) { free(jit); free(vid); dpg_mesh_free(m); return DPG_ERR_INVALID; }
	const double h[2] = {(prm->hi[0] - prm->lo[0])/nx, (prm->hi[1] - prm->lo[1])/ny};
	if (prm->jitter > 0.0) {
		uint64_t st = prm->seed*0x2545F4914F6CDD1Dull + 1;
		for (size_t q = 0; q < (size_t)nx*ny; ++q)
			for (int a = 0; a < 2; ++a) jit[q*2+a] = prm->jitter*h[a]*(2.0*urand(&st) - 1.0);
	}
	static const int corner[2][3][2] = {{{0,0}, {1,0}, {1,1}}, {{0,0}, {1,1}, {0,1}}};
	for (int j = 0; j < ny; ++j)
		for (int i = 0; i < nx; ++i)
			for (int t = 0; t < 2; ++t) {
				const int v = 2*(i + nx*j) + t;
				for (int k = 0; k < 3; ++k) {
					const int gi = i + corner[t][k][0], gj = j + corner[t][k][1];
					const int q = (gi % nx) + nx*(gj % ny);
					vid[(v*3 + k)*2] = gi; vid[(v*3 + k)*2 + 1] = gj;
					double* x = &m->xyz_ve[((size_t)v*DPG_NVE_MAX + k)*3];
					x[0] = prm->lo[0] + gi*h[0] + jit[(size_t)q*2];
					x[1] = prm->lo[1] + gj*h[1] + jit[(size_t)q*2 + 1];
					x[2] = 0.0;
				}
			}
	free(jit);
	/* faces: key = the edge's midpoint in doubled grid units modulo the periodic box (two periodic images of an
	 * edge share it; two edges with the same end vertices on a box two cells wide do not); the first (volume, local
	 * face) with a key is side 0 */
	static const int fve[3][2] = {{1,2}, {0,2}, {0,1}};
	const size_t n_ent = (size_t)n_vol*n_fl;
	struct face_entry* fe = malloc(sizeof *fe*n_ent);
	m->face_vol = malloc(sizeof(int)*n_ent);
	m->face_lf = malloc(sizeof(int)*n_ent);
	int* face_of = malloc(sizeof(int)*n_ent);
	if (!fe || !m->face_vol || !m->face_lf || !face_of) { free(fe); free(face_of); free(vid); dpg_mesh_free(m); return DPG_ERR_INVALID; }
	for (int v = 0; v < n_vol; ++v)
		for (int lf = 0; lf < n_fl; ++lf) {
			struct face_entry* e = &fe[(size_t)v*n_fl + lf];
			const int* a = &vid[(v*3 + fve[lf][0])*2];
			const int* b = &vid[(v*3 + fve[lf][1])*2];
			e->key[0] = (a[0] + b[0]) % (2*nx); e->key[1] = (a[1] + b[1]) % (2*ny); e->key[2] = e->key[3] = -1;
			e->vol = v; e->lf = lf;
		}
	free(vid);
	qsort(fe,n_ent,sizeof *fe,cmp_face);   /* equal keys adjacent, then by (volume, local face) */
	for (size_t q = 0; q < n_ent; ++q) face_of[q] = -1;
	int* partner = malloc(sizeof(int)*n_ent);
	if (!partner) { free(fe); free(face_of); dpg_mesh_free(m); return DPG_ERR_INVALID; }
	for (size_t q = 0; q < n_ent; ++q) partner[q] = -1;
	for (size_t i = 0; i < n_ent;) {
		size_t j = i + 1;
		while (j < n_ent && cmp_key(&fe[i],&fe[j]) == 0) ++j;
		if (j - i != 2) { free(fe); free(face_of); free(partner); dpg_mesh_free(m); return DPG_ERR_INVALID; }
		const size_t ea = (size_t)fe[i].vol*n_fl + fe[i].lf, eb = (size_t)fe[i+1].vol*n_fl + fe[i+1].lf;
		partner[ea] = (int)eb; partner[eb] = (int)ea;
		i = j;
	}
	free(fe);
	int nf = 0;
	for (size_t e = 0; e < n_ent; ++e) {
		if (partner[e] < 0 || (size_t)partner[e] < e) continue;
		m->face_vol[2*nf] = (int)(e / n_fl);                m->face_lf[2*nf] = (int)(e % n_fl);
		m->face_vol[2*nf+1] = (int)(partner[e] / n_fl);     m->face_lf[2*nf+1] = (int)(partner[e] % n_fl);
		++nf;
	}
	free(partner); free(face_of);
	m->n_face = nf;
	m->geom = DPG_GEOM_STRAIGHT;
	return DPG_OK;
}

/* Periodic box of nx x ny x nz cells, each split into six tetrahedra (the Kuhn split along the cell diagonal from
 * corner (0,0,0) to (1,1,1)): for the permutations pi of the axes, in the order (0,1,2), (0,2,1), (1,0,2), (1,2,0),
 * (2,0,1), (2,1,0), the vertices (0,0,0), e_pi0, e_pi0 + e_pi1, (1,1,1) of the cell, the first two swapped where
 * that makes the map's determinant positive (odd permutations); volume 6 (i + nx (j + ny k)) + t.  Vertices jittered
 * by the box's seeded draws of their periodic image (3 per grid point, in grid-point order).  Faces are matched by
 * their centroid in tripled grid units modulo the box; side 0 is the first (volume, local face) of a face. */
int dpg_mesh_tet_structured(const struct dpg_sim_params* prm, struct dpg_mesh* m)
{
	memset(m,0,sizeof *m);
	if (prm->d != 3) return DPG_ERR_UNSUPPORTED;
	const int nx = prm->n_elem[0], ny = prm->n_elem[1], nz = prm->n_elem[2], n_fl = 4;
	if (nx < 1 || ny < 1 || nz < 1) return DPG_ERR_INVALID;
	const int n_vol = 6*nx*ny*nz;
	m->d = 3; m->n_vol = n_vol;
	for (int a = 0; a < 3; ++a) { m->lo[a] = prm->lo[a]; m->hi[a] = prm->hi[a]; }
	m->xyz_ve = calloc((size_t)n_vol*DPG_NVE_MAX*3,sizeof(double));
	double* jit = calloc((size_t)nx*ny*nz*3,sizeof(double));
	int* gv = malloc(sizeof(int)*(size_t)n_vol*4*3);          /* unwrapped grid coordinates of each vertex */
	if (!m->xyz_ve || !jit || !gv) { free(jit); free(gv); dpg_mesh_free(m); return DPG_ERR_INVALID; }
	const double h[3] = {(prm->hi[0] - prm->lo[0])/nx, (prm->hi[1] - prm->lo[1])/ny, (prm->hi[2] - prm->lo[2])/nz};
	if (prm->jitter > 0.0) {
		uint64_t st = prm->seed*0x2545F4914F6CDD1Dull + 1;
		for (size_t q = 0; q < (size_t)nx*ny*nz; ++q)
			for (int a = 0; a < 3; ++a) jit[q*3+a] = prm->jitter*h[a]*(2.0*urand(&st) - 1.0);
	}
	static const int perm[6][3] = {{0,1,2}, {0,2,1}, {1,0,2}, {1,2,0}, {2,0,1}, {2,1,0}};
	static const int odd[6] = {0, 1, 1, 0, 0, 1};
	for (int k = 0; k < nz; ++k)
		for (int j = 0; j < ny; ++j)
			for (int i = 0; i < nx; ++i)
				for (int t = 0; t < 6; ++t) {
					const int v = 6*(i + nx*(j + ny*k)) + t;
					int c[4][3] = {{0,0,0}, {0,0,0}, {0,0,0}, {1,1,1}};
					c[1][perm[t][0]] = 1;
					c[2][perm[t][0]] = 1; c[2][perm[t][1]] = 1;
					if (odd[t]) for (int a = 0; a < 3; ++a) { const int tmp = c[0][a]; c[0][a] = c[1][a]; c[1][a] = tmp; }
					for (int kv = 0; kv < 4; ++kv) {
						const int g[3] = {i + c[kv][0], j + c[kv][1], k + c[kv][2]};
						const size_t q = (size_t)(g[0] % nx) + (size_t)nx*((g[1] % ny) + (size_t)ny*(g[2] % nz));
						double* x = &m->xyz_ve[((size_t)v*DPG_NVE_MAX + kv)*3];
						for (int a = 0; a < 3; ++a) {
							gv[(v*4 + kv)*3 + a] = g[a];
							x[a] = prm->lo[a] + g[a]*h[a] + jit[q*3 + a];
						}
					}
				}
	free(jit);
	static const int fve[4][3] = {{2,3,1}, {2,3,0}, {0,1,3}, {0,1,2}};
	const size_t n_ent = (size_t)n_vol*n_fl;
	struct face_entry* fe = malloc(sizeof *fe*n_ent);
	int* partner = malloc(sizeof(int)*n_ent);
	m->face_vol = malloc(sizeof(int)*n_ent);
	m->face_lf = malloc(sizeof(int)*n_ent);
	if (!fe || !partner || !m->face_vol || !m->face_lf) { free(fe); free(partner); free(gv); dpg_mesh_free(m); return DPG_ERR_INVALID; }
	const int nn[3] = {nx, ny, nz};
	for (int v = 0; v < n_vol; ++v)
		for (int lf = 0; lf < n_fl; ++lf) {
			struct face_entry* e = &fe[(size_t)v*n_fl + lf];
			for (int a = 0; a < 3; ++a) {
				int s3 = 0;
				for (int kv = 0; kv < 3; ++kv) s3 += gv[(v*4 + fve[lf][kv])*3 + a];
				e->key[a] = s3 % (3*nn[a]);
			}
			e->key[3] = -1;
			e->vol = v; e->lf = lf;
		}
	free(gv);
	qsort(fe,n_ent,sizeof *fe,cmp_face);
	for (size_t q = 0; q < n_ent; ++q) partner[q] = -1;
	for (size_t i = 0; i < n_ent;) {
		size_t j = i + 1;
		while (j < n_ent && cmp_key(&fe[i],&fe[j]) == 0) ++j;
		if (j - i != 2) { free(fe); free(partner); dpg_mesh_free(m); return DPG_ERR_INVALID; }
		const size_t ea = (size_t)fe[i].vol*n_fl + fe[i].lf, eb = (size_t)fe[i+1].vol*n_fl + fe[i+1].lf;
		partner[ea] = (int)eb; partner[eb] = (int)ea;
		i = j;
	}
	free(fe);
	int nf = 0;
	for (size_t e = 0; e < n_ent; ++e) {
		if (partner[e] < 0 || (size_t)partner[e] < e) continue;
		m->face_vol[2*nf] = (int)(e / n_fl);                m->face_lf[2*nf] = (int)(e % n_fl);
		m->face_vol[2*nf+1] = (int)(partner[e] / n_fl);     m->face_lf[2*nf+1] = (int)(partner[e] % n_fl);
		++nf;
	}
	free(partner);
	m->n_face = nf;
	m->geom = DPG_GEOM_STRAIGHT;
	return DPG_OK;
}
