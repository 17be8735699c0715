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
 * hexahedra in 3D; points, lines (2D) and boundary quadrilaterals (3D) are read past.  Interior faces are paired
 * by the vertex sets of the volumes' local faces; a boundary face must consist of $Periodic nodes and is paired with
 * its periodic image across the box (the domain of this path: an axis-aligned box, periodic in every direction).
 * A face with no partner carries a boundary condition, which this path does not provide (DPG_ERR_UNSUPPORTED), as
 * do other element types (mixed or curved meshes).
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
	free(m->xyz_ve); free(m->face_vol); free(m->face_lf);
	memset(m,0,sizeof *m);
}

/* ---- structured periodic box ---------------------------------------------------------------------------- */

/* splitmix64: seeded uniform numbers for the vertex jitter */
static uint64_t sm64(uint64_t* s)
{
	uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}
static double urand(uint64_t* s) { return (double)(sm64(s) >> 11) * (1.0/9007199254740992.0); }

int dpg_mesh_structured(const struct dpg_sim_params* prm, struct dpg_mesh* m)
{
	memset(m,0,sizeof *m);
	const int d = prm->d;
	const int nx = prm->n_elem[0], ny = prm->n_elem[1], nz = (d == 3 ? prm->n_elem[2] : 1);
	const int n_vol = nx*ny*nz, n_face = d*n_vol;
	m->d = d; m->n_vol = n_vol; m->n_face = n_face;
	for (int a = 0; a < 3; ++a) { m->lo[a] = prm->lo[a]; m->hi[a] = prm->hi[a]; }
	m->xyz_ve = calloc((size_t)n_vol*DPG_NVE_MAX*3,sizeof(double));
	m->face_vol = calloc((size_t)2*n_face,sizeof(int));
	m->face_lf = calloc((size_t)2*n_face,sizeof(int));
	/* vertex grid with periodic-consistent jitter: vertex (i,j,k), i in [0,nx], is the image of (i mod nx, ...) */
	const int nvx = nx, nvy = ny, nvz = nz;
	double* jit = calloc((size_t)nvx*nvy*nvz*3,sizeof(double));
	if (!m->xyz_ve || !m->face_vol || !m->face_lf || !jit) { free(jit); dpg_mesh_free(m); return DPG_ERR_INVALID; }
	double h[3];
	for (int a = 0; a < 3; ++a) h[a] = (a < d ? (prm->hi[a]-prm->lo[a])/prm->n_elem[a] : 0.0);
	if (prm->jitter > 0.0) {
		uint64_t st = prm->seed*0x2545F4914F6CDD1Dull + 1;
		for (size_t q = 0; q < (size_t)nvx*nvy*nvz; ++q)
			for (int a = 0; a < d; ++a)
				jit[q*3+a] = prm->jitter*h[a]*(2.0*urand(&st) - 1.0);
	}
	for (int k = 0; k < nz; ++k)
	for (int j = 0; j < ny; ++j)
	for (int i = 0; i < nx; ++i) {
		const int v = i + nx*(j + ny*k);
		for (int kv = 0; kv < (1 << d); ++kv) {
			const int bi = kv & 1, bj = (kv >> 1) & 1, bk = (kv >> 2) & 1;
			const int gi = i+bi, gj = j+bj, gk = k+bk;
			const size_t q = (size_t)(gi % nvx) + (size_t)nvx*((gj % nvy) + (size_t)nvy*(d == 3 ? gk % nvz : 0));
			double* x = &m->xyz_ve[((size_t)v*DPG_NVE_MAX + kv)*3];
			x[0] = prm->lo[0] + gi*h[0] + jit[q*3+0];
			x[1] = prm->lo[1] + gj*h[1] + jit[q*3+1];
			x[2] = (d == 3 ? prm->lo[2] + gk*h[2] + jit[q*3+2] : 0.0);
		}
		/* face f = d v + a joins the +a face of v with the -a face of its periodic neighbour nb.  Side 0
		 * (neigh_info[0]) is the smaller (volume, local face), as in the reference, whose constructor_Faces
		 * (computational_elements/face.c:108-148) creates each face from the first volume that reaches it: v for an
		 * interior face, nb across the periodic seam (and the -a face when the volume is its own neighbour).  The
		 * side matters: the Roe-Pike flux with its entropy fix is not antisymmetric in the two states. */
		for (int a = 0; a < d; ++a) {
			const int ii = (a == 0 ? (i+1) % nx : i), jj = (a == 1 ? (j+1) % ny : j), kk = (a == 2 ? (k+1) % nz : k);
			const int f = d*v + a, nb = ii + nx*(jj + ny*kk);
			const int s0 = (nb > v ? 0 : 1);
			m->face_vol[2*f + s0] = v;        m->face_lf[2*f + s0] = 2*a+1;
			m->face_vol[2*f + 1-s0] = nb;     m->face_lf[2*f + 1-s0] = 2*a;
		}
	}
	free(jit);
	return DPG_OK;
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

int dpg_mesh_read_gmsh(const char* path, int d, struct dpg_mesh* m)
{
	memset(m,0,sizeof *m);
	if (d != 2 && d != 3) return DPG_ERR_INVALID;
	FILE* fp = fopen(path,"r");
	if (!fp) return DPG_ERR_IO;
	const int vol_type = (d == 2 ? 3 : 5), n_ve = 1 << d;   /* gmsh: 3 = 4-node quadrilateral, 5 = 8-node hexahedron */
	int rc = DPG_OK;
	int n_nodes = 0, max_id = 0, n_vol = 0, vol_cap = 0, n_pairs = 0, pair_cap = 0;
	int* node_id = NULL;          /* [n_nodes] gmsh node numbers                  */
	double* node_x = NULL;        /* [n_nodes][3]                                 */
	int* vol_nodes = NULL;        /* [n_vol][n_ve] gmsh node numbers, gmsh order  */
	int* pairs = NULL;            /* [n_pairs][2] (slave, master) gmsh numbers    */
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
				} else if (type == 15 || type == 1 || (d == 3 && type == 3)) {
					/* points, boundary lines (2D), boundary quadrilaterals (3D): their faces are found from the volumes */
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

	m->d = d; m->n_vol = n_vol;
	m->xyz_ve = calloc((size_t)n_vol*DPG_NVE_MAX*3,sizeof(double));
	int* vidx = malloc(sizeof(int)*(size_t)n_vol*n_ve);   /* node indices in tensor-product order */
	if (!m->xyz_ve || !vidx) { free(vidx); rc = DPG_ERR_INVALID; goto done; }
	static const int tp_of_gmsh_quad[4] = {0,1,3,2}, tp_of_gmsh_hex[8] = {0,1,3,2,4,5,7,6};
	const int* perm = (d == 2 ? tp_of_gmsh_quad : tp_of_gmsh_hex);
	for (int v = 0; v < n_vol; ++v) {
		int* vi = &vidx[(size_t)v*n_ve];
		for (int k = 0; k < n_ve; ++k) {
			const int id = vol_nodes[(size_t)v*n_ve + perm[k]];
			if (id < 1 || id > max_id || index[id] < 0) { free(vidx); rc = DPG_ERR_IO; goto done; }
			vi[k] = index[id];
		}
		/* right-handed tensor-product map: det[x_1 - x_0, x_2 - x_0 (, x_4 - x_0)] > 0, else mirror the last direction */
		const double* x0 = &node_x[3*vi[0]];
		double e[3][3];
		for (int a = 0; a < d; ++a)
			for (int i = 0; i < 3; ++i) e[a][i] = node_x[3*vi[1 << a] + i] - x0[i];
		const double det = (d == 2 ? e[0][0]*e[1][1] - e[0][1]*e[1][0]
		                           : e[0][0]*(e[1][1]*e[2][2] - e[1][2]*e[2][1]) - e[0][1]*(e[1][0]*e[2][2] - e[1][2]*e[2][0])
		                             + e[0][2]*(e[1][0]*e[2][1] - e[1][1]*e[2][0]));
		if (!(det != 0.0)) { free(vidx); rc = DPG_ERR_INVALID; goto done; }
		if (det < 0.0) {
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
	const int n_fl = 2*d, nvf = n_ve/2;
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
			for (int k = 0; k < n_ve; ++k)
				if (((k >> a) & 1) == side) f->key[c++] = vidx[(size_t)v*n_ve + k];
			for (; c < 4; ++c) f->key[c] = -1;
			qsort(f->key,(size_t)nvf,sizeof(int),cmp_int);
			f->vol = v; f->lf = lf;
		}
	qsort(fe,n_ent,sizeof *fe,cmp_face);
	m->face_vol = malloc(sizeof(int)*n_ent);
	m->face_lf = malloc(sizeof(int)*n_ent);
	struct face_entry* bf = malloc(sizeof *bf*n_ent);
	if (!m->face_vol || !m->face_lf || !bf) { free(vidx); free(periodic_node); free(bf); rc = DPG_ERR_INVALID; goto done; }
	int nf = 0;
	size_t nb = 0;
	for (size_t i = 0; i < n_ent;) {
		size_t j = i + 1;
		while (j < n_ent && cmp_key(&fe[i],&fe[j]) == 0) ++j;
		if (j - i == 2) {
			m->face_vol[2*nf] = fe[i].vol;   m->face_lf[2*nf] = fe[i].lf;
			m->face_vol[2*nf+1] = fe[i+1].vol; m->face_lf[2*nf+1] = fe[i+1].lf;
			++nf;
		} else if (j - i == 1) {
			for (int c = 0; c < nvf; ++c)
				if (!periodic_node[fe[i].key[c]]) { free(vidx); free(periodic_node); free(bf); rc = DPG_ERR_UNSUPPORTED; goto done; }
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
			free(vidx); free(periodic_node); free(bf); rc = DPG_ERR_INVALID; goto done;   /* > 2 volumes on a face */
		}
		i = j;
	}
	free(periodic_node);
	free(vidx);
	qsort(bf,nb,sizeof *bf,cmp_face);
	for (size_t i = 0; i < nb; i += 2) {
		if (i + 1 >= nb || cmp_key(&bf[i],&bf[i+1]) != 0 || (i + 2 < nb && cmp_key(&bf[i+1],&bf[i+2]) == 0)) {
			free(bf); rc = DPG_ERR_UNSUPPORTED; goto done;   /* a boundary face without a periodic image */
		}
		m->face_vol[2*nf] = bf[i].vol;   m->face_lf[2*nf] = bf[i].lf;
		m->face_vol[2*nf+1] = bf[i+1].vol; m->face_lf[2*nf+1] = bf[i+1].lf;
		++nf;
	}
	free(bf);
	m->n_face = nf;
done:
	fclose(fp);
	free(node_id); free(node_x); free(vol_nodes); free(pairs); free(index); free(fe);
	if (rc != DPG_OK) dpg_mesh_free(m);
	return rc;
}
