/* Internal declarations shared by the host-side setup files (nodes, bases, element operators, mesh, geometry,
 * initial solutions).  The public entry points are declared in include/dpg_gb300.h. */
#ifndef DPG_HOST_H
#define DPG_HOST_H

#include <stddef.h>
#include <stdint.h>
#include "dpg_simulation.h"

#ifdef __cplusplus
extern "C" {
#endif

/* nodes + bases (element.c) */
void dpg_nodes_gl (int n, double* x, double* w);
void dpg_nodes_gll(int n, double* x, double* w);
void dpg_nodes_gj10(int n, double* x, double* w);   /* Gauss-Jacobi, weight (1 - x) */
void dpg_nodes_gj(int alpha, int n, double* x, double* w);   /* Gauss-Jacobi, weight (1 - x)^alpha */
void dpg_lagrange_1d(int n, const double* xn, double x, double* val, double* der);
/* tensor-product Lagrange basis on the 1D nodes g (n1 per direction) and its gradient [d][n_s] at r */
void dpg_tp_basis_at(int d, int n1, const double* g, const double* r, double* val, double* grad);
void dpg_kron_rowmajor(int ra, int ca, const double* a, int rb, int cb, const double* b, double* out);
int  dpg_element_ops_build(int e_type, int p, struct dpg_element_ops* ops);
/* TRI (element_tri.c): the operators of order p, and the barycentric P1 basis (v0, v1, v2) with its gradient [2][3] */
int  dpg_element_ops_build_tri(int p, struct dpg_element_ops* ops);
void dpg_tri_p1_at(const double* r, double* val, double* grad);
/* the order-p TRI Lagrange basis of the nodes rst_vs at n_pt points pts[n_pt][2]: out[n_pt][n_s] */
int  dpg_tri_lagrange_at(int p, const double* rst_vs, int n_pt, const double* pts, double* out);
/* TET (element_tet.c): the operators of order p (1..4), the barycentric P1 basis with its gradient [3][4], and the
 * order-p Lagrange basis of the nodes rst_vs at n_pt points pts[n_pt][3]: out[n_pt][n_s] */
int  dpg_element_ops_build_tet(int p, struct dpg_element_ops* ops);
void dpg_tet_p1_at(const double* r, double* val, double* grad);
int  dpg_tet_lagrange_at(int p, const double* rst_vs, int n_pt, const double* pts, double* out);
/* mixed orders: ov's basis at the face cubature of the higher-order operators of (ov->cv0_vs_fcp[of->p], ...) */
int  dpg_element_face_ops_build(struct dpg_element_ops* ov, const struct dpg_element_ops* of);
void dpg_element_ops_free(struct dpg_element_ops* ops);

/* dense linear algebra (linalg.c) */
int  dpg_lu_factor(int n, double* a, int* piv);
void dpg_lu_solve (int n, const double* lu, const int* piv, double* b);
int  dpg_invert   (int n, const double* a, double* a_inv);
int  dpg_simplex_bezier_ops(struct dpg_element_ops* ops, const double (*V)[3]);
void dpg_matmul   (int m, int n, int k, double alpha, const double* a, const double* b, double beta, double* c);

/* mesh sources (mesh_gmsh.c): volume vertices in tensor-product order and the two (volume, local face) sides of
 * every face */
struct dpg_sim_params;
struct dpg_mesh {
	int d, n_vol, n_face;
	double* xyz_ve;      /* [n_vol][DPG_NVE_MAX][3]                          */
	int* face_vol;       /* [n_face][2] volume of side 0 / side 1            */
	int* face_lf;        /* [n_face][2] local face of side 0 / side 1        */
	int* face_bc;        /* [n_face] BC code of a boundary face (side 1 = -1), else 0; may be NULL */
	double lo[3], hi[3]; /* bounding box (its extents: the periodic lengths; 0: not periodic) */
	int geom;            /* DPG_GEOM_*: for DPG_GEOM_CYLINDER xyz_ve hold (r, theta) */
	int* vol_p;          /* [n_vol] given volume orders, or NULL (prm->p, or draws from p .. p_max) */
};
uint64_t dpg_splitmix64(uint64_t* state);
int  dpg_mesh_structured(const struct dpg_sim_params* prm, struct dpg_mesh* m);
int  dpg_mesh_annulus(const struct dpg_sim_params* prm, struct dpg_mesh* m);
int  dpg_mesh_tri_structured(const struct dpg_sim_params* prm, struct dpg_mesh* m);
int  dpg_mesh_tet_structured(const struct dpg_sim_params* prm, struct dpg_mesh* m);
/* gmsh 2.2 ASCII mesh of QUADs / HEXs (e_type DPG_QUAD / DPG_HEX), TRIs (DPG_TRI) or TETs (DPG_TET); DPG_OK or a
 * DPG_ERR_* status */
int  dpg_mesh_read_gmsh(const char* path, int d, int e_type, struct dpg_mesh* m);
void dpg_mesh_free(struct dpg_mesh* m);

/* restart files (restart.c): the inverse of a tensor-product volume's multilinear map, vertices x[2^d][3] */
int  dpg_p1_inverse_map(int d, const double (*x)[3], const double* y, double* r);

/* geometry (geometry.c) */
int  dpg_setup_geometry(struct dpg_sim* sim);
int  dpg_setup_mass_inverse(struct dpg_sim* sim);

/* initial / exact solutions (solution.c) */
void dpg_exact_solution(const struct dpg_sim* sim, double t, const double* xyz, double* u);
void dpg_set_initial_solution(struct dpg_sim* sim);

#ifdef __cplusplus
}
#endif
#endif
