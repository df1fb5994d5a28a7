/*
 * hp3d_oracle.h -- CPU FP64 restatement of the hp3D element pass.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it to
 * produce reference answers.  The product (libhp3dg, include/hp3dg.h) never
 * links, loads or calls it.
 *
 * Every routine restates a routine of Oden-EAG/hp3d (paths relative to the
 * project's trunk/), cited beside its declaration.  Arrays follow the Fortran
 * conventions of the reference: matrices are column-major with an explicit
 * leading dimension, GradH-style arrays are (3, k) with the component index
 * fastest, and all integer tables are 0-based in C where the reference is
 * 1-based (noted per argument).
 *
 * Parity pin: the reference ships no element-level golden vectors (its tests
 * pin results only end-to-end through MUMPS).  The restatement is pinned by
 * restating those end-to-end tests (test/poly_pois.F90, test/conv_pois.F90)
 * plus the reference's own debug self-checks (monomial integration,
 * set_3D_int.F90:407-457) in tests/test_oracle_*.py.
 */
#ifndef HP3D_ORACLE_H
#define HP3D_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* element types (data_structure3D node types MDLB/MDLP/MDLN) */
#define ORC_HEXA  1
#define ORC_PRISM 2
#define ORC_TET   3

#define ORC_MAXP 6          /* parameters.F90:17 */
#define ORC_MAX_NINT3 392   /* parameters.F90 MAX_NINT3 = (MAXP+1)**2*(MAXP+2) */
#define ORC_MAXBRICKH 343   /* (MAXP+1)**3 */

/* 1D Gauss-Legendre rule with n points rescaled to [0,1]
 * (gauss_quadrature.F90:518-660 tables, rescale 749-750). */
int orc_gauss1d(int n, double *x, double *w);

/* set_3D_int for a hexahedron (set_3D_int.F90:47-64 + find_order_loc
 * find_order.F90:68-108 + set_3Dint_aux BRICK branch 155-245).
 * norder: Norder(19); nori_face: Norient_face(6); returns nint. */
int orc_set_3D_int_hexa(const int32_t *norder, const int32_t *nori_face,
                        int integration, double *xiloc, double *waloc);

/* set_3D_int for a tetrahedron (Duffy-collapsed Gauss rule,
 * gauss_quadrature.F90 tet section + set_3Dint_aux TETRA branch). */
int orc_set_3D_int_tet(const int32_t *norder, int integration,
                       double *xiloc, double *waloc);

/* celndof H1 count for a hexa / tet (celndof.F90:24-149). */
int orc_nrdofH_hexa(const int32_t *norder);
int orc_nrdofH_tet(const int32_t *norder);
/* number of interior (bubble) H1 dof (ndof_nod, element_data.F90:808-884) */
int orc_nrdofH_bubble(int etype, const int32_t *norder);

/* shape3DHHexa (Hexahedron.F90:33-210): values and gradients (3,k). */
int orc_shape3DH_hexa(const double *xi, const int32_t *nord,
                      const int32_t *nori_edge, const int32_t *nori_face,
                      double *shap, double *grad);

/* shape3DHTet (Tetrahedron.F90:33-234). */
int orc_shape3DH_tet(const double *xi, const int32_t *nord,
                     const int32_t *nori_edge, const int32_t *nori_face,
                     double *shap, double *grad);

/* Prism: celndof count, set_3D_int (triangle rule x Gauss, set_3D_int.F90:
 * 264-300 on find_order_loc orders) and shape3DHPris (Prism.F90:33-330). */
int orc_nrdofH_prism(const int32_t *norder);
int orc_set_3D_int_prism(const int32_t *norder, const int32_t *nori_face, int integration,
                         double *xiloc, double *waloc);
int orc_shape3DH_prism(const double *xi, const int32_t *nord,
                       const int32_t *nori_edge, const int32_t *nori_face,
                       double *shap, double *grad);

/* geom (geom.F90:30-138): det and cofactor inverse; returns Iflag. */
int orc_geom(const double *dxdxi, double *dxidx, double *rjac);

/* source term f = -Laplace(u) of the manufactured solution
 * (common/getf.F90:63, common/solution.F90:45-134).  isol 0,1,2 are the
 * reference's cases; 10 = sin(pi x)sin(pi y)sin(pi z), 11 = f==1,
 * 12 = u = x*y*z (test/poly_pois.F90:390-395), 13 = u = 1 + x + 2y + 3z. */
double orc_getf(int isol, const double *x);
/* exact solution value and gradient (for error evaluation) */
void orc_exact(int isol, const double *x, double *u, double *gradu);

/* elem_opt (problems/POISSON/GALERKIN/elem_opt.F90:22-141) extended with a
 * per-element coefficient kappa (K = kappa * A_TEST A_TEST^T).
 * xnod: (3, nrdofH) geometry dof.  Writes zaloc (ld x n, column-major,
 * both triangles) and zbloc (n).  Returns 0, or 1 for a negative Jacobian.
 * variant 0 = BLAS-3 form (DSYRK), 1 = scalar elem_poisson form
 * (elem.F90:78-250). */
int orc_elem(int etype, const int32_t *norder, const int32_t *nori_edge,
             const int32_t *nori_face, const double *xnod, double kappa,
             int isol, int integration, int variant,
             double *zaloc, int ld, double *zbloc);

/* stc_fwd_gen (stc.F90:443-509): LU with partial pivoting of the bubble
 * block; A (n x n, ld) holds the element matrix with interface dof first.
 * Outputs Aii (ni x ni, ld ni), Bi (ni), ASchur = inv(Abb) Abi (nb x ni,
 * ld nb), BSchur = inv(Abb) Bb (nb).  method 0 = LU (stc_fwd_gen),
 * 1 = Cholesky (stc_fwd_herm, stc.F90:338-416).  Returns 0 or -1 on a zero
 * pivot / non-positive Cholesky pivot. */
/* Optional optimised BLAS-3 / LAPACK routines (Fortran calling convention):
 * DSYRK for elem_opt.F90:131 and DGETRF / DGETRS / DGEMM for stc.F90:462-507.
 * NULL pointers restore the oracle's own loops. */
void orc_set_blas(void *dsyrk, void *dgetrf, void *dgetrs, void *dgemm);
int orc_blas_active(void);

int orc_stc_fwd(int ni, int nb, const double *a, int lda, const double *b,
                int method, double *aii, double *bi, double *aschur,
                double *bschur);

/* stc_bwd (stc.F90:661-679): xb = BSchur - ASchur xi. */
void orc_stc_bwd(int ni, int nb, const double *aschur, const double *bschur,
                 const double *xi, double *xb);

/* Per-node H1 dof counts of an element in element node order
 * (vertices, edges, faces; ndof_nod).  Returns number of nodes (26 hexa,
 * 14 tet). */
int orc_node_ndof(int etype, const int32_t *norder, int32_t *ndof);

/* celem_systemI extraction + Dirichlet lift + compression
 * (celem_systemI.F90:290-510, 812-845) for a conforming element (identity
 * constraints, logic.F90 active-node branch).
 * aii (ni x ni, ld ni) and bi: condensed system in element dof order;
 * bcflag: per element node (26 hexa) 1 = Dirichlet; zdofd: per interface
 * dof Dirichlet value (may be NULL = homogeneous).
 * Outputs nextract (0-based interface index per compressed dof), zbload
 * (nrdofc), zastif (nrdofc^2 row-major, ISYM_FLAG=2), ndofm (per node
 * number of active dof).  Returns nrdofc. */
int orc_celem_compress(int etype, const int32_t *norder, const int32_t *bcflag,
                       const double *aii, const double *bi,
                       const double *zdofd, int32_t *nextract, double *zbload,
                       double *zastif, int32_t *ndofm);

/* The same over an arbitrary node list (the modified element nodes of a
 * constrained element): nn nodes with nd dof each (modified dof numbered node
 * by node, forward), bcflag per node. */
int orc_celem_compress_nodes(int nn, const int32_t *nd, const int32_t *bcflag,
                             const double *aii, const double *bi, const double *zdofd,
                             int32_t *nextract, double *zbload, double *zastif,
                             int32_t *ndofm);

/* Constraint transform of the condensed element system (celem_systemI.F90:
 * 541-760, CONTIN branch): amod = C^T aii C, bmod = C^T bi with the
 * coefficients of logic (constrs/logic.F90) given as triplets (element
 * interface dof k, modified dof l, coefficient), in the reference's loop
 * order (k, then its connected dof).  aii ni x ni and amod nmod x nmod,
 * column-major.  Returns 0, or <0 for an index out of range. */
int orc_constrain(int ni, const double *aii, const double *bi, int ncoef, const int32_t *ck,
                  const int32_t *cl, const double *cv, int nmod, double *amod, double *bmod);

/* update_Ddof for one hexahedron whose geometry block is the element itself
 * (eta = xi; x(eta) trilinear in the vertices): Dirichlet values of the
 * nodes with bcflag set, per interface dof in element order (zeros
 * elsewhere) -- vertex values (dhpvert.F90), then the tangential
 * H1-seminorm projections on edges (edge/dhpedgeH.F90) and faces
 * (face/dhpfaceH.F90) of what the lower-order part leaves.  Returns the
 * number of interface dof, or -1. */
int orc_dirichlet_hexa(const int32_t *norder, const int32_t *nori_edge, const int32_t *nori_face,
                       const double *xvert, const int32_t *bcflag, int isol, double *zd);

/* update_gdof for one hexahedron (update_gdof.F90:80-200 and 404-435,
 * hpvert.F90, hpedge.F90, hpface.F90, hpmdle.F90): its geometry dof xnod
 * (nrdofH x 3, row-major, element dof order) from the geometry block's map
 * x(eta), evaluated by gmap at block coordinates eta (x and dxdeta row-major,
 * dxdeta[3 i + j] = d x_i / d eta_j).  etav: the element's 8 vertices in the
 * block's coordinates (refel); eta(xi) is trilinear in them.  Vertex dof are
 * x at the vertices; edge, face and interior dof are the eta-space H1
 * projections (tangential, surface, full gradient) of x minus the lower-order
 * part, with the quadrature of set_1Dint / set_2Dint / set_3Dint at
 * INTEGRATION = integration.  linear != 0: vertices only (a 'Linear' block).
 * Returns nrdofH, or -1 for a singular projection. */
typedef void (*orc_gmap_fn)(const double *eta, double *x, double *dxdeta, void *user);
int orc_gdof_hexa(const int32_t *norder, const int32_t *nori_edge, const int32_t *nori_face,
                  const double *etav, int integration, orc_gmap_fn gmap, void *user, int linear,
                  double *xnod);

/* mumps_sc STEP 1 offsets + STEP 2 connectivities
 * (solver/omp_mumps/mumps_sc.F90:102-188, 266-299).
 * nodes: nelem x nnode_max global node ids (element node order),
 * ndofm: nelem x nnode_max active dof counts, nnode: nodes per element.
 * Outputs nfirst_dof (nnodes_global, -1 for unvisited), lcon (concatenated
 * per element, 1-based global dof as in the reference), lcon_off (nelem+1),
 * elem_nnz (nelem+1, int64 prefix of nrdofc^2).  Returns total nrdof. */
int64_t orc_index_maps(int nelem, int nnode_max, const int32_t *nnode,
                       const int32_t *nodes, const int32_t *ndofm,
                       int nnodes_global, int32_t *nfirst_dof, int32_t *lcon,
                       int64_t *lcon_off, int64_t *elem_nnz);

/* element_error (compute_error.F90:226-360): squared H1 error / norm. */
int orc_element_error(int etype, const int32_t *norder, const int32_t *nori_edge,
                      const int32_t *nori_face, const double *xnod, const double *dof,
                      int isol, double *err2, double *norm2);

/* Whole element pass over a batch of elements (OpenMP over elements):
 * elem -> stc_fwd -> celem compression.  Descriptor arrays are per element:
 * etype[e], norder[e*19], nori_edge[e*12], nori_face[e*6], bcflag[e*26],
 * xvert[e*3*8] vertex coordinates (trilinear/linear geometry, higher-order
 * geometry dof zero), kappa[e].  Output offsets follow the compressed sizes:
 * zastif at elem_nnz[e], zbload/nextract at lcon_off[e]; aschur/bschur at
 * schur_off[e] (nb*ni) / bub_off[e] (nb).  Pass NULL for outputs not wanted.
 * nthreads <= 0 means all cores.  Returns 0, or 1+e of the first element
 * with a negative Jacobian / failed factorisation. */
int orc_element_pass(int nelem, const int32_t *etype, const int32_t *norder,
                     const int32_t *nori_edge, const int32_t *nori_face,
                     const int32_t *bcflag, const double *xvert,
                     const double *kappa, int isol, int integration,
                     int stc_method, int nthreads,
                     const int64_t *elem_nnz, const int64_t *lcon_off,
                     const int64_t *schur_off, const int64_t *bub_off,
                     double *zastif, double *zbload, double *aschur,
                     double *bschur);

/* ------------------------------------------------------------------------ */
/* Ultraweak DPG Maxwell on hexahedra (problems/MAXWELL/ULTRAWEAK_DPG),       */
/* hp3d_oracle_dpg.c.  Complex arrays are interleaved (re, im) doubles.       */
/* ------------------------------------------------------------------------ */

/* commonParam.F90 / set_environment.F90: OMEGA, MU, EPSILON, GAMMA,
 * ALPHA_NORM, IBCFLAG (0 Dirichlet, 2 impedance by penalty), NORD_ADD,
 * ISOL (mfd_solutions cases 0-2) and ICOMP_EXACT (1-based component of E). */
typedef struct {
  double omega, mu, epsilon, gamma, alpha;
  int32_t ibcflag, nord_add, isol, icomp;
} orc_maxw_params;

/* H(curl) count of shape3DEHexa for Norder (celndof E branch) */
int orc_nrdofE_hexa(const int32_t *norder);
/* shape3DEHexa (Hexahedron.F90:240-440): values and curls (3,k) */
int orc_shape3DE_hexa(const double *xi, const int32_t *nord, const int32_t *nori_edge,
                      const int32_t *nori_face, double *shapE, double *curlE);
/* shape3DQHexa (Hexahedron.F90:640-698) */
int orc_shape3DQ_hexa(const double *xi, const int32_t *nord, double *shapQ);
/* shape3EE for a brick -> shape3DEBrokenHexa (BrokenHexahedron.F90:139-258);
 * nordP = the enriched middle-node order code (e.g. 444) */
int orc_shape3EE_hexa(const double *xi, int nordP, double *shapE, double *curlE);
/* set_2D_int(_DPG) of a quad face (set_2D_int.F90:72-247): norderf = face_order
 * (4 edge orders + face code), maxp = MAXP (6) or MAXPP (7) */
int orc_set_2D_int_quad(const int32_t *norderf, int nori, int integration, int maxp,
                        double *tloc, double *wtloc);
/* exact E, H and source J of mfd_solutions case isol (exact.F90, getf.F90);
 * eps = EPSILON * eps_r of the element */
void orc_maxw_exact(int isol, int icomp, double omega, double mu, double eps_re, double eps_im,
                    const double *X, double *E, double *H, double *J);
/* sizes[5] = {NrdofEi, NrdofQ, NrdofEE, NrTest, NrTrial} (elem.F90:78-103) */
int orc_dpg_sizes(const int32_t *norder, int nord_add, int32_t *sizes);
/* elem_maxwell (elem/elem_maxwell.F90:24-676) with the impedance penalty
 * (imp_penalty 679-876) on the faces of imp_mask (bit f: ibc(f,2) = 2) and a
 * scalar complex relative permittivity eps_r per element (get_permittivity
 * returns eps_r * I).  zaloc: NrTrial x NrTrial, column-major, rows/columns
 * [E,H traces interleaved per shape function | 6 L2 components per shape
 * function]; zbloc: NrTrial.  Returns NrTrial, -1 (negative Jacobian) or -2
 * (Gram not positive definite). */
int orc_dpg_maxwell_elem(const int32_t *norder, const int32_t *nori_edge, const int32_t *nori_face,
                         const double *xvert, double eps_re, double eps_im, int32_t imp_mask,
                         const orc_maxw_params *prm, double *zaloc, double *zbloc);
/* stc_fwd_herm (stc.F90:338-416), complex Hermitian */
int orc_stc_fwd_z(int ni, int nb, const double *a, int lda, const double *b, double *aii,
                  double *bi, double *aschur, double *bschur);
/* H(curl) shape functions per element node (26: vertices, edges, faces) */
int orc_node_nshapeE(const int32_t *norder, int32_t *nsh);
/* celem_systemI H(curl) branch with the two EHtrc components + compression;
 * bcflag bit 0 = E known, bit 1 = H known.  Returns nrdofc. */
int orc_celem_compress_z(const int32_t *norder, const int32_t *bcflag, const double *aii,
                         const double *bi, const double *zdofd, int32_t *nextract,
                         double *zbload, double *zastif, int32_t *ndofm);
/* batch pass elem_maxwell -> stc_fwd_herm -> compression (OpenMP) */
int orc_dpg_pass(int nelem, const int32_t *norder, const int32_t *nori_edge,
                 const int32_t *nori_face, const int32_t *bcflag, const int32_t *imp_mask,
                 const double *xvert, const double *eps, const orc_maxw_params *prm, int nthreads,
                 const int64_t *elem_nnz, const int64_t *lcon_off, const int64_t *schur_off,
                 const int64_t *bub_off, double *zastif, double *zbload, double *aschur,
                 double *bschur);

#ifdef __cplusplus
}
#endif

#endif
