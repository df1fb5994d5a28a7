/*
 * hp3dg.h -- C ABI of the GB300 element pass for hp3D.
 *
 * One batched, device-resident pass replaces hp3D's per-element work inside
 * the assembly loop of the MUMPS driver (Oden-EAG/hp3d, paths relative to
 * trunk/):
 *
 *   solver/omp_mumps/mumps_sc.F90:253-330   element loop (OpenMP)
 *     -> constrs/celem_systemI.F90:54-951   modified element, compression
 *        -> problems/POISSON/GALERKIN/elem.F90:20-55 / elem_opt.F90:22-141
 *           (set_3D_int, shape3DH, geom3D, getf, A_TEST, DSYRK)
 *        -> modules/stc.F90:182-509         static condensation
 *     -> mumps_sc.F90:266-321               LCON / triplets
 *
 * The caller describes each element as find_order/find_orient/nodcor/
 * get_index would (hp3dg_elem_desc), submits the batch once before the
 * element loop, runs it, and then reads per element exactly what the
 * reference routines return.  All entry points are plain C: pointers and
 * sizes, no C++ or torch types.  Every result is computed on the GPU; there
 * is no CPU fallback.  A call returns HP3DG_OK (0) or a negative error code.
 *
 * Thread safety: submit/run/download are called by one thread (the
 * reference's STEP 1.5, before its parallel region).  The hp3dg_get_* calls
 * only read host buffers filled by hp3dg_batch_download and may be called
 * concurrently from the OpenMP threads of the element loop.
 */
#ifndef HP3DG_H
#define HP3DG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference stops on these conditions: geom.F90:70-71
 * negative Jacobian, stc.F90:464-488 LAPACK info /= 0) */
#define HP3DG_OK 0
#define HP3DG_ERR_NEG_JACOBIAN -1 /* det J < 0 at a quadrature point */
#define HP3DG_ERR_NOT_SPD -2      /* bubble block not positive definite */
#define HP3DG_ERR_BAD_ORDER -3    /* order outside 1..MAXP or unsupported type */
#define HP3DG_ERR_ALLOC -4        /* device or pinned allocation failed */
#define HP3DG_ERR_CUDA -5         /* a CUDA call failed */
#define HP3DG_ERR_TIMEOUT -6      /* a bounded device wait gave up */
#define HP3DG_ERR_ARG -7          /* invalid argument */
#define HP3DG_ERR_STATE -8        /* call out of order (e.g. get before run) */
#define HP3DG_ERR_UNSUPPORTED -9  /* feature not available on this device */

/* element types: node types MDLB / MDLP / MDLN of data_structure3D */
#define HP3DG_HEXA 1
#define HP3DG_PRISM 2
#define HP3DG_TET 3

/* precision of the B^T D B contraction */
#define HP3DG_FP64 0  /* FP64 on CUDA cores (the plain GPU form) */
#define HP3DG_MIXED 1 /* split-BF16 digits on tcgen05 tensor cores, exact
                         FP32 accumulation per digit level, FP64 recombination */

#define HP3DG_MAXP 6 /* parameters.F90:17 */

typedef struct hp3dg_ctx hp3dg_ctx;

typedef struct hp3dg_opts {
  int32_t precision;   /* HP3DG_FP64 or HP3DG_MIXED */
  int32_t integration; /* control INTEGRATION: quadrature order p+INTEGRATION
                          (set_3D_int.F90:236-244), capped at MAXP */
  int32_t isol;        /* source selector of getf (common/getf.F90:63):
                          0,1,2 as common/solution.F90; 10 = sin sin sin;
                          11 = f == 1; 12 = u = xyz (f = 0);
                          13 = u = 1 + x + 2y + 3z (f = 0) */
  int32_t keep_elem;   /* 1: keep the unconstrained element matrices so that
                          hp3dg_get_elem can serve the elem() contract */
  int32_t timing;      /* 1: record per-phase CUDA-event timings */
  int32_t device;      /* CUDA device ordinal */
  int32_t ozaki_radix; /* mixed: bits per BF16 digit (0 = default 7) */
  int32_t ozaki_digits;/* mixed: digits per operand (0 = default 7) */
  int32_t stc_method;  /* condensation: 0 = Cholesky (the Poisson bubble block
                          is SPD); reserved for an LU variant */
  int32_t launch_mode; /* 0 = hp3dg_batch_run replays one CUDA graph of the pass
                          (captured on the first run after a submit);
                          1 = direct stream launches */
  int32_t schur_fp64;  /* HP3DG_MIXED only: 0 = the Schur update of the
                          condensation (K_ii - Y^T Y) on tensor cores with
                          split-BF16 digits where the bin fits, 1 = FP64 */
  int32_t download_chunks; /* 0/1: one piece; N = 2..8: for a batch of one bin
                          the pass runs in N element chunks and
                          hp3dg_batch_download copies each chunk's outputs
                          as soon as it is done, overlapping the copies with
                          the rest of the pass (same results) */
  int32_t fault_inject;  /* testing only, 0 otherwise.  1: the mixed
                          contraction's loader withholds one stage, so the
                          kernel's bounded waits run out (with a short limit)
                          and hp3dg_batch_sync returns HP3DG_ERR_TIMEOUT; the
                          context stays usable.  2: every device allocation
                          of a submit that allocates fails, which returns
                          HP3DG_ERR_ALLOC; the context can be ended. */
  int32_t tune;        /* 0: per-bin kernel variants from the tuning table
                          (hp3dg_tune_load, or the file named by the
                          environment variable HP3DG_TUNE_FILE), where it has
                          an entry for the bin; 1: built-in rules only */
  int32_t reserved[2];
} hp3dg_opts;

/* Element descriptor: what find_order (datstrs/find_order.F90:5),
 * find_orient (datstrs/find_orient.F90:8), elem_nodes and get_index
 * (datstrs/get_index.F90:27) return for element Mdle. */
typedef struct hp3dg_elem_desc {
  int32_t etype;         /* HP3DG_HEXA, HP3DG_PRISM or HP3DG_TET */
  int32_t mdle;          /* middle node id, returned back for bookkeeping */
  int32_t norder[19];    /* Norder.  hexa: 12 edges, 6 faces (MODORDER=10
                            packed), interior (3 digits); prism: 6 mixed and
                            3 vertical edges, 2 triangle faces, 3 quad faces
                            (packed), interior (ph*10+pz), 15 used; tet:
                            6 edges, 4 faces, interior, 11 used */
  int32_t nori_edge[12]; /* NoriE: 0/1 (prism 9, tet 6 used) */
  int32_t nori_face[6];  /* NoriF: quad faces 0..7 (OrientQuad), triangle
                            faces 0..5 (OrientTri); prism: 2 triangles then
                            3 quads; tet: 4 triangles */
  int32_t nodes[26];     /* global ids of vertex, edge, face nodes in element
                            order (hexa 26, prism 20, tet 14 used) */
  int32_t bcflag[26];    /* 1: every dof of this node is Dirichlet (index=1) */
} hp3dg_elem_desc;

/* Create a context on opts->device (NULL opts = defaults: FP64,
 * INTEGRATION=0, isol=10). */
int hp3dg_batch_begin(const hp3dg_opts *opts, hp3dg_ctx **ctx);

/* Bind the context to an existing CUDA stream (cudaStream_t passed as
 * void*; NULL = the context's own stream). */
int hp3dg_set_stream(hp3dg_ctx *ctx, void *stream);

/* Submit a batch: n_elem descriptors in ELEM_ORDER, vertex coordinates
 * xvert (n_elem x 8 x 3, the nodcor geometry dof of a trilinear map, a
 * tetrahedron using the first 4 vertex slots; higher-order geometry dof are
 * zero; a prism the first 6), per-element coefficient kappa
 * (NULL = 1), Dirichlet data zdofd (NULL = homogeneous; else for each
 * element its interface dof values in element dof order, concatenated),
 * and the number of global nodes (size of NFIRST_DOF).
 * Validates orders and copies the batch to the device.  A resubmit whose
 * descriptors, node count and Dirichlet layout equal the current batch's
 * (a new geometry, coefficient or Dirichlet data on the same mesh) only
 * uploads xvert, kappa and zdofd: device buffers, bin tables, the captured
 * pass and the pinned result buffers are kept.
 * Replaces: mumps_sc.F90 STEP 1 (102-188). */
int hp3dg_batch_submit(hp3dg_ctx *ctx, int32_t n_elem, const hp3dg_elem_desc *desc,
                       const double *xvert, const double *kappa, const double *zdofd,
                       int32_t n_nodes_global);

/* Isoparametric (curved) geometry: the element's nrdofH geometry dof, as
 * nodcor returns them (constrs/nodcor.F90:19-196) and geom3D consumes them
 * (element/util/geom3D.F90:30-112): per element 3 values (x, y, z) per dof
 * in element dof order (vertices, edges, faces, interior; the element's
 * orientation), elements concatenated in ELEM_ORDER -- 3 * nrdofH(e) values
 * for element e.  The vertex dof are the vertex coordinates; a trilinear
 * element has zero higher-order dof.  Call after hp3dg_batch_submit; the
 * next runs use this geometry until the next submit (which returns to the
 * vertex coordinates).  NULL returns to the vertex coordinates now.  With
 * this geometry hp3dg_element_error, hp3dg_adjoint and hp3dg_dirichlet_dofs
 * return HP3DG_ERR_UNSUPPORTED. */
int hp3dg_batch_set_geometry(hp3dg_ctx *ctx, const double *xnod);

/* Constrained approximation (hanging nodes): for each constrained element,
 * what logic (constrs/logic.F90) returns for it, as celem_systemI consumes it
 * (celem_systemI.F90:541-760):
 *   the modified element nodes Nodm (without the middle node), their H1 dof
 *   counts and Dirichlet flags; and the coefficients constrH of every
 *   element interface dof k (element order, 0-based) on the modified dof l
 *   (modified nodes in order, each node's dof forward, 0-based) as triplets,
 *   listed per element in the order logic gives them (k, then its connected
 *   dof).
 * The condensed element system becomes C^T A C, C^T b; extraction,
 * Dirichlet lift and compression run over the modified nodes, and the index
 * maps walk Nodm (mumps_sc.F90:102-188 with celem's Nodm). */
typedef struct hp3dg_constraints {
  int32_t n;               /* number of constrained elements */
  const int32_t *iel;      /* their batch indices, strictly increasing */
  const int64_t *node_off; /* n+1 offsets into nodm / ndof / bcflag */
  const int32_t *nodm;     /* modified element nodes (global ids) */
  const int32_t *ndof;     /* H1 dof per modified node */
  const int32_t *bcflag;   /* 1: the node's dof are Dirichlet */
  const int64_t *coef_off; /* n+1 offsets into coef_k / coef_l / coef_v */
  const int32_t *coef_k;
  const int32_t *coef_l;
  const double *coef_v;
  const double *zdofd;     /* Dirichlet values per modified dof, concatenated
                              per element (node_off order); NULL = 0 */
} hp3dg_constraints;

/* hp3dg_batch_submit for a batch with constrained elements (cons may be
 * NULL).  Back-substitution, element errors and the adjoint are not
 * available for a constrained batch (HP3DG_ERR_UNSUPPORTED). */
int hp3dg_batch_submit_constrained(hp3dg_ctx *ctx, int32_t n_elem, const hp3dg_elem_desc *desc,
                                   const double *xvert, const double *kappa,
                                   const double *zdofd, int32_t nnodes,
                                   const hp3dg_constraints *cons);

/* Run the whole element pass on the device (asynchronous on the context's
 * stream; errors of the pass are reported by hp3dg_batch_sync).
 * Replaces: the STEP 2 element loop (mumps_sc.F90:253-330). */
int hp3dg_batch_run(hp3dg_ctx *ctx);

/* Wait for the pass and return its status (first bad element via
 * hp3dg_last_bad_element). */
int hp3dg_batch_sync(hp3dg_ctx *ctx);

/* Copy all outputs into pinned host buffers owned by the context. */
int hp3dg_batch_download(hp3dg_ctx *ctx);

/* elem() contract (problems/POISSON/GALERKIN/elem.F90:20-55): unconstrained
 * stiffness ALOC(1,1) written with leading dimension ld (= ALOC(1,1)%nrow)
 * and load BLOC(1).  Needs opts.keep_elem = 1. */
int hp3dg_get_elem(const hp3dg_ctx *ctx, int32_t iel, double *aloc, int32_t ld,
                   double *bloc);

/* celem_systemI contract (constrs/celem_systemI.F90:812-845, ISYM_FLAG=2):
 * compressed condensed load Zbload(nrdofc) and row-major stiffness
 * Zastif(nrdofc**2); nrdofc returned. */
int hp3dg_get_condensed(const hp3dg_ctx *ctx, int32_t iel, double *zbload,
                        double *zastif, int32_t *nrdofc);

/* Schur blocks kept for back-substitution (stc.F90:273-277): ASchur =
 * inv(Abb) Abi (nb x ni column-major), BSchur = inv(Abb) Bb (nb). */
int hp3dg_get_schur(const hp3dg_ctx *ctx, int32_t iel, double *aschur, double *bschur,
                    int32_t *nb, int32_t *ni);

/* Index maps of mumps_sc (STEP 1 NFIRST_DOF, STEP 2 LCON): nfirst_dof
 * (n_nodes_global, -1 for unvisited), elem_nnz (n_elem+1 prefix of
 * nrdofc**2), lcon_off (n_elem+1 prefix of nrdofc), lcon (1-based global
 * dof, nodes in reverse order), nrdof (number of interface dof).  Any
 * pointer may be NULL. */
int hp3dg_index_map(const hp3dg_ctx *ctx, int32_t *nfirst_dof, int64_t *elem_nnz,
                    int64_t *lcon_off, int32_t *lcon, int64_t *nrdof);

/* Back-substitution after the global solve (stc_bwd_wrapper / stc_bwd /
 * stc_solout, modules/stc.F90:529-991; called from solout,
 * solver/frontal/interf/solout.F90:457): x_global holds the nrdof interface
 * unknowns (host memory, 1-based LCON numbering).  Builds every element's
 * full dof vector (interface dof from x_global or the submitted Dirichlet
 * data, bubbles = BSchur - ASchur xi) on the device and copies it to the
 * host; read it with hp3dg_get_dofs. */
int hp3dg_backsub(hp3dg_ctx *ctx, const double *x_global);

/* Full dof vector of element iel (interface dof then bubbles, element dof
 * order) after hp3dg_backsub; n returned. */
int hp3dg_get_dofs(const hp3dg_ctx *ctx, int32_t iel, double *dof, int32_t *n);

/* Squared H1 error and squared H1 norm of every element against the
 * manufactured solution isol (element_error, element/util/compute_error.F90:
 * 226-360, H1 branch with the INTEGRATION = 2 rule), using the dof of the
 * last hp3dg_backsub.  err2, nrm2: host arrays of n_elem. */
int hp3dg_element_error(hp3dg_ctx *ctx, int32_t isol, double *err2, double *nrm2);

/* Compliance sensitivities (J = f^T u with K u = f, adjoint lambda = u):
 * dJ/dkappa_e = -u_e^T (dK_e/dkappa_e) u_e for every element, and the
 * element contributions to dJ/dx of its 8 vertices (n_elem x 8 x 3; sum
 * them over elements sharing a vertex), including the dependence of the
 * load on the geometry.  dofs: host array of the full element dof vectors
 * concatenated in element order, or NULL to use those of hp3dg_backsub.
 * No counterpart in the reference solver (used for design optimisation on
 * top of its element pass). */
int hp3dg_adjoint(hp3dg_ctx *ctx, const double *dofs, double *djdkappa, double *djdx);

/* Sizes of the batch outputs (for the caller's allocation). */
int hp3dg_output_sizes(const hp3dg_ctx *ctx, int64_t *nnz_total, int64_t *lcon_total,
                       int64_t *schur_total, int64_t *bubble_total);

/* Device pointers of the outputs (for consumers that stay on the GPU). */
int hp3dg_device_outputs(const hp3dg_ctx *ctx, const double **zastif,
                         const double **zbload, const double **aschur,
                         const double **bschur, const int32_t **lcon);

/* Per-phase device times (ms) of the last run when opts.timing = 1:
 * [0] tables, [1] geometry+load, [2] contraction, [3] condensation,
 * [4] index maps, [5] whole pass.  n = number of entries wanted. */
int hp3dg_phase_times(const hp3dg_ctx *ctx, float *ms, int32_t n);

/* Mixed-precision configuration of the context's first bin: bits per digit,
 * digits per operand, number of digit-pair products (tensor-core passes).
 * Returns HP3DG_ERR_STATE before a mixed-precision submit. */
int hp3dg_mixed_config(const hp3dg_ctx *ctx, int32_t *radix, int32_t *digits, int32_t *pairs);

/* Statistics of the pass as it runs after the last submit.
 * kernels: kernel launches per hp3dg_batch_run, counted from the kernel nodes
 *   of the captured CUDA graph (-1 before the first run or with launch_mode
 *   = 1, where nothing is captured).
 * contraction_flops: algorithmic floating-point operations of the contraction
 *   per run, summed over the bins: mixed precision, digit-pair products x
 *   2 (6 nint) n(n+1)/2 per element; FP64, n(n+1) 3 nint per element (the
 *   DSYRK count of elem_opt). */
int hp3dg_pass_stats(const hp3dg_ctx *ctx, int64_t *kernels, double *contraction_flops);

/* Geometry dof by projection-based interpolation of the geometry-block maps
 * (update_gdof, hpinterp/update_gdof.F90:6; hpvert, hpedge, hpface,
 * hpmdle), hexahedra.  The block maps stay with the caller (the reference's
 * GMP routines hexa(No, eta, x, dxdeta) and their kin); the projections run
 * on the GPU.  Two calls:
 *   hp3dg_gdof_points: the points in block coordinates at which the caller
 *     evaluates its maps: per element (batch order) its 8 vertices, then per
 *     edge, face and the interior carrying dof the quadrature points of
 *     set_1Dint / set_2Dint / set_3Dint at the context's INTEGRATION.
 *     etav: n_elem x 8 x 3, each element's vertices in its block's
 *     coordinates (refel); eta(xi) is trilinear in them.  *npts = number of
 *     points; eta (nullable) receives npts x 3 block coordinates.
 *   hp3dg_update_gdof: x (npts x 3) and dxdeta (npts x 9, row-major
 *     dx_i/deta_j) of the maps at those points -> the geometry dof of every
 *     element in the layout of hp3dg_batch_set_geometry (xnod, nullable).
 *     Vertex dof are x at the vertices; edge, face and interior dof are the
 *     eta-space H1 projections (tangential derivative, surface gradient, full
 *     gradient) of x minus the lower-order part.  Each node takes the values
 *     of the first element (batch order) that contains it, as the reference
 *     projects each node once.  linear (nullable, n_elem): 1 = a 'Linear'
 *     block, vertices only.  apply = 1 makes the result the pass's geometry
 *     (as hp3dg_batch_set_geometry).  A singular projection returns
 *     HP3DG_ERR_NOT_SPD (hp3dg_last_bad_element names the element).
 * Other element types return HP3DG_ERR_UNSUPPORTED. */
int hp3dg_gdof_points(hp3dg_ctx *ctx, const double *etav, double *eta, int64_t *npts);
int hp3dg_update_gdof(hp3dg_ctx *ctx, const double *etav, const double *x, const double *dxdeta,
                      const int32_t *linear, double *xnod, int32_t apply);

/* Tuning table (JSON, written by hp3d_gb300/autotune.py from timings on the
 * target GPU): per (element type, n, nb, quadrature points, precision) bin
 * the condensation variant and the contraction's raster group, and the
 * contraction's pipeline depth.  Process-wide; read by every later submit of
 * a context with opts.tune = 0 that builds its bins (a resubmit of the same
 * descriptors keeps the batch's variants).  path = NULL clears the table.  Returns
 * HP3DG_ERR_ARG for an unreadable or malformed file (the table is then left
 * as it was); *nrec = bin entries loaded. */
int hp3dg_tune_load(const char *path, int32_t *nrec);

/* The table's entry for a bin: cond (0 = built-in rule, 1 = fused
 * tensor-core condensation, 2 = FP64 factor + tensor-core Schur update,
 * 3 = FP64), grp (contraction column blocks per raster group, 0 = built-in)
 * and the table's ring depth nstage (0 = as many as fit).  HP3DG_ERR_ARG
 * when the table has no entry (cond = grp = 0). */
int hp3dg_tune_lookup(int32_t etype, int32_t n, int32_t nb, int32_t nint, int32_t precision,
                      int32_t *cond, int32_t *grp, int32_t *nstage);

/* Bins of the last submit: *nbins, and for bin b (0 <= b < nbins)
 * info[0..7] = etype, n, nb, nint (quadrature points), elements, the
 * condensation variant in use (1, 2, 3 as in hp3dg_tune_lookup; FP64
 * precision: 3), the contraction raster group requested (0 = built-in),
 * and 1 if the table supplied the bin's variant.  bin_of (nullable, n_elem
 * entries): each element's bin. */
int hp3dg_bin_info(const hp3dg_ctx *ctx, int32_t *nbins, int32_t b, int32_t *info,
                   int32_t *bin_of);

/* Size of the fixed device scratch array used by hp3dg_condense_noalloc:
 * 2^20 doubles (8 MiB), resident on every GPU that loads the library. */
#define HP3DG_NOALLOC_SCRATCH_DOUBLES (1 << 20)

/* Static condensation of caller-supplied dense element matrices, with no
 * allocation of any kind.  This entry point has no counterpart in the
 * reference: it exists for callers that cannot allocate device memory (an
 * element loop inside an OpenMP region of a host solver, where cudaMalloc
 * would serialise the threads and synchronise the device; applications
 * whose device memory belongs to their own pool or to a solver sharing the
 * GPU).  All pointers are device pointers supplied by the caller:
 *   K      n_elem x (n x n) column-major element matrices, interface dof
 *          first and the nb bubble dof last (the order of stc_fwd_wrapper)
 *   b      n_elem x n loads
 *   aii    n_elem x (ni x ni) column-major condensed matrices, ni = n - nb
 *   bi     n_elem x ni condensed loads
 *   aschur n_elem x (nb x ni) column-major inv(Abb) Abi
 *   bschur n_elem x nb inv(Abb) Bb
 * Scratch: the packed Schur triangles, n_elem * ni*(ni+1)/2 doubles, live in
 * a fixed device array of HP3DG_NOALLOC_SCRATCH_DOUBLES - 1 usable doubles
 * (90 elements of a p = 5 hexahedron, ni = 152); larger batches are rejected
 * with HP3DG_ERR_ARG (split them).  One element's bubble block, [K_bi | b_b]
 * and condensed load, (nb^2 + nb(ni+1) + ni) doubles, must fit in the
 * device's opt-in shared memory per block: hexahedra up to p = 5 do, p = 6
 * (345 KB) returns HP3DG_ERR_UNSUPPORTED.  Calls share the scratch array:
 * calls whose kernels overlap on the GPU race and must be ordered by the
 * caller.  The first call on a device looks up the array's device address;
 * make it before any stream capture begins.  The call waits for its kernel
 * on `stream` (NULL = legacy default stream).  *bad_element is set to -1, or
 * on HP3DG_ERR_NOT_SPD to the first element whose bubble block is not
 * positive definite.  n_elem = 0 returns HP3DG_OK. */
int hp3dg_condense_noalloc(int32_t n_elem, int32_t n, int32_t nb, const double *K,
                           const double *b, double *aii, double *bi, double *aschur,
                           double *bschur, int32_t *bad_element, void *stream);

/* The contraction kernel of HP3DG_MIXED on caller-supplied FP64 operands:
 * out[r, c] = sum_q D[r, q] M[q, c] for D nrows x K, M K x ncols and out
 * nrows x ncols, all row-major device pointers.  Both operands are split
 * into balanced BF16 digits of `radix` bits (0 = 7), `digits` per operand
 * (0 = 7), with power-of-two row / column scales; the digit products of
 * each level are summed on tcgen05 tensor cores in FP32 accumulators that
 * are restarted before any partial sum can exceed 2^24, so every level sum
 * is exact, and the levels are recombined exactly as 64-bit integers before
 * one rounding to FP64.  Allocates its digit buffers, runs on `stream`
 * (NULL = legacy default stream) and waits for it.  No counterpart in the
 * reference: the element pass applies this kernel with K = 6 nint and M the
 * bin's shape-function products (elem_opt.F90:86-137); this entry point
 * takes operands of any content, so the exactness bound can be checked on
 * worst-case data. */
int hp3dg_mixed_contract(int32_t nrows, int32_t K, int32_t ncols, const double *D,
                         const double *M, double *out, int32_t radix, int32_t digits,
                         void *stream);

/* Dirichlet data of the submitted batch by projection-based interpolation
 * (update_Ddof, hpinterp/update_Ddof.F90 with dhpvert, dhpedgeH, dhpfaceH)
 * of the manufactured solution isol, computed on the GPU: for every element
 * the values of its interface dof on the nodes with bcflag set (vertex
 * values, then tangential H1-seminorm projections on edges and faces), in
 * the layout hp3dg_batch_submit takes as zdofd (element order, n_i per
 * element; zeros elsewhere).  Hexahedra whose geometry block is the element
 * (trilinear vertex geometry).  zdofd = NULL returns the length in *n. */
int hp3dg_dirichlet_dofs(hp3dg_ctx *ctx, int32_t isol, double *zdofd, int64_t *n);

/* First element (0-based) that failed in the last run, or -1. */
int32_t hp3dg_last_bad_element(const hp3dg_ctx *ctx);

/* Release everything. */
void hp3dg_batch_end(hp3dg_ctx *ctx);

/* Message for a status code. */
const char *hp3dg_strerror(int status);

/* ------------------------------------------------------------------------ */
/* Ultraweak DPG Maxwell on hexahedra (problems/MAXWELL/ULTRAWEAK_DPG).       */
/* Replaces elem (elem/elem.F90:15 -> elem_maxwell / elem_opt, complex) with  */
/* the automatic static condensation of the L2 fields (stc_fwd_herm,          */
/* HERM_STC) and celem_systemI's compression for the EHtrc attribute, over    */
/* a batch of hexahedra of one isotropic trial order p (1..5, test order      */
/* p + NORD_ADD).  Complex arrays are interleaved (re, im) doubles, the       */
/* layout of Fortran complex(8).                                              */
/* ------------------------------------------------------------------------ */
typedef struct hp3dg_dpg_ctx hp3dg_dpg_ctx;

typedef struct hp3dg_dpg_opts {
  double omega;      /* OMEGA (commonParam.F90; default 2 pi) */
  double mu;         /* MU */
  double epsilon;    /* EPSILON (times the element's relative permittivity) */
  double gamma;      /* GAMMA, impedance constant */
  double alpha;      /* ALPHA_NORM of the scaled adjoint graph test norm */
  int32_t ibcflag;   /* IBCFLAG: 0 Dirichlet only, 2 impedance by penalty */
  int32_t nord_add;  /* NORD_ADD: test enrichment (1) */
  int32_t isol;      /* source: mfd_solutions case 0 (none), 1 (sin), 2 (polynomial) */
  int32_t icomp;     /* ICOMP_EXACT: component (1..3) of E in the manufactured solution */
  int32_t device;
  int32_t timing;    /* record phase times */
  int32_t keep_elem; /* keep the uncondensed DPG element matrices (hp3dg_dpg_get_elem) */
  int32_t precision; /* HP3DG_FP64: contractions and dense algebra in FP64.  HP3DG_MIXED:
                        the contractions (M_FF, M_CC, P, R, T) and every O(n^3) product of
                        the dense algebra and the L2-field condensation on tensor cores from
                        split-BF16 digits, as one partial Cholesky of the augmented matrix
                        [[G, [B|l]], [[B|l]^H, 0]] with FP64 64 x 64 diagonal blocks */
  int32_t reserved[4];
} hp3dg_dpg_opts;

int hp3dg_dpg_begin(const hp3dg_dpg_opts *opts, hp3dg_dpg_ctx **ctx);
/* desc: as for hp3dg_batch_submit with etype HP3DG_HEXA and isotropic order p
 * on every edge, face and the interior.  bcflag per node: bit 0 = the E
 * trace is known (perfect conductor, homogeneous), bit 1 = the H trace is
 * known; on a face node bit 2 = the face lies on the impedance boundary
 * (ibc = 2).  xvert: 3 x 8 vertex coordinates per element (trilinear
 * geometry).  eps: complex relative permittivity per element (the
 * permittivity tensor is EPSILON * eps * I). */
int hp3dg_dpg_submit(hp3dg_dpg_ctx *ctx, int32_t n_elem, const hp3dg_elem_desc *desc,
                     const double *xvert, const double *eps, int32_t nnodes);
int hp3dg_dpg_run(hp3dg_dpg_ctx *ctx);
int hp3dg_dpg_sync(hp3dg_dpg_ctx *ctx);
int hp3dg_dpg_download(hp3dg_dpg_ctx *ctx);
/* Sizes of one element: trial dof (2 nEi + 6 nQ), interface (2 nEi), L2 (6 nQ). */
int hp3dg_dpg_sizes(const hp3dg_dpg_ctx *ctx, int32_t *ntrial, int32_t *ni, int32_t *nb);
/* The DPG element matrix B^H G^-1 B (ld x ntrial, column-major, complex) and
 * load before condensation, rows/columns [E,H traces per trace function |
 * six L2 components per L2 function] (needs keep_elem). */
int hp3dg_dpg_get_elem(const hp3dg_dpg_ctx *ctx, int32_t iel, double *zaloc, int32_t ld,
                       double *zbloc);
/* Condensed and compressed element system (row-major, complex), as
 * celem_systemI returns it to the MUMPS driver. */
int hp3dg_dpg_get_condensed(const hp3dg_dpg_ctx *ctx, int32_t iel, double *zbload,
                            double *zastif, int32_t *nrdofc);
/* ASchur (nb x ni, column-major) and BSchur (nb), complex. */
int hp3dg_dpg_get_schur(const hp3dg_dpg_ctx *ctx, int32_t iel, double *aschur, double *bschur,
                        int32_t *nb, int32_t *ni);
/* NFIRST_DOF / LCON of the EHtrc unknowns, as hp3dg_index_map. */
int hp3dg_dpg_index_map(const hp3dg_dpg_ctx *ctx, int32_t *nfirst, int64_t *elem_nnz,
                        int64_t *lcon_off, int32_t *lcon, int64_t *nrdof);
/* [0] geometry + contractions + assembly, [1] Cholesky + solve + X^H X,
 * [2] condensation + compression, [3] index maps, [4] whole pass (ms). */
int hp3dg_dpg_phase_times(const hp3dg_dpg_ctx *ctx, float *ms, int32_t n);
/* Kernels launched on the device by the last hp3dg_dpg_run (the dense
 * algebra of the tensor-core path is a sequence of per-panel launches). */
int hp3dg_dpg_pass_stats(const hp3dg_dpg_ctx *ctx, int64_t *kernels);
int32_t hp3dg_dpg_last_bad_element(const hp3dg_dpg_ctx *ctx);
void hp3dg_dpg_end(hp3dg_dpg_ctx *ctx);

#ifdef __cplusplus
}
#endif

#endif /* HP3DG_H */
