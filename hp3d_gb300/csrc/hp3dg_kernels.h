// hp3dg_kernels.h -- host launchers of the device kernels (internal).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace hp3dg {

// Raises the dynamic shared-memory limit of a kernel (on the current device)
// to at least `bytes`.  The limit only grows, so a launch enqueued earlier
// (into a graph being captured, or a stream that has not reached it) stays
// valid when a later launch of the same kernel needs less.
cudaError_t raise_smem_limit(const void* func, size_t bytes);

// 1D Gauss-Legendre rule of the reference's tables on [0,1] (n <= 10)
int gauss_rule01(int n, double* x, double* w);

// element types as in the C ABI (HP3DG_HEXA / HP3DG_PRISM / HP3DG_TET)
constexpr int ETYPE_HEXA = 1, ETYPE_PRISM = 2, ETYPE_TET = 3;

// bin tables: nord_loc = the bin's full orders (hexa: 19 local orders; tet:
// every entry the bin order), face_nori = orientation of each face in the
// tables (tets: the orientation class of each triangle face)
void launch_tables(int etype, const int* nord_loc, const int* face_nori, int nint, int n,
                   const double* d_xi, double* d_shap, double* d_grad, cudaStream_t st);
void launch_orient(int etype, int nel, const int* d_elist, const int* d_norder, const int* d_nori_e,
                   const int* d_nori_f, const int* full, int nfull, uint32_t* d_perm,
                   cudaStream_t st);
// geometry per point; d_xnod != NULL: isoparametric, from every element's
// nrdofH geometry dof (3 per dof, element order, at 3 * d_dof_off[e]) through
// its dof map d_perm (j * n + a); else trilinear/linear from d_xvert
void launch_geom(int nel, int nvert, const int* d_elist, int nint, int n, const double* d_wq,
                 const double* d_shap, const double* d_grad, const double* d_xvert,
                 const double* d_kappa, int isol, double* d_D, double* d_F, int* d_bad,
                 cudaStream_t st, const double* d_xnod = nullptr,
                 const int64_t* d_dof_off = nullptr, const uint32_t* d_perm = nullptr);
void launch_load_hexa(int nel, int nint, int n, const double* d_shap, const double* d_F,
                      double* d_b0, cudaStream_t st);

// Grouped launches of the per-element stage kernels over several bins: one
// segment per bin (device arrays built at submit), block offsets per kernel.
// The per-element arithmetic is the one of the per-bin kernels.
struct StageSeg {
  int etype, nvert, n, nint, nel;
  int full[19];              // bin orders (tet: full[0] = the orientation class)
  const int* elist;
  const double *wq, *shap, *grad;
  double *D, *F, *b0;
  uint32_t* perm;
  // mixed precision: the digits of D
  int K, nk, radix, digits;
  uint16_t* ddig;
  double* dscale;
};
struct StageGroup {
  StageSeg* segs = nullptr;  // device
  int nseg = 0;
  int *pre_el = nullptr, *pre_geom = nullptr, *pre_dsc = nullptr, *pre_slice = nullptr;  // device
  std::vector<int> h_pre;    // host copies: [el | geom | dsc | slice] x (nseg + 1)
  int max_nint = 0;
};
// orientation maps, vertex geometry and loads of the group's segments k0..k1-1
// (one launch per kernel)
void launch_stage0_grouped(const StageGroup& g, int k0, int k1, const int* d_norder,
                           const int* d_nori_e, const int* d_nori_f, const double* d_xvert,
                           const double* d_kappa, int isol, int* d_bad, cudaStream_t st);
// row scales and digit tiles of D of the segments k0..k1-1 (mixed)
int launch_slice_d_grouped(const StageGroup& g, int k0, int k1, cudaStream_t st);
void launch_contract_fp64(int nel, int nint, int n, int ni, int nb, const double* d_grad,
                          const double* d_D, double* d_PK, cudaStream_t st);
size_t condense_smem(int ni, int nb);
size_t condense_smem_small(int ni, int nb);
// Factor mode of the condensation (mixed pass): instead of the FP64 Schur
// update and the compression, write Y = L^-1 K_bi as balanced BF16 digits
// (per element ebytes: digit, k-block, nr x 16 canonical tile) with one
// power-of-two exponent per column, and the condensed load bi (nif per element).
struct TcFactorOut {
  uint8_t* ydig = nullptr;
  int* yexp = nullptr;
  double* bi = nullptr;
  int nr = 0, nkb = 0, digits = 0, radix = 0;
  size_t ebytes = 0;
};
int launch_condense(int nel, int nfull, int nif, int nbf, const int* d_elist, const int* d_ni_e,
                    const int* d_nb_e, const double* d_PK, const double* d_b0,
                    const uint32_t* d_perm, const int* d_nextract, const int64_t* d_lcon_off,
                    const int64_t* d_elem_nnz, const int64_t* d_schur_off,
                    const int64_t* d_bub_off, const int64_t* d_zd_off, const double* d_zdofd,
                    const uint8_t* d_dmask, double* d_S, double* d_zastif, double* d_zbload,
                    double* d_aschur, double* d_bschur, double* d_Yg, int* d_bad_spd,
                    cudaStream_t st, const TcFactorOut* tco = nullptr);
// compression after the tensor-core update: S = K_ii (through the dof map)
// - W, then Zastif / Zbload as compress_out
void launch_compress(int nel, int nfull, int nif, int nbf, const int* d_elist, const int* d_ni_e,
                     const double* d_PK, const uint32_t* d_perm, const double* d_W,
                     const double* d_bi, const int* d_nextract, const int64_t* d_lcon_off,
                     const int64_t* d_elem_nnz, const int64_t* d_zd_off, const double* d_zdofd,
                     const uint8_t* d_dmask, double* d_zastif, double* d_zbload, cudaStream_t st);
// condensation with every product on tensor cores (nb <= 64) -- k_cond_tc.cu
// Digits of its operands: with K = nb <= 64 a level sum of radix-8 digits is
// at most (2^16 + 4 * 2^14) * 64 = 2^23 < 2^24 (exact in FP32).
constexpr int COND_TC_RADIX = 8, COND_TC_DIGITS = 6;
struct CondTcBufs {
  uint8_t *kbd = nullptr, *lid = nullptr, *ltd = nullptr;  // digits of K_bi^T, Li, Li^T
  int *ekb = nullptr, *eli = nullptr, *elt = nullptr;      // row exponents
  double* bi = nullptr;                                     // condensed load
  int nr = 0, nbr = 0, nkb = 0, digits = 0, radix = 0;
  size_t bytes_a = 0, bytes_b = 0;                          // per element
};
// Grouped launches of the fused condensation (k_cond_chol, k_cond_kbi,
// k_cond_tc, k_compress) over several bins or element chunks: one segment
// each, tables built once per batch; an element's arithmetic is the same in
// any batch.  Segments with nbf = 0 (no bubbles: S = K_ii, the condensed load
// is b_i) come after the tensor-core ones and only enter the compression.
struct CondSegIn {
  int nfull, nif, nbf, nel;
  const int* elist;
  const double *PK, *b0;
  const uint32_t* perm;
  double* W;             // Schur scratch, nif(nif+1)/2 per element
  CondTcBufs t;          // digit buffers offset to the segment's first element
  const uint8_t* dmask;  // Dirichlet mask, nif per element
};
struct CompressSeg {
  int nfull, nif, nbf;
  const int* elist;
  const double* PK;
  const uint32_t* perm;
  const double* W;
  const double* bi;
  const uint8_t* dmask;
  const double* b0;  // nbf = 0: the load, b_i gathered through perm
};
struct CondGroup {
  void* segs = nullptr;           // device segment table of the fused kernels
  CompressSeg* csegs = nullptr;   // device
  int nseg = 0;
  int ntc = 0;                    // segments 0..ntc-1 use the tensor-core kernels
  size_t smem_plain = 0;          // compression of nbf = 0 segments: b_i in shared memory
  int *pre_chol = nullptr, *pre_kbi = nullptr, *pre_el = nullptr;  // device block offsets
  std::vector<int> h_pre;         // host copies: [chol | kbi | el] x (nseg + 1)
  std::vector<CondSegIn> h_in;    // the segments as built (one-segment launches)
  size_t smem_chol = 0, smem_tc = 0;
};
// builds the device tables (allocations appended to *allocs, freed by the caller)
int cond_tc_group_build(const std::vector<CondSegIn>& in, CondGroup* g,
                        std::vector<void*>* allocs);
// Cholesky + inverse, K_bi digits, the fused tensor-core kernel, for the
// segments k0..k1-1
int launch_cond_tc_group(const CondGroup& g, int k0, int k1, const int* d_ni_e, const int* d_nb_e,
                         const int64_t* d_schur_off, const int64_t* d_bub_off, double* d_aschur,
                         double* d_bschur, int* d_bad_spd, int* d_flag, cudaStream_t st);
// S = K_ii - W, compression and lift for the segments k0..k1-1
void launch_compress_group(const CondGroup& g, int k0, int k1, const int* d_ni_e,
                           const int* d_nextract, const int64_t* d_lcon_off,
                           const int64_t* d_elem_nnz, const int64_t* d_zd_off,
                           const double* d_zdofd, double* d_zastif, double* d_zbload,
                           cudaStream_t st);
bool cond_tc_supported(int nif, int nbf, int digits);
void cond_tc_make_out(int nif, int nbf, int radix, int digits, CondTcBufs& b);
int launch_cond_tc(int nel, int nfull, int nif, int nbf, const int* d_elist, const int* d_ni_e,
                   const int* d_nb_e, const double* d_PK, const double* d_b0,
                   const uint32_t* d_perm, const int64_t* d_schur_off, const int64_t* d_bub_off,
                   double* d_W, double* d_aschur, double* d_bschur, const CondTcBufs& b,
                   int* d_bad_spd, int* d_flag, cudaStream_t st);
// tensor-core Schur update S = K_ii - Y^T Y -- k_schur.cu
int schur_tc_rows(int nif);
int schur_tc_kblocks(int nbf);
size_t schur_tc_elem_bytes(int nif, int nbf, int digits);
bool schur_tc_supported(int nif, int nbf, int digits);
int launch_schur_tc(int nel, int nfull, int nif, int nbf, int radix, int digits,
                    const uint8_t* d_ydig, const int* d_yexp, const int* d_elist,
                    const int* d_ni_e, double* d_W, int* d_flag, cudaStream_t st);
int launch_index_maps(int nel, int nnode, int nnodes_global, const int* d_nodes, const int* d_ndofm,
                      const int64_t* d_lcon_off, int* d_first, int* d_cnt, int64_t* d_scan,
                      int64_t* d_blk, int64_t* d_total, int* d_nfirst, int* d_lcon,
                      cudaStream_t st);

// after the solve -- k_post.cu
void launch_backsub(int nel, int nif, const int* d_elist, const int* d_ni_e, const int* d_nb_e,
                    const int* d_nextract,
                    const int64_t* d_lcon_off, const int* d_lcon, const double* d_x,
                    const int64_t* d_zd_off, const double* d_zdofd, const int64_t* d_schur_off,
                    const int64_t* d_bub_off, const double* d_aschur, const double* d_bschur,
                    const int64_t* d_dof_off, double* d_dofs, cudaStream_t st);
void launch_element_error(int nel, int nvert, int nint, int n, int isol, const int* d_elist,
                          const int* d_n_e,
                          const double* d_wq,
                          const double* d_shap, const double* d_grad, const double* d_xvert,
                          const uint32_t* d_perm, const int64_t* d_dof_off, const double* d_dofs,
                          double* d_err2, double* d_nrm2, cudaStream_t st);
void launch_adjoint(int nel, int nvert, int nint, int n, int isol, const int* d_elist,
                    const int* d_n_e,
                    const double* d_wq,
                    const double* d_shap, const double* d_grad, const double* d_xvert,
                    const double* d_kappa, const uint32_t* d_perm, const int64_t* d_dof_off,
                    const double* d_dofs, double* d_djdk, double* d_djdx, cudaStream_t st);

// Dirichlet data by projection-based interpolation (hexahedra) -- k_post.cu.
// d_gx / d_gw: the n-point Gauss rules on [0,1] at [16 n + l], n <= 10.
size_t dirichlet_work_doubles(int nel);
// geometry dof by projection of block maps (k_post.cu): per-thread scratch
// for projections of up to nmax dof; the three phases with the first-visit
// gathers between them, elements in chunks of `chunk` threads' scratch
size_t gdof_work_doubles(int nmax);
int launch_gdof(int nel, const int* d_norder, const int* d_nori_e, const int* d_nori_f,
                const double* d_etav, const int64_t* d_node_pt, const double* d_pts,
                const double* d_x, const double* d_dxdeta, const int* d_linear,
                const int* d_src, const int64_t* d_dof_off, double* d_xnod, double* d_work,
                int64_t wstride, int chunk, int* d_bad, cudaStream_t st);
void launch_dirichlet(int nel, const int* d_norder, const int* d_nori_e, const int* d_nori_f,
                      const int* d_bc, const double* d_xvert, const int64_t* d_zd_off,
                      const double* d_gx, const double* d_gw, int isol, double* d_work,
                      double* d_zdofd, int* d_bad, cudaStream_t st);

// mixed precision (split-BF16 digits on tcgen05) -- k_ozaki.cu
struct OzakiPlan {
  int radix;      // bits per digit
  int digits;     // digits per operand
  int levels;     // number of exact FP32 level accumulators
  int kdim;       // 6*nint rounded up to the K tile
  int ncols;      // n(n+1)/2 rounded up to the N tile
  int kreal = 0, nreal = 0;  // dense plans: K and columns before rounding
};
int ozaki_plan(int nint, int n, int radix, int digits, OzakiPlan* plan);
// build the M digit table of a bin (once): B operand, column scales
int launch_ozaki_build_m(const OzakiPlan& plan, int nint, int n, int ni, int nb,
                         const double* d_grad, uint16_t* d_mdig, double* d_mscale,
                         double* d_work, cudaStream_t st);
size_t ozaki_m_bytes(const OzakiPlan& plan);
// slice the per-element D rows into digits (A operand) with row scales
int launch_ozaki_slice_d(const OzakiPlan& plan, int nel, int nint, const double* d_D,
                         uint16_t* d_ddig, double* d_dscale, cudaStream_t st);
size_t ozaki_d_bytes(const OzakiPlan& plan, int nel);
int ozaki_pairs(const OzakiPlan& plan);
// k-blocks (16 q each) per exact accumulation run of the contraction
int ozaki_kchunk(const OzakiPlan& plan);
// the tensor-core contraction: PK = dscale*mscale*sum_s 2^-radix*s acc_s.
// fault = 1 (testing only): the loader withholds one stage, so the bounded
// waits run out and the kernel reports through d_flag instead of finishing.
int launch_ozaki_gemm(const OzakiPlan& plan, int nel, int n, const uint16_t* d_ddig,
                      const double* d_dscale, const uint16_t* d_mdig, const double* d_mscale,
                      double* d_PK, int* d_flag, cudaStream_t st, int fault = 0,
                      int grp = 0);
// The contraction of several bins (same radix and digits) in one persistent
// launch over their joint tile space (split into launches of at most
// OZAKI_MAXBINS bins): out[r, c] = sum_q D[r, q] M[q, c] per bin.
constexpr int OZAKI_MAXBINS = 352;
struct OzakiGemmItem {
  const OzakiPlan* plan;
  int nrows;        // elements (rows of D)
  int ncols_real;   // columns of the output (n(n+1)/2, or a dense plan's nreal)
  const uint16_t* ddig;
  const double* dscale;
  const uint16_t* mdig;
  const double* mscale;
  double* out;
  int grp = 0;      // column blocks per raster group (0 = sized for L2)
};
int launch_ozaki_gemm_group(const OzakiGemmItem* items, int nitems, int* d_flag,
                            cudaStream_t st, int fault = 0);

// the same contraction for a dense bin-constant M (K x ncols, row-major FP64):
// OUT[r, c] = sum_q D[r, q] M[q, c] for rows r of D (K per row)
int ozaki_plan_dense(int K, int ncols, int radix, int digits, OzakiPlan* plan);
int launch_ozaki_build_m_dense(const OzakiPlan& plan, const double* d_M, uint16_t* d_mdig,
                               double* d_mscale, cudaStream_t st);
int launch_ozaki_slice_d_dense(const OzakiPlan& plan, int nrows, const double* d_D,
                               uint16_t* d_ddig, double* d_dscale, cudaStream_t st);
int launch_ozaki_gemm_dense(const OzakiPlan& plan, int nrows, const uint16_t* d_ddig,
                            const double* d_dscale, const uint16_t* d_mdig, const double* d_mscale,
                            double* d_out, int* d_flag, cudaStream_t st);

// constrained approximation (hanging nodes) -- k_constrain.cu
struct ConstrainArgs {
  const int* cidx;                 // per element: constrained index j, or -1
  const int64_t *lcon_off, *elem_nnz;    // final layout
  double *zastif, *zbload;
  const int64_t *wlcon_off, *welem_nnz;  // work layout of the compression
  const double *zwork, *bwork;
  const int* nmod;                 // per constrained element: modified dof
  const int64_t* gptr_off;         // per constrained element: offset of its nmod+1 row pointers
  const int* gptr;                 // row pointers into gk / gv (absolute)
  const int* gk;                   // element interface dof
  const double* gv;                // coefficient
  const int64_t* aux_off;          // scratch nmod x ni per constrained element
  double* aux;
  const int* cnextract;            // final extraction over the modified dof (at lcon_off)
  const int64_t* mdof_off;         // per constrained element: offset into mdir / mzd
  const uint8_t* mdir;             // modified dof is Dirichlet
  const double* mzd;               // Dirichlet values (or nullptr)
};
void launch_constrain(int nel, const ConstrainArgs& a, cudaStream_t st);

// ultraweak DPG Maxwell on hexahedra -- k_dpg.cu
constexpr int DPG_GV = 36;  // doubles per volume point: D1(6) D2(6) wJ^-1(9) wJ/detJ(9) g(6)
struct DpgDims {
  int p, q;            // trial order, test order p + NORD_ADD
  int nEE, nEi, nQ;    // test functions per field, trace functions, L2 functions
  int nr;              // trial dof: 2 nEi + 6 nQ
  int nv, nfp, nip;    // volume points, face points per face (DPG rule), impedance points per face
  double dxidt[6][3][2];  // face parametrisations (face_param)
  double nsign[6];        // outward normal signs (Nsign_param)
};
struct DpgPhys {
  double omega, mu, epsilon, gamma, alpha;
  int ibcflag, isol, icomp;
};
struct DpgTables {
  double *vs = nullptr, *vc = nullptr, *vq = nullptr;     // volume: test values, curls, L2
  double *fs = nullptr, *fscratch = nullptr, *ft = nullptr;  // faces: test values, traces
  double* it = nullptr;                                   // impedance points: traces
};
struct DpgTcBufs {
  uint8_t *a = nullptr, *b = nullptr;  // digit operands (per element dpg_tc_a_bytes / _b_bytes)
  int *ea = nullptr, *eb = nullptr;    // row exponents (per element dpg_tc_ex_slots)
};
struct DpgWork {
  const double *xiV, *wV, *xiF, *wF, *xiI, *wI;
  double *gV, *gF, *gI;            // per element point data
  double *MFF, *MCC, *MFC;         // real Gram parts (MFC per bin)
  double *P, *R, *T, *load;        // real coupling blocks, complex load
  double *G, *S, *Z;               // complex: Gram, [B|l] -> X, DPG matrix (nr+1)^2
  bool tc = false;                 // dense algebra on tensor cores
  DpgTcBufs tb;
  // tensor-core path: augmented matrix (nt + nr + 1)^2 per element, the
  // inverse diagonal blocks of the panels (64 x 64 each), ASchur workspace
  double *M = nullptr, *W = nullptr, *Y = nullptr;
  // M_FF (0) and M_CC (1) as split-BF16 contractions (k_ozaki.cu): the test
  // function tables as bin-constant digit operands, the per-point metrics as
  // per-element rows; MFF / MCC then hold packed upper triangles
  OzakiPlan gplan{};
  uint16_t* gmdig[2] = {nullptr, nullptr};
  double* gmscale[2] = {nullptr, nullptr};
  uint16_t* gddig[2] = {nullptr, nullptr};
  double* gdscale[2] = {nullptr, nullptr};
  double* gD[2] = {nullptr, nullptr};
  // P (0), R (1), T (2) the same way, with dense bin-constant tables:
  // P/R rows (element, component c) over (point, i), T rows per element over
  // (face point, a, b); the dense tables are staged in bMd once per batch
  OzakiPlan bplan[3]{};
  uint16_t* bmdig[3] = {nullptr, nullptr, nullptr};
  double* bmscale[3] = {nullptr, nullptr, nullptr};
  uint16_t* bddig = nullptr;
  double* bdscale = nullptr;
  double *bDP = nullptr, *bDR = nullptr, *bMd = nullptr;
};
// the digit tables of the test functions (once per batch, tensor-core path)
int launch_dpg_gram_tables(const DpgDims& d, const DpgTables& t, const DpgWork& w, cudaStream_t st);
void launch_dpg_tables(const DpgDims& d, const double* xiV, const double* wV, const double* xiF,
                       const double* xiI, const DpgTables& t, double* mfc, cudaStream_t st);
// the dense DPG algebra on tensor cores -- k_dpg_tc.cu
size_t dpg_tc_ex_slots(int rows);
size_t dpg_tc_a_bytes(int rows);
size_t dpg_tc_b_bytes(int rows);
// the augmented partial factorization: part 1 eliminates the test unknowns
// (trailing block -> Z), 2 the L2 fields (-> Schur complement, ASchur), 3
// writes Z in the interface order [E | Q | l] (full) to zkeep.  Returns the
// number of kernels launched, or -1.
int dpg_aug_wslots(int nt, int nq);
int launch_dpg_aug_tc(int part, int nel, int nt, int n1, int nq, const DpgWork& w, double* zkeep,
                      int* bad, int* err, cudaStream_t st);
int launch_dpg_aug_out(int nel, int nt, int n1, int nq, const DpgWork& w, const int* nextract,
                        const int64_t* lcon_off, const int64_t* elem_nnz,
                        const int64_t* schur_off, const int64_t* bub_off, double* zastif,
                        double* zbload, double* aschur, double* bschur, cudaStream_t st);

// stage 0: geometry, real contractions, assembly of G and [B|l];
// 1: Cholesky of G, forward solve, Z = X^H X, impedance penalty;
// 2: condensation of the L2 fields and compression.  Returns the number of
// kernels launched, or -1.
int launch_dpg_stage(int stage, int nel, const DpgDims& d, const DpgPhys& ph,
                      const DpgTables& t, const DpgWork& w, const double* xvert, const double* eps,
                      const int* imp_mask, const uint32_t* perm, const int* nextract,
                      const int64_t* lcon_off, const int64_t* elem_nnz, const int64_t* schur_off,
                      const int64_t* bub_off, double* zastif, double* zbload, double* aschur,
                      double* bschur, double* zkeep, int* flags, cudaStream_t st);

// tuning table (tune.cu): the entry of a bin, the contraction's ring stages
struct TuneRec {
  int etype = 0, n = 0, nb = 0, nint = 0, precision = 0;
  int cond = 0;  // 0 = built-in rule, 1 = fused tensor-core, 2 = FP64 factor +
                 // tensor-core Schur update, 3 = FP64
  int grp = 0;   // contraction raster group (column blocks), 0 = built-in
};
bool tune_lookup(int etype, int n, int nb, int nint, int precision, TuneRec* out);
int tune_nstage();

}  // namespace hp3dg
