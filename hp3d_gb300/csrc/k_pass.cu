// k_pass.cu -- FP64 kernels of the element pass (sm_103a).
//
// Each kernel restates one stage of hp3D's per-element work as a batched
// device pass over one bin (elements with the same type and local orders):
//   k_tables_*      shape3DHHexa / shape3DHTet / shape3DHPris at the
//                   set_3D_int points, once per bin (shape_1/Hexahedron.F90:
//                   33-210, Tetrahedron.F90:33-234, Prism.F90:33-330,
//                   quadrature/set_3D_int.F90)
//   k_orient_*      signed permutation of the element's oriented dof onto the
//                   bin's reference enumeration (shape_1/Orient.F90:9-162)
//   k_geom          geom3D + geom + getf per point (util/geom3D.F90:30-112,
//                   util/geom.F90:30-138, common/getf.F90:63)
//   k_load_hexa     load vector (elem_opt.F90:118)
//   k_contract_fp64 B^T D B in FP64 (elem_opt.F90:86-137 DSYRK)
//   k_condense      static condensation + compression + Dirichlet lift
//                   (modules/stc.F90:182-509, constrs/celem_systemI.F90:800-845)
//   k_index_*       NFIRST_DOF / LCON (solver/omp_mumps/mumps_sc.F90:149-157, 266-299)
#include "hp3dg_internal.cuh"
#include "hp3dg_kernels.h"
#include "hp3dg_simplex.cuh"

#include <math.h>

#include <map>
#include <mutex>
#include <utility>

namespace hp3dg {

cudaError_t raise_smem_limit(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> cur;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  size_t& have = cur[{dev, func}];
  if (bytes <= have) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) have = bytes;
  return e;
}


// ---------------------------------------------------------------------------
// tables
// ---------------------------------------------------------------------------
struct Ord19 { int v[19]; };

__global__ void k_tables_hexa(Ord19 ord, int nint, int n, const double* __restrict__ xi,
                              double* __restrict__ tab_shap, double* __restrict__ tab_grad) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nint) return;
  double x[3] = {xi[3 * l], xi[3 * l + 1], xi[3 * l + 2]};
  // write straight to the tables: shap row l, grad rows (l,c)
  hexa_shape0(x, ord.v, tab_shap + (size_t)l * n, tab_grad + (size_t)l * 3 * n, n);
}

// tetrahedron tables: edge orientation 0, face orientations = the bin's
// orientation classes (fo)
__global__ void k_tables_tet(Ord19 ord, Ord19 fo, int nint, int n, const double* __restrict__ xi,
                             double* __restrict__ tab_shap, double* __restrict__ tab_grad) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nint) return;
  double x[3] = {xi[3 * l], xi[3 * l + 1], xi[3 * l + 2]};
  const int oe[6] = {0, 0, 0, 0, 0, 0};
  tet_shape(x, ord.v, oe, fo.v, tab_shap + (size_t)l * n, tab_grad + (size_t)l * 3 * n, n);
}

// prism tables: edge and quad-face orientation 0, triangle faces in the
// bin's orientation classes (fo[0..1])
__global__ void k_tables_prism(Ord19 ord, Ord19 fo, int nint, int n, const double* __restrict__ xi,
                               double* __restrict__ tab_shap, double* __restrict__ tab_grad) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nint) return;
  double x[3] = {xi[3 * l], xi[3 * l + 1], xi[3 * l + 2]};
  const int oe[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  prism_shape(x, ord.v, oe, fo.v, tab_shap + (size_t)l * n, tab_grad + (size_t)l * 3 * n, n);
}

void launch_tables(int etype, const int* nord_loc, const int* face_nori, int nint, int n,
                   const double* d_xi, double* d_shap, double* d_grad, cudaStream_t st) {
  Ord19 o, f;
  for (int i = 0; i < 19; ++i) o.v[i] = nord_loc[i];
  for (int i = 0; i < 19; ++i) f.v[i] = i < 6 ? face_nori[i] : 0;
  if (etype == ETYPE_TET)
    k_tables_tet<<<(nint + 63) / 64, 64, 0, st>>>(o, f, nint, n, d_xi, d_shap, d_grad);
  else if (etype == ETYPE_PRISM)
    k_tables_prism<<<(nint + 63) / 64, 64, 0, st>>>(o, f, nint, n, d_xi, d_shap, d_grad);
  else
    k_tables_hexa<<<(nint + 63) / 64, 64, 0, st>>>(o, nint, n, d_xi, d_shap, d_grad);
}

// ---------------------------------------------------------------------------
// dof maps: perm[j][a] = bin dof of the element's oriented dof a (bit31 sign)
// ---------------------------------------------------------------------------
__global__ void k_orient_hexa(int nel, const int* __restrict__ elist, const int* __restrict__ norder,
                              const int* __restrict__ nori_e, const int* __restrict__ nori_f,
                              Ord19 full, int nfull, uint32_t* __restrict__ perm) {
  int j = blockIdx.x;
  if (j >= nel) return;
  int e = elist[j];
  __shared__ int no[19], oe[12], of[6];
  if (threadIdx.x < 19) no[threadIdx.x] = norder[19 * e + threadIdx.x];
  if (threadIdx.x < 12) oe[threadIdx.x] = nori_e[12 * e + threadIdx.x];
  if (threadIdx.x < 6) of[threadIdx.x] = nori_f[6 * e + threadIdx.x];
  __syncthreads();
  const int n = hexa_ndof(no);
  for (int a = threadIdx.x; a < nfull; a += blockDim.x)
    perm[(size_t)j * nfull + a] = a < n ? hexa_dof_map(a, no, oe, of, full.v) : 0u;
}

__global__ void k_orient_tet(int nel, const int* __restrict__ elist, const int* __restrict__ norder,
                             const int* __restrict__ nori_e, const int* __restrict__ nori_f, int pm,
                             int nfull, uint32_t* __restrict__ perm) {
  int j = blockIdx.x;
  if (j >= nel) return;
  int e = elist[j];
  __shared__ int no[19], oe[12], of[6];
  if (threadIdx.x < 19) no[threadIdx.x] = norder[19 * e + threadIdx.x];
  if (threadIdx.x < 12) oe[threadIdx.x] = nori_e[12 * e + threadIdx.x];
  if (threadIdx.x < 6) of[threadIdx.x] = nori_f[6 * e + threadIdx.x];
  __syncthreads();
  const int n = tet_ndof(no);
  for (int a = threadIdx.x; a < nfull; a += blockDim.x)
    perm[(size_t)j * nfull + a] = a < n ? tet_dof_map(a, no, oe, of, pm) : 0u;
}

__global__ void k_orient_prism(int nel, const int* __restrict__ elist, const int* __restrict__ norder,
                               const int* __restrict__ nori_e, const int* __restrict__ nori_f,
                               Ord19 full, int nfull, uint32_t* __restrict__ perm) {
  int j = blockIdx.x;
  if (j >= nel) return;
  int e = elist[j];
  __shared__ int no[19], oe[12], of[6];
  if (threadIdx.x < 19) no[threadIdx.x] = norder[19 * e + threadIdx.x];
  if (threadIdx.x < 12) oe[threadIdx.x] = nori_e[12 * e + threadIdx.x];
  if (threadIdx.x < 6) of[threadIdx.x] = nori_f[6 * e + threadIdx.x];
  __syncthreads();
  const int n = prism_ndof(no);
  for (int a = threadIdx.x; a < nfull; a += blockDim.x)
    perm[(size_t)j * nfull + a] = a < n ? prism_dof_map(a, no, oe, of, full.v) : 0u;
}

void launch_orient(int etype, int nel, const int* d_elist, const int* d_norder, const int* d_nori_e,
                   const int* d_nori_f, const int* full, int nfull, uint32_t* d_perm,
                   cudaStream_t st) {
  if (nel <= 0) return;
  if (etype == ETYPE_PRISM) {
    Ord19 o;
    for (int i = 0; i < 19; ++i) o.v[i] = full[i];
    k_orient_prism<<<nel, 128, 0, st>>>(nel, d_elist, d_norder, d_nori_e, d_nori_f, o, nfull, d_perm);
    return;
  }
  if (etype == ETYPE_TET) {
    k_orient_tet<<<nel, 128, 0, st>>>(nel, d_elist, d_norder, d_nori_e, d_nori_f, full[0], nfull,
                                      d_perm);
    return;
  }
  Ord19 o;
  for (int i = 0; i < 19; ++i) o.v[i] = full[i];
  k_orient_hexa<<<nel, 128, 0, st>>>(nel, d_elist, d_norder, d_nori_e, d_nori_f, o, nfull, d_perm);
}

// ---------------------------------------------------------------------------
// geometry: D and F per (element, point)
// ---------------------------------------------------------------------------
__device__ inline double getf_dev(int isol, double x1, double x2, double x3) {
  const double PI = 3.141592653589793238462643383279502884;
  switch (isol) {
    case 0: {
      double fx = pow(x1, 6.0), fy = pow(x2, 6.0), fz = pow(x3, 6.0);
      double ddx = 30.0 * pow(x1, 4.0), ddy = 30.0 * pow(x2, 4.0), ddz = 30.0 * pow(x3, 4.0);
      return -(ddx * fy * fz + fx * ddy * fz + fx * fy * ddz);
    }
    case 1: return 0.0 * sin(x1 * PI) * sinh(x2 * PI);
    case 2: {
      double s = sin(x1 * PI) * sinh(x2 * PI);
      return -(-PI * PI * s * (x3 * x3) + PI * PI * s * (x3 * x3) + 2.0 * s);
    }
    case 10: return 3.0 * PI * PI * sin(PI * x1) * sin(PI * x2) * sin(PI * x3);
    case 11: return 1.0;
    default: return 0.0;
  }
}

// per point: det J (rule of Sarrus), cofactor inverse, D = w kappa detJ
// J^-1 J^-T (upper 00 11 22 01 02 12) and F = getf(x) w detJ (geom.F90:57-113)
__device__ __forceinline__ void geom_point(int e, int j, int l, int nint, const double (&dx)[3][3],
                                           const double (&X)[3], const double* __restrict__ wq,
                                           const double* __restrict__ kappa, int isol,
                                           double* __restrict__ D, double* __restrict__ F,
                                           int* __restrict__ bad) {
  double r = dx[0][0] * dx[1][1] * dx[2][2] + dx[1][0] * dx[2][1] * dx[0][2] +
             dx[2][0] * dx[0][1] * dx[1][2] - dx[2][0] * dx[1][1] * dx[0][2] -
             dx[0][0] * dx[2][1] * dx[1][2] - dx[1][0] * dx[0][1] * dx[2][2];
  if (!(r > 0.0)) atomicMin(bad, e);
  double ir = 1.0 / r;
  double a[3][3];  // a[i][k] = d xi_i / d x_k
  a[0][0] = (dx[1][1] * dx[2][2] - dx[2][1] * dx[1][2]) * ir;
  a[1][0] = (-dx[1][0] * dx[2][2] + dx[2][0] * dx[1][2]) * ir;
  a[2][0] = (dx[1][0] * dx[2][1] - dx[2][0] * dx[1][1]) * ir;
  a[0][1] = (dx[2][1] * dx[0][2] - dx[0][1] * dx[2][2]) * ir;
  a[1][1] = (dx[0][0] * dx[2][2] - dx[2][0] * dx[0][2]) * ir;
  a[2][1] = (-dx[0][0] * dx[2][1] + dx[2][0] * dx[0][1]) * ir;
  a[0][2] = (dx[0][1] * dx[1][2] - dx[1][1] * dx[0][2]) * ir;
  a[1][2] = (-dx[0][0] * dx[1][2] + dx[1][0] * dx[0][2]) * ir;
  a[2][2] = (dx[0][0] * dx[1][1] - dx[1][0] * dx[0][1]) * ir;
  double weight = r * wq[l];
  double kw = kappa[e] * weight;
  double* Dp = D + ((size_t)j * nint + l) * 6;
  Dp[0] = kw * (a[0][0] * a[0][0] + a[0][1] * a[0][1] + a[0][2] * a[0][2]);
  Dp[1] = kw * (a[1][0] * a[1][0] + a[1][1] * a[1][1] + a[1][2] * a[1][2]);
  Dp[2] = kw * (a[2][0] * a[2][0] + a[2][1] * a[2][1] + a[2][2] * a[2][2]);
  Dp[3] = kw * (a[0][0] * a[1][0] + a[0][1] * a[1][1] + a[0][2] * a[1][2]);
  Dp[4] = kw * (a[0][0] * a[2][0] + a[0][1] * a[2][1] + a[0][2] * a[2][2]);
  Dp[5] = kw * (a[1][0] * a[2][0] + a[1][1] * a[2][1] + a[1][2] * a[2][2]);
  F[(size_t)j * nint + l] = getf_dev(isol, X[0], X[1], X[2]) * weight;
}

// x and dx/dxi at point l from the NV vertex functions of the bin tables
template <int NV>
__device__ __forceinline__ void vertex_map(int l, int n, const double* __restrict__ tab_shap,
                                           const double* __restrict__ tab_grad, const double* xv,
                                           double (&dx)[3][3], double (&X)[3]) {
  const double* gs = tab_shap + (size_t)l * n;
  const double* gg = tab_grad + (size_t)l * 3 * n;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    double s = gs[v];
    double g0 = gg[v], g1 = gg[n + v], g2 = gg[2 * n + v];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double xi_ = xv[3 * v + i];
      X[i] += xi_ * s;
      dx[i][0] += xi_ * g0;
      dx[i][1] += xi_ * g1;
      dx[i][2] += xi_ * g2;
    }
  }
}

template <int NV>
__global__ void k_geom(int nel, const int* __restrict__ elist, int nint, int n,
                            const double* __restrict__ wq, const double* __restrict__ tab_shap,
                            const double* __restrict__ tab_grad, const double* __restrict__ xvert,
                            const double* __restrict__ kappa, int isol, double* __restrict__ D,
                            double* __restrict__ F, int* __restrict__ bad) {
  int j = blockIdx.y;
  int e = elist[j];
  __shared__ double xv[24];
  if (threadIdx.x < 24) xv[threadIdx.x] = xvert[(size_t)e * 24 + threadIdx.x];
  __syncthreads();
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nint) return;
  double dx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // dx[i][c] = d x_i / d xi_c
  double X[3] = {0, 0, 0};
  vertex_map<NV>(l, n, tab_shap, tab_grad, xv, dx, X);
  geom_point(e, j, l, nint, dx, X, wq, kappa, isol, D, F, bad);
}

// isoparametric geometry (geom3D.F90:30-112 with the element's nrdofH
// geometry dof Xnod): the dof are mapped to the bin's canonical functions
// through the element's signed dof map, then x and dx/dxi are sums over all
// n functions of the bin tables
__global__ void k_geom_iso(int nel, const int* __restrict__ elist, int nint, int n,
                           const double* __restrict__ wq, const double* __restrict__ tab_shap,
                           const double* __restrict__ tab_grad, const double* __restrict__ xnod,
                           const int64_t* __restrict__ dof_off, const uint32_t* __restrict__ perm,
                           const double* __restrict__ kappa, int isol, double* __restrict__ D,
                           double* __restrict__ F, int* __restrict__ bad) {
  extern __shared__ double xc[];  // 3 x n in the bin's dof order
  const int j = blockIdx.y;
  const int e = elist[j];
  const int64_t o = dof_off[e];
  const int ne = (int)(dof_off[e + 1] - o);
  for (int t = threadIdx.x; t < 3 * n; t += blockDim.x) xc[t] = 0.0;
  __syncthreads();
  for (int a = threadIdx.x; a < ne && a < n; a += blockDim.x) {
    const uint32_t pm = perm[(size_t)j * n + a];
    const int k = (int)(pm & 0x7fffffffu);
    const double sg = (pm >> 31) ? -1.0 : 1.0;
    for (int i = 0; i < 3; ++i) xc[3 * k + i] = sg * xnod[3 * (o + a) + i];
  }
  __syncthreads();
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nint) return;
  double dx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double X[3] = {0, 0, 0};
  const double* gs = tab_shap + (size_t)l * n;
  const double* gg = tab_grad + (size_t)l * 3 * n;
  for (int k = 0; k < n; ++k) {
    const double s = gs[k], g0 = gg[k], g1 = gg[n + k], g2 = gg[2 * n + k];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double xk = xc[3 * k + i];
      X[i] = fma(xk, s, X[i]);
      dx[i][0] = fma(xk, g0, dx[i][0]);
      dx[i][1] = fma(xk, g1, dx[i][1]);
      dx[i][2] = fma(xk, g2, dx[i][2]);
    }
  }
  geom_point(e, j, l, nint, dx, X, wq, kappa, isol, D, F, bad);
}

void launch_geom(int nel, int nvert, const int* d_elist, int nint, int n, const double* d_wq,
                 const double* d_shap, const double* d_grad, const double* d_xvert,
                 const double* d_kappa, int isol, double* d_D, double* d_F, int* d_bad,
                 cudaStream_t st, const double* d_xnod, const int64_t* d_dof_off,
                 const uint32_t* d_perm) {
  if (nel <= 0) return;
  dim3 g((nint + 127) / 128, nel);
  if (d_xnod) {
    k_geom_iso<<<g, 128, (size_t)3 * n * sizeof(double), st>>>(
        nel, d_elist, nint, n, d_wq, d_shap, d_grad, d_xnod, d_dof_off, d_perm, d_kappa, isol, d_D,
        d_F, d_bad);
    return;
  }
  if (nvert == 4)
    k_geom<4><<<g, 128, 0, st>>>(nel, d_elist, nint, n, d_wq, d_shap, d_grad, d_xvert, d_kappa,
                                 isol, d_D, d_F, d_bad);
  else if (nvert == 6)
    k_geom<6><<<g, 128, 0, st>>>(nel, d_elist, nint, n, d_wq, d_shap, d_grad, d_xvert, d_kappa,
                                 isol, d_D, d_F, d_bad);
  else
    k_geom<8><<<g, 128, 0, st>>>(nel, d_elist, nint, n, d_wq, d_shap, d_grad, d_xvert, d_kappa,
                                 isol, d_D, d_F, d_bad);
}

// b0[j][k] = sum_l shap[l][k] F[j][l]   (reference enumeration)
__device__ __forceinline__ void load_elem(int j, int nint, int n, const double* __restrict__ tab_shap,
                                          const double* __restrict__ F, double* __restrict__ b0,
                                          double* fs) {
  for (int l = threadIdx.x; l < nint; l += blockDim.x) fs[l] = F[(size_t)j * nint + l];
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double s = 0.0;
    for (int l = 0; l < nint; ++l) s += tab_shap[(size_t)l * n + k] * fs[l];
    b0[(size_t)j * n + k] = s;
  }
}

__global__ void k_load_hexa(int nint, int n, const double* __restrict__ tab_shap,
                            const double* __restrict__ F, double* __restrict__ b0) {
  extern __shared__ double fs[];
  load_elem(blockIdx.x, nint, n, tab_shap, F, b0, fs);
}

void launch_load_hexa(int nel, int nint, int n, const double* d_shap, const double* d_F,
                      double* d_b0, cudaStream_t st) {
  if (nel > 0) k_load_hexa<<<nel, 256, nint * sizeof(double), st>>>(nint, n, d_shap, d_F, d_b0);
}

// ---------------------------------------------------------------------------
// grouped launches: the per-element stage kernels of many bins in one launch
// ---------------------------------------------------------------------------
// The segment (bin) of block b: pre holds nseg + 1 block offsets.
__device__ __forceinline__ int seg_of(const int* __restrict__ pre, int nseg, int b) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// orientation maps of every element of every bin: one block per element
__global__ void k_orient_grp(const StageSeg* __restrict__ segs, const int* __restrict__ pre,
                             int nseg, int off, const int* __restrict__ norder,
                             const int* __restrict__ nori_e, const int* __restrict__ nori_f) {
  const int blk = blockIdx.x + off;
  const int s = seg_of(pre, nseg, blk);
  const StageSeg& G = segs[s];
  const int j = blk - pre[s];
  const int e = G.elist[j];
  __shared__ int no[19], oe[12], of[6];
  if (threadIdx.x < 19) no[threadIdx.x] = norder[19 * e + threadIdx.x];
  if (threadIdx.x < 12) oe[threadIdx.x] = nori_e[12 * e + threadIdx.x];
  if (threadIdx.x < 6) of[threadIdx.x] = nori_f[6 * e + threadIdx.x];
  __syncthreads();
  const int nfull = G.n;
  uint32_t* perm = G.perm + (size_t)j * nfull;
  if (G.etype == ETYPE_TET) {
    const int n = tet_ndof(no);
    for (int a = threadIdx.x; a < nfull; a += blockDim.x)
      perm[a] = a < n ? tet_dof_map(a, no, oe, of, G.full[0]) : 0u;
  } else if (G.etype == ETYPE_PRISM) {
    const int n = prism_ndof(no);
    for (int a = threadIdx.x; a < nfull; a += blockDim.x)
      perm[a] = a < n ? prism_dof_map(a, no, oe, of, G.full) : 0u;
  } else {
    const int n = hexa_ndof(no);
    for (int a = threadIdx.x; a < nfull; a += blockDim.x)
      perm[a] = a < n ? hexa_dof_map(a, no, oe, of, G.full) : 0u;
  }
}

// geometry (vertex maps): ceil(nint / 128) blocks of 128 points per element
__global__ void k_geom_grp(const StageSeg* __restrict__ segs, const int* __restrict__ pre, int nseg,
                           int off, const double* __restrict__ xvert,
                           const double* __restrict__ kappa, int isol, int* __restrict__ bad) {
  const int blk = blockIdx.x + off;
  const int s = seg_of(pre, nseg, blk);
  const StageSeg& G = segs[s];
  const int nbx = (G.nint + 127) / 128;
  const int loc = blk - pre[s];
  const int j = loc / nbx, bx = loc - j * nbx;
  const int e = G.elist[j];
  __shared__ double xv[24];
  if (threadIdx.x < 24) xv[threadIdx.x] = xvert[(size_t)e * 24 + threadIdx.x];
  __syncthreads();
  const int l = bx * blockDim.x + threadIdx.x;
  if (l >= G.nint) return;
  double dx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double X[3] = {0, 0, 0};
  if (G.nvert == 4) vertex_map<4>(l, G.n, G.shap, G.grad, xv, dx, X);
  else if (G.nvert == 6) vertex_map<6>(l, G.n, G.shap, G.grad, xv, dx, X);
  else vertex_map<8>(l, G.n, G.shap, G.grad, xv, dx, X);
  geom_point(e, j, l, G.nint, dx, X, G.wq, kappa, isol, G.D, G.F, bad);
}

// loads: one block per element, the element's F in shared memory
__global__ void k_load_grp(const StageSeg* __restrict__ segs, const int* __restrict__ pre,
                           int nseg, int off) {
  extern __shared__ double fs[];
  const int blk = blockIdx.x + off;
  const int s = seg_of(pre, nseg, blk);
  const StageSeg& G = segs[s];
  load_elem(blk - pre[s], G.nint, G.n, G.shap, G.F, G.b0, fs);
}

void launch_stage0_grouped(const StageGroup& g, int k0, int k1, const int* d_norder,
                           const int* d_nori_e, const int* d_nori_f, const double* d_xvert,
                           const double* d_kappa, int isol, int* d_bad, cudaStream_t st) {
  if (k1 <= k0) return;
  const int* h = g.h_pre.data();  // host copies: [el | geom | dsc | slice] x (nseg + 1)
  const int ns = g.nseg + 1;
  const int el0 = h[k0], el1 = h[k1], ge0 = h[ns + k0], ge1 = h[ns + k1];
  if (el1 > el0) {
    k_orient_grp<<<el1 - el0, 128, 0, st>>>(g.segs, g.pre_el, g.nseg, el0, d_norder, d_nori_e,
                                            d_nori_f);
    k_geom_grp<<<ge1 - ge0, 128, 0, st>>>(g.segs, g.pre_geom, g.nseg, ge0, d_xvert, d_kappa, isol,
                                          d_bad);
    k_load_grp<<<el1 - el0, 256, (size_t)g.max_nint * sizeof(double), st>>>(g.segs, g.pre_el,
                                                                            g.nseg, el0);
  }
}

// ---------------------------------------------------------------------------
// FP64 contraction: PK[j] = sum_l G_l^T D_l G_l  (64x64 output tiles, I <= J)
// ---------------------------------------------------------------------------
constexpr int CT = 64;      // tile
constexpr int CPTS = 8;     // points per k-chunk
constexpr int CK = 3 * CPTS;

__global__ void __launch_bounds__(256) k_contract_fp64(int nint, int n, int ni, int nb, int ntb,
                                                       const double* __restrict__ tab_grad,
                                                       const double* __restrict__ D,
                                                       double* __restrict__ PK) {
  // decode the upper tile pair (I, J) from blockIdx.x
  int t = blockIdx.x, I = 0;
  while (t >= ntb - I) { t -= ntb - I; ++I; }
  int J = I + t;
  int j = blockIdx.y;
  __shared__ double As[CK][CT];
  __shared__ double Bs[CK][CT];
  __shared__ double Ds[CPTS][6];
  int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s) acc[r][s] = 0.0;
  const double* Dj = D + (size_t)j * nint * 6;
  for (int l0 = 0; l0 < nint; l0 += CPTS) {
    int np = min(CPTS, nint - l0);
    __syncthreads();
    if (threadIdx.x < CPTS * 6) {
      int p = threadIdx.x / 6, c = threadIdx.x % 6;
      Ds[p][c] = (p < np) ? Dj[(size_t)(l0 + p) * 6 + c] : 0.0;
    }
    for (int idx = threadIdx.x; idx < CK * CT; idx += 256) {
      int k = idx / CT, c = idx % CT;
      int p = k / 3;
      int col = I * CT + c;
      As[k][c] = (p < np && col < n) ? tab_grad[((size_t)(l0 + p) * 3 + (k % 3)) * n + col] : 0.0;
    }
    __syncthreads();
    // T rows: T[(p,i)][b] = sum_m D_p[i][m] G[(p,m)][b]
    for (int idx = threadIdx.x; idx < CPTS * CT; idx += 256) {
      int p = idx / CT, c = idx % CT;
      int col = J * CT + c;
      double g0 = 0, g1 = 0, g2 = 0;
      if (p < np && col < n) {
        const double* gp = tab_grad + (size_t)(l0 + p) * 3 * n + col;
        g0 = gp[0]; g1 = gp[n]; g2 = gp[2 * n];
      }
      double d00 = Ds[p][0], d11 = Ds[p][1], d22 = Ds[p][2], d01 = Ds[p][3], d02 = Ds[p][4],
             d12 = Ds[p][5];
      Bs[3 * p + 0][c] = d00 * g0 + d01 * g1 + d02 * g2;
      Bs[3 * p + 1][c] = d01 * g0 + d11 * g1 + d12 * g2;
      Bs[3 * p + 2][c] = d02 * g0 + d12 * g1 + d22 * g2;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < 3 * np; ++k) {
      double av[4], bv[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) av[r] = As[k][ty + 16 * r];
#pragma unroll
      for (int s = 0; s < 4; ++s) bv[s] = Bs[k][tx + 16 * s];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int s = 0; s < 4; ++s) acc[r][s] += av[r] * bv[s];
    }
  }
  double* PKj = PK + (size_t)j * ((size_t)n * (n + 1) / 2);
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      int a = I * CT + ty + 16 * r, b = J * CT + tx + 16 * s;
      if (a < n && b < n && a <= b) PKj[pk_index(a, b, ni, nb)] = acc[r][s];
    }
}

void launch_contract_fp64(int nel, int nint, int n, int ni, int nb, const double* d_grad,
                          const double* d_D, double* d_PK, cudaStream_t st) {
  if (nel <= 0) return;
  int ntb = (n + CT - 1) / CT;
  dim3 g(ntb * (ntb + 1) / 2, nel);
  k_contract_fp64<<<g, 256, 0, st>>>(nint, n, ni, nb, ntb, d_grad, d_D, d_PK);
}

// ---------------------------------------------------------------------------
// condensation + compression (one CTA per element)
// ---------------------------------------------------------------------------
// smem: L (nb*nb, row-major lower) | Ys (nb x (ni+1), [r*(ni+1)+c]) | bi (ni) | yb (nb)
// Cholesky of the SPD bubble block, Y = L^-1 [K_bi | b_b], S = K_ii - Y^T Y,
// Bi = b_i - Y^T y_b, then ASchur = L^-T Y, BSchur = L^-T y_b.
constexpr int CND_THREADS = 256;

__device__ inline void upper_decode(int64_t idx, int& a, int& b) {
  int bb = (int)((sqrtf(8.0f * (float)idx + 1.0f) - 1.0f) * 0.5f);
  while ((int64_t)(bb + 1) * (bb + 2) / 2 <= idx) ++bb;
  while ((int64_t)bb * (bb + 1) / 2 > idx) --bb;
  b = bb;
  a = (int)(idx - (int64_t)bb * (bb + 1) / 2);
}

// celem_systemI compression (constrs/celem_systemI.F90:800-845) of one
// element: Zastif row-major over the extracted dof (NEXTRACT), Zbload with
// the Dirichlet lift bi - S zd over the Dirichlet dof.  S is the element's
// packed upper Schur complement, bi its condensed load.
__device__ inline void compress_out(int e, int j, int ni, int nif, const double* __restrict__ S,
                                    const double* __restrict__ bi, const int* __restrict__ nextract,
                                    const int64_t* __restrict__ lcon_off,
                                    const int64_t* __restrict__ elem_nnz,
                                    const int64_t* __restrict__ zd_off,
                                    const double* __restrict__ zdofd,
                                    const uint8_t* __restrict__ dmask, double* __restrict__ zastif,
                                    double* __restrict__ zbload) {
  const int tid = threadIdx.x;
  {
    const int64_t lo = lcon_off[e];
    const int nc = (int)(lcon_off[e + 1] - lo);
    const int* nx = nextract + lo;
    double* Z = zastif + elem_nnz[e];
    for (int64_t idx = tid; idx < (int64_t)nc * nc; idx += CND_THREADS) {
      int l1 = (int)(idx / nc), l2 = (int)(idx % nc);
      int k1 = nx[l1], k2 = nx[l2];
      int a = k1 < k2 ? k1 : k2, b = k1 < k2 ? k2 : k1;
      Z[idx] = S[(int64_t)b * (b + 1) / 2 + a];
    }
    const double* zd = zdofd ? zdofd + zd_off[e] : nullptr;
    const uint8_t* dm = dmask + (size_t)j * nif;
    for (int l1 = tid; l1 < nc; l1 += CND_THREADS) {
      int k1 = nx[l1];
      double v = bi[k1];
      if (zd) {
        for (int k2 = 0; k2 < ni; ++k2)
          if (dm[k2]) {
            int a = k1 < k2 ? k1 : k2, b = k1 < k2 ? k2 : k1;
            v -= S[(int64_t)b * (b + 1) / 2 + a] * zd[k2];
          }
      }
      zbload[lo + l1] = v;
    }
  }
}


__global__ void __launch_bounds__(CND_THREADS) k_condense(
    int nfull, int nif, int nbf, const int* __restrict__ elist, const int* __restrict__ ni_e,
    const int* __restrict__ nb_e, const double* __restrict__ PK, const double* __restrict__ b0,
    const uint32_t* __restrict__ perm, const int* __restrict__ nextract,
    const int64_t* __restrict__ lcon_off, const int64_t* __restrict__ elem_nnz,
    const int64_t* __restrict__ schur_off, const int64_t* __restrict__ bub_off,
    const int64_t* __restrict__ zd_off, const double* __restrict__ zdofd,
    const uint8_t* __restrict__ dmask, double* __restrict__ Sbuf, double* __restrict__ zastif,
    double* __restrict__ zbload, double* __restrict__ aschur, double* __restrict__ bschur,
    double* __restrict__ Yg, int* __restrict__ bad_spd, TcFactorOut tco) {
  extern __shared__ double sm[];
  const int j = blockIdx.x;
  const int e = elist[j];
  const int ni = ni_e[e], nb = nb_e[e];  // this element's dof (a subset of the bin's)
  const double* PKj = PK + (size_t)j * ((size_t)nfull * (nfull + 1) / 2);
  const uint32_t* pm = perm + (size_t)j * nfull;
  const double* bj = b0 + (size_t)j * nfull;
  const int ld = ni + 1;
  // L and the condensed load live in shared memory; Y = L^-1 [K_bi | b_b]
  // too, unless the bin is too large, then in a global scratch slab (Yg)
  double* L = sm;
  double* Ys = Yg ? Yg + (size_t)j * nbf * (nif + 1) : sm + (size_t)nb * nb;
  double* bi = Yg ? sm + (size_t)nb * nb : Ys + (size_t)nb * ld;
  __shared__ int fail;
  const int tid = threadIdx.x;
  if (tid == 0) fail = 0;
  double* S = Sbuf + (size_t)j * ((size_t)nif * (nif + 1) / 2);
  // ---- gather K_bb and [K_bi | b_b] through the dof map ----
  for (int idx = tid; idx < nb * nb; idx += CND_THREADS) {
    int r = idx / nb, c = idx % nb;
    L[idx] = pk_get(PKj, pm, ni + r, ni + c, nif, nbf);
  }
  for (int idx = tid; idx < nb * ni; idx += CND_THREADS) {
    int c = idx / nb, r = idx % nb;
    Ys[r * ld + c] = pk_get(PKj, pm, ni + r, c, nif, nbf);
  }
  for (int r = tid; r < nb; r += CND_THREADS) {
    uint32_t m = pm[ni + r];
    double v = bj[m & 0x7fffffffu];
    Ys[r * ld + ni] = (m & 0x80000000u) ? -v : v;
  }
  __syncthreads();
  // ---- Cholesky K_bb = L L^T (reciprocals of the pivots kept in rd: the
  // FP64 pipe is the bound, one division per pivot instead of per entry) ----
  __shared__ double rd[128];
  for (int k = 0; k < nb; ++k) {
    if (tid == 0) {
      double d = L[k * nb + k];
      if (!(d > 0.0)) { fail = 1; d = 1.0; }
      d = sqrt(d);
      L[k * nb + k] = d;
      rd[k] = 1.0 / d;
    }
    __syncthreads();
    const double rk = rd[k];
    for (int i = k + 1 + tid; i < nb; i += CND_THREADS) L[i * nb + k] *= rk;
    __syncthreads();
    int m = nb - k - 1;
    for (int idx = tid; idx < m * m; idx += CND_THREADS) {
      int ii = k + 1 + idx / m, jj = k + 1 + idx % m;
      if (jj <= ii) L[ii * nb + jj] -= L[ii * nb + k] * L[jj * nb + k];
    }
    __syncthreads();
  }
  if (fail && tid == 0) atomicMin(bad_spd, e);
  // ---- forward solve, one column per thread ----
  for (int c = tid; c < ld; c += CND_THREADS) {
    for (int r = 0; r < nb; ++r) {
      double s = Ys[r * ld + c];
      for (int k = 0; k < r; ++k) s -= L[r * nb + k] * Ys[k * ld + c];
      Ys[r * ld + c] = s * rd[r];
    }
  }
  __syncthreads();
  // ---- condensed load and Schur complement (upper, col-major) ----
  for (int a = tid; a < ni; a += CND_THREADS) {
    uint32_t ma = pm[a];
    double v = bj[ma & 0x7fffffffu];
    if (ma & 0x80000000u) v = -v;
    double s = 0.0;
    for (int r = 0; r < nb; ++r) s += Ys[r * ld + a] * Ys[r * ld + ni];
    bi[a] = v - s;
  }
  if (tco.ydig) {
    // ---- factor mode: Y's columns as balanced digits for the tensor-core
    // Schur update, the condensed load for the compression kernel ----
    __shared__ int yex[256];
    // column exponents e_c (max |Y[:, c]| = m 2^e_c, m in [0.5, 1)), from the
    // bit patterns: magnitudes of finite doubles order like their bits
    for (int c = tid; c < tco.nr; c += CND_THREADS) {
      unsigned long long mb = 0;
      if (c < ni)
        for (int r = 0; r < nb; ++r) {
          unsigned long long bits = (unsigned long long)__double_as_longlong(Ys[r * ld + c]) &
                                    0x7fffffffffffffffull;
          mb = bits > mb ? bits : mb;
        }
      const int E = (int)(mb >> 52);
      const int ex = mb ? E - 1022 : 0;
      yex[c] = ex;
      tco.yexp[(size_t)j * tco.nr + c] = ex;
    }
    for (int a = tid; a < ni; a += CND_THREADS) tco.bi[(size_t)j * nif + a] = bi[a];
    __syncthreads();
    // balanced digits in integer arithmetic: X = round(Y 2^(radix*D - e_c)),
    // a fixed-point integer below 2^(radix*D) in magnitude, then
    // X = sum_i d_i 2^(radix (D-i)) with |d_1| <= 2^radix, |d_i| <= 2^(radix-1)
    uint8_t* Yd = tco.ydig + (size_t)j * tco.ebytes;
    const int R = tco.radix, DG = tco.digits, half = 1 << (R - 1);
    for (int it = tid; it < tco.nr * tco.nkb * 2; it += CND_THREADS) {
      const int c = it % tco.nr, kg = (it / tco.nr) & 1, kb = it / (2 * tco.nr);
      long long X[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int r = kb * 16 + kg * 8 + t;
        X[t] = 0;
        if (c < ni && r < nb) {
          const long long bits = __double_as_longlong(Ys[r * ld + c]);
          const int E = (int)((bits >> 52) & 0x7ff);
          if (E > 0) {
            const long long M = (bits & 0xfffffffffffffLL) | (1LL << 52);
            const int sh = E - 1075 - yex[c] + R * DG;  // X = M 2^sh
            long long v = 0;
            if (sh >= 0) v = M << sh;
            else if (sh > -54) v = (M + (1LL << (-sh - 1))) >> (-sh);
            X[t] = bits < 0 ? -v : v;
          }
        }
      }
      uint8_t* dst = Yd + (size_t)kb * tco.nr * 32 + (size_t)(c >> 3) * 256 + (size_t)kg * 128 +
                     (size_t)(c & 7) * 16;
      for (int dg = DG - 1; dg >= 0; --dg) {  // least significant digit first
        uint32_t h[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          long long d;
          if (dg > 0) {
            const long long q = (X[t] + half) >> R;  // floor division
            d = X[t] - (q << R);
            X[t] = q;
          } else {
            d = X[t];
          }
          h[t] = __float_as_uint((float)(int)d) >> 16;  // exact in BF16
        }
        uint4 w;
        w.x = h[0] | (h[1] << 16);
        w.y = h[2] | (h[3] << 16);
        w.z = h[4] | (h[5] << 16);
        w.w = h[6] | (h[7] << 16);
        *(uint4*)(dst + (size_t)dg * tco.nkb * tco.nr * 32) = w;
      }
    }
    __syncthreads();  // the backward solve below overwrites Y in place
  } else {
    // ---- Schur complement (upper, col-major), then compression ----
    const int64_t nup = (int64_t)ni * (ni + 1) / 2;
    for (int64_t idx = tid; idx < nup; idx += CND_THREADS) {
      int a, b;
      upper_decode(idx, a, b);
      double v = pk_get(PKj, pm, a, b, nif, nbf);
      double s = 0.0;
      for (int r = 0; r < nb; ++r) s += Ys[r * ld + a] * Ys[r * ld + b];
      S[idx] = v - s;
    }
    __syncthreads();
    compress_out(e, j, ni, nif, S, bi, nextract, lcon_off, elem_nnz, zd_off, zdofd, dmask, zastif,
                 zbload);
  }
  // ---- ASchur = L^-T Y, BSchur = L^-T y_b ----
  for (int c = tid; c < ld; c += CND_THREADS) {
    for (int r = nb - 1; r >= 0; --r) {
      double s = Ys[r * ld + c];
      for (int k = r + 1; k < nb; ++k) s -= L[k * nb + r] * Ys[k * ld + c];
      Ys[r * ld + c] = s * rd[r];
    }
  }
  __syncthreads();
  if (nb > 0) {
    double* AS = aschur + schur_off[e];
    for (int idx = tid; idx < nb * ni; idx += CND_THREADS) {
      int c = idx / nb, r = idx % nb;
      AS[idx] = Ys[r * ld + c];
    }
    for (int r = tid; r < nb; r += CND_THREADS) bschur[bub_off[e] + r] = Ys[r * ld + ni];
  }
}

size_t condense_smem(int ni, int nb) {
  return ((size_t)nb * nb + (size_t)nb * (ni + 1) + ni + nb) * sizeof(double);
}
// shared memory when Y is kept in global memory (large bubble blocks)
size_t condense_smem_small(int ni, int nb) {
  return ((size_t)nb * nb + ni + nb) * sizeof(double);
}

int launch_condense(int nel, int nfull, int nif, int nbf, const int* d_elist, const int* d_ni_e,
                    const int* d_nb_e, const double* d_PK, const double* d_b0,
                    const uint32_t* d_perm, const int* d_nextract, const int64_t* d_lcon_off,
                    const int64_t* d_elem_nnz, const int64_t* d_schur_off,
                    const int64_t* d_bub_off, const int64_t* d_zd_off, const double* d_zdofd,
                    const uint8_t* d_dmask, double* d_S, double* d_zastif, double* d_zbload,
                    double* d_aschur, double* d_bschur, double* d_Yg, int* d_bad_spd,
                    cudaStream_t st, const TcFactorOut* tco) {
  if (nel <= 0) return 0;
  size_t smem = d_Yg ? condense_smem_small(nif, nbf) : condense_smem(nif, nbf);
  if (smem > 227 * 1024) return -2;
  if (raise_smem_limit((const void*)k_condense, smem) != cudaSuccess) return -1;
  TcFactorOut none{};
  k_condense<<<nel, CND_THREADS, smem, st>>>(nfull, nif, nbf, d_elist, d_ni_e, d_nb_e, d_PK, d_b0,
                                              d_perm, d_nextract, d_lcon_off, d_elem_nnz,
                                              d_schur_off, d_bub_off, d_zd_off, d_zdofd, d_dmask,
                                              d_S, d_zastif, d_zbload, d_aschur, d_bschur,
                                              d_Yg, d_bad_spd, tco ? *tco : none);
  return 0;
}

// compression after the tensor-core Schur update: one block per element.
// S = K_ii - W is formed in place (K_ii gathered through the dof map), then
// compressed as in the FP64 path.
__device__ __forceinline__ void compress_elem(
    int j, int nfull, int nif, int nbf, const int* __restrict__ elist, const int* __restrict__ ni_e,
    const double* __restrict__ PK, const uint32_t* __restrict__ perm, double* __restrict__ Wbuf,
    const double* __restrict__ Bi, const int* __restrict__ nextract,
    const int64_t* __restrict__ lcon_off, const int64_t* __restrict__ elem_nnz,
    const int64_t* __restrict__ zd_off, const double* __restrict__ zdofd,
    const uint8_t* __restrict__ dmask, double* __restrict__ zastif, double* __restrict__ zbload) {
  const int e = elist[j];
  const int ni = ni_e[e];
  const double* PKj = PK + (size_t)j * ((size_t)nfull * (nfull + 1) / 2);
  const uint32_t* pm = perm + (size_t)j * nfull;
  double* S = Wbuf + (size_t)j * ((size_t)nif * (nif + 1) / 2);
  const int64_t nup = (int64_t)ni * (ni + 1) / 2;
  for (int64_t idx = threadIdx.x; idx < nup; idx += CND_THREADS) {
    int a, b;
    upper_decode(idx, a, b);
    S[idx] = pk_get(PKj, pm, a, b, nif, nbf) - S[idx];
  }
  __syncthreads();
  compress_out(e, j, ni, nif, S, Bi + (size_t)j * nif, nextract, lcon_off, elem_nnz, zd_off, zdofd,
               dmask, zastif, zbload);
}

__global__ void __launch_bounds__(CND_THREADS) k_compress(
    int nfull, int nif, int nbf, const int* __restrict__ elist, const int* __restrict__ ni_e,
    const double* __restrict__ PK, const uint32_t* __restrict__ perm, double* __restrict__ Wbuf,
    const double* __restrict__ Bi, const int* __restrict__ nextract,
    const int64_t* __restrict__ lcon_off, const int64_t* __restrict__ elem_nnz,
    const int64_t* __restrict__ zd_off, const double* __restrict__ zdofd,
    const uint8_t* __restrict__ dmask, double* __restrict__ zastif, double* __restrict__ zbload) {
  compress_elem(blockIdx.x, nfull, nif, nbf, elist, ni_e, PK, perm, Wbuf, Bi, nextract, lcon_off,
                elem_nnz, zd_off, zdofd, dmask, zastif, zbload);
}

// the same over the segments of a condensation group: one block per element
__global__ void __launch_bounds__(CND_THREADS) k_compress_grp(
    const CompressSeg* __restrict__ segs, const int* __restrict__ pre, int nseg, int off,
    const int* __restrict__ ni_e, const int* __restrict__ nextract,
    const int64_t* __restrict__ lcon_off, const int64_t* __restrict__ elem_nnz,
    const int64_t* __restrict__ zd_off, const double* __restrict__ zdofd,
    double* __restrict__ zastif, double* __restrict__ zbload) {
  const int blk = blockIdx.x + off;
  const int s = seg_of(pre, nseg, blk);
  const CompressSeg& G = segs[s];
  const int j = blk - pre[s];
  if (G.nbf > 0) {
    compress_elem(j, G.nfull, G.nif, G.nbf, G.elist, ni_e, G.PK, G.perm, (double*)G.W, G.bi,
                  nextract, lcon_off, elem_nnz, zd_off, zdofd, G.dmask, zastif, zbload);
    return;
  }
  // no bubbles: S = K_ii and the condensed load b_i, in k_condense's
  // arithmetic (v - 0.0 with an empty bubble sum, which is v)
  extern __shared__ double bsm[];
  const int e = G.elist[j];
  const int ni = ni_e[e];
  const double* PKj = G.PK + (size_t)j * ((size_t)G.nfull * (G.nfull + 1) / 2);
  const uint32_t* pm = G.perm + (size_t)j * G.nfull;
  const double* bj = G.b0 + (size_t)j * G.nfull;
  double* S = (double*)G.W + (size_t)j * ((size_t)G.nif * (G.nif + 1) / 2);
  const int64_t nup = (int64_t)ni * (ni + 1) / 2;
  for (int64_t idx = threadIdx.x; idx < nup; idx += CND_THREADS) {
    int a, b;
    upper_decode(idx, a, b);
    S[idx] = pk_get(PKj, pm, a, b, G.nif, 0);
  }
  for (int a = threadIdx.x; a < ni; a += CND_THREADS) {
    const uint32_t ma = pm[a];
    const double v = bj[ma & 0x7fffffffu];
    bsm[a] = (ma & 0x80000000u) ? -v : v;
  }
  __syncthreads();
  compress_out(e, j, ni, G.nif, S, bsm, nextract, lcon_off, elem_nnz, zd_off, zdofd, G.dmask,
               zastif, zbload);
}

void launch_compress_group(const CondGroup& g, int k0, int k1, const int* d_ni_e,
                           const int* d_nextract, const int64_t* d_lcon_off,
                           const int64_t* d_elem_nnz, const int64_t* d_zd_off,
                           const double* d_zdofd, double* d_zastif, double* d_zbload,
                           cudaStream_t st) {
  if (k1 <= k0) return;
  if (k1 == k0 + 1 && g.h_in[k0].nbf > 0) {
    // one bin or chunk on the tensor-core path: the kernel with the
    // segment's parameters in the launch arguments (the same device body)
    const CondSegIn& q = g.h_in[k0];
    launch_compress(q.nel, q.nfull, q.nif, q.nbf, q.elist, d_ni_e, q.PK, q.perm, q.W, q.t.bi,
                    d_nextract, d_lcon_off, d_elem_nnz, d_zd_off, d_zdofd, q.dmask, d_zastif,
                    d_zbload, st);
    return;
  }
  const int ns = g.nseg + 1;
  const int e0 = g.h_pre[2 * ns + k0], e1 = g.h_pre[2 * ns + k1];
  if (e1 > e0)
    k_compress_grp<<<e1 - e0, CND_THREADS, g.smem_plain, st>>>(g.csegs, g.pre_el, g.nseg, e0, d_ni_e,
                                                    d_nextract, d_lcon_off, d_elem_nnz, d_zd_off,
                                                    d_zdofd, d_zastif, d_zbload);
}

void launch_compress(int nel, int nfull, int nif, int nbf, const int* d_elist, const int* d_ni_e,
                     const double* d_PK, const uint32_t* d_perm, const double* d_W,
                     const double* d_bi, const int* d_nextract, const int64_t* d_lcon_off,
                     const int64_t* d_elem_nnz, const int64_t* d_zd_off, const double* d_zdofd,
                     const uint8_t* d_dmask, double* d_zastif, double* d_zbload, cudaStream_t st) {
  if (nel <= 0) return;
  k_compress<<<nel, CND_THREADS, 0, st>>>(nfull, nif, nbf, d_elist, d_ni_e, d_PK, d_perm,
                                          (double*)d_W, d_bi, d_nextract, d_lcon_off, d_elem_nnz,
                                          d_zd_off, d_zdofd, d_dmask, d_zastif, d_zbload);
}

// ---------------------------------------------------------------------------
// index maps
// ---------------------------------------------------------------------------
__global__ void k_first_visit(int64_t nslots, const int* __restrict__ nodes, int* __restrict__ first) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s < nslots && nodes[s] >= 0) atomicMin(&first[nodes[s]], (int)s);
}

__global__ void k_slot_counts(int64_t nslots, const int* __restrict__ nodes,
                              const int* __restrict__ first, const int* __restrict__ ndofm,
                              int* __restrict__ cnt) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s < nslots) cnt[s] = (nodes[s] >= 0 && first[nodes[s]] == (int)s) ? ndofm[s] : 0;
}

// block-local exclusive scan (1024 per block) + block totals
__global__ void k_scan_local(int64_t n, const int* __restrict__ in, int64_t* __restrict__ out,
                             int64_t* __restrict__ blk) {
  __shared__ int64_t buf[1024];
  int64_t i = blockIdx.x * 1024 + threadIdx.x;
  int64_t v = (i < n) ? in[i] : 0;
  buf[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    int64_t t = (threadIdx.x >= (unsigned)off) ? buf[threadIdx.x - off] : 0;
    __syncthreads();
    buf[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = buf[threadIdx.x] - v;
  if (threadIdx.x == 1023) blk[blockIdx.x] = buf[1023];
}

__global__ void k_scan_blocks(int nb, int64_t* __restrict__ blk, int64_t* __restrict__ total) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int64_t s = 0;
    for (int b = 0; b < nb; ++b) { int64_t t = blk[b]; blk[b] = s; s += t; }
    *total = s;
  }
}

__global__ void k_scan_add(int64_t n, int64_t* __restrict__ out, const int64_t* __restrict__ blk) {
  int64_t i = blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += blk[blockIdx.x];
}

__global__ void k_nfirst(int nnodes, int64_t nslots, const int* __restrict__ first,
                         const int64_t* __restrict__ scan, int* __restrict__ nfirst) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < nnodes) {
    int s = first[g];
    nfirst[g] = (s < 0 || (int64_t)s >= nslots) ? -1 : (int)scan[s];
  }
}

__global__ void k_lcon(int nel, int nnode, const int* __restrict__ nodes, const int* __restrict__ ndofm,
                       const int* __restrict__ nfirst, const int64_t* __restrict__ lcon_off,
                       int* __restrict__ lcon) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  int64_t l = lcon_off[e];
  for (int i = nnode - 1; i >= 0; --i) {
    int g = nodes[(size_t)e * nnode + i];
    if (g < 0) continue;  // padding slot of an element with fewer nodes
    int nd = ndofm[(size_t)e * nnode + i];
    int base = nfirst[g];
    for (int q = 1; q <= nd; ++q) lcon[l++] = base + q;
  }
}

int launch_index_maps(int nel, int nnode, int nnodes_global, const int* d_nodes, const int* d_ndofm,
                      const int64_t* d_lcon_off, int* d_first, int* d_cnt, int64_t* d_scan,
                      int64_t* d_blk, int64_t* d_total, int* d_nfirst, int* d_lcon,
                      cudaStream_t st) {
  int64_t ns = (int64_t)nel * nnode;
  if (ns == 0) return 0;
  // 0x7f7f7f7f exceeds every slot index, so untouched nodes read as unvisited
  cudaMemsetAsync(d_first, 0x7f, sizeof(int) * (size_t)nnodes_global, st);
  k_first_visit<<<(unsigned)((ns + 255) / 256), 256, 0, st>>>(ns, d_nodes, d_first);
  k_slot_counts<<<(unsigned)((ns + 255) / 256), 256, 0, st>>>(ns, d_nodes, d_first, d_ndofm, d_cnt);
  int nblk = (int)((ns + 1023) / 1024);
  k_scan_local<<<nblk, 1024, 0, st>>>(ns, d_cnt, d_scan, d_blk);
  k_scan_blocks<<<1, 32, 0, st>>>(nblk, d_blk, d_total);
  k_scan_add<<<nblk, 1024, 0, st>>>(ns, d_scan, d_blk);
  k_nfirst<<<(nnodes_global + 255) / 256, 256, 0, st>>>(nnodes_global, ns, d_first, d_scan, d_nfirst);
  k_lcon<<<(nel + 127) / 128, 128, 0, st>>>(nel, nnode, d_nodes, d_ndofm, d_nfirst, d_lcon_off, d_lcon);
  return 0;
}

}  // namespace hp3dg
