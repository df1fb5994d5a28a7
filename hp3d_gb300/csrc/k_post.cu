// k_post.cu -- kernels that run after the global solve (sm_103a).
//
//   k_backsub        interface solution -> element dof: xi from the global
//                    vector through LCON/NEXTRACT (Dirichlet dof from the
//                    submitted data), bubbles xb = BSchur - ASchur xi
//                    (modules/stc.F90:529-679 stc_bwd_wrapper / stc_bwd,
//                    solver/frontal/interf/solout.F90:457)
//   k_element_error  squared H1 error and norm per element against the
//                    manufactured solution (element/util/compute_error.F90:
//                    226-360, H1 branch, INTEGRATION = 2 rule)
//   k_adjoint        compliance sensitivities: dJ/dkappa_e and dJ/dx of the
//                    element's vertices (vertex slots beyond the element
//                    type's vertex count are written as zero)
#include "hp3dg_internal.cuh"
#include "hp3dg_kernels.h"

#include <math.h>

namespace hp3dg {

// one block per element
__global__ void k_backsub(const int* __restrict__ elist, const int* __restrict__ ni_e,
                          const int* __restrict__ nb_e, const int* __restrict__ nextract, const int64_t* __restrict__ lcon_off,
                          const int* __restrict__ lcon, const double* __restrict__ xglob,
                          const int64_t* __restrict__ zd_off, const double* __restrict__ zdofd,
                          const int64_t* __restrict__ schur_off, const int64_t* __restrict__ bub_off,
                          const double* __restrict__ aschur, const double* __restrict__ bschur,
                          const int64_t* __restrict__ dof_off, double* __restrict__ dofs) {
  extern __shared__ double xi[];
  const int j = blockIdx.x, e = elist[j];
  const int ni = ni_e[e], nb = nb_e[e];
  double* out = dofs + dof_off[e];
  // Dirichlet (or zero) values first, then the active dof from the solution
  for (int k = threadIdx.x; k < ni; k += blockDim.x) xi[k] = zdofd ? zdofd[zd_off[e] + k] : 0.0;
  __syncthreads();
  const int64_t lo = lcon_off[e];
  const int nc = (int)(lcon_off[e + 1] - lo);
  for (int l = threadIdx.x; l < nc; l += blockDim.x) xi[nextract[lo + l]] = xglob[lcon[lo + l] - 1];
  __syncthreads();
  for (int k = threadIdx.x; k < ni; k += blockDim.x) out[k] = xi[k];
  const double* A = aschur + schur_off[e];  // nb x ni column-major
  const double* B = bschur + bub_off[e];
  for (int r = threadIdx.x; r < nb; r += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < ni; ++k) s += A[(size_t)k * nb + r] * xi[k];
    out[ni + r] = B[r] - s;
  }
}

void launch_backsub(int nel, int nif, const int* d_elist, const int* d_ni_e, const int* d_nb_e,
                    const int* d_nextract, const int64_t* d_lcon_off, const int* d_lcon,
                    const double* d_x, const int64_t* d_zd_off, const double* d_zdofd,
                    const int64_t* d_schur_off, const int64_t* d_bub_off, const double* d_aschur,
                    const double* d_bschur, const int64_t* d_dof_off, double* d_dofs,
                    cudaStream_t st) {
  if (nel <= 0) return;
  k_backsub<<<nel, 128, nif * sizeof(double), st>>>(d_elist, d_ni_e, d_nb_e, d_nextract, d_lcon_off,
                                                    d_lcon, d_x, d_zd_off, d_zdofd, d_schur_off,
                                                    d_bub_off, d_aschur, d_bschur, d_dof_off, d_dofs);
}

// manufactured solutions (common/solution.F90:45-134, plus 10, 12 and 13)
__device__ inline void exact_dev(int isol, const double* X, double& u, double* g) {
  const double PI = 3.141592653589793238462643383279502884;
  double x1 = X[0], x2 = X[1], x3 = X[2];
  u = 0.0; g[0] = g[1] = g[2] = 0.0;
  switch (isol) {
    case 0: {
      double fx = pow(x1, 6.0), fy = pow(x2, 6.0), fz = pow(x3, 6.0);
      u = fx * fy * fz;
      g[0] = 6.0 * pow(x1, 5.0) * fy * fz; g[1] = fx * 6.0 * pow(x2, 5.0) * fz;
      g[2] = fx * fy * 6.0 * pow(x3, 5.0);
      break;
    }
    case 1:
      u = sin(x1 * PI) * sinh(x2 * PI);
      g[0] = PI * cos(x1 * PI) * sinh(x2 * PI); g[1] = PI * sin(x1 * PI) * cosh(x2 * PI);
      break;
    case 2:
      u = sin(x1 * PI) * sinh(x2 * PI) * (x3 * x3);
      g[0] = PI * cos(x1 * PI) * sinh(x2 * PI) * (x3 * x3);
      g[1] = PI * sin(x1 * PI) * cosh(x2 * PI) * (x3 * x3);
      g[2] = 2.0 * sin(x1 * PI) * sinh(x2 * PI) * x3;
      break;
    case 10: {
      double s1 = sin(PI * x1), s2 = sin(PI * x2), s3 = sin(PI * x3);
      u = s1 * s2 * s3;
      g[0] = PI * cos(PI * x1) * s2 * s3; g[1] = PI * s1 * cos(PI * x2) * s3;
      g[2] = PI * s1 * s2 * cos(PI * x3);
      break;
    }
    case 12:
      u = x1 * x2 * x3; g[0] = x2 * x3; g[1] = x1 * x3; g[2] = x1 * x2;
      break;
    case 13:
      u = 1.0 + x1 + 2.0 * x2 + 3.0 * x3; g[0] = 1.0; g[1] = 2.0; g[2] = 3.0;
      break;
    default: break;
  }
}

// geometry at point l from the nvert vertex functions of the bin's tables
__device__ inline double geom_point(const double* xv, int nvert, const double* ts, const double* tg,
                                    int n, double* X, double a[3][3]) {
  double dx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  X[0] = X[1] = X[2] = 0.0;
  for (int v = 0; v < nvert; ++v) {
    double s = ts[v], g0 = tg[v], g1 = tg[n + v], g2 = tg[2 * n + v];
    for (int i = 0; i < 3; ++i) {
      double xi_ = xv[3 * v + i];
      X[i] += xi_ * s; dx[i][0] += xi_ * g0; dx[i][1] += xi_ * g1; dx[i][2] += xi_ * g2;
    }
  }
  double r = dx[0][0] * dx[1][1] * dx[2][2] + dx[1][0] * dx[2][1] * dx[0][2] +
             dx[2][0] * dx[0][1] * dx[1][2] - dx[2][0] * dx[1][1] * dx[0][2] -
             dx[0][0] * dx[2][1] * dx[1][2] - dx[1][0] * dx[0][1] * dx[2][2];
  double ir = 1.0 / r;
  a[0][0] = (dx[1][1] * dx[2][2] - dx[2][1] * dx[1][2]) * ir;
  a[1][0] = (-dx[1][0] * dx[2][2] + dx[2][0] * dx[1][2]) * ir;
  a[2][0] = (dx[1][0] * dx[2][1] - dx[2][0] * dx[1][1]) * ir;
  a[0][1] = (dx[2][1] * dx[0][2] - dx[0][1] * dx[2][2]) * ir;
  a[1][1] = (dx[0][0] * dx[2][2] - dx[2][0] * dx[0][2]) * ir;
  a[2][1] = (-dx[0][0] * dx[2][1] + dx[2][0] * dx[0][1]) * ir;
  a[0][2] = (dx[0][1] * dx[1][2] - dx[1][1] * dx[0][2]) * ir;
  a[1][2] = (-dx[0][0] * dx[1][2] + dx[1][0] * dx[0][2]) * ir;
  a[2][2] = (dx[0][0] * dx[1][1] - dx[1][0] * dx[0][1]) * ir;
  return r;
}

// Element dof in the bin's enumeration: dref[pi(a)] = sign_a dof_a, zero for
// bin dof the element does not have.  Ends with a block barrier.
__device__ inline void to_reference(const double* dof, const uint32_t* pm, int n, int nfull,
                                    double* dref) {
  for (int r = threadIdx.x; r < nfull; r += blockDim.x) dref[r] = 0.0;
  __syncthreads();
  for (int a = threadIdx.x; a < n; a += blockDim.x) {
    uint32_t m = pm[a];
    double v = dof[a];
    dref[m & 0x7fffffffu] = (m & 0x80000000u) ? -v : v;
  }
}

// one block per element, one warp per point (lanes split the dof sum)
__global__ void k_element_error(int nvert, int nint, int n, int isol, const int* __restrict__ elist,
                                const int* __restrict__ n_e,
                                const double* __restrict__ wq, const double* __restrict__ ts,
                                const double* __restrict__ tg, const double* __restrict__ xvert,
                                const uint32_t* __restrict__ perm, const int64_t* __restrict__ dof_off,
                                const double* __restrict__ dofs, double* __restrict__ err2,
                                double* __restrict__ nrm2) {
  extern __shared__ double dref[];
  __shared__ double xv[24];
  __shared__ double red[2][32];
  const int j = blockIdx.x, e = elist[j];
  if (threadIdx.x < 24) xv[threadIdx.x] = xvert[(size_t)e * 24 + threadIdx.x];
  to_reference(dofs + dof_off[e], perm + (size_t)j * n, n_e[e], n, dref);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  double e2 = 0.0, r2 = 0.0;
  for (int l = warp; l < nint; l += nw) {
    const double* s = ts + (size_t)l * n;
    const double* g = tg + (size_t)l * 3 * n;
    double u = 0.0, gu[3] = {0, 0, 0};
    for (int r = lane; r < n; r += 32) {
      double d = dref[r];
      u += d * s[r]; gu[0] += d * g[r]; gu[1] += d * g[n + r]; gu[2] += d * g[2 * n + r];
    }
    for (int o = 16; o > 0; o >>= 1) {
      u += __shfl_xor_sync(0xffffffffu, u, o);
      for (int c = 0; c < 3; ++c) gu[c] += __shfl_xor_sync(0xffffffffu, gu[c], o);
    }
    if (lane == 0) {
      double X[3], a[3][3];
      double rjac = geom_point(xv, nvert, s, g, n, X, a);
      double gx[3];
      for (int c = 0; c < 3; ++c) gx[c] = gu[0] * a[0][c] + gu[1] * a[1][c] + gu[2] * a[2][c];
      double ue, ge[3];
      exact_dev(isol, X, ue, ge);
      double w = wq[l] * rjac;
      for (int c = 0; c < 3; ++c) { e2 += (ge[c] - gx[c]) * (ge[c] - gx[c]) * w; r2 += ge[c] * ge[c] * w; }
      e2 += (ue - u) * (ue - u) * w;
      r2 += ue * ue * w;
    }
  }
  if (lane == 0) { red[0][warp] = e2; red[1][warp] = r2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < nw; ++w) { a += red[0][w]; b += red[1][w]; }
    err2[e] = a;
    nrm2[e] = b;
  }
}

void launch_element_error(int nel, int nvert, int nint, int n, int isol, const int* d_elist,
                          const int* d_n_e,
                          const double* d_wq,
                          const double* d_shap, const double* d_grad, const double* d_xvert,
                          const uint32_t* d_perm, const int64_t* d_dof_off, const double* d_dofs,
                          double* d_err2, double* d_nrm2, cudaStream_t st) {
  if (nel <= 0) return;
  k_element_error<<<nel, 256, n * sizeof(double), st>>>(nvert, nint, n, isol, d_elist, d_n_e, d_wq, d_shap, d_grad,
                                                        d_xvert, d_perm, d_dof_off, d_dofs, d_err2,
                                                        d_nrm2);
}

// ---------------------------------------------------------------------------
// adjoint: compliance J = b^T u (K u = b, lambda = u)
//   dJ/dkappa_e = -u_e^T (K_e / kappa_e) u_e
//   dJ/dX_{v,k} = -u_e^T (dK_e/dX_{v,k}) u_e + 2 u_e^T (db_e/dX_{v,k})
// per point: e = kappa w detJ |J^-T g|^2 with g = G_l u_e (reference
// gradient), v = J^-T g, q = J^-1 v:
//   de/dJ_{ij} = kappa w detJ ( (J^-1)_{ji} |v|^2 - 2 v_i q_j )
// load: b = sum_l phi f(x_l) w detJ; with u_h(l) = phi_l . u_e:
//   d(u_h f w detJ)/dJ_{ij} = u_h w ( f detJ (J^-1)_{ji} ) + u_h w detJ (df/dx_i) phi_v-part
// J_{ij} = sum_v X_{v,i} dphi_v/dxi_j, x_i = sum_v X_{v,i} phi_v.
// ---------------------------------------------------------------------------
__device__ inline void source_grad(int isol, const double* X, double& f, double* df) {
  const double PI = 3.141592653589793238462643383279502884;
  df[0] = df[1] = df[2] = 0.0;
  switch (isol) {
    case 10: {
      double s1 = sin(PI * X[0]), s2 = sin(PI * X[1]), s3 = sin(PI * X[2]);
      double c = 3.0 * PI * PI;
      f = c * s1 * s2 * s3;
      df[0] = c * PI * cos(PI * X[0]) * s2 * s3;
      df[1] = c * PI * s1 * cos(PI * X[1]) * s3;
      df[2] = c * PI * s1 * s2 * cos(PI * X[2]);
      break;
    }
    case 11: f = 1.0; break;
    default: f = 0.0; break;
  }
}

__global__ void k_adjoint(int nvert, int nint, int n, int isol, const int* __restrict__ elist,
                          const int* __restrict__ n_e,
                          const double* __restrict__ wq, const double* __restrict__ ts,
                          const double* __restrict__ tg, const double* __restrict__ xvert,
                          const double* __restrict__ kappa, const uint32_t* __restrict__ perm,
                          const int64_t* __restrict__ dof_off, const double* __restrict__ dofs,
                          double* __restrict__ djdk, double* __restrict__ djdx) {
  extern __shared__ double dref[];
  __shared__ double xv[24];
  __shared__ double red[8][25];
  const int j = blockIdx.x, e = elist[j];
  if (threadIdx.x < 24) xv[threadIdx.x] = xvert[(size_t)e * 24 + threadIdx.x];
  to_reference(dofs + dof_off[e], perm + (size_t)j * n, n_e[e], n, dref);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const double kap = kappa[e];
  double acc[25];  // [0] energy/kappa, [1..24] dJ/dX
  for (int i = 0; i < 25; ++i) acc[i] = 0.0;
  for (int l = warp; l < nint; l += nw) {
    const double* s = ts + (size_t)l * n;
    const double* g = tg + (size_t)l * 3 * n;
    double u = 0.0, gu[3] = {0, 0, 0};
    for (int r = lane; r < n; r += 32) {
      double d = dref[r];
      u += d * s[r]; gu[0] += d * g[r]; gu[1] += d * g[n + r]; gu[2] += d * g[2 * n + r];
    }
    for (int o = 16; o > 0; o >>= 1) {
      u += __shfl_xor_sync(0xffffffffu, u, o);
      for (int c = 0; c < 3; ++c) gu[c] += __shfl_xor_sync(0xffffffffu, gu[c], o);
    }
    if (lane == 0) {
      double X[3], a[3][3];  // a = J^-1: a[i][k] = dxi_i/dx_k
      double det = geom_point(xv, nvert, s, g, n, X, a);
      double w = wq[l];
      double v[3], q[3];
      for (int c = 0; c < 3; ++c) v[c] = gu[0] * a[0][c] + gu[1] * a[1][c] + gu[2] * a[2][c];
      for (int c = 0; c < 3; ++c) q[c] = a[c][0] * v[0] + a[c][1] * v[1] + a[c][2] * v[2];
      double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      acc[0] += w * det * vv;  // energy density without kappa
      double f, df[3];
      source_grad(isol, X, f, df);
      // dJ/dJ_{ik} (matrix T): stiffness part (with the minus sign) + load part
      double T[3][3];
      for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k)
          T[i][k] = -kap * w * det * (a[k][i] * vv - 2.0 * v[i] * q[k]) +
                    2.0 * u * w * f * det * a[k][i];
      for (int vtx = 0; vtx < nvert; ++vtx) {
        double gv[3] = {g[vtx], g[n + vtx], g[2 * n + vtx]};
        for (int i = 0; i < 3; ++i) {
          double t = T[i][0] * gv[0] + T[i][1] * gv[1] + T[i][2] * gv[2];
          t += 2.0 * u * w * det * df[i] * s[vtx];  // d f(x_l) / d X_{vtx,i}
          acc[1 + 3 * vtx + i] += t;
        }
      }
    }
  }
  if (lane == 0)
    for (int i = 0; i < 25; ++i) red[warp][i] = acc[i];
  __syncthreads();
  if (threadIdx.x < 25) {
    double sum = 0.0;
    for (int w = 0; w < nw; ++w) sum += red[w][threadIdx.x];
    if (threadIdx.x == 0) djdk[e] = -sum;  // -u^T (K/kappa) u
    else djdx[(size_t)e * 24 + threadIdx.x - 1] = sum;
  }
}

void launch_adjoint(int nel, int nvert, int nint, int n, int isol, const int* d_elist,
                    const int* d_n_e,
                    const double* d_wq,
                    const double* d_shap, const double* d_grad, const double* d_xvert,
                    const double* d_kappa, const uint32_t* d_perm, const int64_t* d_dof_off,
                    const double* d_dofs, double* d_djdk, double* d_djdx, cudaStream_t st) {
  if (nel <= 0) return;
  k_adjoint<<<nel, 256, n * sizeof(double), st>>>(nvert, nint, n, isol, d_elist, d_n_e, d_wq, d_shap, d_grad,
                                                  d_xvert, d_kappa, d_perm, d_dof_off, d_dofs, d_djdk,
                                                  d_djdx);
}

// ---------------------------------------------------------------------------
// Dirichlet data by projection-based interpolation (update_Ddof.F90:70-250):
// vertex values (dhpvert.F90), then tangential H1-seminorm projections on
// the boundary edges (edge/dhpedgeH.F90) and faces (face/dhpfaceH.F90) of
// what the lower-order part leaves, in the element's reference coordinates
// (the element is its own geometry block: eta = xi, x(eta) trilinear).  The
// values depend only on the node's trace, so every element computes its own
// boundary nodes; one thread per element.  Output per interface dof in
// element order (zeros on non-Dirichlet nodes).
// ---------------------------------------------------------------------------
namespace {

__device__ inline int lu_small(int n, double* A, double* b) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (fabs(A[i + n * k]) > fabs(A[p + n * k])) p = i;
    if (A[p + n * k] == 0.0) return -1;
    if (p != k) {
      for (int j = 0; j < n; ++j) { double t = A[k + n * j]; A[k + n * j] = A[p + n * j]; A[p + n * j] = t; }
      double t = b[k]; b[k] = b[p]; b[p] = t;
    }
    for (int i = k + 1; i < n; ++i) {
      double f = A[i + n * k] / A[k + n * k];
      A[i + n * k] = f;
      for (int j = k + 1; j < n; ++j) A[i + n * j] -= f * A[k + n * j];
      b[i] -= f * b[k];
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    double t = b[k];
    for (int j = k + 1; j < n; ++j) t -= A[k + n * j] * b[j];
    b[k] = t / A[k + n * k];
  }
  return 0;
}

__device__ const double DBRICK_XI[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                           {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
__device__ const int DBRICK_E2V[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6},
                                          {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
__device__ const int DBRICK_F2V[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                         {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}};
__device__ const int DBRICK_F2E[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 9, 4, 8},
                                         {1, 10, 5, 9}, {2, 10, 6, 11}, {3, 11, 7, 8}};

// gradient (in xi) of the element's oriented function a at xi, from the
// reference-enumeration gradients of the element's local orders
__device__ inline void grad_oriented(int a, const int* nord, const int* ne, const int* nf,
                                     const int* loc, const double* grad, double* g) {
  const uint32_t m = hexa_dof_map(a, nord, ne, nf, loc);
  const int r = (int)(m & 0x7fffffffu);
  const double sg = (m >> 31) ? -1.0 : 1.0;
  for (int c = 0; c < 3; ++c) g[c] = sg * grad[c * MAXN + r];
}

__device__ void trilin_dev(const double* xv, const double* xi, double* x, double J[3][3]) {
  double Mu[2][3];
  for (int a = 0; a < 3; ++a) { Mu[0][a] = 1.0 - xi[a]; Mu[1][a] = xi[a]; }
  for (int i = 0; i < 3; ++i) {
    x[i] = 0.0;
    for (int j = 0; j < 3; ++j) J[i][j] = 0.0;
  }
  for (int v = 0; v < 8; ++v) {
    const int s0 = hexa_v(v, 0), s1 = hexa_v(v, 1), s2 = hexa_v(v, 2);
    const double b0 = Mu[s0][0], b1 = Mu[s1][1], b2 = Mu[s2][2];
    const double gg[3] = {(s0 ? 1.0 : -1.0) * b1 * b2, b0 * (s1 ? 1.0 : -1.0) * b2,
                          b0 * b1 * (s2 ? 1.0 : -1.0)};
    for (int i = 0; i < 3; ++i) {
      x[i] += xv[3 * v + i] * b0 * b1 * b2;
      for (int j = 0; j < 3; ++j) J[i][j] += xv[3 * v + i] * gg[j];
    }
  }
}

__global__ void k_dirichlet(int nel, const int* __restrict__ norder, const int* __restrict__ nori_e,
                            const int* __restrict__ nori_f, const int* __restrict__ nodes_bc,
                            const double* __restrict__ xvert, const int64_t* __restrict__ zd_off,
                            const double* __restrict__ gx, const double* __restrict__ gw,
                            int isol, double* __restrict__ work, double* __restrict__ zdofd,
                            int* __restrict__ bad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  const int* bc = nodes_bc + (size_t)26 * e;
  bool any = false;
  for (int i = 0; i < 26; ++i) any |= bc[i] != 0;
  double* zd = zdofd + zd_off[e];
  const int ni = (int)(zd_off[e + 1] - zd_off[e]);
  for (int k = 0; k < ni; ++k) zd[k] = 0.0;
  if (!any) return;
  int nord[19], ne[12], nf[6], loc[19];
  for (int i = 0; i < 19; ++i) nord[i] = norder[19 * (size_t)e + i];
  for (int i = 0; i < 12; ++i) ne[i] = nori_e[12 * (size_t)e + i];
  for (int i = 0; i < 6; ++i) nf[i] = nori_f[6 * (size_t)e + i];
  hexa_order_loc(nord, nf, loc);
  const double* xv = xvert + (size_t)24 * e;
  // per-thread scratch: shape values and gradients, the small system
  double* shap = work + (size_t)e * (4 * MAXN + 64 * 64 + 64);
  double* grad = shap + MAXN;
  double* A = grad + 3 * MAXN;
  double* rhs = A + 64 * 64;
  int nd[26], first[27];
  first[0] = 0;
  for (int i = 0; i < 26; ++i) {
    if (i < 8) nd[i] = 1;
    else if (i < 20) nd[i] = nord[i - 8] > 1 ? nord[i - 8] - 1 : 0;
    else { int a, b; decod2(nord[12 + i - 20], a, b); nd[i] = (a > 1 && b > 1) ? (a - 1) * (b - 1) : 0; }
    first[i + 1] = first[i] + nd[i];
  }
  for (int v = 0; v < 8; ++v)
    if (bc[v]) {
      double u, g[3];
      exact_dev(isol, &xv[3 * v], u, g);
      zd[v] = u;
    }
  // edges, then faces (the faces subtract the edges' values)
  for (int node = 8; node < 26; ++node) {
    const int n = nd[node];
    if (!bc[node] || n == 0) continue;
    const bool edge = node < 20;
    const int id = edge ? node - 8 : node - 20;
    int nx, ny;
    double x1[3], t1[3], t2[3];
    if (edge) {
      const int p = nord[id];
      nx = min(p + 1, MAXP) + 1;
      ny = 1;
      for (int c = 0; c < 3; ++c) {
        x1[c] = DBRICK_XI[DBRICK_E2V[id][0]][c];
        t1[c] = DBRICK_XI[DBRICK_E2V[id][1]][c] - x1[c];
        t2[c] = 0.0;
      }
    } else {
      int h, v; decod2(nord[12 + id], h, v);
      const int* fe = DBRICK_F2E[id];
      nx = min(max(max(nord[fe[0]], nord[fe[2]]), h) + 1, MAXP) + 1;
      ny = min(max(max(nord[fe[1]], nord[fe[3]]), v) + 1, MAXP) + 1;
      for (int c = 0; c < 3; ++c) {
        x1[c] = DBRICK_XI[DBRICK_F2V[id][0]][c];
        t1[c] = DBRICK_XI[DBRICK_F2V[id][1]][c] - x1[c];
        t2[c] = DBRICK_XI[DBRICK_F2V[id][3]][c] - x1[c];
      }
    }
    // the lower part: vertices (edges) or vertices and all edges (faces)
    const int nlow = edge ? 8 : first[20];
    const int a0 = first[node];
    for (int q = 0; q < n * n; ++q) A[q] = 0.0;
    for (int q = 0; q < n; ++q) rhs[q] = 0.0;
    double rn[3] = {t1[1] * t2[2] - t1[2] * t2[1], t1[2] * t2[0] - t1[0] * t2[2],
                    t1[0] * t2[1] - t1[1] * t2[0]};
    double bjac;
    if (edge) {
      bjac = sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
      for (int c = 0; c < 3; ++c) rn[c] = t1[c] / bjac;  // the unit tangent
    } else {
      bjac = sqrt(rn[0] * rn[0] + rn[1] * rn[1] + rn[2] * rn[2]);
      for (int c = 0; c < 3; ++c) rn[c] /= bjac;  // the unit normal (its sign is immaterial)
    }
    for (int l2 = 0; l2 < ny; ++l2)
      for (int l1 = 0; l1 < nx; ++l1) {
        const double s1 = gx[16 * nx + l1], s2 = edge ? 0.0 : gx[16 * ny + l2];
        const double w = gw[16 * nx + l1] * (edge ? 1.0 : gw[16 * ny + l2]) * bjac;
        double xi[3];
        for (int c = 0; c < 3; ++c) xi[c] = x1[c] + s1 * t1[c] + s2 * t2[c];
        hexa_shape0(xi, loc, shap, grad, MAXN);
        double x[3], J[3][3];
        trilin_dev(xv, xi, x, J);
        double u, gu[3];
        exact_dev(isol, x, u, gu);
        double du[3];
        for (int i = 0; i < 3; ++i) du[i] = gu[0] * J[0][i] + gu[1] * J[1][i] + gu[2] * J[2][i];
        for (int k = 0; k < nlow; ++k) {
          if (zd[k] == 0.0) continue;
          double g[3];
          grad_oriented(k, nord, ne, nf, loc, grad, g);
          for (int i = 0; i < 3; ++i) du[i] -= zd[k] * g[i];
        }
        for (int j = 0; j < n; ++j) {
          double gj[3], dv[3];
          grad_oriented(a0 + j, nord, ne, nf, loc, grad, gj);
          const double pr = gj[0] * rn[0] + gj[1] * rn[1] + gj[2] * rn[2];
          for (int c = 0; c < 3; ++c) dv[c] = edge ? pr * rn[c] : gj[c] - pr * rn[c];
          rhs[j] += (du[0] * dv[0] + du[1] * dv[1] + du[2] * dv[2]) * w;
          for (int i = 0; i < n; ++i) {
            double gi[3];
            grad_oriented(a0 + i, nord, ne, nf, loc, grad, gi);
            A[j + n * i] += (dv[0] * gi[0] + dv[1] * gi[1] + dv[2] * gi[2]) * w;
          }
        }
      }
    if (lu_small(n, A, rhs)) { atomicMin(bad, e); return; }
    for (int j = 0; j < n; ++j) zd[a0 + j] = rhs[j];
  }
}

// ---------------------------------------------------------------------------
// geometry dof by projection-based interpolation of a geometry-block map
// (update_gdof.F90:80-200 and 404-435; hpvert / hpedge / hpface / hpmdle),
// hexahedra.  The host evaluates its block maps x(eta), dx/deta at the
// points of hp3dg_gdof_points; here, one thread per element, each node's dof
// solve the eta-space H1 projection of what the lower-order dof leave:
// tangential derivative on edges, surface gradient on faces, full gradient
// in the interior.  Phase 0: vertices and edges; 1: faces; 2: the interior.
// Between phases every node takes the values of the first element (in batch
// order) that contains it, as the reference projects each node once.
// ---------------------------------------------------------------------------
__device__ inline int lu_small3(int n, double* A, double* b) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (fabs(A[i + n * k]) > fabs(A[p + n * k])) p = i;
    if (A[p + n * k] == 0.0) return -1;
    if (p != k) {
      for (int j = 0; j < n; ++j) { double t = A[k + n * j]; A[k + n * j] = A[p + n * j]; A[p + n * j] = t; }
      for (int c = 0; c < 3; ++c) { double t = b[c * n + k]; b[c * n + k] = b[c * n + p]; b[c * n + p] = t; }
    }
    for (int i = k + 1; i < n; ++i) {
      const double f = A[i + n * k] / A[k + n * k];
      A[i + n * k] = f;
      for (int j = k + 1; j < n; ++j) A[i + n * j] -= f * A[k + n * j];
      for (int c = 0; c < 3; ++c) b[c * n + i] -= f * b[c * n + k];
    }
  }
  for (int c = 0; c < 3; ++c)
    for (int k = n - 1; k >= 0; --k) {
      double t = b[c * n + k];
      for (int j = k + 1; j < n; ++j) t -= A[k + n * j] * b[c * n + j];
      b[c * n + k] = t / A[k + n * k];
    }
  return 0;
}

__device__ inline void inv3(const double J[3][3], double Ji[3][3], double& det) {
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const double r = 1.0 / det;
  Ji[0][0] = c00 * r; Ji[1][0] = c01 * r; Ji[2][0] = c02 * r;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
}

// dof count of node i (0..7 vertices, 8..19 edges, 20..25 faces, 26 the
// interior) of a hexahedron, and the element dof of its first function
__device__ inline int hexa_node_n(const int* nord, int i) {
  if (i < 8) return 1;
  if (i < 20) return nord[i - 8] > 1 ? nord[i - 8] - 1 : 0;
  if (i < 26) {
    int a, b;
    decod2(nord[12 + i - 20], a, b);
    return (a > 1 && b > 1) ? (a - 1) * (b - 1) : 0;
  }
  int x, y, z;
  decod3(nord[18], x, y, z);
  return (x > 1 && y > 1 && z > 1) ? (x - 1) * (y - 1) * (z - 1) : 0;
}
__device__ inline int hexa_node_a0(const int* nord, int i) {
  int s = 0;
  for (int k = 0; k < i; ++k) s += hexa_node_n(nord, k);
  return s;
}

__global__ void k_gdof(int phase, int e0, int e1, const int* __restrict__ norder,
                       const int* __restrict__ nori_e, const int* __restrict__ nori_f,
                       const double* __restrict__ etav, const int64_t* __restrict__ node_pt,
                       const double* __restrict__ pts, const double* __restrict__ xg,
                       const double* __restrict__ jg, const int* __restrict__ linear,
                       const int64_t* __restrict__ dof_off, double* __restrict__ xnod,
                       double* __restrict__ work, int64_t wstride, int* __restrict__ bad) {
  const int e = e0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= e1) return;
  int nord[19], ne[12], nf[6], loc[19];
  for (int i = 0; i < 19; ++i) nord[i] = norder[19 * (size_t)e + i];
  for (int i = 0; i < 12; ++i) ne[i] = nori_e[12 * (size_t)e + i];
  for (int i = 0; i < 6; ++i) nf[i] = nori_f[6 * (size_t)e + i];
  hexa_order_loc(nord, nf, loc);
  const double* ev = etav + (size_t)24 * e;
  const int64_t* np = node_pt + (size_t)28 * e;
  double* X = xnod + 3 * dof_off[e];
  double* shap = work + (size_t)(e - e0) * wstride;
  double* grad = shap + MAXN;
  double* A = grad + 3 * MAXN;
  if (phase == 0) {
    for (int v = 0; v < 8; ++v)
      for (int c = 0; c < 3; ++c) X[3 * v + c] = xg[3 * np[v] + c];
    const int ndof = hexa_node_a0(nord, 27);
    for (int k = 3 * 8; k < 3 * ndof; ++k) X[k] = 0.0;
  }
  if (linear && linear[e]) return;
  const int n0 = phase == 0 ? 8 : (phase == 1 ? 20 : 26);
  const int n1 = phase == 0 ? 20 : (phase == 1 ? 26 : 27);
  for (int node = n0; node < n1; ++node) {
    const int n = hexa_node_n(nord, node);
    if (n == 0) continue;
    const int kind = node < 20 ? 0 : (node < 26 ? 1 : 2);
    const int a0 = hexa_node_a0(nord, node);
    const int nlow = kind == 0 ? 8 : hexa_node_a0(nord, node < 26 ? 20 : 26);
    double* b = A + (size_t)n * n;
    for (int q = 0; q < n * n; ++q) A[q] = 0.0;
    for (int q = 0; q < 3 * n; ++q) b[q] = 0.0;
    double t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
    if (kind == 0) {
      const int id = node - 8;
      for (int c = 0; c < 3; ++c)
        t1[c] = DBRICK_XI[DBRICK_E2V[id][1]][c] - DBRICK_XI[DBRICK_E2V[id][0]][c];
    } else if (kind == 1) {
      const int id = node - 20;
      for (int c = 0; c < 3; ++c) {
        t1[c] = DBRICK_XI[DBRICK_F2V[id][1]][c] - DBRICK_XI[DBRICK_F2V[id][0]][c];
        t2[c] = DBRICK_XI[DBRICK_F2V[id][3]][c] - DBRICK_XI[DBRICK_F2V[id][0]][c];
      }
    }
    for (int64_t l = np[node]; l < np[node + 1]; ++l) {
      const double* pq = pts + 4 * l;
      const double xi[3] = {pq[0], pq[1], pq[2]};
      hexa_shape0(xi, loc, shap, grad, MAXN);
      double eta[3], J[3][3], Ji[3][3], det;
      trilin_dev(ev, xi, eta, J);  // eta(xi) and d eta / d xi (refgeom3D)
      inv3(J, Ji, det);
      double w = pq[3], rv[3] = {0, 0, 0};
      if (kind == 0) {
        for (int i = 0; i < 3; ++i) rv[i] = J[i][0] * t1[0] + J[i][1] * t1[1] + J[i][2] * t1[2];
        const double bj = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
        for (int i = 0; i < 3; ++i) rv[i] /= bj;
        w *= bj;
      } else if (kind == 1) {
        double a1[3], a2[3];
        for (int i = 0; i < 3; ++i) {
          a1[i] = J[i][0] * t1[0] + J[i][1] * t1[1] + J[i][2] * t1[2];
          a2[i] = J[i][0] * t2[0] + J[i][1] * t2[1] + J[i][2] * t2[2];
        }
        rv[0] = a1[1] * a2[2] - a1[2] * a2[1];
        rv[1] = a1[2] * a2[0] - a1[0] * a2[2];
        rv[2] = a1[0] * a2[1] - a1[1] * a2[0];
        const double bj = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
        for (int i = 0; i < 3; ++i) rv[i] /= bj;  // the unit normal (its sign is immaterial)
        w *= bj;
      } else {
        w *= det;
      }
      // what the lower-order dof leave of dx/deta
      double R[3][3];
      for (int c = 0; c < 3; ++c)
        for (int i = 0; i < 3; ++i) R[c][i] = jg[9 * l + 3 * c + i];
      for (int k = 0; k < nlow; ++k) {
        double gx[3], g[3];
        grad_oriented(k, nord, ne, nf, loc, grad, gx);
        for (int i = 0; i < 3; ++i) g[i] = gx[0] * Ji[0][i] + gx[1] * Ji[1][i] + gx[2] * Ji[2][i];
        for (int c = 0; c < 3; ++c) {
          const double xk = X[3 * k + c];
          for (int i = 0; i < 3; ++i) R[c][i] -= xk * g[i];
        }
      }
      for (int j = 0; j < n; ++j) {
        double gx[3], dv[3];
        grad_oriented(a0 + j, nord, ne, nf, loc, grad, gx);
        for (int i = 0; i < 3; ++i) dv[i] = gx[0] * Ji[0][i] + gx[1] * Ji[1][i] + gx[2] * Ji[2][i];
        if (kind == 0) {
          const double pr = dv[0] * rv[0] + dv[1] * rv[1] + dv[2] * rv[2];
          for (int i = 0; i < 3; ++i) dv[i] = pr * rv[i];
        } else if (kind == 1) {
          const double pr = dv[0] * rv[0] + dv[1] * rv[1] + dv[2] * rv[2];
          for (int i = 0; i < 3; ++i) dv[i] -= pr * rv[i];
        }
        for (int c = 0; c < 3; ++c)
          b[c * n + j] += (R[c][0] * dv[0] + R[c][1] * dv[1] + R[c][2] * dv[2]) * w;
        for (int i = 0; i < n; ++i) {
          double gi[3], du[3];
          grad_oriented(a0 + i, nord, ne, nf, loc, grad, gi);
          for (int m = 0; m < 3; ++m)
            du[m] = gi[0] * Ji[0][m] + gi[1] * Ji[1][m] + gi[2] * Ji[2][m];
          A[j + n * i] += (dv[0] * du[0] + dv[1] * du[1] + dv[2] * du[2]) * w;
        }
      }
    }
    if (lu_small3(n, A, b)) { atomicMin(bad, e); return; }
    for (int j = 0; j < n; ++j)
      for (int c = 0; c < 3; ++c) X[3 * (a0 + j) + c] = b[c * n + j];
  }
}

// every node of phase `phase` (0: vertices and edges, 1: faces) takes the
// values of its first element: one thread per (element, node slot)
__global__ void k_gdof_gather(int phase, int nel, const int* __restrict__ norder,
                              const int* __restrict__ src, const int64_t* __restrict__ dof_off,
                              double* __restrict__ xnod) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)nel * 26) return;
  const int e = (int)(t / 26), slot = (int)(t % 26);
  if (phase == 0 ? slot >= 20 : slot < 20) return;
  const int sv = src[t];
  if (sv < 0) return;
  const int f = sv / 26, fs = sv % 26;
  int nord[19], nordf[19];
  for (int i = 0; i < 19; ++i) { nord[i] = norder[19 * (size_t)e + i]; nordf[i] = norder[19 * (size_t)f + i]; }
  int n = hexa_node_n(nord, slot);
  const int nfs = hexa_node_n(nordf, fs);
  n = n < nfs ? n : nfs;
  const double* s = xnod + 3 * (dof_off[f] + hexa_node_a0(nordf, fs));
  double* d = xnod + 3 * (dof_off[e] + hexa_node_a0(nord, slot));
  for (int k = 0; k < 3 * n; ++k) d[k] = s[k];
}

}  // namespace

size_t dirichlet_work_doubles(int nel) { return (size_t)nel * (4 * MAXN + 64 * 64 + 64); }
size_t gdof_work_doubles(int nmax) { return (size_t)4 * MAXN + (size_t)nmax * nmax + 3 * (size_t)nmax; }

int launch_gdof(int nel, const int* d_norder, const int* d_nori_e, const int* d_nori_f,
                const double* d_etav, const int64_t* d_node_pt, const double* d_pts,
                const double* d_x, const double* d_dxdeta, const int* d_linear,
                const int* d_src, const int64_t* d_dof_off, double* d_xnod, double* d_work,
                int64_t wstride, int chunk, int* d_bad, cudaStream_t st) {
  if (nel <= 0) return 0;
  for (int phase = 0; phase < 3; ++phase) {
    for (int e0 = 0; e0 < nel; e0 += chunk) {
      const int e1 = e0 + chunk < nel ? e0 + chunk : nel;
      k_gdof<<<(e1 - e0 + 63) / 64, 64, 0, st>>>(phase, e0, e1, d_norder, d_nori_e, d_nori_f,
                                                 d_etav, d_node_pt, d_pts, d_x, d_dxdeta,
                                                 d_linear, d_dof_off, d_xnod, d_work, wstride,
                                                 d_bad);
    }
    if (phase < 2) {
      const int64_t nt = (int64_t)nel * 26;
      k_gdof_gather<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(phase, nel, d_norder, d_src,
                                                                 d_dof_off, d_xnod);
    }
  }
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}


void launch_dirichlet(int nel, const int* d_norder, const int* d_nori_e, const int* d_nori_f,
                      const int* d_bc, const double* d_xvert, const int64_t* d_zd_off,
                      const double* d_gx, const double* d_gw, int isol, double* d_work,
                      double* d_zdofd, int* d_bad, cudaStream_t st) {
  if (nel <= 0) return;
  k_dirichlet<<<(nel + 63) / 64, 64, 0, st>>>(nel, d_norder, d_nori_e, d_nori_f, d_bc, d_xvert,
                                              d_zd_off, d_gx, d_gw, isol, d_work, d_zdofd, d_bad);
}

}  // namespace hp3dg
