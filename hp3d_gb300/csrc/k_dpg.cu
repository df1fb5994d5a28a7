// k_dpg.cu -- the ultraweak DPG Maxwell element pass on hexahedra, FP64.
//
// elem_maxwell (problems/MAXWELL/ULTRAWEAK_DPG/elem/elem_maxwell.F90:24-676)
// per element, rewritten around the structure of the graph-norm Gram matrix:
// with a scalar permittivity per element (get_permittivity = eps_r I) every
// entry of G is a combination of three real matrices of the test functions
//   M_FF = sum_l w detJ (J^-T phi_k1).(J^-T phi_k2)      (geometry metric D1)
//   M_CC = sum_l w / detJ (J curl phi_k1).(J curl phi_k2) (metric D2)
//   M_FC = sum_l w phi_k1 . curl phi_k2                   (Piola maps cancel:
//                                                          one matrix per bin)
// so the element-dependent work before the dense algebra is two symmetric
// contractions with a 3x3 metric per point (the structure of the H1
// stiffness), the L2-field coupling P, R and the trace coupling T.  Then, per
// element on one CTA: G = L L^H, X = L^-1 [B | l], Z = X^H X; the impedance
// penalty on the trace block; the condensation of the L2 fields (stc_fwd_herm)
// and the compression.
#include "hp3dg_dpg.cuh"
#include "hp3dg_kernels.h"
#include "hp3dg_zla.cuh"

namespace hp3dg {

namespace {
using namespace zla;

// ---------------------------------------------------------------------------
// tables and geometry
// ---------------------------------------------------------------------------
__global__ void k_dpg_tables(DpgDims d, const double* xiV, const double* xiF, const double* xiI,
                             DpgTables t) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nF = 6 * d.nfp, nI = 6 * d.nip;
  if (tid < d.nv) {
    const double* xi = &xiV[3 * tid];
    dpg_test_shape(xi, d.q, t.vs + (size_t)tid * 3 * d.nEE, t.vc + (size_t)tid * 3 * d.nEE, d.nEE);
    dpg_l2_shape(xi, d.p, t.vq + (size_t)tid * d.nQ);
  } else if (tid < d.nv + nF) {
    const int l = tid - d.nv;
    const double* xi = &xiF[3 * l];
    double* s = t.fs + (size_t)l * 3 * d.nEE;
    // the curls of the test functions are not used on faces (scratch rows)
    dpg_test_shape(xi, d.q, s, t.fscratch + (size_t)l * 3 * d.nEE, d.nEE);
    dpg_trace_shape0(xi, d.p, t.ft + (size_t)l * 3 * d.nEi, d.nEi);
  } else if (tid < d.nv + nF + nI) {
    const int l = tid - d.nv - nF;
    dpg_trace_shape0(&xiI[3 * l], d.p, t.it + (size_t)l * 3 * d.nEi, d.nEi);
  }
}

// M_FC = sum_l w_l phi_k1 . curl phi_k2 (bin constant)
__global__ void k_dpg_mfc(DpgDims d, const double* wV, DpgTables t, double* mfc) {
  const int k1 = blockIdx.x * blockDim.x + threadIdx.x, k2 = blockIdx.y;
  if (k1 >= d.nEE) return;
  double s = 0.0;
  for (int l = 0; l < d.nv; ++l) {
    const double* vs = t.vs + (size_t)l * 3 * d.nEE;
    const double* vc = t.vc + (size_t)l * 3 * d.nEE;
    s += wV[l] * (vs[k1] * vc[k2] + vs[d.nEE + k1] * vc[d.nEE + k2] +
                  vs[2 * d.nEE + k1] * vc[2 * d.nEE + k2]);
  }
  mfc[k1 + (size_t)k2 * d.nEE] = s;
}

__device__ void trilinear(const double* xv, const double* xi, double* x, double J[3][3]) {
  double Mu[2][3];
  for (int a = 0; a < 3; ++a) { Mu[0][a] = 1.0 - xi[a]; Mu[1][a] = xi[a]; }
  for (int i = 0; i < 3; ++i) {
    x[i] = 0.0;
    for (int j = 0; j < 3; ++j) J[i][j] = 0.0;
  }
  for (int v = 0; v < 8; ++v) {
    const int s0 = hexa_v(v, 0), s1 = hexa_v(v, 1), s2 = hexa_v(v, 2);
    const double b0 = Mu[s0][0], b1 = Mu[s1][1], b2 = Mu[s2][2];
    const double g[3] = {(s0 ? 1.0 : -1.0) * b1 * b2, b0 * (s1 ? 1.0 : -1.0) * b2,
                         b0 * b1 * (s2 ? 1.0 : -1.0)};
    const double sh = b0 * b1 * b2;
    for (int i = 0; i < 3; ++i) {
      x[i] += xv[3 * v + i] * sh;
      for (int j = 0; j < 3; ++j) J[i][j] += xv[3 * v + i] * g[j];
    }
  }
}

// determinant and cofactor inverse (geom.F90:57-113); returns det
__device__ double inv3(const double J[3][3], double Ji[3][3]) {
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const double r = 1.0 / det;
  Ji[0][0] = c00 * r;
  Ji[1][0] = c01 * r;
  Ji[2][0] = c02 * r;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
  return det;
}

// mfd_solutions cases 1 and 2 (component icomp of E), H = curl E/(-i w mu),
// J = curl H - i w eps E (common/mfd_solutions.F90, exact.F90, getf.F90)
__device__ void dpg_source(const DpgPhys& ph, double epr, double epi, const double* X, double2* J) {
  double p[2] = {0, 0}, g2[3][3][2];  // the scalar p and its second derivatives
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) g2[i][j][0] = g2[i][j][1] = 0.0;
  const double x = X[0], y = X[1], z = X[2];
  if (ph.isol == 1) {
    const double w = ph.omega, sx = sin(w * x), sy = sin(w * y), sz = sin(w * z);
    const double cx = cos(w * x), cy = cos(w * y), cz = cos(w * z);
    double v = sx * sy * sz;  // times (1 + i)
    p[0] = p[1] = v;
    double h[3][3] = {{-w * w * v, w * w * cx * cy * sz, w * w * cx * sy * cz},
                      {w * w * cx * cy * sz, -w * w * v, w * w * sx * cy * cz},
                      {w * w * cx * sy * cz, w * w * sx * cy * cz, -w * w * v}};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) g2[i][j][0] = g2[i][j][1] = h[i][j];
  } else if (ph.isol == 2) {
    const double cn = 100.0;
    p[0] = -cn * x * y * z * (x - 1.0) * (y - 1.0) * (z - 1.0);
    g2[0][0][0] = cn * y * z * (y - 1.0) * (z - 1.0) * (-2.0);
    g2[1][1][0] = cn * x * z * (x - 1.0) * (z - 1.0) * (-2.0);
    g2[2][2][0] = cn * x * y * (x - 1.0) * (y - 1.0) * (-2.0);
    g2[0][1][0] = g2[1][0][0] = -cn * z * (2.0 * x - 1.0) * (2.0 * y - 1.0) * (z - 1.0);
    g2[0][2][0] = g2[2][0][0] = -cn * y * (2.0 * x - 1.0) * (2.0 * z - 1.0) * (y - 1.0);
    g2[1][2][0] = g2[2][1][0] = -cn * x * (2.0 * y - 1.0) * (2.0 * z - 1.0) * (x - 1.0);
  }
  const int c = ph.icomp - 1;
  // curl curl (p e_c) = grad(d_c p) - lap(p) e_c ;  J = that/(-i w mu) - i w eps p e_c
  const double lap[2] = {g2[0][0][0] + g2[1][1][0] + g2[2][2][0],
                         g2[0][0][1] + g2[1][1][1] + g2[2][2][1]};
  // 1/(-i w mu) = i/(w mu)
  const double s = 1.0 / (ph.omega * ph.mu);
  for (int i = 0; i < 3; ++i) {
    double cr = g2[i][c][0] - (i == c ? lap[0] : 0.0), ci = g2[i][c][1] - (i == c ? lap[1] : 0.0);
    double2 v = make_double2(-ci * s, cr * s);  // i s (cr + i ci)
    if (i == c) {
      // - i w eps p, eps = EPSILON (epr + i epi)
      const double er = ph.epsilon * epr, ei = ph.epsilon * epi;
      const double tr = er * p[0] - ei * p[1], ti = er * p[1] + ei * p[0];  // eps p
      v.x += ph.omega * ti;
      v.y -= ph.omega * tr;
    }
    J[i] = v;
  }
}

// Per element and point: volume metrics D1, D2 (upper 00 11 22 01 02 12),
// A = w J^-1, B = w J / detJ (row-major), g = w detJ J^-1 zJ (complex);
// face points: the trace metric w_f bjac J^-1 [n]x J^-T; impedance points:
// the four penalty metrics (bgeom3D, geom3D.F90:149-203).
__global__ void k_dpg_geom(DpgDims d, DpgPhys ph, const double* xiV, const double* wV,
                           const double* xiF, const double* wF, const double* xiI,
                           const double* wI, const double* xvert, const double* eps,
                           double* gV, double* gF, double* gI, int* bad) {
  const int e = blockIdx.x;
  const double* xv = xvert + (size_t)24 * e;
  const int nF = 6 * d.nfp, nI = 6 * d.nip;
  for (int t = threadIdx.x; t < d.nv + nF + nI; t += blockDim.x) {
    double x[3], J[3][3], Ji[3][3];
    if (t < d.nv) {
      trilinear(xv, &xiV[3 * t], x, J);
      const double det = inv3(J, Ji);
      if (!(det > 0.0)) atomicMin(bad, e);
      const double w = wV[t];
      double* o = gV + ((size_t)e * d.nv + t) * DPG_GV;
      const int pr[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
      for (int k = 0; k < 6; ++k) {
        const int a = pr[k][0], b = pr[k][1];
        double s1 = 0.0, s2 = 0.0;
        for (int m = 0; m < 3; ++m) {
          s1 += Ji[a][m] * Ji[b][m];
          s2 += J[m][a] * J[m][b];
        }
        o[k] = w * det * s1;
        o[6 + k] = w * s2 / det;
      }
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          o[12 + 3 * a + b] = w * Ji[a][b];
          o[21 + 3 * a + b] = w * J[a][b] / det;
        }
      double2 zJ[3];
      dpg_source(ph, eps[2 * e], eps[2 * e + 1], x, zJ);
      for (int a = 0; a < 3; ++a) {
        double2 s = make_double2(0.0, 0.0);
        for (int b = 0; b < 3; ++b) s = zadd(s, zscale(Ji[a][b], zJ[b]));
        o[30 + 2 * a] = w * det * s.x;
        o[31 + 2 * a] = w * det * s.y;
      }
      continue;
    }
    const bool imp = t >= d.nv + nF;
    const int l = imp ? t - d.nv - nF : t - d.nv;
    const int f = imp ? l / d.nip : l / d.nfp;
    const double* xi = imp ? &xiI[3 * l] : &xiF[3 * l];
    trilinear(xv, xi, x, J);
    inv3(J, Ji);
    // face tangents dx/dt = J dxi/dt (face_param), outward unit normal
    double t1[3], t2[3], rn[3];
    for (int i = 0; i < 3; ++i) {
      t1[i] = t2[i] = 0.0;
      for (int j = 0; j < 3; ++j) {
        t1[i] += J[i][j] * d.dxidt[f][j][0];
        t2[i] += J[i][j] * d.dxidt[f][j][1];
      }
    }
    rn[0] = t1[1] * t2[2] - t1[2] * t2[1];
    rn[1] = t1[2] * t2[0] - t1[0] * t2[2];
    rn[2] = t1[0] * t2[1] - t1[1] * t2[0];
    const double bjac = sqrt(rn[0] * rn[0] + rn[1] * rn[1] + rn[2] * rn[2]);
    for (int i = 0; i < 3; ++i) rn[i] = rn[i] * d.nsign[f] / bjac;
    const double w = bjac * (imp ? wI[l] : wF[l]);
    const double N[3][3] = {{0.0, -rn[2], rn[1]}, {rn[2], 0.0, -rn[0]}, {-rn[1], rn[0], 0.0}};
    if (!imp) {
      double* o = gF + ((size_t)e * nF + l) * 9;
      // (J^-T phi) . (n x J^-T psi) = phi^T (J^-1 N J^-T) psi
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          double s = 0.0;
          for (int m = 0; m < 3; ++m)
            for (int q = 0; q < 3; ++q) s += Ji[a][m] * N[m][q] * Ji[b][q];
          o[3 * a + b] = w * s;
        }
    } else {
      double N2[3][3];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          N2[a][b] = 0.0;
          for (int m = 0; m < 3; ++m) N2[a][b] += N[a][m] * N[m][b];
        }
      // K_P = J^-1 P^T Q J^-T for the pairs (P,Q) = (N2,N2), (N2,N), (N,N2), (N,N)
      const double(*Ps[4])[3] = {N2, N2, N, N};
      const double(*Qs[4])[3] = {N2, N, N2, N};
      const double sc[4] = {ph.gamma * ph.gamma, -ph.gamma, -ph.gamma, 1.0};
      double* o = gI + ((size_t)e * nI + l) * 36;
      for (int k = 0; k < 4; ++k) {
        double PQ[3][3];
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) {
            PQ[a][b] = 0.0;
            for (int m = 0; m < 3; ++m) PQ[a][b] += Ps[k][m][a] * Qs[k][m][b];
          }
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int m = 0; m < 3; ++m)
              for (int q = 0; q < 3; ++q) s += Ji[a][m] * PQ[m][q] * Ji[b][q];
            o[9 * k + 3 * a + b] = sc[k] * w * s;
          }
      }
    }
  }
}

// the metrics D1 and D2 of every volume point as rows [e][l][6] (the
// per-element operand of the split-BF16 contraction)
__global__ void k_dpg_dpack(DpgDims d, const double* gV, double* D1, double* D2) {
  const int e = blockIdx.x;
  for (int x = threadIdx.x; x < 6 * d.nv; x += blockDim.x) {
    const double* g = gV + ((size_t)e * d.nv + x / 6) * DPG_GV;
    D1[(size_t)e * 6 * d.nv + x] = g[x % 6];
    D2[(size_t)e * 6 * d.nv + x] = g[6 + x % 6];
  }
}

// dense bin-constant tables of the couplings (row-major K x ncols):
//   which 0 (P): [(l, i)][(k1, k2)] = phi_k1,i(l) q_k2(l)
//   which 1 (R): [(l, i)][(k1, k2)] = (curl phi_k1)_i(l) q_k2(l)
//   which 2 (T): [(l, a, b)][(k1, m)] = phi_k1,a(l) psi_m,b(l), l over face points
__global__ void k_dpg_bdense(DpgDims d, DpgTables t, int which, double* Md) {
  const int nE = d.nEE;
  const int64_t ncols = which < 2 ? (int64_t)nE * d.nQ : (int64_t)nE * d.nEi;
  const int64_t K = which < 2 ? 3 * (int64_t)d.nv : 9 * 6 * (int64_t)d.nfp;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < K * ncols;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = x / ncols, c = x % ncols;
    const int k1 = (int)(c % nE), k2 = (int)(c / nE);
    double v;
    if (which < 2) {
      const int l = (int)(q / 3), i = (int)(q % 3);
      const double* T = which ? t.vc : t.vs;
      v = T[(size_t)l * 3 * nE + (size_t)i * nE + k1] * t.vq[(size_t)l * d.nQ + k2];
    } else {
      const int l = (int)(q / 9), a = (int)(q % 9) / 3, b = (int)(q % 3);
      v = t.fs[(size_t)l * 3 * nE + (size_t)a * nE + k1] *
          t.ft[(size_t)l * 3 * d.nEi + (size_t)b * d.nEi + k2];
    }
    Md[x] = v;
  }
}

// D rows of P and R: row (e, c) = A(l)_{i,c} (A = w J^-1) and B(l)_{c,i}
// (B = w J / detJ) over (l, i)
__global__ void k_dpg_dpackPR(DpgDims d, const double* gV, double* DP, double* DR) {
  const int e = blockIdx.x, K = 3 * d.nv;
  for (int x = threadIdx.x; x < 3 * K; x += blockDim.x) {
    const int c = x / K, q = x % K, l = q / 3, i = q % 3;
    const double* g = gV + ((size_t)e * d.nv + l) * DPG_GV;
    DP[((size_t)3 * e + c) * K + q] = g[12 + 3 * i + c];
    DR[((size_t)3 * e + c) * K + q] = g[21 + 3 * c + i];
  }
}

// M_FF (which 0, metric D1, values) and M_CC (which 1, metric D2, curls):
// C[k1][k2] = sum_l phi_k1(l)^T D_l phi_k2(l), upper 64x64 tiles, mirrored.
constexpr int GR_PTS = 8;
__global__ void __launch_bounds__(256) k_dpg_gram(DpgDims d, DpgTables t, const double* gV,
                                                  double* MFF, double* MCC) {
  const int e = blockIdx.x, which = blockIdx.z;
  const int nt = (d.nEE + 63) / 64;
  int ti = 0, tj = 0, cnt = blockIdx.y;
  for (ti = 0; ti < nt; ++ti) {
    if (cnt < nt - ti) { tj = ti + cnt; break; }
    cnt -= nt - ti;
  }
  const double* T = which ? t.vc : t.vs;
  double* C = (which ? MCC : MFF) + (size_t)e * d.nEE * d.nEE;
  __shared__ double rowS[GR_PTS][3][64], colS[GR_PTS][3][64];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  double acc[4][4] = {};
  for (int l0 = 0; l0 < d.nv; l0 += GR_PTS) {
    for (int x = tid; x < GR_PTS * 64; x += 256) {
      const int lp = x / 64, r = x % 64, l = l0 + lp;
      const int k1 = ti * 64 + r, k2 = tj * 64 + r;
      double a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
      if (l < d.nv) {
        const double* tl = T + (size_t)l * 3 * d.nEE;
        if (k1 < d.nEE)
          for (int c = 0; c < 3; ++c) a[c] = tl[c * d.nEE + k1];
        if (k2 < d.nEE) {
          const double* D = gV + ((size_t)e * d.nv + l) * DPG_GV + 6 * which;
          const double p0 = tl[k2], p1 = tl[d.nEE + k2], p2 = tl[2 * d.nEE + k2];
          b[0] = D[0] * p0 + D[3] * p1 + D[4] * p2;
          b[1] = D[3] * p0 + D[1] * p1 + D[5] * p2;
          b[2] = D[4] * p0 + D[5] * p1 + D[2] * p2;
        }
      }
      for (int c = 0; c < 3; ++c) {
        rowS[lp][c][r] = a[c];
        colS[lp][c][r] = b[c];
      }
    }
    __syncthreads();
#pragma unroll
    for (int lp = 0; lp < GR_PTS; ++lp)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        double a[4], b[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = rowS[lp][c][ty * 4 + r];
#pragma unroll
        for (int q = 0; q < 4; ++q) b[q] = colS[lp][c][tx * 4 + q];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[r][q] = fma(a[r], b[q], acc[r][q]);
      }
    __syncthreads();
  }
  for (int r = 0; r < 4; ++r)
    for (int q = 0; q < 4; ++q) {
      const int k1 = ti * 64 + ty * 4 + r, k2 = tj * 64 + tx * 4 + q;
      if (k1 >= d.nEE || k2 >= d.nEE || k1 > k2) continue;
      C[k1 + (size_t)k2 * d.nEE] = acc[r][q];
      C[k2 + (size_t)k1 * d.nEE] = acc[r][q];
    }
}

// P[k1][(k2,c)] = sum_l q_k2 (J^-T phi_k1)_c w, R[k1][(k2,c)] = sum_l q_k2
// (J curl phi_k1)_c w / detJ (blockIdx.z = chunk of 8 L2 functions), T[k1][k2]
// (reference trace order) and the load (blockIdx.z = nzq .. ).
constexpr int BQ_CH = 8, BT_CH = 12;
__global__ void __launch_bounds__(128) k_dpg_bmat(DpgDims d, DpgTables t, const double* gV,
                                                  const double* gF, double* P, double* R,
                                                  double* Tm, double* load, int zbase) {
  const int e = blockIdx.x, k1 = blockIdx.y * blockDim.x + threadIdx.x;
  const int nzq = (d.nQ + BQ_CH - 1) / BQ_CH, nzt = (d.nEi + BT_CH - 1) / BT_CH;
  const int z = zbase + blockIdx.z;
  if (k1 >= d.nEE) return;
  const int n3q = 3 * d.nQ;
  if (z < nzq) {
    const int q0 = z * BQ_CH;
    double ap[BQ_CH][3] = {}, ar[BQ_CH][3] = {};
    for (int l = 0; l < d.nv; ++l) {
      const double* g = gV + ((size_t)e * d.nv + l) * DPG_GV;
      const double* vs = t.vs + (size_t)l * 3 * d.nEE;
      const double* vc = t.vc + (size_t)l * 3 * d.nEE;
      const double ph[3] = {vs[k1], vs[d.nEE + k1], vs[2 * d.nEE + k1]};
      const double cu[3] = {vc[k1], vc[d.nEE + k1], vc[2 * d.nEE + k1]};
      double u[3], v[3];
      for (int c = 0; c < 3; ++c) {
        u[c] = g[12 + c] * ph[0] + g[15 + c] * ph[1] + g[18 + c] * ph[2];  // (A^T phi)_c
        v[c] = g[21 + 3 * c] * cu[0] + g[22 + 3 * c] * cu[1] + g[23 + 3 * c] * cu[2];
      }
      const double* qv = t.vq + (size_t)l * d.nQ;
#pragma unroll
      for (int k = 0; k < BQ_CH; ++k) {
        const double qk = (q0 + k < d.nQ) ? qv[q0 + k] : 0.0;
        for (int c = 0; c < 3; ++c) {
          ap[k][c] = fma(qk, u[c], ap[k][c]);
          ar[k][c] = fma(qk, v[c], ar[k][c]);
        }
      }
    }
    for (int k = 0; k < BQ_CH && q0 + k < d.nQ; ++k)
      for (int c = 0; c < 3; ++c) {
        const size_t o = (size_t)e * d.nEE * n3q + k1 + (size_t)(3 * (q0 + k) + c) * d.nEE;
        P[o] = ap[k][c];
        R[o] = ar[k][c];
      }
  } else if (z < nzq + nzt) {
    const int m0 = (z - nzq) * BT_CH;
    double at[BT_CH] = {};
    for (int l = 0; l < 6 * d.nfp; ++l) {
      const double* M = gF + ((size_t)e * 6 * d.nfp + l) * 9;
      const double* fs = t.fs + (size_t)l * 3 * d.nEE;
      const double ph[3] = {fs[k1], fs[d.nEE + k1], fs[2 * d.nEE + k1]};
      double u[3];
      for (int b = 0; b < 3; ++b) u[b] = ph[0] * M[b] + ph[1] * M[3 + b] + ph[2] * M[6 + b];
      const double* ft = t.ft + (size_t)l * 3 * d.nEi;
#pragma unroll
      for (int k = 0; k < BT_CH; ++k) {
        const int m = m0 + k;
        if (m < d.nEi)
          at[k] += u[0] * ft[m] + u[1] * ft[d.nEi + m] + u[2] * ft[2 * d.nEi + m];
      }
    }
    for (int k = 0; k < BT_CH && m0 + k < d.nEi; ++k)
      Tm[(size_t)e * d.nEE * d.nEi + k1 + (size_t)(m0 + k) * d.nEE] = at[k];
  } else {
    double lr = 0.0, li = 0.0;
    for (int l = 0; l < d.nv; ++l) {
      const double* g = gV + ((size_t)e * d.nv + l) * DPG_GV;
      const double* vs = t.vs + (size_t)l * 3 * d.nEE;
      for (int c = 0; c < 3; ++c) {
        const double ph = vs[c * d.nEE + k1];
        lr = fma(ph, g[30 + 2 * c], lr);
        li = fma(ph, g[31 + 2 * c], li);
      }
    }
    load[2 * ((size_t)e * d.nEE + k1)] = lr;
    load[2 * ((size_t)e * d.nEE + k1) + 1] = li;
  }
}

// G (lower) and [B | l] in complex FP64 from the real parts.
// AUG = false: G (nt x nt, lower) and S = [B | l] (nt x (nr+1)), column-major.
// AUG = true: the lower triangle of the augmented Hermitian matrix
// [[G, S], [S^H, 0]] (N = nt + nr + 1, column-major) with the trial unknowns
// in the order [L2 fields | traces | load], for the partial factorization of
// the tensor-core path; the trailing block starts at zero.
template <bool AUG>
__global__ void k_dpg_assemble(DpgDims d, DpgPhys ph, const double* eps, const double* MFF,
                               const double* MCC, const double* MFC, const double* P,
                               const double* R, const double* Tm, const double* load,
                               const uint32_t* perm, double2* G, double2* S) {
  const int e = blockIdx.x;
  const int nE = d.nEE, nt = 2 * nE, ni = 2 * d.nEi, nr = d.nr;
  const double er = ph.epsilon * eps[2 * e], ei = ph.epsilon * eps[2 * e + 1];
  const double2 za = make_double2(-ph.omega * ei, ph.omega * er);  // i w eps
  const double2 zc1 = make_double2(0.0, ph.omega * ph.mu);
  const double za2 = za.x * za.x + za.y * za.y, zc2 = zc1.y * zc1.y;
  const size_t mst = AUG ? (size_t)nE * (nE + 1) / 2 : (size_t)nE * nE;
  const double* mff = MFF + (size_t)e * mst;
  const double* mcc = MCC + (size_t)e * mst;
  const int n1 = d.nr + 1, NA = nt + n1;
  const size_t ldg = AUG ? (size_t)NA : (size_t)nt;
  double2* g = AUG ? G + (size_t)e * NA * NA : G + (size_t)e * nt * nt;
  const size_t ntot = (size_t)nt * nt;
  for (size_t x = blockIdx.y * blockDim.x + threadIdx.x; x < ntot; x += (size_t)gridDim.y * blockDim.x) {
    const int r = (int)(x % nt), c = (int)(x / nt);
    if (r < c) continue;
    const int k1 = r >> 1, a = r & 1, k2 = c >> 1, b = c & 1;
    double2 v;
    if (a == b) {
      const double s = (a == 0 ? za2 : zc2) + ph.alpha;
      // AUG: M_FF and M_CC as packed upper triangles (k_ozaki.cu layout)
      const size_t ix = AUG ? (k1 < k2 ? (size_t)k2 * (k2 + 1) / 2 + k1 : (size_t)k1 * (k1 + 1) / 2 + k2)
                            : k1 + (size_t)k2 * nE;
      v = make_double2(s * mff[ix] + mcc[ix], 0.0);
    } else {
      const double f12 = MFC[k1 + (size_t)k2 * nE], f21 = MFC[k2 + (size_t)k1 * nE];
      if (a == 0)  // -za M_FC(k1,k2) + conj(zc1) M_FC(k2,k1)
        v = make_double2(-za.x * f12 + zc1.x * f21, -za.y * f12 - zc1.y * f21);
      else         // -conj(za) M_FC(k2,k1) + zc1 M_FC(k1,k2)
        v = make_double2(-za.x * f21 + zc1.x * f12, za.y * f21 + zc1.y * f12);
    }
    g[r + (size_t)c * ldg] = v;
  }
  if (AUG)  // trailing block (lower): zero
    for (size_t x = blockIdx.y * blockDim.x + threadIdx.x; x < (size_t)n1 * n1;
         x += (size_t)gridDim.y * blockDim.x) {
      const int r = (int)(x % n1), c = (int)(x / n1);
      if (r >= c) g[(nt + r) + (size_t)(nt + c) * ldg] = make_double2(0.0, 0.0);
    }
  const int n3q = 3 * d.nQ;
  const double* pe = P + (size_t)e * nE * n3q;
  const double* re = R + (size_t)e * nE * n3q;
  const double* te = Tm + (size_t)e * nE * d.nEi;
  const uint32_t* pm = perm + (size_t)e * d.nEi;
  double2* s = AUG ? nullptr : S + (size_t)e * nt * (nr + 1);
  const size_t stot = (size_t)nt * (nr + 1);
  const int nq = nr - ni;
  for (size_t x = blockIdx.y * blockDim.x + threadIdx.x; x < stot; x += (size_t)gridDim.y * blockDim.x) {
    const int r = (int)(x % nt), c = (int)(x / nt);
    const int k1 = r >> 1, a = r & 1;
    double2 v = make_double2(0.0, 0.0);
    if (c < ni) {
      const int m = c >> 1, comp = c & 1;
      if (comp != a) {  // <n x H, F> and <n x E, G>
        const uint32_t pv = pm[m];
        double tv = te[k1 + (size_t)(pv & 0x7fffffffu) * nE];
        v.x = (pv >> 31) ? -tv : tv;
      }
    } else if (c < nr) {
      const int k2 = (c - ni) / 6, comp = (c - ni) % 6;
      const int cc = comp % 3;
      // AUG: P and R from the split-BF16 contraction, rows (element, cc)
      const size_t pix = AUG ? k1 + (size_t)(cc * d.nQ + k2) * nE : k1 + (size_t)(3 * k2 + cc) * nE;
      const double pv = pe[pix], rv = re[pix];
      if (a == 0) v = comp < 3 ? make_double2(-za.x * pv, -za.y * pv) : make_double2(rv, 0.0);
      else v = comp < 3 ? make_double2(rv, 0.0) : make_double2(zc1.x * pv, zc1.y * pv);
    } else if (a == 0) {
      v = make_double2(load[2 * ((size_t)e * nE + k1)], load[2 * ((size_t)e * nE + k1) + 1]);
    }
    if (AUG) {  // row nt + c' of S^H, c' the position of trial unknown c in [Q | E | l]
      const int ca = c < ni ? nq + c : (c < nr ? c - ni : nr);
      g[(nt + ca) + (size_t)r * ldg] = make_double2(v.x, -v.y);
    } else {
      s[x] = v;
    }
  }
}

// G = L L^H; X = L^-1 [B|l]; Z = X^H X (lower, then mirrored).
__global__ void __launch_bounds__(LA_THREADS) k_dpg_dpg(DpgDims d, double2* G, double2* S,
                                                        double2* Z, int* bad) {
  __shared__ double2 sm[2 * TK * TM];
  const int e = blockIdx.x;
  const int nt = 2 * d.nEE, n1 = d.nr + 1;
  double2* g = G + (size_t)e * nt * nt;
  double2* s = S + (size_t)e * nt * n1;
  double2* z = Z + (size_t)e * n1 * n1;
  if (cta_zpotrf(g, nt, nt, sm) && threadIdx.x == 0) atomicMin(bad, e);
  cta_ztrsm_fwd(g, nt, nt, s, nt, n1, sm);
  cta_zgemm(n1, n1, nt, s, nt, true, s, nt, false, z, n1, 1.0, false, true, sm);
  for (size_t x = threadIdx.x; x < (size_t)n1 * n1; x += LA_THREADS) {
    const int i = (int)(x % n1), j = (int)(x / n1);
    if (i < j) z[x] = zconj(z[j + (size_t)i * n1]);
  }
}

// impedance penalty (imp_penalty, elem_maxwell.F90:679-876) on the trace
// block of Z, in the element's oriented trace functions.
// the penalty is added to the trace block of Z, which starts at row and
// column `off` of a column-major matrix with leading dimension n1
__global__ void k_dpg_imp(DpgDims d, const int* imp_mask, DpgTables t, const double* gI,
                          const uint32_t* perm, double2* Z, int64_t estride, int off, int n1) {
  const int e = blockIdx.x;
  const int mask = imp_mask[e];
  if (!mask) return;
  const int nE = d.nEi;
  const uint32_t* pm = perm + (size_t)e * nE;
  double2* z = Z + (size_t)e * estride + off + (size_t)off * n1;
  for (int x = blockIdx.y * blockDim.x + threadIdx.x; x < nE * nE; x += gridDim.y * blockDim.x) {
    const int m1 = x % nE, m2 = x / nE;
    const uint32_t p1 = pm[m1], p2 = pm[m2];
    const int c1 = p1 & 0x7fffffff, c2 = p2 & 0x7fffffff;
    const double sg = ((p1 ^ p2) >> 31) ? -1.0 : 1.0;
    double acc[4] = {0, 0, 0, 0};
    for (int f = 0; f < 6; ++f) {
      if (!((mask >> f) & 1)) continue;
      for (int l = f * d.nip; l < (f + 1) * d.nip; ++l) {
        const double* it = t.it + (size_t)l * 3 * nE;
        const double a[3] = {it[c1], it[nE + c1], it[2 * nE + c1]};
        const double b[3] = {it[c2], it[nE + c2], it[2 * nE + c2]};
        const double* K = gI + ((size_t)e * 6 * d.nip + l) * 36;
        for (int k = 0; k < 4; ++k) {
          double s = 0.0;
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) s += a[i] * K[9 * k + 3 * i + j] * b[j];
          acc[k] += s;
        }
      }
    }
    const int r0 = 2 * m1, c0 = 2 * m2;
    z[r0 + (size_t)c0 * n1].x += sg * acc[0];
    z[r0 + (size_t)(c0 + 1) * n1].x += sg * acc[1];
    z[(r0 + 1) + (size_t)c0 * n1].x += sg * acc[2];
    z[(r0 + 1) + (size_t)(c0 + 1) * n1].x += sg * acc[3];
  }
}

// condensation of the L2 fields (stc_fwd_herm) and compression
__global__ void __launch_bounds__(LA_THREADS) k_dpg_condense(
    DpgDims d, double2* Z, const int* nextract, const int64_t* lcon_off, const int64_t* elem_nnz,
    const int64_t* schur_off, const int64_t* bub_off, double2* zastif, double2* zbload,
    double2* aschur, double2* bschur, int* bad) {
  __shared__ double2 sm[2 * TK * TM];
  const int e = blockIdx.x;
  const int n1 = d.nr + 1, ni = 2 * d.nEi, nq = 6 * d.nQ;
  double2* z = Z + (size_t)e * n1 * n1;
  double2* L = z + ni + (size_t)ni * n1;       // Z_QQ
  double2* Y = z + ni;                         // Z_QE (nq x ni)
  double2* y = z + ni + (size_t)d.nr * n1;     // z_Q (load)
  if (cta_zpotrf(L, n1, nq, sm) && threadIdx.x == 0) atomicMin(bad, e);
  cta_ztrsm_fwd(L, n1, nq, Y, n1, ni, sm);
  cta_ztrsm_fwd(L, n1, nq, y, n1, 1, sm);
  // S = Z_EE - Y^H Y ; zb = z_E - Y^H y
  cta_zgemm(ni, ni, nq, Y, n1, true, Y, n1, false, z, n1, -1.0, true, false, sm);
  cta_zgemm(ni, 1, nq, Y, n1, true, y, n1, false, z + (size_t)d.nr * n1, n1, -1.0, true, false, sm);
  // ASchur = L^-H Y, BSchur = L^-H y
  cta_ztrsm_bwd(L, n1, nq, Y, n1, ni, sm);
  cta_ztrsm_bwd(L, n1, nq, y, n1, 1, sm);
  double2* as = aschur + schur_off[e];
  for (size_t x = threadIdx.x; x < (size_t)nq * ni; x += LA_THREADS) {
    const int i = (int)(x % nq), j = (int)(x / nq);
    as[x] = Y[i + (size_t)j * n1];
  }
  for (int i = threadIdx.x; i < nq; i += LA_THREADS) bschur[bub_off[e] + i] = y[i];
  const int64_t lo = lcon_off[e];
  const int nc = (int)(lcon_off[e + 1] - lo);
  const int* nx = nextract + lo;
  double2* za = zastif + elem_nnz[e];
  for (size_t x = threadIdx.x; x < (size_t)nc * nc; x += LA_THREADS) {
    const int l1 = (int)(x / nc), l2 = (int)(x % nc);
    za[x] = z[nx[l1] + (size_t)nx[l2] * n1];
  }
  for (int l1 = threadIdx.x; l1 < nc; l1 += LA_THREADS)
    zbload[lo + l1] = z[nx[l1] + (size_t)d.nr * n1];
}

}  // namespace

void launch_dpg_tables(const DpgDims& d, const double* xiV, const double* wV, const double* xiF,
                       const double* xiI, const DpgTables& t, double* mfc, cudaStream_t st) {
  const int n = d.nv + 6 * d.nfp + 6 * d.nip;
  k_dpg_tables<<<(n + 63) / 64, 64, 0, st>>>(d, xiV, xiF, xiI, t);
  k_dpg_mfc<<<dim3((d.nEE + 127) / 128, d.nEE), 128, 0, st>>>(d, wV, t, mfc);
}

int launch_dpg_gram_tables(const DpgDims& d, const DpgTables& t, const DpgWork& w,
                           cudaStream_t st) {
  for (int which = 0; which < 2; ++which)
    if (launch_ozaki_build_m(w.gplan, d.nv, d.nEE, d.nEE, 0, which ? t.vc : t.vs, w.gmdig[which],
                             w.gmscale[which], nullptr, st))
      return -1;
  for (int which = 0; which < 3; ++which) {
    k_dpg_bdense<<<1024, 256, 0, st>>>(d, t, which, w.bMd);
    if (launch_ozaki_build_m_dense(w.bplan[which], w.bMd, w.bmdig[which], w.bmscale[which], st))
      return -1;
  }
  return 0;
}

int launch_dpg_stage(int stage, int nel, const DpgDims& d, const DpgPhys& ph,
                     const DpgTables& t, const DpgWork& w, const double* xvert, const double* eps,
                     const int* imp_mask, const uint32_t* perm, const int* nextract,
                     const int64_t* lcon_off, const int64_t* elem_nnz, const int64_t* schur_off,
                     const int64_t* bub_off, double* zastif, double* zbload, double* aschur,
                     double* bschur, double* zkeep, int* flags, cudaStream_t st) {
  if (nel <= 0) return 0;
  int nk = 0;
  bool fail = false;
  auto sub = [&](int rc, int kernels) {  // a sub-launcher: 0 or its count, -1 on error
    if (rc < 0) fail = true;
    else nk += kernels > 0 ? kernels : rc;
  };
  if (stage == 0) {
    k_dpg_geom<<<nel, 128, 0, st>>>(d, ph, w.xiV, w.wV, w.xiF, w.wF, w.xiI, w.wI, xvert, eps,
                                    w.gV, w.gF, w.gI, flags);
    ++nk;
    if (w.tc) {
      k_dpg_dpack<<<nel, 256, 0, st>>>(d, w.gV, w.gD[0], w.gD[1]);
      ++nk;
      for (int which = 0; which < 2; ++which) {
        sub(launch_ozaki_slice_d(w.gplan, nel, d.nv, w.gD[which], w.gddig[which],
                                 w.gdscale[which], st), 2);
        sub(launch_ozaki_gemm(w.gplan, nel, d.nEE, w.gddig[which], w.gdscale[which],
                              w.gmdig[which], w.gmscale[which], which ? w.MCC : w.MFF, flags + 2,
                              st), 1);
      }
    } else {
      const int nt = (d.nEE + 63) / 64;
      k_dpg_gram<<<dim3(nel, nt * (nt + 1) / 2, 2), 256, 0, st>>>(d, t, w.gV, w.MFF, w.MCC);
      ++nk;
    }
    const int nzq = (d.nQ + BQ_CH - 1) / BQ_CH, nzt = (d.nEi + BT_CH - 1) / BT_CH;
    if (w.tc) {
      k_dpg_dpackPR<<<nel, 256, 0, st>>>(d, w.gV, w.bDP, w.bDR);
      ++nk;
      for (int which = 0; which < 3; ++which) {
        const int rows = which < 2 ? 3 * nel : nel;
        const double* D = which == 0 ? w.bDP : (which == 1 ? w.bDR : w.gF);
        double* out = which == 0 ? w.P : (which == 1 ? w.R : w.T);
        sub(launch_ozaki_slice_d_dense(w.bplan[which], rows, D, w.bddig, w.bdscale, st), 2);
        sub(launch_ozaki_gemm_dense(w.bplan[which], rows, w.bddig, w.bdscale, w.bmdig[which],
                                    w.bmscale[which], out, flags + 2, st), 1);
      }
      // the load only
      k_dpg_bmat<<<dim3(nel, (d.nEE + 127) / 128, 1), 128, 0, st>>>(d, t, w.gV, w.gF, w.P, w.R,
                                                                    w.T, w.load, nzq + nzt);
      k_dpg_assemble<true><<<dim3(nel, 32), 256, 0, st>>>(d, ph, eps, w.MFF, w.MCC, w.MFC, w.P,
                                                          w.R, w.T, w.load, perm,
                                                          (double2*)w.M, nullptr);
    } else {
      k_dpg_bmat<<<dim3(nel, (d.nEE + 127) / 128, nzq + nzt + 1), 128, 0, st>>>(
          d, t, w.gV, w.gF, w.P, w.R, w.T, w.load, 0);
      k_dpg_assemble<false><<<dim3(nel, 32), 256, 0, st>>>(d, ph, eps, w.MFF, w.MCC, w.MFC, w.P,
                                                           w.R, w.T, w.load, perm,
                                                           (double2*)w.G, (double2*)w.S);
    }
    nk += 2;
  } else if (stage == 1) {
    const int n1 = d.nr + 1;
    const dim3 gimp(nel, (d.nEi * d.nEi + 255) / 256);
    if (w.tc) {
      // test block of the augmented matrix -> -Z in the trailing block -> Z
      const int nt = 2 * d.nEE, na = nt + n1, nq = 6 * d.nQ;
      sub(launch_dpg_aug_tc(1, nel, nt, n1, nq, w, zkeep, flags + 1, flags + 2, st), 0);
      if (ph.ibcflag == 2) {
        k_dpg_imp<<<gimp, 256, 0, st>>>(d, imp_mask, t, w.gI, perm, (double2*)w.M,
                                        (int64_t)na * na, nt + nq, na);
        ++nk;
      }
      if (zkeep) sub(launch_dpg_aug_tc(3, nel, nt, n1, nq, w, zkeep, flags + 1, flags + 2, st), 0);
    } else {
      k_dpg_dpg<<<nel, LA_THREADS, 0, st>>>(d, (double2*)w.G, (double2*)w.S, (double2*)w.Z,
                                            flags + 1);
      ++nk;
      if (ph.ibcflag == 2) {
        k_dpg_imp<<<gimp, 256, 0, st>>>(d, imp_mask, t, w.gI, perm, (double2*)w.Z,
                                        (int64_t)n1 * n1, 0, n1);
        ++nk;
      }
    }
  } else if (w.tc) {
    // L2 block of Z -> Schur complement, ASchur/BSchur, compression
    const int nt = 2 * d.nEE, n1 = d.nr + 1, nq = 6 * d.nQ;
    sub(launch_dpg_aug_tc(2, nel, nt, n1, nq, w, nullptr, flags + 1, flags + 2, st), 0);
    sub(launch_dpg_aug_out(nel, nt, n1, nq, w, nextract, lcon_off, elem_nnz, schur_off, bub_off,
                           zastif, zbload, aschur, bschur, st), 0);
  } else {
    k_dpg_condense<<<nel, LA_THREADS, 0, st>>>(d, (double2*)w.Z, nextract, lcon_off, elem_nnz,
                                               schur_off, bub_off, (double2*)zastif,
                                               (double2*)zbload, (double2*)aschur,
                                               (double2*)bschur, flags + 1);
    ++nk;
  }
  if (fail || cudaPeekAtLastError() != cudaSuccess) return -1;
  return nk;
}

}  // namespace hp3dg
