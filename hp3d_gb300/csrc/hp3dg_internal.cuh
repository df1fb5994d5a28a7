// hp3dg_internal.cuh -- shared device helpers of the GB300 element pass.
//
// Data layout in HBM (one "bin" = elements of one type and one local order
// tuple, plus, for triangle faces, one orientation class per face):
//   tab_shap [nint][n]          reference-element H1 values (orientation 0)
//   tab_grad [nint][3][n]       reference gradients, row (l,c) contiguous in k
//   D        [E][nint][6]       kappa*w*detJ*(dxi/dx)(dxi/dx)^T, upper (00,11,22,01,02,12)
//   F        [E][nint]          f(x_l)*w_l*detJ_l
//   PK       [E][n(n+1)/2]      element stiffness, packed blocks
//                               [BB upper col-major | BI nb x ni col-major | II upper col-major]
//   perm     [E][n]             oriented dof -> reference dof (bit 31 = sign)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hp3dg {

constexpr int MAXP = 6;
constexpr int MAXN = 343;  // (MAXP+1)^3

struct HexaOrders {
  int nord[19];  // local (find_order_loc) orders of the bin
};

// integrated Legendre of the pair with s0+s1=1 (HomILegendre Idec=.true.,
// shape_1/Polynomials.F90:494-530): L_i(x), dL_i/dx = P_{i-1}(x), i=2..p.
__host__ __device__ inline void ileg(double x, int p, double* L, double* dL) {
  double P[MAXP + 2];
  P[0] = 1.0;
  double y = 2.0 * x - 1.0;
  if (p >= 1) P[1] = y;
  for (int i = 2; i <= p; ++i) P[i] = ((2 * i - 1) * y * P[i - 1] - (i - 1) * P[i - 2]) / i;
  for (int i = 2; i <= p; ++i) {
    L[i] = (P[i] - P[i - 2]) / (4 * i - 2);
    dL[i] = P[i - 1];
  }
}

__host__ __device__ inline void decod2(int v, int& a, int& b) { a = v / 10; b = v % 10; }
__host__ __device__ inline void decod3(int v, int& a, int& b, int& c) {
  a = v / 100; b = (v / 10) % 10; c = v % 10;
}

// vertex -> side of Mu per axis (BlendHexaV)
__host__ __device__ inline int hexa_v(int v, int ax) {
  const int T[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                       {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  return T[v][ax];
}
// edge -> (side1, axis1, side2, axis2, projection axis) (BlendProjectHexaE)
__host__ __device__ inline int hexa_e(int e, int k) {
  const int T[12][5] = {{0, 1, 0, 2, 0}, {1, 0, 0, 2, 1}, {1, 1, 0, 2, 0}, {0, 0, 0, 2, 1},
                        {0, 1, 1, 2, 0}, {1, 0, 1, 2, 1}, {1, 1, 1, 2, 0}, {0, 0, 1, 2, 1},
                        {0, 0, 0, 1, 2}, {1, 0, 0, 1, 2}, {1, 0, 1, 1, 2}, {0, 0, 1, 1, 2}};
  return T[e][k];
}
// face -> (blend side, blend axis, pair-1 axis, pair-2 axis) (BlendProjectHexaF)
__host__ __device__ inline int hexa_f(int f, int k) {
  const int T[6][4] = {{0, 2, 0, 1}, {1, 2, 0, 1}, {0, 1, 0, 2},
                       {1, 0, 1, 2}, {1, 1, 0, 2}, {0, 0, 1, 2}};
  return T[f][k];
}
// OrientQuad (shape_1/Orient.F90:59-116): OrPa(1:2)-1, OrGS(0:1), OrGT(0:1)
__host__ __device__ inline int orq(int o, int k) {
  const int T[8][6] = {{0, 1, 0, 1, 0, 1}, {1, 0, 0, 1, 1, 0}, {0, 1, 1, 0, 1, 0},
                       {1, 0, 1, 0, 0, 1}, {1, 0, 0, 1, 0, 1}, {0, 1, 1, 0, 0, 1},
                       {1, 0, 1, 0, 1, 0}, {0, 1, 0, 1, 1, 0}};
  return T[o][k];
}
// NFAXES(3,o): the orientation swaps the face axes (element_data.F90:246-249)
__host__ __device__ inline int nfaxes_swap(int o) {
  const int T[8] = {0, 1, 0, 1, 1, 0, 1, 0};
  return T[o & 7];
}

// Number of H1 dof of a hexa with orders nord (celndof).
__host__ __device__ inline int hexa_ndof(const int* nord) {
  int n = 8;
  for (int e = 0; e < 12; ++e) n += nord[e] > 1 ? nord[e] - 1 : 0;
  for (int f = 0; f < 6; ++f) {
    int a, b; decod2(nord[12 + f], a, b);
    n += (a > 1 && b > 1) ? (a - 1) * (b - 1) : 0;
  }
  int x, y, z; decod3(nord[18], x, y, z);
  n += (x > 1 && y > 1 && z > 1) ? (x - 1) * (y - 1) * (z - 1) : 0;
  return n;
}
__host__ __device__ inline int hexa_nbub(const int* nord) {
  int x, y, z; decod3(nord[18], x, y, z);
  return (x > 1 && y > 1 && z > 1) ? (x - 1) * (y - 1) * (z - 1) : 0;
}

// H1 shape functions of the hexahedron at xi in the reference (orientation 0)
// enumeration: vertices, edges, faces, bubbles (Hexahedron.F90:33-210).
// grad is written as grad[c*ldg + k].
__host__ __device__ inline int hexa_shape0(const double* xi, const int* nord, double* shap,
                                           double* grad, int ldg) {
  double Mu[2][3];
  for (int d = 0; d < 3; ++d) { Mu[0][d] = 1.0 - xi[d]; Mu[1][d] = xi[d]; }
  // d Mu[s][d] / d xi_c = (c==d) ? (s ? 1 : -1) : 0
  int m = 0;
  for (int v = 0; v < 8; ++v) {
    int s0 = hexa_v(v, 0), s1 = hexa_v(v, 1), s2 = hexa_v(v, 2);
    double b0 = Mu[s0][0], b1 = Mu[s1][1], b2 = Mu[s2][2];
    shap[m] = b0 * b1 * b2;
    grad[0 * ldg + m] = (s0 ? 1.0 : -1.0) * b1 * b2;
    grad[1 * ldg + m] = b0 * (s1 ? 1.0 : -1.0) * b2;
    grad[2 * ldg + m] = b0 * b1 * (s2 ? 1.0 : -1.0);
    ++m;
  }
  double L[MAXP + 2], dL[MAXP + 2];
  for (int e = 0; e < 12; ++e) {
    int p = nord[e];
    if (p < 2) continue;
    int sa = hexa_e(e, 0), aa = hexa_e(e, 1), sb = hexa_e(e, 2), ab = hexa_e(e, 3),
        ax = hexa_e(e, 4);
    double m1 = Mu[sa][aa], m2 = Mu[sb][ab];
    ileg(xi[ax], p, L, dL);
    for (int i = 2; i <= p; ++i) {
      shap[m] = m1 * m2 * L[i];
      for (int c = 0; c < 3; ++c) {
        double g = 0.0;
        if (c == ax) g += m1 * m2 * dL[i];
        if (c == ab) g += m1 * (sb ? 1.0 : -1.0) * L[i];
        if (c == aa) g += (sa ? 1.0 : -1.0) * m2 * L[i];
        grad[c * ldg + m] = g;
      }
      ++m;
    }
  }
  for (int f = 0; f < 6; ++f) {
    int p1, p2; decod2(nord[12 + f], p1, p2);
    if (p1 < 2 || p2 < 2) continue;
    int sf = hexa_f(f, 0), af = hexa_f(f, 1), a1 = hexa_f(f, 2), a2 = hexa_f(f, 3);
    double mb = Mu[sf][af];
    double Ls[MAXP + 2], dLs[MAXP + 2], Lt[MAXP + 2], dLt[MAXP + 2];
    ileg(xi[a1], p1, Ls, dLs);
    ileg(xi[a2], p2, Lt, dLt);
    for (int j = 2; j <= p2; ++j)
      for (int i = 2; i <= p1; ++i) {
        double pq = Ls[i] * Lt[j];
        shap[m] = mb * pq;
        for (int c = 0; c < 3; ++c) {
          double g = 0.0;
          if (c == a1) g += mb * dLs[i] * Lt[j];
          if (c == a2) g += mb * Ls[i] * dLt[j];
          if (c == af) g += (sf ? 1.0 : -1.0) * pq;
          grad[c * ldg + m] = g;
        }
        ++m;
      }
  }
  int px, py, pz; decod3(nord[18], px, py, pz);
  if (px >= 2 && py >= 2 && pz >= 2) {
    double Lx[MAXP + 2], dLx[MAXP + 2], Ly[MAXP + 2], dLy[MAXP + 2], Lz[MAXP + 2], dLz[MAXP + 2];
    ileg(xi[0], px, Lx, dLx);
    ileg(xi[1], py, Ly, dLy);
    ileg(xi[2], pz, Lz, dLz);
    for (int k = 2; k <= pz; ++k)
      for (int j = 2; j <= py; ++j)
        for (int i = 2; i <= px; ++i) {
          shap[m] = Lx[i] * Ly[j] * Lz[k];
          grad[0 * ldg + m] = dLx[i] * Ly[j] * Lz[k];
          grad[1 * ldg + m] = Lx[i] * dLy[j] * Lz[k];
          grad[2 * ldg + m] = Lx[i] * Ly[j] * dLz[k];
          ++m;
        }
  }
  return m;
}

// Full (bin) orders of a hexa from its local orders: per axis the maximum
// over edges, faces and interior -- the orders set_3Dint_aux integrates
// exactly (quadrature/set_3D_int.F90:193-230).  Every element of the bin
// uses the bin's quadrature, and its dof are a subset of the bin element's
// (the H1 basis is hierarchical: an edge of order p carries the first p-1
// edge functions of any higher order, a face the leading sub-rectangle).
__host__ __device__ inline void hexa_bin_orders(const int* loc, int* full) {
  int nx = 0, ny = 0, nz = 0;
  for (int e = 0; e < 12; ++e) {
    int ax = hexa_e(e, 4);
    if (ax == 0) nx = loc[e] > nx ? loc[e] : nx;
    else if (ax == 1) ny = loc[e] > ny ? loc[e] : ny;
    else nz = loc[e] > nz ? loc[e] : nz;
  }
  for (int f = 0; f < 6; ++f) {
    int h, v; decod2(loc[12 + f], h, v);
    int a1 = hexa_f(f, 2), a2 = hexa_f(f, 3);
    int* m1 = a1 == 0 ? &nx : (a1 == 1 ? &ny : &nz);
    int* m2 = a2 == 0 ? &nx : (a2 == 1 ? &ny : &nz);
    if (h > *m1) *m1 = h;
    if (v > *m2) *m2 = v;
  }
  int x, y, z; decod3(loc[18], x, y, z);
  nx = x > nx ? x : nx; ny = y > ny ? y : ny; nz = z > nz ? z : nz;
  for (int e = 0; e < 12; ++e) {
    int ax = hexa_e(e, 4);
    full[e] = ax == 0 ? nx : (ax == 1 ? ny : nz);
  }
  for (int f = 0; f < 6; ++f) {
    int a1 = hexa_f(f, 2), a2 = hexa_f(f, 3);
    int o1 = a1 == 0 ? nx : (a1 == 1 ? ny : nz), o2 = a2 == 0 ? nx : (a2 == 1 ? ny : nz);
    full[12 + f] = 10 * o1 + o2;
  }
  full[18] = 100 * nx + 10 * ny + nz;
}

// Oriented dof a of an element with (global-frame) orders nord and
// orientations -> dof of the bin element (orders `full`, orientation 0),
// with sign.  Edge reversal multiplies L_i by (-1)^i; a face orientation
// swaps and/or reverses the two face axes (OrientE / OrientQuad,
// shape_1/Orient.F90:9-116).  Returns (bin dof) | (sign < 0 ? 0x80000000 : 0).
__host__ __device__ inline uint32_t hexa_dof_map(int a, const int* nord, const int* nori_e,
                                                 const int* nori_f, const int* full) {
  if (a < 8) return (uint32_t)a;
  int off = 8, boff = 8;  // element / bin offsets
  for (int e = 0; e < 12; ++e) {
    int nd = nord[e] > 1 ? nord[e] - 1 : 0;
    if (a < off + nd) {
      int i = a - off + 2;
      bool neg = (nori_e[e] == 1) && (i & 1);
      return (uint32_t)(boff + i - 2) | (neg ? 0x80000000u : 0u);
    }
    off += nd;
    boff += full[e] > 1 ? full[e] - 1 : 0;
  }
  for (int f = 0; f < 6; ++f) {
    int n1, n2; decod2(nord[12 + f], n1, n2);
    int b1, b2; decod2(full[12 + f], b1, b2);
    int nd = (n1 > 1 && n2 > 1) ? (n1 - 1) * (n2 - 1) : 0;
    if (a < off + nd) {
      int r = a - off;
      int i = r % (n1 - 1) + 2, j = r / (n1 - 1) + 2;
      int o = nori_f[f] & 7;
      bool swap = orq(o, 0) == 1;
      // GS1 = Mu[OrGS(1)] of pair OrPa(1): reversed when OrGS(1)==0
      bool negs = (orq(o, 3) == 0) && (i & 1);
      bool negt = (orq(o, 5) == 0) && (j & 1);
      int il = swap ? j : i, jl = swap ? i : j;  // local face indices
      int ref = boff + (jl - 2) * (b1 - 1) + (il - 2);
      return (uint32_t)ref | ((negs != negt) ? 0x80000000u : 0u);
    }
    off += nd;
    boff += (b1 > 1 && b2 > 1) ? (b1 - 1) * (b2 - 1) : 0;
  }
  int px, py, pz; decod3(nord[18], px, py, pz);
  int bx, by, bz; decod3(full[18], bx, by, bz);
  int r = a - off;
  int i = r % (px - 1) + 2, t = r / (px - 1), j = t % (py - 1) + 2, k = t / (py - 1) + 2;
  (void)bz;
  return (uint32_t)(boff + ((k - 2) * (by - 1) + (j - 2)) * (bx - 1) + (i - 2));
}

// Local (bin) orders of a hexa: find_order_loc (datstrs/find_order.F90:68-108).
__host__ __device__ inline void hexa_order_loc(const int* nord, const int* nori_f, int* loc) {
  for (int i = 0; i < 19; ++i) loc[i] = nord[i];
  for (int f = 0; f < 6; ++f)
    if (nfaxes_swap(nori_f[f])) {
      int h, v; decod2(nord[12 + f], h, v);
      loc[12 + f] = v * 10 + h;
    }
}

// packed element-matrix index (see layout note at the top)
__host__ __device__ inline int64_t pk_index(int a, int b, int ni, int nb) {
  if (a > b) { int t = a; a = b; b = t; }
  if (b < ni) return (int64_t)nb * (nb + 1) / 2 + (int64_t)nb * ni + (int64_t)b * (b + 1) / 2 + a;
  if (a < ni) return (int64_t)nb * (nb + 1) / 2 + (int64_t)a * nb + (b - ni);
  int r = a - ni, c = b - ni;
  return (int64_t)c * (c + 1) / 2 + r;
}

// entry (a, b) of an element's matrix (element dof a, b) from the bin
// element's packed matrix through the element's signed dof map pm
__device__ inline double pk_get(const double* PKj, const uint32_t* pm, int a, int b, int ni,
                                int nb) {
  uint32_t ma = pm[a], mb = pm[b];
  int ra = (int)(ma & 0x7fffffffu), rb = (int)(mb & 0x7fffffffu);
  double v = PKj[pk_index(ra, rb, ni, nb)];
  return ((ma ^ mb) & 0x80000000u) ? -v : v;
}

}  // namespace hp3dg
