// hp3dg_simplex.cuh -- H1 shape functions of the tetrahedron (and the
// triangle factors shared with the prism) for the bin tables, plus the
// element -> bin dof map of tetrahedra.
//
// Restates shape_1/Tetrahedron.F90:33-234 (shape3DHTet) with the ancillary
// routines it calls: AncPhiE / AncPhiTri (Ancillary.F90:37-58, 397-442),
// HomILegendre / HomIJacobi / PolyIJacobi / PolyJacobi (Polynomials.F90:
// 197-431, 497-646), OrientE / OrientTri (Orient.F90:9-37, 119-162),
// AffineTetrahedron (AffineCoordinates.F90:74-89) and ProjectTetE/F
// (BlendProject.F90:470-560).
#pragma once
#include "hp3dg_internal.cuh"

namespace hp3dg {

// Homogenized integrated Legendre of the pair (s0, s1), t = s0 + s1
// (HomILegendre with Idec false): L_i(s1; t), i = 2..p, and its gradient
// dL_i = P_{i-1} ds1 + R_{i-1} (ds0 + ds1), R_{i-1} = -(P_{i-1} + t P_{i-2}) / 2.
__host__ __device__ inline void hom_leg(double s0, double s1, const double* d0, const double* d1,
                                        int p, double* L, double (*dL)[3]) {
  double t = s0 + s1, y = 2.0 * s1 - t, tt = t * t;
  double P[MAXP + 2];
  P[0] = 1.0;
  P[1] = y;
  for (int i = 2; i <= p; ++i) P[i] = ((2 * i - 1) * y * P[i - 1] - (i - 1) * tt * P[i - 2]) / i;
  for (int i = 2; i <= p; ++i) {
    L[i] = (P[i] - tt * P[i - 2]) / (4 * i - 2);
    double R = -(P[i - 1] + t * P[i - 2]) / 2.0;
    for (int c = 0; c < 3; ++c) dL[i][c] = P[i - 1] * d1[c] + R * (d0[c] + d1[c]);
  }
}

// Homogenized integrated Jacobi L^alpha_j(x; t), j = 1..p (PolyIJacobi for
// one alpha): value L[j], x-derivative Px[j] = P^alpha_{j-1}(x; t) and
// t-derivative Rt[j].
__host__ __device__ inline void hom_jac(double x, double t, int alpha, int p, double* L,
                                        double* Px, double* Rt) {
  double P[MAXP + 2];
  double y = 2.0 * x - t, tt = t * t;
  P[0] = 1.0;
  P[1] = y + alpha * x;
  for (int i = 2; i <= p; ++i) {
    double a = 2.0 * i * (i + alpha) * (2 * i + alpha - 2);
    double b = 2 * i + alpha - 1;
    double c = (2.0 * i + alpha) * (2 * i + alpha - 2);
    double d = 2.0 * (i + alpha - 1) * (i - 1) * (2 * i + alpha);
    P[i] = (b * (c * y + (double)alpha * alpha * t) * P[i - 1] - d * tt * P[i - 2]) / a;
  }
  L[1] = x;
  Px[1] = 1.0;
  Rt[1] = 0.0;
  for (int i = 2; i <= p; ++i) {
    int ti = 2 * i + alpha;
    double A = (double)(i + alpha) / ((ti - 1.0) * ti);
    double B = (double)alpha / ((ti - 2.0) * ti);
    double C = (i - 1.0) / ((ti - 2.0) * (ti - 1.0));
    L[i] = A * P[i] + B * t * P[i - 1] - C * tt * P[i - 2];
    Px[i] = P[i - 1];
    Rt[i] = -(i - 1.0) * (P[i - 1] + t * P[i - 2]) / (ti - 2.0);
  }
}

// number of triangle-face functions of order p: (p-1)(p-2)/2
__host__ __device__ inline int tri_ndof(int p) { return p > 2 ? (p - 1) * (p - 2) / 2 : 0; }
__host__ __device__ inline int tet_nbub(int p) { return p > 3 ? (p - 1) * (p - 2) * (p - 3) / 6 : 0; }

// Triangle ancillary functions (AncPhiTri with Idec false) of the oriented
// affine triple (s0, s1, s2) with gradients ds[k][c]:
//   phi_{ij} = phiE_i(s0, s1) * L^{2i}_j(s2; s0 + s1 + s2), i >= 2, j >= 1,
// enumerated by n = i + j = 3..p, then i = 2..n-1 (the reference order).
// Writes value and gradient of function q at out[q], dout[q][c].
__host__ __device__ inline int anc_tri(const double* s, const double (*ds)[3], int p,
                                       double* out, double (*dout)[3]) {
  if (p < 3) return 0;
  double E[MAXP + 2], dE[MAXP + 2][3];
  hom_leg(s[0], s[1], ds[0], ds[1], p - 1, E, dE);
  double t = s[0] + s[1] + s[2];
  double dt[3] = {ds[0][0] + ds[1][0] + ds[2][0], ds[0][1] + ds[1][1] + ds[2][1],
                  ds[0][2] + ds[1][2] + ds[2][2]};
  // one Jacobi family per i (alpha = 2i), orders j = 1..p-i
  double J[MAXP + 1][MAXP + 2], Jx[MAXP + 1][MAXP + 2], Jt[MAXP + 1][MAXP + 2];
  for (int i = 2; i <= p - 1; ++i) hom_jac(s[2], t, 2 * i, p - i, J[i], Jx[i], Jt[i]);
  int q = 0;
  for (int n = 3; n <= p; ++n)
    for (int i = 2; i <= n - 1; ++i, ++q) {
      int j = n - i;
      out[q] = E[i] * J[i][j];
      for (int c = 0; c < 3; ++c)
        dout[q][c] = J[i][j] * dE[i][c] + E[i] * (Jx[i][j] * ds[2][c] + Jt[i][j] * dt[c]);
    }
  return q;
}

// OrientTri: GS(k) = S(Or(nori, k))
__host__ __device__ inline int ortri(int o, int k) {
  const int T[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 0}};
  return T[o][k];
}
// Orientation codes o and o' of a triangle face give the same functions up
// to (-1)^i when they differ only by swapping GS(0) and GS(1): the class
// {0,4} puts vertex 2 last, {1,5} vertex 0, {2,3} vertex 1.  tri_class is
// the class (and its canonical code), tri_flip whether o is the swapped one.
__host__ __device__ inline int tri_class(int o) {
  const int T[6] = {0, 1, 2, 2, 0, 1};
  return T[o];
}
__host__ __device__ inline bool tri_flip(int o) { return o >= 3; }

__host__ __device__ inline int tet_e(int e, int k) {
  const int T[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  return T[e][k];
}
__host__ __device__ inline int tet_f(int f, int k) {
  const int T[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};
  return T[f][k];
}

// H1 dof of a tetrahedron with orders nord[0..10] (6 edges, 4 faces, interior).
__host__ __device__ inline int tet_ndof(const int* nord) {
  int n = 4;
  for (int e = 0; e < 6; ++e) n += nord[e] > 1 ? nord[e] - 1 : 0;
  for (int f = 0; f < 4; ++f) n += tri_ndof(nord[6 + f]);
  return n + tet_nbub(nord[10]);
}

// shape3DHTet at xi: orders nord[0..10], edge orientations nori_e[6], face
// orientations nori_f[4]; grad written as grad[c*ldg + k].
__host__ __device__ inline int tet_shape(const double* xi, const int* nord, const int* nori_e,
                                         const int* nori_f, double* shap, double* grad, int ldg) {
  const double lam[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
  const double DL[4][3] = {{-1.0, -1.0, -1.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  int m = 0;
  for (int v = 0; v < 4; ++v, ++m) {
    shap[m] = lam[v];
    for (int c = 0; c < 3; ++c) grad[c * ldg + m] = DL[v][c];
  }
  double L[MAXP + 2], dL[MAXP + 2][3];
  for (int e = 0; e < 6; ++e) {
    int p = nord[e];
    if (p < 2) continue;
    int v0 = tet_e(e, 0), v1 = tet_e(e, 1);
    if (nori_e[e] == 1) { int t = v0; v0 = v1; v1 = t; }
    hom_leg(lam[v0], lam[v1], DL[v0], DL[v1], p, L, dL);
    for (int i = 2; i <= p; ++i, ++m) {
      shap[m] = L[i];
      for (int c = 0; c < 3; ++c) grad[c * ldg + m] = dL[i][c];
    }
  }
  double F[28], dF[28][3];  // up to tri_ndof(MAXP + 1)
  for (int f = 0; f < 4; ++f) {
    int p = nord[6 + f];
    if (tri_ndof(p) == 0) continue;
    double s[3], ds[3][3];
    for (int k = 0; k < 3; ++k) {
      int v = tet_f(f, ortri(nori_f[f], k));
      s[k] = lam[v];
      for (int c = 0; c < 3; ++c) ds[k][c] = DL[v][c];
    }
    int q = anc_tri(s, ds, p, F, dF);
    for (int r = 0; r < q; ++r, ++m) {
      shap[m] = F[r];
      for (int c = 0; c < 3; ++c) grad[c * ldg + m] = dF[r][c];
    }
  }
  int pb = nord[10];
  if (tet_nbub(pb) > 0) {
    // triangle functions of (lam0, lam1, lam2) up to pb-1, times
    // L^{2(i+j)}_k(lam3; 1), enumerated by i+j+k, then i+j, then i
    double s[3] = {lam[0], lam[1], lam[2]}, ds[3][3];
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) ds[k][c] = DL[k][c];
    anc_tri(s, ds, pb - 1, F, dF);
    double K[MAXP + 1][MAXP + 2], Kx[MAXP + 1][MAXP + 2], Kt[MAXP + 1][MAXP + 2];
    for (int n = 3; n <= pb - 1; ++n) hom_jac(lam[3], 1.0, 2 * n, pb - n, K[n], Kx[n], Kt[n]);
    for (int nk = 4; nk <= pb; ++nk)
      for (int n = 3; n <= nk - 1; ++n)
        for (int i = 2; i <= n - 1; ++i, ++m) {
          int k = nk - n;
          int r = (n - 3) * (n - 2) / 2 + (i - 2);  // index of (i, n-i) in F
          double hv = K[n][k], hx = Kx[n][k];
          shap[m] = F[r] * hv;
          for (int c = 0; c < 3; ++c) grad[c * ldg + m] = hv * dF[r][c] + F[r] * hx * DL[3][c];
        }
  }
  return m;
}

// Oriented dof a of a tetrahedron (orders nord, orientations nori_e/nori_f)
// -> dof of its bin element (all orders pm, edge orientation 0, face
// orientation tri_class(nori_f)), with sign.  The hierarchical enumeration
// makes each node's functions a prefix of the bin's.
__host__ __device__ inline uint32_t tet_dof_map(int a, const int* nord, const int* nori_e,
                                                const int* nori_f, int pm) {
  if (a < 4) return (uint32_t)a;
  int off = 4, boff = 4;
  for (int e = 0; e < 6; ++e) {
    int nd = nord[e] > 1 ? nord[e] - 1 : 0;
    if (a < off + nd) {
      int i = a - off + 2;
      bool neg = (nori_e[e] == 1) && (i & 1);
      return (uint32_t)(boff + i - 2) | (neg ? 0x80000000u : 0u);
    }
    off += nd;
    boff += pm - 1;
  }
  for (int f = 0; f < 4; ++f) {
    int nd = tri_ndof(nord[6 + f]);
    if (a < off + nd) {
      int r = a - off, n = 3;
      while (tri_ndof(n) <= r) ++n;
      int i = 2 + r - tri_ndof(n - 1);
      bool neg = tri_flip(nori_f[f]) && (i & 1);
      return (uint32_t)(boff + r) | (neg ? 0x80000000u : 0u);
    }
    off += nd;
    boff += tri_ndof(pm);
  }
  return (uint32_t)(boff + (a - off));
}

}  // namespace hp3dg
