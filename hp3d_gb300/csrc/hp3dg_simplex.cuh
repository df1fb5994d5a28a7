// hp3dg_simplex.cuh -- H1 shape functions of the tetrahedron and the prism
// for the bin tables, plus the element -> bin dof maps of both.
//
// Restates shape_1/Tetrahedron.F90:33-234 (shape3DHTet) with the ancillary
// routines it calls: AncPhiE / AncPhiTri (Ancillary.F90:37-58, 397-442),
// HomILegendre / HomIJacobi / PolyIJacobi / PolyJacobi (Polynomials.F90:
// 197-431, 497-646), OrientE / OrientTri (Orient.F90:9-37, 119-162),
// AffineTetrahedron (AffineCoordinates.F90:74-89) and ProjectTetE/F
// (BlendProject.F90:470-560); and shape_1/Prism.F90:33-330 (shape3DHPris)
// with AffinePrism, BlendPrisV, BlendProjectPrisME/QE/TF, ProjectPrisQF
// (BlendProject.F90:562-804), OrientQuad (Orient.F90:39-116) and AncPhiQuad
// (Ancillary.F90:171-206).
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
// unit_t: the triple sums to one identically (AncPhiTri with Idec true):
// the Jacobi factor then uses t = 1 and has no t-derivative.
__host__ __device__ inline int anc_tri(const double* s, const double (*ds)[3], int p,
                                       double* out, double (*dout)[3], bool unit_t = false) {
  if (p < 3) return 0;
  double E[MAXP + 2], dE[MAXP + 2][3];
  hom_leg(s[0], s[1], ds[0], ds[1], p - 1, E, dE);
  double t = unit_t ? 1.0 : s[0] + s[1] + s[2];
  double dt[3] = {ds[0][0] + ds[1][0] + ds[2][0], ds[0][1] + ds[1][1] + ds[2][1],
                  ds[0][2] + ds[1][2] + ds[2][2]};
  if (unit_t) dt[0] = dt[1] = dt[2] = 0.0;
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

// ---------------------------------------------------------------------------
// prism
// ---------------------------------------------------------------------------
// Norder layout (15 used): [0..5] mixed (horizontal) edges, [6..8] quad
// (vertical) edges, [9..10] triangle faces, [11..13] quad faces (h*10+v in
// the face's frame), [14] interior (ph*10+pz).
__host__ __device__ inline int prism_nupair(int k, int s) {
  const int T[3][2] = {{0, 1}, {1, 2}, {0, 2}};
  return T[k][s];
}
__host__ __device__ inline int prism_nbub(const int* nord) {
  int ph = nord[14] / 10, pz = nord[14] % 10;
  return pz > 1 ? tri_ndof(ph) * (pz - 1) : 0;
}
__host__ __device__ inline int prism_ndof(const int* nord) {
  int n = 6;
  for (int e = 0; e < 9; ++e) n += nord[e] > 1 ? nord[e] - 1 : 0;
  for (int f = 0; f < 2; ++f) n += tri_ndof(nord[9 + f]);
  for (int f = 0; f < 3; ++f) {
    int h, v; decod2(nord[11 + f], h, v);
    n += (h > 1 && v > 1) ? (h - 1) * (v - 1) : 0;
  }
  return n + prism_nbub(nord);
}

// integrated Legendre L_i(x; 1), i = 2..p, gradient P_{i-1}(x) dx
__host__ __device__ inline void leg_unit(double x, const double* dx, int p, double* L,
                                         double (*dL)[3]) {
  double l[MAXP + 2], dl[MAXP + 2];
  ileg(x, p, l, dl);
  for (int i = 2; i <= p; ++i) {
    L[i] = l[i];
    for (int c = 0; c < 3; ++c) dL[i][c] = dl[i] * dx[c];
  }
}

__host__ __device__ inline int prism_shape(const double* xi, const int* nord, const int* nori_e,
                                           const int* nori_f, double* shap, double* grad, int ldg) {
  const double Nu[3] = {1.0 - xi[0] - xi[1], xi[0], xi[1]};
  const double DNu[3][3] = {{-1.0, -1.0, 0.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}};
  const double Mu[2] = {1.0 - xi[2], xi[2]};
  const double DMu[2][3] = {{0.0, 0.0, -1.0}, {0.0, 0.0, 1.0}};
  int m = 0;
  for (int v = 0; v < 6; ++v, ++m) {
    int a = v % 3, b = v / 3;
    shap[m] = Nu[a] * Mu[b];
    for (int c = 0; c < 3; ++c) grad[c * ldg + m] = DNu[a][c] * Mu[b] + Nu[a] * DMu[b][c];
  }
  double L[MAXP + 2], dL[MAXP + 2][3];
  for (int e = 0; e < 6; ++e) {  // mixed edges: Nu pair (homogenized) x Mu blend
    int p = nord[e];
    if (p < 2) continue;
    int a = prism_nupair(e % 3, 0), b = prism_nupair(e % 3, 1), mb = e / 3;
    if (nori_e[e] == 1) { int t = a; a = b; b = t; }
    hom_leg(Nu[a], Nu[b], DNu[a], DNu[b], p, L, dL);
    for (int i = 2; i <= p; ++i, ++m) {
      shap[m] = L[i] * Mu[mb];
      for (int c = 0; c < 3; ++c) grad[c * ldg + m] = dL[i][c] * Mu[mb] + L[i] * DMu[mb][c];
    }
  }
  for (int e = 0; e < 3; ++e) {  // quad edges: Mu pair (t = 1) x Nu blend
    int p = nord[6 + e];
    if (p < 2) continue;
    int o1 = nori_e[6 + e] == 1 ? 0 : 1;
    leg_unit(Mu[o1], DMu[o1], p, L, dL);
    for (int i = 2; i <= p; ++i, ++m) {
      shap[m] = L[i] * Nu[e];
      for (int c = 0; c < 3; ++c) grad[c * ldg + m] = dL[i][c] * Nu[e] + L[i] * DNu[e][c];
    }
  }
  double F[28], dF[28][3];
  for (int f = 0; f < 2; ++f) {  // triangle faces: oriented Nu triple (t = 1) x Mu blend
    int p = nord[9 + f];
    if (tri_ndof(p) == 0) continue;
    double sv[3], ds[3][3];
    for (int k = 0; k < 3; ++k) {
      int a = ortri(nori_f[f], k);
      sv[k] = Nu[a];
      for (int c = 0; c < 3; ++c) ds[k][c] = DNu[a][c];
    }
    int q = anc_tri(sv, ds, p, F, dF, true);
    for (int r = 0; r < q; ++r, ++m) {
      shap[m] = F[r] * Mu[f];
      for (int c = 0; c < 3; ++c) grad[c * ldg + m] = dF[r][c] * Mu[f] + F[r] * DMu[f][c];
    }
  }
  for (int f = 0; f < 3; ++f) {  // quad faces: OrientQuad of (Nu pair, Mu pair)
    int h, v; decod2(nord[11 + f], h, v);
    if (h < 2 || v < 2) continue;
    int o = nori_f[2 + f] & 7;
    const int na = prism_nupair(f, 0), nb = prism_nupair(f, 1);
    // pair q, end k: value and gradient (pair 0 = Nu, general; pair 1 = Mu, t = 1)
    auto st = [&](int k, int q) { return q == 0 ? Nu[k ? nb : na] : Mu[k]; };
    auto dst = [&](int k, int q) { return q == 0 ? DNu[k ? nb : na] : DMu[k]; };
    double LS[MAXP + 2], dLS[MAXP + 2][3], LT[MAXP + 2], dLT[MAXP + 2][3];
    int pa1 = orq(o, 0), pa2 = orq(o, 1);
    if (pa1 == 0) hom_leg(st(orq(o, 2), 0), st(orq(o, 3), 0), dst(orq(o, 2), 0), dst(orq(o, 3), 0), h, LS, dLS);
    else leg_unit(st(orq(o, 3), 1), dst(orq(o, 3), 1), h, LS, dLS);
    if (pa2 == 0) hom_leg(st(orq(o, 4), 0), st(orq(o, 5), 0), dst(orq(o, 4), 0), dst(orq(o, 5), 0), v, LT, dLT);
    else leg_unit(st(orq(o, 5), 1), dst(orq(o, 5), 1), v, LT, dLT);
    for (int j = 2; j <= v; ++j)
      for (int i = 2; i <= h; ++i, ++m) {
        shap[m] = LS[i] * LT[j];
        for (int c = 0; c < 3; ++c) grad[c * ldg + m] = LS[i] * dLT[j][c] + LT[j] * dLS[i][c];
      }
  }
  int ph = nord[14] / 10, pz = nord[14] % 10;
  if (tri_ndof(ph) > 0 && pz >= 2) {  // bubbles: triangle(Nu; t = 1) x L_k(z)
    double sv[3] = {Nu[0], Nu[1], Nu[2]}, ds[3][3];
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) ds[k][c] = DNu[k][c];
    int q = anc_tri(sv, ds, ph, F, dF, true);
    leg_unit(Mu[1], DMu[1], pz, L, dL);
    for (int k = 2; k <= pz; ++k)
      for (int r = 0; r < q; ++r, ++m) {
        shap[m] = F[r] * L[k];
        for (int c = 0; c < 3; ++c) grad[c * ldg + m] = dF[r][c] * L[k] + F[r] * dL[k][c];
      }
  }
  return m;
}

// Local (bin) orders of a prism: quad faces in the element's own frame
// (find_order_loc, datstrs/find_order.F90:88-94), then the per-direction
// maxima (horizontal ph, vertical pz) that set_3Dint_aux integrates
// (quadrature/set_3D_int.F90:264-290), spread over every node.
__host__ __device__ inline void prism_bin_orders(const int* nord, const int* nori_f, int* full) {
  int ph = 0, pz = 0;
  for (int e = 0; e < 6; ++e) ph = nord[e] > ph ? nord[e] : ph;
  for (int e = 6; e < 9; ++e) pz = nord[e] > pz ? nord[e] : pz;
  for (int f = 9; f < 11; ++f) ph = nord[f] > ph ? nord[f] : ph;
  for (int f = 0; f < 4; ++f) {
    int h, v; decod2(nord[11 + f], h, v);
    if (f < 3 && nfaxes_swap(nori_f[2 + f])) { int t = h; h = v; v = t; }
    ph = h > ph ? h : ph;
    pz = v > pz ? v : pz;
  }
  for (int i = 0; i < 19; ++i) full[i] = 0;
  for (int e = 0; e < 6; ++e) full[e] = ph;
  for (int e = 6; e < 9; ++e) full[e] = pz;
  full[9] = full[10] = ph;
  for (int f = 11; f < 15; ++f) full[f] = 10 * ph + pz;
}

// Oriented dof a of a prism (orders nord in the global frames, orientations
// nori_e / nori_f) -> dof of its bin element (orders full from
// prism_bin_orders, edge and quad-face orientation 0, triangle faces in the
// class tri_class(nori_f)), with sign.
__host__ __device__ inline uint32_t prism_dof_map(int a, const int* nord, const int* nori_e,
                                                  const int* nori_f, const int* full) {
  if (a < 6) return (uint32_t)a;
  const int ph = full[14] / 10, pz = full[14] % 10;
  int off = 6, boff = 6;
  for (int e = 0; e < 9; ++e) {
    int nd = nord[e] > 1 ? nord[e] - 1 : 0;
    if (a < off + nd) {
      int i = a - off + 2;
      bool neg = (nori_e[e] == 1) && (i & 1);
      return (uint32_t)(boff + i - 2) | (neg ? 0x80000000u : 0u);
    }
    off += nd;
    boff += (e < 6 ? ph : pz) - 1;
  }
  for (int f = 0; f < 2; ++f) {
    int nd = tri_ndof(nord[9 + f]);
    if (a < off + nd) {
      int r = a - off, n = 3;
      while (tri_ndof(n) <= r) ++n;
      int i = 2 + r - tri_ndof(n - 1);
      bool neg = tri_flip(nori_f[f]) && (i & 1);
      return (uint32_t)(boff + r) | (neg ? 0x80000000u : 0u);
    }
    off += nd;
    boff += tri_ndof(ph);
  }
  for (int f = 0; f < 3; ++f) {
    int n1, n2; decod2(nord[11 + f], n1, n2);
    int nd = (n1 > 1 && n2 > 1) ? (n1 - 1) * (n2 - 1) : 0;
    if (a < off + nd) {
      int r = a - off;
      int i = r % (n1 - 1) + 2, j = r / (n1 - 1) + 2;
      int o = nori_f[2 + f] & 7;
      bool swap = orq(o, 0) == 1;
      bool negs = (orq(o, 3) == 0) && (i & 1);
      bool negt = (orq(o, 5) == 0) && (j & 1);
      int il = swap ? j : i, jl = swap ? i : j;  // indices in the element's own frame
      return (uint32_t)(boff + (jl - 2) * (ph - 1) + (il - 2)) | ((negs != negt) ? 0x80000000u : 0u);
    }
    off += nd;
    boff += (ph - 1) * (pz - 1);
  }
  int eh = nord[14] / 10;
  int r = a - off, te = tri_ndof(eh);
  int k = r / te, t = r % te;
  return (uint32_t)(boff + k * tri_ndof(ph) + t);
}

}  // namespace hp3dg
