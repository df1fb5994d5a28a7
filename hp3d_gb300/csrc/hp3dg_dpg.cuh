// hp3dg_dpg.cuh -- shape functions and layouts of the ultraweak DPG Maxwell
// element on hexahedra (problems/MAXWELL/ULTRAWEAK_DPG), isotropic order p.
//
// Spaces of an element of trial order p (elem.F90:78-103, elem_maxwell.F90):
//   test   broken H(curl) of order p+NORD_ADD, two fields (F, G): 2 nEE
//   trial  H(curl) interface traces of order p, two components (E, H): 2 nEi
//          L2 fields of order p, six components (E, H):                6 nQ
// The element matrix rows/columns are [traces, component fastest | L2
// fields, six components per shape function]; the test functions are
// interleaved (F, G) per shape function.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hp3dg_internal.cuh"

namespace hp3dg {

constexpr int DPG_MAXP = 5;  // trial order; the test order p+1 <= MAXP

__host__ __device__ inline int dpg_nEE(int q) { return 3 * q * (q + 1) * (q + 1); }
__host__ __device__ inline int dpg_nEi(int p) { return 12 * p + 6 * 2 * p * (p - 1); }
__host__ __device__ inline int dpg_nQ(int p) { return p * p * p; }

// Legendre P_0..P_n of x on [0,1] (PolyLegendre with t = 1)
__host__ __device__ inline void leg01(double x, int n, double* P) {
  double y = 2.0 * x - 1.0;
  P[0] = 1.0;
  if (n >= 1) P[1] = y;
  for (int i = 2; i <= n; ++i) P[i] = ((2 * i - 1) * y * P[i - 1] - (i - 1) * P[i - 2]) / i;
}

// 1D broken H1 (1-x, x, integrated Legendre 2..q) and L2 (Legendre 0..q-1)
// functions of the segment (Segment.F90:30-199)
__host__ __device__ inline void seg_hq(double x, int q, double* h, double* dh, double* l2) {
  h[0] = 1.0 - x; dh[0] = -1.0;
  h[1] = x; dh[1] = 1.0;
  double L[MAXP + 2], dL[MAXP + 2];
  ileg(x, q, L, dL);
  for (int i = 2; i <= q; ++i) { h[i] = L[i]; dh[i] = dL[i]; }
  leg01(x, q - 1, l2);
}

// Broken H(curl) test functions of order q (shape3DEBrokenHexa,
// BrokenHexahedron.F90:139-258): value and curl of function k, written as
// s[c*lds + k], cu[c*lds + k].
__host__ __device__ inline int dpg_test_shape(const double* xi, int q, double* s, double* cu,
                                              int lds) {
  double h[3][MAXP + 2], dh[3][MAXP + 2], l2[3][MAXP + 2];
  for (int d = 0; d < 3; ++d) seg_hq(xi[d], q, h[d], dh[d], l2[d]);
  const int nh = q + 1, nq = q;
  int m = 0;
  for (int k = 0; k < nh; ++k)
    for (int j = 0; j < nh; ++j)
      for (int i = 0; i < nq; ++i, ++m) {
        s[m] = l2[0][i] * h[1][j] * h[2][k]; s[lds + m] = 0.0; s[2 * lds + m] = 0.0;
        cu[m] = 0.0;
        cu[lds + m] = l2[0][i] * h[1][j] * dh[2][k];
        cu[2 * lds + m] = -l2[0][i] * dh[1][j] * h[2][k];
      }
  for (int k = 0; k < nh; ++k)
    for (int j = 0; j < nq; ++j)
      for (int i = 0; i < nh; ++i, ++m) {
        s[m] = 0.0; s[lds + m] = h[0][i] * l2[1][j] * h[2][k]; s[2 * lds + m] = 0.0;
        cu[m] = -h[0][i] * l2[1][j] * dh[2][k];
        cu[lds + m] = 0.0;
        cu[2 * lds + m] = dh[0][i] * l2[1][j] * h[2][k];
      }
  for (int k = 0; k < nq; ++k)
    for (int j = 0; j < nh; ++j)
      for (int i = 0; i < nh; ++i, ++m) {
        s[m] = 0.0; s[lds + m] = 0.0; s[2 * lds + m] = h[0][i] * h[1][j] * l2[2][k];
        cu[m] = h[0][i] * dh[1][j] * l2[2][k];
        cu[lds + m] = -dh[0][i] * h[1][j] * l2[2][k];
        cu[2 * lds + m] = 0.0;
      }
  return m;
}

// L2 functions of order p (shape3DQHexa, Hexahedron.F90:640-698)
__host__ __device__ inline int dpg_l2_shape(const double* xi, int p, double* q) {
  double P[3][MAXP + 2];
  for (int d = 0; d < 3; ++d) leg01(xi[d], p - 1, P[d]);
  int m = 0;
  for (int k = 0; k < p; ++k)
    for (int j = 0; j < p; ++j)
      for (int i = 0; i < p; ++i) q[m++] = P[0][i] * P[1][j] * P[2][k];
  return m;
}

// H(curl) interface traces of order p in the reference enumeration
// (orientation 0): edges (E-type along the edge times the edge blend), then
// per face the two families (shape3DEHexa, Hexahedron.F90:240-400; AncEE /
// AncEQuad with Idec = .true.).  Values only: s[c*lds + k].
__host__ __device__ inline int dpg_trace_shape0(const double* xi, int p, double* s, int lds) {
  double Mu[2][3];
  for (int d = 0; d < 3; ++d) { Mu[0][d] = 1.0 - xi[d]; Mu[1][d] = xi[d]; }
  int m = 0;
  double P[3][MAXP + 2], L[3][MAXP + 2], dL[3][MAXP + 2];
  for (int d = 0; d < 3; ++d) {
    leg01(xi[d], p - 1, P[d]);
    ileg(xi[d], p, L[d], dL[d]);
  }
  for (int e = 0; e < 12; ++e) {
    const double mb = Mu[hexa_e(e, 0)][hexa_e(e, 1)] * Mu[hexa_e(e, 2)][hexa_e(e, 3)];
    const int ax = hexa_e(e, 4);
    for (int i = 0; i < p; ++i, ++m) {
      for (int c = 0; c < 3; ++c) s[c * lds + m] = 0.0;
      s[ax * lds + m] = mb * P[ax][i];  // P_i(xi_ax) grad(xi_ax)
    }
  }
  for (int f = 0; f < 6; ++f) {
    const double mbf = Mu[hexa_f(f, 0)][hexa_f(f, 1)];
    const int a1 = hexa_f(f, 2), a2 = hexa_f(f, 3);
    // family 0: E along axis a1 (index i), phi along a2 (index j); j outer
    for (int j = 2; j <= p; ++j)
      for (int i = 0; i < p; ++i, ++m) {
        for (int c = 0; c < 3; ++c) s[c * lds + m] = 0.0;
        s[a1 * lds + m] = mbf * P[a1][i] * L[a2][j];
      }
    // family 1: E along axis a2 (index i), phi along a1 (index j); i outer
    for (int i = 0; i < p; ++i)
      for (int j = 2; j <= p; ++j, ++m) {
        for (int c = 0; c < 3; ++c) s[c * lds + m] = 0.0;
        s[a2 * lds + m] = mbf * P[a2][i] * L[a1][j];
      }
  }
  return m;
}

// Element trace function k (with the element's edge and face orientation
// codes) = sign * reference function perm[k]: OrientE reverses the edge
// coordinate (P_i(1-x) grad(1-x) = (-1)^(i+1) P_i(x) grad x); OrientQuad
// may swap the face axes (exchanging the families) and reverse either axis
// ((-1)^(i+1) on the E-type factor, (-1)^j on the integrated Legendre one).
// Encoded as perm | (sign < 0) << 31.
__host__ __device__ inline void dpg_trace_perm(int p, const int* nori_e, const int* nori_f,
                                               uint32_t* perm) {
  int m = 0;
  for (int e = 0; e < 12; ++e)
    for (int i = 0; i < p; ++i, ++m) {
      const bool neg = nori_e[e] == 1 && ((i + 1) & 1);
      perm[m] = (uint32_t)m | (neg ? 0x80000000u : 0u);
    }
  const int nf = p * (p - 1);  // functions per family
  for (int f = 0; f < 6; ++f) {
    const int base = 12 * p + f * 2 * nf;
    const int o = nori_f[f] & 7;
    const int swap = orq(o, 0), r1 = orq(o, 2), r2 = orq(o, 4);
    for (int fam = 0; fam < 2; ++fam) {
      // element function (fam, i, j): E along GS (fam 0) or GT (fam 1)
      const int re = fam == 0 ? r1 : r2, rp = fam == 0 ? r2 : r1;
      const int tfam = swap ? 1 - fam : fam;  // reference family with the same axes
      for (int o1 = 0; o1 < (fam == 0 ? p - 1 : p); ++o1)
        for (int o2 = 0; o2 < (fam == 0 ? p : p - 1); ++o2, ++m) {
          const int i = fam == 0 ? o2 : o1, j = fam == 0 ? o1 + 2 : o2 + 2;
          const int t = tfam == 0 ? (j - 2) * p + i : nf + i * (p - 1) + (j - 2);
          const int par = re * (i + 1) + rp * j;
          perm[m] = (uint32_t)(base + t) | ((par & 1) ? 0x80000000u : 0u);
        }
    }
  }
}

}  // namespace hp3dg
