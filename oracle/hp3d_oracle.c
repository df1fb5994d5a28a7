/*
 * hp3d_oracle.c -- CPU FP64 restatement of the hp3D element pass.
 *
 * TEST INFRASTRUCTURE ONLY (see hp3d_oracle.h).  Compiled with
 * -ffp-contract=off so that x86-64 and aarch64 hosts give identical bits.
 * Citations are to Oden-EAG/hp3d, paths relative to trunk/.
 */
#include "hp3d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* 1D Gauss-Legendre tables on [-1,1].  The reference tabulates them as      */
/* 15-digit literals (src/element/quadrature/gauss_quadrature.F90:518-660,   */
/* 25 digits for n=10); an oracle that wants the reference's element         */
/* matrices bit for bit must use the same rounded values, so these are the   */
/* same decimal numbers (the standard Gauss nodes/weights at that precision). */
/* ------------------------------------------------------------------------ */
static const double GAUSS_X[10][10] = {
    {0.0},
    {-.577350269189626, .577350269189626},
    {-.774596669241483, .000000000000000, .774596669241483},
    {-.861136311594053, -.339981043584856, .339981043584856, .861136311594053},
    {-.906179845938664, -.538469310105683, .000000000000000, .538469310105683,
     .906179845938664},
    {-.932469514203152, -.661209386466265, -.238619186083197, .238619186083197,
     .661209386466265, .932469514203152},
    {-.949107912342759, -.741531185599394, -.405845151377397, .000000000000000,
     .405845151377397, .741531185599394, .949107912342759},
    {-.960289856497536, -.796666477413627, -.525532409916329, -.183434642495650,
     .183434642495650, .525532409916329, .796666477413627, .960289856497536},
    {-.968160239507626, -.836031107326636, -.613371432700590, -.324253423403809,
     .000000000000000, .324253423403809, .613371432700590, .836031107326636,
     .968160239507626},
    {-.9739065285171717200779640, -.8650633666889845107320967,
     -.6794095682990244062343274, -.4333953941292471907992659,
     -.1488743389816312108848260, .1488743389816312108848260,
     .4333953941292471907992659, .6794095682990244062343274,
     .8650633666889845107320967, .9739065285171717200779640}};

static const double GAUSS_W[10][10] = {
    {2.000000000000000},
    {1.000000000000000, 1.000000000000000},
    {.555555555555556, .888888888888889, .555555555555556},
    {.347854845137454, .652145154862546, .652145154862546, .347854845137454},
    {.236926885056189, .478628670499366, .568888888888889, .478628670499366,
     .236926885056189},
    {.171324492379170, .360761573048139, .467913934572691, .467913934572691,
     .360761573048139, .171324492379170},
    {.129484966168870, .279705391489277, .381830050505119, .417959183673469,
     .381830050505119, .279705391489277, .129484966168870},
    {.101228536290376, .222381034453374, .313706645877887, .362683783378362,
     .362683783378362, .313706645877887, .222381034453374, .101228536290376},
    {.081274388361574, .180648160694857, .260610696402935, .312347077040003,
     .330239355001260, .312347077040003, .260610696402935, .180648160694857,
     .081274388361574},
    {.0666713443086881375935688, .1494513491505805931457763,
     .2190863625159820439955349, .2692667193099963550912269,
     .2955242247147528701738930, .2955242247147528701738930,
     .2692667193099963550912269, .2190863625159820439955349,
     .1494513491505805931457763, .0666713443086881375935688}};

/* rescale to [0,1]: gauss_quadrature.F90:749-750 */
int orc_gauss1d(int n, double *x, double *w) {
  if (n < 1 || n > 10) return -1;
  for (int j = 0; j < n; ++j) {
    x[j] = 0.5 * (1.0 + GAUSS_X[n - 1][j]);
    w[j] = 0.5 * GAUSS_W[n - 1][j];
  }
  return 0;
}

/* decod (utility/decod.F90): split Nick into n digits base mod, most
 * significant first. */
static void decod(int nick, int mod, int n, int *arr) {
  int nick1 = nick;
  for (int i = 1; i <= n - 1; ++i) {
    int nick2 = nick1 / mod;
    arr[n - i] = nick1 - nick2 * mod;
    nick1 = nick2;
  }
  arr[0] = nick1;
}

/* NFAXES(3,j): 1 when orientation j swaps the two face axes
 * (modules/element_data.F90:246-249). */
static const int NFAXES3[8] = {0, 1, 0, 1, 1, 0, 1, 0};

static int imax(int a, int b) { return a > b ? a : b; }
static int imin(int a, int b) { return a < b ? a : b; }

/* set_3D_int BRICK branch (set_3D_int.F90:47-64, 155-245) with the face
 * order swap of find_order_loc (datstrs/find_order.F90:68-108). */
int orc_set_3D_int_hexa(const int32_t *norder, const int32_t *nori_face,
                        int integration, double *xiloc, double *waloc) {
  int nl[19];
  for (int i = 0; i < 19; ++i) nl[i] = norder[i];
  for (int j = 0; j < 6; ++j) {
    if (NFAXES3[nori_face[j] & 7] == 1) {
      int hv[2];
      decod(norder[12 + j], 10, 2, hv);
      nl[12 + j] = hv[1] * 10 + hv[0];
    }
  }
  int nx = 0, ny = 0, nz = 0;
  for (int i = 1; i <= 19; ++i) {
    int hv[2], xyz[3];
    switch (i) {
      case 1: case 3: case 5: case 7: nx = imax(nx, nl[i - 1]); break;
      case 2: case 4: case 6: case 8: ny = imax(ny, nl[i - 1]); break;
      case 9: case 10: case 11: case 12: nz = imax(nz, nl[i - 1]); break;
      case 13: case 14:
        decod(nl[i - 1], 10, 2, hv); nx = imax(nx, hv[0]); ny = imax(ny, hv[1]);
        break;
      case 15: case 17:
        decod(nl[i - 1], 10, 2, hv); nx = imax(nx, hv[0]); nz = imax(nz, hv[1]);
        break;
      case 16: case 18:
        decod(nl[i - 1], 10, 2, hv); ny = imax(ny, hv[0]); nz = imax(nz, hv[1]);
        break;
      case 19:
        decod(nl[i - 1], 10, 3, xyz);
        nx = imax(nx, xyz[0]); ny = imax(ny, xyz[1]); nz = imax(nz, xyz[2]);
        break;
    }
  }
  nx = imin(nx + integration, ORC_MAXP);
  ny = imin(ny + integration, ORC_MAXP);
  nz = imin(nz + integration, ORC_MAXP);
  int nix = nx + 1, niy = ny + 1, niz = nz + 1;
  double gx[10], gwx[10], gy[10], gwy[10], gz[10], gwz[10];
  orc_gauss1d(nix, gx, gwx);
  orc_gauss1d(niy, gy, gwy);
  orc_gauss1d(niz, gz, gwz);
  int l = 0;
  for (int l3 = 0; l3 < niz; ++l3)
    for (int l2 = 0; l2 < niy; ++l2)
      for (int l1 = 0; l1 < nix; ++l1) {
        xiloc[3 * l + 0] = gx[l1];
        xiloc[3 * l + 1] = gy[l2];
        xiloc[3 * l + 2] = gz[l3];
        waloc[l] = gwx[l1] * gwy[l2] * gwz[l3];
        ++l;
      }
  return l;
}

/* ------------------------------------------------------------------------ */
/* Polynomials (src/element/shape_1/Polynomials.F90)                         */
/* ------------------------------------------------------------------------ */

/* PolyLegendre (Polynomials.F90:34-80): shifted scaled Legendre P(0:nord). */
static void poly_legendre(double x, double t, int nord, double *p) {
  p[0] = 1.0;
  double y = 0.0;
  if (nord >= 1) {
    y = 2.0 * x - t;
    p[1] = y;
  }
  if (nord >= 2) {
    double tt = t * t;
    for (int i = 2; i <= nord; ++i) {
      p[i] = (double)(2 * i - 1) * y * p[i - 1] - (double)(i - 1) * tt * p[i - 2];
      p[i] = p[i] / (double)i;
    }
  }
}

/* PolyILegendre (Polynomials.F90:113-160): integrated Legendre L(2:nord),
 * x-derivative P(1:nord-1) and t-derivative R(1:nord-1). Arrays are indexed
 * by the polynomial order (L[i], P[i-1] stored at index i-1). */
static void poly_ilegendre(double x, double t, int nord, int idec, double *L,
                           double *P, double *R) {
  double pt[16];
  poly_legendre(x, t, nord, pt);
  for (int i = 1; i <= nord - 1; ++i) P[i] = pt[i];
  double tt = t * t;
  for (int i = 2; i <= nord; ++i) {
    int ifact = 4 * i - 2;
    L[i] = (pt[i] - tt * pt[i - 2]) / (double)ifact;
    if (!idec) R[i - 1] = -(pt[i - 1] + t * pt[i - 2]) / 2.0;
  }
}

/* HomILegendre (Polynomials.F90:494-530): homogenized integrated Legendre of
 * the pair S=(s0,s1) with gradients DS(3,0:1); outputs HomL(i), DHomL(3,i)
 * for i=2..nord (stored at index i). */
static void hom_ilegendre(const double *S, const double DS[3][2], int nord,
                          int idec, double *homL, double dhomL[][3]) {
  double homP[16], homR[16];
  if (idec) {
    poly_ilegendre(S[1], 1.0, nord, 1, homL, homP, homR);
    for (int i = 2; i <= nord; ++i)
      for (int c = 0; c < 3; ++c) dhomL[i][c] = homP[i - 1] * DS[c][1];
  } else {
    poly_ilegendre(S[1], S[0] + S[1], nord, 0, homL, homP, homR);
    double ds01[3];
    for (int c = 0; c < 3; ++c) ds01[c] = DS[c][0] + DS[c][1];
    for (int i = 2; i <= nord; ++i)
      for (int c = 0; c < 3; ++c)
        dhomL[i][c] = homP[i - 1] * DS[c][1] + homR[i - 1] * ds01[c];
  }
}

/* ------------------------------------------------------------------------ */
/* Hexahedron H1 (Hexahedron.F90:33-210; AffineHexahedron,                    */
/* AffineCoordinates.F90:56-72; BlendHexaV / BlendProjectHexaE/F,             */
/* BlendProject.F90:197-439; OrientE / OrientQuad, Orient.F90:9-116).         */
/* ------------------------------------------------------------------------ */

/* vertex -> (which Mu per axis) : BlendHexaV */
static const int HEXA_V[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                 {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
/* edge -> blend1 (side, axis), blend2 (side, axis), projection axis :
 * BlendProjectHexaE */
static const int HEXA_E[12][5] = {
    {0, 1, 0, 2, 0}, {1, 0, 0, 2, 1}, {1, 1, 0, 2, 0}, {0, 0, 0, 2, 1},
    {0, 1, 1, 2, 0}, {1, 0, 1, 2, 1}, {1, 1, 1, 2, 0}, {0, 0, 1, 2, 1},
    {0, 0, 0, 1, 2}, {1, 0, 0, 1, 2}, {1, 0, 1, 1, 2}, {0, 0, 1, 1, 2}};
/* face -> blend (side, axis), pair-1 axis, pair-2 axis : BlendProjectHexaF */
static const int HEXA_F[6][4] = {{0, 2, 0, 1}, {1, 2, 0, 1}, {0, 1, 0, 2},
                                 {1, 0, 1, 2}, {1, 1, 0, 2}, {0, 0, 1, 2}};
/* OrientQuad tables (Orient.F90:59-116): OrPa(1:2), OrGS(0:1), OrGT(0:1)
 * with pairs 0-based. */
static const int ORQ[8][6] = {{0, 1, 0, 1, 0, 1}, {1, 0, 0, 1, 1, 0},
                              {0, 1, 1, 0, 1, 0}, {1, 0, 1, 0, 0, 1},
                              {1, 0, 0, 1, 0, 1}, {0, 1, 1, 0, 0, 1},
                              {1, 0, 1, 0, 1, 0}, {0, 1, 0, 1, 1, 0}};

int orc_nrdofH_hexa(const int32_t *norder) {
  int n = 8;
  for (int e = 0; e < 12; ++e) n += imax(norder[e] - 1, 0);
  for (int f = 0; f < 6; ++f) {
    int hv[2];
    decod(norder[12 + f], 10, 2, hv);
    n += imax(hv[0] - 1, 0) * imax(hv[1] - 1, 0);
  }
  int b[3];
  decod(norder[18], 10, 3, b);
  n += imax(b[0] - 1, 0) * imax(b[1] - 1, 0) * imax(b[2] - 1, 0);
  return n;
}

int orc_nrdofH_bubble(int etype, const int32_t *norder) {
  if (etype == ORC_HEXA) {
    int b[3];
    decod(norder[18], 10, 3, b);
    return imax(b[0] - 1, 0) * imax(b[1] - 1, 0) * imax(b[2] - 1, 0);
  }
  if (etype == ORC_TET) {
    int p = norder[10];
    return (p - 3) * (p - 2) * (p - 1) / 6 > 0 ? (p - 3) * (p - 2) * (p - 1) / 6 : 0;
  }
  if (etype == ORC_PRISM) {
    int ph = norder[14] / 10, pz = norder[14] % 10;
    return (ph > 2 && pz > 1) ? (ph - 1) * (ph - 2) / 2 * (pz - 1) : 0;
  }
  return -1;
}

int orc_shape3DH_hexa(const double *xi, const int32_t *nord,
                      const int32_t *nori_edge, const int32_t *nori_face,
                      double *shap, double *grad) {
  /* AffineHexahedron */
  double Mu[2][3], DMu[3][2][3];
  for (int d = 0; d < 3; ++d) {
    Mu[0][d] = 1.0 - xi[d];
    Mu[1][d] = xi[d];
    for (int c = 0; c < 3; ++c) {
      DMu[c][0][d] = 0.0;
      DMu[c][1][d] = 0.0;
    }
    DMu[d][0][d] = -1.0;
    DMu[d][1][d] = 1.0;
  }
  int m = 0;
  /* vertices */
  for (int v = 0; v < 8; ++v) {
    const int *s = HEXA_V[v];
    double b1 = Mu[s[0]][0], b2 = Mu[s[1]][1], b3 = Mu[s[2]][2];
    shap[m] = b1 * b2 * b3;
    for (int c = 0; c < 3; ++c)
      grad[3 * m + c] = b1 * b2 * DMu[c][s[2]][2] + b1 * DMu[c][s[1]][1] * b3 +
                        DMu[c][s[0]][0] * b2 * b3;
    ++m;
  }
  /* edges */
  for (int e = 0; e < 12; ++e) {
    int ndofE = nord[e] - 1;
    if (ndofE <= 0) continue;
    const int *t = HEXA_E[e];
    double mb1 = Mu[t[0]][t[1]], mb2 = Mu[t[2]][t[3]];
    double dmb1[3], dmb2[3];
    for (int c = 0; c < 3; ++c) {
      dmb1[c] = DMu[c][t[0]][t[1]];
      dmb2[c] = DMu[c][t[2]][t[3]];
    }
    int ax = t[4];
    /* OrientE: Nori=1 swaps the pair */
    int o0 = (nori_edge[e] == 1) ? 1 : 0, o1 = 1 - o0;
    double GS[2] = {Mu[o0][ax], Mu[o1][ax]};
    double GDS[3][2];
    for (int c = 0; c < 3; ++c) {
      GDS[c][0] = DMu[c][o0][ax];
      GDS[c][1] = DMu[c][o1][ax];
    }
    double phi[16], dphi[16][3];
    hom_ilegendre(GS, GDS, nord[e], 1, phi, dphi);
    for (int i = 2; i <= nord[e]; ++i) {
      shap[m] = mb1 * mb2 * phi[i];
      for (int c = 0; c < 3; ++c)
        grad[3 * m + c] = mb1 * mb2 * dphi[i][c] + mb1 * dmb2[c] * phi[i] +
                          dmb1[c] * mb2 * phi[i];
      ++m;
    }
  }
  /* faces */
  for (int f = 0; f < 6; ++f) {
    int nf[2];
    decod(nord[12 + f], 10, 2, nf);
    int ndofF = (nf[0] - 1) * (nf[1] - 1);
    if (nf[0] < 2 || nf[1] < 2 || ndofF <= 0) continue;
    const int *t = HEXA_F[f];
    double mbf = Mu[t[0]][t[1]];
    double dmbf[3];
    for (int c = 0; c < 3; ++c) dmbf[c] = DMu[c][t[0]][t[1]];
    /* local pairs ST(0:1, 1:2) */
    int axes[2] = {t[2], t[3]};
    const int *oq = ORQ[nori_face[f] & 7];
    /* GST(:,1) = ST(OrGS(:), OrPa(1)); GST(:,2) = ST(OrGT(:), OrPa(2)) */
    double GS[2], GT[2], GDS[3][2], GDT[3][2];
    int pa1 = axes[oq[0]], pa2 = axes[oq[1]];
    GS[0] = Mu[oq[2]][pa1];
    GS[1] = Mu[oq[3]][pa1];
    GT[0] = Mu[oq[4]][pa2];
    GT[1] = Mu[oq[5]][pa2];
    for (int c = 0; c < 3; ++c) {
      GDS[c][0] = DMu[c][oq[2]][pa1];
      GDS[c][1] = DMu[c][oq[3]][pa1];
      GDT[c][0] = DMu[c][oq[4]][pa2];
      GDT[c][1] = DMu[c][oq[5]][pa2];
    }
    double phs[16], dphs[16][3], pht[16], dpht[16][3];
    hom_ilegendre(GS, GDS, nf[0], 1, phs, dphs);
    hom_ilegendre(GT, GDT, nf[1], 1, pht, dpht);
    for (int j = 2; j <= nf[1]; ++j)
      for (int i = 2; i <= nf[0]; ++i) {
        double pq = phs[i] * pht[j];
        shap[m] = mbf * pq;
        for (int c = 0; c < 3; ++c) {
          double dpq = phs[i] * dpht[j][c] + pht[j] * dphs[i][c];
          grad[3 * m + c] = mbf * dpq + dmbf[c] * pq;
        }
        ++m;
      }
  }
  /* bubbles */
  int nb[3];
  decod(nord[18], 10, 3, nb);
  if (nb[0] >= 2 && nb[1] >= 2 && nb[2] >= 2) {
    double S0[2] = {Mu[0][0], Mu[1][0]}, S1[2] = {Mu[0][1], Mu[1][1]},
           S2[2] = {Mu[0][2], Mu[1][2]};
    double D0[3][2], D1[3][2], D2[3][2];
    for (int c = 0; c < 3; ++c) {
      D0[c][0] = DMu[c][0][0]; D0[c][1] = DMu[c][1][0];
      D1[c][0] = DMu[c][0][1]; D1[c][1] = DMu[c][1][1];
      D2[c][0] = DMu[c][0][2]; D2[c][1] = DMu[c][1][2];
    }
    double px[16], dpx[16][3], py[16], dpy[16][3], pz[16], dpz[16][3];
    hom_ilegendre(S0, D0, nb[0], 1, px, dpx);
    hom_ilegendre(S1, D1, nb[1], 1, py, dpy);
    hom_ilegendre(S2, D2, nb[2], 1, pz, dpz);
    for (int k = 2; k <= nb[2]; ++k)
      for (int j = 2; j <= nb[1]; ++j)
        for (int i = 2; i <= nb[0]; ++i) {
          double pq = px[i] * py[j];
          shap[m] = pq * pz[k];
          for (int c = 0; c < 3; ++c) {
            double dpq = px[i] * dpy[j][c] + py[j] * dpx[i][c];
            grad[3 * m + c] = pq * dpz[k][c] + dpq * pz[k];
          }
          ++m;
        }
  }
  return m;
}

/* ------------------------------------------------------------------------ */
/* Geometry (src/element/util/geom.F90:30-138)                               */
/* dxdxi[i + 3*j] = dx_i/dxi_j (Fortran Dxdxi(i,j)); same for dxidx.          */
/* ------------------------------------------------------------------------ */
#define A(i, j) dxdxi[(i - 1) + 3 * (j - 1)]
#define B(i, j) dxidx[(i - 1) + 3 * (j - 1)]
int orc_geom(const double *dxdxi, double *dxidx, double *rjac) {
  int iflag = 0;
  double r = A(1, 1) * A(2, 2) * A(3, 3) + A(2, 1) * A(3, 2) * A(1, 3) +
             A(3, 1) * A(1, 2) * A(2, 3) - A(3, 1) * A(2, 2) * A(1, 3) -
             A(1, 1) * A(3, 2) * A(2, 3) - A(2, 1) * A(1, 2) * A(3, 3);
  if (r < 0.0) iflag = 1;
  double d1, d2, d3;
  d1 = A(2, 2) * A(3, 3) - A(3, 2) * A(2, 3);
  d2 = -A(2, 1) * A(3, 3) + A(3, 1) * A(2, 3);
  d3 = A(2, 1) * A(3, 2) - A(3, 1) * A(2, 2);
  B(1, 1) = d1 / r; B(2, 1) = d2 / r; B(3, 1) = d3 / r;
  d1 = A(3, 2) * A(1, 3) - A(1, 2) * A(3, 3);
  d2 = A(1, 1) * A(3, 3) - A(3, 1) * A(1, 3);
  d3 = -A(1, 1) * A(3, 2) + A(3, 1) * A(1, 2);
  B(1, 2) = d1 / r; B(2, 2) = d2 / r; B(3, 2) = d3 / r;
  d1 = A(1, 2) * A(2, 3) - A(2, 2) * A(1, 3);
  d2 = -A(1, 1) * A(2, 3) + A(2, 1) * A(1, 3);
  d3 = A(1, 1) * A(2, 2) - A(2, 1) * A(1, 2);
  B(1, 3) = d1 / r; B(2, 3) = d2 / r; B(3, 3) = d3 / r;
  *rjac = r;
  return iflag;
}
#undef A
#undef B

/* ------------------------------------------------------------------------ */
/* Manufactured solutions (problems/POISSON/GALERKIN/common/solution.F90,     */
/* getf.F90: f = -(u_xx + u_yy + u_zz)).                                      */
/* PI = 4*atan(1) (modules/common_prob_data.F90:51).                          */
/* ------------------------------------------------------------------------ */
static void solution(int isol, const double *X, double *u, double *gu,
                     double *hess_trace) {
  const double PI = 4.0 * atan(1.0);
  double x1 = X[0], x2 = X[1], x3 = X[2];
  *u = 0.0; gu[0] = gu[1] = gu[2] = 0.0; *hess_trace = 0.0;
  switch (isol) {
    case 0: {
      double np = 6.0;
      double fx = pow(x1, np), fy = pow(x2, np), fz = pow(x3, np);
      double dfx = np * pow(x1, np - 1.0), dfy = np * pow(x2, np - 1.0),
             dfz = np * pow(x3, np - 1.0);
      double ddfx = np * (np - 1.0) * pow(x1, np - 2.0);
      double ddfy = np * (np - 1.0) * pow(x2, np - 2.0);
      double ddfz = np * (np - 1.0) * pow(x3, np - 2.0);
      *u = fx * fy * fz;
      gu[0] = dfx * fy * fz; gu[1] = fx * dfy * fz; gu[2] = fx * fy * dfz;
      double h11 = ddfx * fy * fz, h22 = fx * ddfy * fz, h33 = fx * fy * ddfz;
      *hess_trace = h11 + h22 + h33;
      break;
    }
    case 1: {
      *u = sin(x1 * PI) * sinh(x2 * PI);
      gu[0] = PI * cos(x1 * PI) * sinh(x2 * PI);
      gu[1] = PI * sin(x1 * PI) * cosh(x2 * PI);
      double h11 = -PI * PI * sin(x1 * PI) * sinh(x2 * PI);
      double h22 = PI * PI * sin(x1 * PI) * sinh(x2 * PI);
      *hess_trace = h11 + h22 + 0.0;
      break;
    }
    case 2: {
      *u = sin(x1 * PI) * sinh(x2 * PI) * (x3 * x3);
      gu[0] = PI * cos(x1 * PI) * sinh(x2 * PI) * (x3 * x3);
      gu[1] = PI * sin(x1 * PI) * cosh(x2 * PI) * (x3 * x3);
      gu[2] = 2. * sin(x1 * PI) * sinh(x2 * PI) * x3;
      double h11 = -PI * PI * sin(x1 * PI) * sinh(x2 * PI) * (x3 * x3);
      double h22 = PI * PI * sin(x1 * PI) * sinh(x2 * PI) * (x3 * x3);
      double h33 = 2. * sin(x1 * PI) * sinh(x2 * PI);
      *hess_trace = h11 + h22 + h33;
      break;
    }
    case 10: { /* u = sin(pi x) sin(pi y) sin(pi z), f = 3 pi^2 u */
      double s1 = sin(PI * x1), s2 = sin(PI * x2), s3 = sin(PI * x3);
      *u = s1 * s2 * s3;
      gu[0] = PI * cos(PI * x1) * s2 * s3;
      gu[1] = PI * s1 * cos(PI * x2) * s3;
      gu[2] = PI * s1 * s2 * cos(PI * x3);
      *hess_trace = -3.0 * PI * PI * (*u);
      break;
    }
    case 11: /* f == 1, no closed-form u */
      *hess_trace = -1.0;
      break;
    case 12: /* u = x y z (test/poly_pois.F90:390-395) */
      *u = x1 * x2 * x3;
      gu[0] = x2 * x3; gu[1] = x1 * x3; gu[2] = x1 * x2;
      *hess_trace = 0.0;
      break;
    case 13: /* u = 1 + x + 2y + 3z: in the space of every order (f = 0) */
      *u = 1.0 + x1 + 2.0 * x2 + 3.0 * x3;
      gu[0] = 1.0; gu[1] = 2.0; gu[2] = 3.0;
      *hess_trace = 0.0;
      break;
    default:
      break;
  }
}

double orc_getf(int isol, const double *x) {
  double u, gu[3], tr;
  solution(isol, x, &u, gu, &tr);
  return -tr;
}

void orc_exact(int isol, const double *x, double *u, double *gradu) {
  double tr;
  solution(isol, x, u, gradu, &tr);
}

/* ------------------------------------------------------------------------ */
/* Element routine                                                           */
/* ------------------------------------------------------------------------ */
static int shape_dispatch(int etype, const double *xi, const int32_t *norder,
                          const int32_t *noriE, const int32_t *noriF,
                          double *shap, double *grad) {
  if (etype == ORC_HEXA) return orc_shape3DH_hexa(xi, norder, noriE, noriF, shap, grad);
  if (etype == ORC_TET) return orc_shape3DH_tet(xi, norder, noriE, noriF, shap, grad);
  if (etype == ORC_PRISM) return orc_shape3DH_prism(xi, norder, noriE, noriF, shap, grad);
  return -1;
}

static int quad_dispatch(int etype, const int32_t *norder, const int32_t *noriF,
                         int integration, double *xi, double *w) {
  if (etype == ORC_HEXA) return orc_set_3D_int_hexa(norder, noriF, integration, xi, w);
  if (etype == ORC_TET) return orc_set_3D_int_tet(norder, integration, xi, w);
  if (etype == ORC_PRISM) return orc_set_3D_int_prism(norder, noriF, integration, xi, w);
  return -1;
}

/* ------------------------------------------------------------------------ */
/* Optional BLAS-3 / LAPACK kernels (the reference calls DSYRK in elem_opt and  */
/* DGETRF / DGETRS / DGEMM in stc_fwd_gen).  The caller (the Python harness)   */
/* passes pointers to an optimised library's routines with the Fortran         */
/* calling convention (all arguments by reference); without them the oracle   */
/* runs its own loops in the same order of operations.                        */
/* ------------------------------------------------------------------------ */
typedef void (*orc_dsyrk_t)(char *, char *, int *, int *, double *, double *, int *, double *,
                            double *, int *);
typedef void (*orc_dgetrf_t)(int *, int *, double *, int *, int *, int *);
typedef void (*orc_dgetrs_t)(char *, int *, int *, double *, int *, int *, double *, int *, int *);
typedef void (*orc_dgemm_t)(char *, char *, int *, int *, int *, double *, double *, int *,
                            double *, int *, double *, double *, int *);
static struct {
  orc_dsyrk_t dsyrk;
  orc_dgetrf_t dgetrf;
  orc_dgetrs_t dgetrs;
  orc_dgemm_t dgemm;
} g_blas;

void orc_set_blas(void *dsyrk, void *dgetrf, void *dgetrs, void *dgemm) {
  g_blas.dsyrk = (orc_dsyrk_t)dsyrk;
  g_blas.dgetrf = (orc_dgetrf_t)dgetrf;
  g_blas.dgetrs = (orc_dgetrs_t)dgetrs;
  g_blas.dgemm = (orc_dgemm_t)dgemm;
}

int orc_blas_active(void) { return g_blas.dsyrk && g_blas.dgetrf && g_blas.dgetrs && g_blas.dgemm; }

int orc_elem(int etype, const int32_t *norder, const int32_t *nori_edge,
             const int32_t *nori_face, const double *xnod, double kappa,
             int isol, int integration, int variant, double *zaloc, int ld,
             double *zbloc) {
  double xiloc[3 * ORC_MAX_NINT3 + 3 * 200], waloc[ORC_MAX_NINT3 + 200];
  int nint = quad_dispatch(etype, norder, nori_face, integration, xiloc, waloc);
  if (nint <= 0) return -2;
  double *shap = (double *)malloc(sizeof(double) * ORC_MAXBRICKH);
  double *grad = (double *)malloc(sizeof(double) * 3 * ORC_MAXBRICKH);
  int n = 0, iflag_any = 0;
  double *atest = NULL;
  int nda = 3 * nint;
  for (int l = 0; l < nint; ++l) {
    const double *xi = &xiloc[3 * l];
    double wa = waloc[l];
    n = shape_dispatch(etype, xi, norder, nori_edge, nori_face, shap, grad);
    if (l == 0) {
      for (int j = 0; j < n; ++j) {
        zbloc[j] = 0.0;
        for (int i = 0; i < n; ++i) zaloc[i + (size_t)ld * j] = 0.0;
      }
      if (variant == 0) atest = (double *)malloc(sizeof(double) * (size_t)n * nda);
    }
    /* geom3D isoparametric branch (geom3D.F90:60-85) */
    double X[3] = {0, 0, 0}, dxdxi[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < n; ++k) {
      for (int c = 0; c < 3; ++c) X[c] = X[c] + xnod[3 * k + c] * shap[k];
      for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c)
          dxdxi[c + 3 * i] = dxdxi[c + 3 * i] + xnod[3 * k + c] * grad[3 * k + i];
    }
    double dxidx[9], rjac;
    int iflag = orc_geom(dxdxi, dxidx, &rjac);
    if (iflag) iflag_any = 1;
    double weight = rjac * wa;
    double fval = orc_getf(isol, X);
    if (variant == 0) {
      double sw = sqrt(weight);
      for (int k = 0; k < n; ++k) {
        double q = shap[k];
        double dq[3];
        for (int j = 0; j < 3; ++j)
          dq[j] = grad[3 * k + 0] * dxidx[0 + 3 * j] + grad[3 * k + 1] * dxidx[1 + 3 * j] +
                  grad[3 * k + 2] * dxidx[2 + 3 * j];
        zbloc[k] = zbloc[k] + q * fval * weight;
        for (int j = 0; j < 3; ++j) atest[k + (size_t)n * (3 * l + j)] = dq[j] * sw;
      }
    } else {
      /* elem_poisson scalar form (elem.F90:200-245) */
      double *dq = (double *)malloc(sizeof(double) * 3 * n);
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < 3; ++j)
          dq[3 * k + j] = grad[3 * k + 0] * dxidx[0 + 3 * j] + grad[3 * k + 1] * dxidx[1 + 3 * j] +
                          grad[3 * k + 2] * dxidx[2 + 3 * j];
      for (int k1 = 0; k1 < n; ++k1) {
        zbloc[k1] = zbloc[k1] + shap[k1] * fval * weight;
        for (int k2 = 0; k2 < n; ++k2)
          zaloc[k1 + (size_t)ld * k2] =
              zaloc[k1 + (size_t)ld * k2] +
              weight * (dq[3 * k1] * dq[3 * k2] + dq[3 * k1 + 1] * dq[3 * k2 + 1] +
                        dq[3 * k1 + 2] * dq[3 * k2 + 2]);
      }
      free(dq);
    }
  }
  if (variant == 0) {
    /* DSYRK('U','N') + lower fill (elem_opt.F90:131-137) */
    if (g_blas.dsyrk) {
      char up = 'U', no = 'N';
      int nn = n, kk = nda, lda = n, ldc = ld;
      double one = 1.0, zero = 0.0;
      g_blas.dsyrk(&up, &no, &nn, &kk, &one, atest, &lda, &zero, zaloc, &ldc);
    } else {
      for (int j = 0; j < n; ++j)
        for (int i = 0; i <= j; ++i) {
          double s = 0.0;
          for (int k = 0; k < nda; ++k) s += atest[i + (size_t)n * k] * atest[j + (size_t)n * k];
          zaloc[i + (size_t)ld * j] = s;
        }
    }
    for (int k = 0; k < n; ++k)
      for (int i = k + 1; i < n; ++i) zaloc[i + (size_t)ld * k] = zaloc[k + (size_t)ld * i];
    free(atest);
  }
  if (kappa != 1.0)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) zaloc[i + (size_t)ld * j] *= kappa;
  free(shap);
  free(grad);
  return iflag_any;
}

/* ------------------------------------------------------------------------ */
/* Static condensation (src/modules/stc.F90:182-509)                          */
/* ------------------------------------------------------------------------ */
int orc_stc_fwd(int ni, int nb, const double *a, int lda, const double *b,
                int method, double *aii, double *bi, double *aschur,
                double *bschur) {
  /* split (stc.F90:227-261): interface dof first, bubbles last */
  double *abb = (double *)malloc(sizeof(double) * (size_t)nb * nb);
  double *aib = (double *)malloc(sizeof(double) * (size_t)ni * nb);
  for (int j = 0; j < ni; ++j)
    for (int i = 0; i < ni; ++i) aii[i + (size_t)ni * j] = a[i + (size_t)lda * j];
  for (int j = 0; j < ni; ++j)
    for (int i = 0; i < nb; ++i) aschur[i + (size_t)nb * j] = a[ni + i + (size_t)lda * j];
  for (int j = 0; j < nb; ++j)
    for (int i = 0; i < ni; ++i) aib[i + (size_t)ni * j] = a[i + (size_t)lda * (ni + j)];
  for (int j = 0; j < nb; ++j)
    for (int i = 0; i < nb; ++i) abb[i + (size_t)nb * j] = a[ni + i + (size_t)lda * (ni + j)];
  for (int i = 0; i < ni; ++i) bi[i] = b[i];
  for (int i = 0; i < nb; ++i) bschur[i] = b[ni + i];
  int rc = 0;
  if (method == 0 && g_blas.dgetrf && nb > 0) {
    /* stc_fwd_gen with the library: DGETRF, DGETRS on [Abi | Bb], then
       DGEMM / the load update (stc.F90:462-507) */
    int *piv = (int *)malloc(sizeof(int) * nb);
    int nn = nb, info = 0;
    g_blas.dgetrf(&nn, &nn, abb, &nn, piv, &info);
    if (info != 0) rc = -1;
    if (rc == 0) {
      char no = 'N';
      int one_i = 1, nrhs = ni;
      g_blas.dgetrs(&no, &nn, &nrhs, abb, &nn, piv, aschur, &nn, &info);
      g_blas.dgetrs(&no, &nn, &one_i, abb, &nn, piv, bschur, &nn, &info);
      double m1 = -1.0, p1 = 1.0;
      int mi = ni;
      g_blas.dgemm(&no, &no, &mi, &mi, &nn, &m1, aib, &mi, aschur, &nn, &p1, aii, &mi);
      g_blas.dgemm(&no, &no, &mi, &one_i, &nn, &m1, aib, &mi, bschur, &nn, &p1, bi, &mi);
    }
    free(piv);
    free(abb);
    free(aib);
    return rc;
  }
  if (method == 0) {
    /* DGETRF: right-looking LU with partial pivoting (first max |.|) */
    int *piv = (int *)malloc(sizeof(int) * (nb > 0 ? nb : 1));
    for (int k = 0; k < nb; ++k) {
      int p = k;
      double amax = fabs(abb[k + (size_t)nb * k]);
      for (int i = k + 1; i < nb; ++i)
        if (fabs(abb[i + (size_t)nb * k]) > amax) { amax = fabs(abb[i + (size_t)nb * k]); p = i; }
      piv[k] = p;
      if (abb[p + (size_t)nb * k] == 0.0) { rc = -1; break; }
      if (p != k)
        for (int j = 0; j < nb; ++j) {
          double t = abb[k + (size_t)nb * j];
          abb[k + (size_t)nb * j] = abb[p + (size_t)nb * j];
          abb[p + (size_t)nb * j] = t;
        }
      double rp = 1.0 / abb[k + (size_t)nb * k];
      for (int i = k + 1; i < nb; ++i) abb[i + (size_t)nb * k] *= rp;
      for (int j = k + 1; j < nb; ++j) {
        double akj = abb[k + (size_t)nb * j];
        for (int i = k + 1; i < nb; ++i) abb[i + (size_t)nb * j] -= abb[i + (size_t)nb * k] * akj;
      }
    }
    if (rc == 0) {
      /* DGETRS on [Bb | Abi] */
      for (int c = -1; c < ni; ++c) {
        double *x = (c < 0) ? bschur : &aschur[(size_t)nb * c];
        for (int k = 0; k < nb; ++k)
          if (piv[k] != k) { double t = x[k]; x[k] = x[piv[k]]; x[piv[k]] = t; }
        for (int k = 0; k < nb; ++k)
          for (int i = k + 1; i < nb; ++i) x[i] -= abb[i + (size_t)nb * k] * x[k];
        for (int k = nb - 1; k >= 0; --k) {
          x[k] /= abb[k + (size_t)nb * k];
          for (int i = 0; i < k; ++i) x[i] -= abb[i + (size_t)nb * k] * x[k];
        }
      }
    }
    free(piv);
  } else {
    /* Cholesky A = U^T U (stc_fwd_herm restated with dense storage) */
    for (int j = 0; j < nb && rc == 0; ++j) {
      double s = abb[j + (size_t)nb * j];
      for (int k = 0; k < j; ++k) s -= abb[k + (size_t)nb * j] * abb[k + (size_t)nb * j];
      if (!(s > 0.0)) { rc = -1; break; }
      double ujj = sqrt(s);
      abb[j + (size_t)nb * j] = ujj;
      for (int i = j + 1; i < nb; ++i) {
        double t = abb[j + (size_t)nb * i];
        for (int k = 0; k < j; ++k) t -= abb[k + (size_t)nb * j] * abb[k + (size_t)nb * i];
        abb[j + (size_t)nb * i] = t / ujj;
      }
    }
    if (rc == 0)
      for (int c = -1; c < ni; ++c) {
        double *x = (c < 0) ? bschur : &aschur[(size_t)nb * c];
        for (int k = 0; k < nb; ++k) { /* U^T y = x */
          double t = x[k];
          for (int i = 0; i < k; ++i) t -= abb[i + (size_t)nb * k] * x[i];
          x[k] = t / abb[k + (size_t)nb * k];
        }
        for (int k = nb - 1; k >= 0; --k) { /* U z = y */
          double t = x[k];
          for (int i = k + 1; i < nb; ++i) t -= abb[k + (size_t)nb * i] * x[i];
          x[k] = t / abb[k + (size_t)nb * k];
        }
      }
  }
  if (rc == 0) {
    /* Bi -= Aib * Bb ; Aii -= Aib * Abi (stc.F90:493-507) */
    for (int i = 0; i < ni; ++i) {
      double s = 0.0;
      for (int k = 0; k < nb; ++k) s += aib[i + (size_t)ni * k] * bschur[k];
      bi[i] = bi[i] - s;
    }
    for (int j = 0; j < ni; ++j)
      for (int i = 0; i < ni; ++i) {
        double s = 0.0;
        for (int k = 0; k < nb; ++k) s += aib[i + (size_t)ni * k] * aschur[k + (size_t)nb * j];
        aii[i + (size_t)ni * j] = aii[i + (size_t)ni * j] - s;
      }
  }
  free(abb);
  free(aib);
  return rc;
}

void orc_stc_bwd(int ni, int nb, const double *aschur, const double *bschur,
                 const double *xi, double *xb) {
  for (int i = 0; i < nb; ++i) {
    double s = 0.0;
    for (int k = 0; k < ni; ++k) s += aschur[i + (size_t)nb * k] * xi[k];
    xb[i] = bschur[i] - s;
  }
}

/* ------------------------------------------------------------------------ */
/* Node dof counts, compression, index maps                                  */
/* ------------------------------------------------------------------------ */
int orc_node_ndof(int etype, const int32_t *norder, int32_t *ndof) {
  if (etype == ORC_HEXA) {
    for (int v = 0; v < 8; ++v) ndof[v] = 1;
    for (int e = 0; e < 12; ++e) ndof[8 + e] = imax(norder[e] - 1, 0);
    for (int f = 0; f < 6; ++f) {
      int hv[2];
      decod(norder[12 + f], 10, 2, hv);
      ndof[20 + f] = imax(hv[0] - 1, 0) * imax(hv[1] - 1, 0);
    }
    return 26;
  }
  if (etype == ORC_TET) {
    for (int v = 0; v < 4; ++v) ndof[v] = 1;
    for (int e = 0; e < 6; ++e) ndof[4 + e] = imax(norder[e] - 1, 0);
    for (int f = 0; f < 4; ++f) {
      int p = norder[6 + f];
      ndof[10 + f] = (p - 2) * (p - 1) / 2 > 0 ? (p - 2) * (p - 1) / 2 : 0;
    }
    return 14;
  }
  if (etype == ORC_PRISM) {
    for (int v = 0; v < 6; ++v) ndof[v] = 1;
    for (int e = 0; e < 9; ++e) ndof[6 + e] = imax(norder[e] - 1, 0);
    for (int f = 0; f < 2; ++f) {
      int p = norder[9 + f];
      ndof[15 + f] = (p - 2) * (p - 1) / 2 > 0 ? (p - 2) * (p - 1) / 2 : 0;
    }
    for (int f = 0; f < 3; ++f) {
      int h = norder[11 + f] / 10, v = norder[11 + f] % 10;
      ndof[17 + f] = imax(h - 1, 0) * imax(v - 1, 0);
    }
    return 20;
  }
  return -1;
}

int orc_celem_compress(int etype, const int32_t *norder, const int32_t *bcflag,
                       const double *aii, const double *bi,
                       const double *zdofd, int32_t *nextract, double *zbload,
                       double *zastif, int32_t *ndofm) {
  int32_t nd[32];
  int nn = orc_node_ndof(etype, norder, nd);
  return orc_celem_compress_nodes(nn, nd, bcflag, aii, bi, zdofd, nextract, zbload, zastif,
                                  ndofm);
}

int orc_celem_compress_nodes(int nn, const int32_t *nd, const int32_t *bcflag,
                             const double *aii, const double *bi, const double *zdofd,
                             int32_t *nextract, double *zbload, double *zastif,
                             int32_t *ndofm) {
  int first[256], ni = 0;
  if (nn > 256) return -1;
  for (int i = 0; i < nn; ++i) { first[i] = ni; ni += nd[i]; }
  /* NEXTRACT: nodes in reverse order, dof in forward order, skip Dirichlet
   * (celem_systemI.F90:290-350) */
  int k = 0;
  for (int i = nn - 1; i >= 0; --i) {
    int kold = k;
    if (!bcflag[i])
      for (int j = 0; j < nd[i]; ++j) nextract[k++] = first[i] + j;
    ndofm[i] = k - kold;
  }
  int nrdofc = k;
  /* Dirichlet lift (celem_systemI.F90:800-812) then compression (812-845) */
  double *zb = (double *)malloc(sizeof(double) * (ni > 0 ? ni : 1));
  for (int i = 0; i < ni; ++i) zb[i] = bi[i];
  if (zdofd) {
    for (int i2 = 0; i2 < nn; ++i2) {
      if (!bcflag[i2]) continue;
      for (int j2 = 0; j2 < nd[i2]; ++j2) {
        int k2 = first[i2] + j2;
        for (int k1 = 0; k1 < ni; ++k1) zb[k1] = zb[k1] - aii[k1 + (size_t)ni * k2] * zdofd[k2];
      }
    }
  }
  for (int l1 = 0; l1 < nrdofc; ++l1) {
    int k1 = nextract[l1];
    zbload[l1] = zb[k1];
    for (int l2 = 0; l2 < nrdofc; ++l2)
      zastif[(size_t)l1 * nrdofc + l2] = aii[k1 + (size_t)ni * nextract[l2]];
  }
  free(zb);
  return nrdofc;
}

int64_t orc_index_maps(int nelem, int nnode_max, const int32_t *nnode,
                       const int32_t *nodes, const int32_t *ndofm,
                       int nnodes_global, int32_t *nfirst_dof, int32_t *lcon,
                       int64_t *lcon_off, int64_t *elem_nnz) {
  for (int i = 0; i < nnodes_global; ++i) nfirst_dof[i] = -1;
  int64_t nrdof = 0, nnz = 0, off = 0;
  for (int e = 0; e < nelem; ++e) {
    const int32_t *nod = &nodes[(size_t)e * nnode_max];
    const int32_t *nd = &ndofm[(size_t)e * nnode_max];
    int ndof = 0;
    for (int i = 0; i < nnode[e]; ++i) {
      ndof += nd[i];
      if (nfirst_dof[nod[i]] >= 0) continue;
      nfirst_dof[nod[i]] = (int32_t)nrdof;
      nrdof += nd[i];
    }
    elem_nnz[e] = nnz;
    nnz += (int64_t)ndof * ndof;
    lcon_off[e] = off;
    off += ndof;
  }
  elem_nnz[nelem] = nnz;
  lcon_off[nelem] = off;
  for (int e = 0; e < nelem; ++e) {
    const int32_t *nod = &nodes[(size_t)e * nnode_max];
    const int32_t *nd = &ndofm[(size_t)e * nnode_max];
    int64_t l = lcon_off[e];
    for (int i = nnode[e] - 1; i >= 0; --i)
      for (int j = 1; j <= nd[i]; ++j) lcon[l++] = nfirst_dof[nod[i]] + j;
  }
  return nrdof;
}

/* ------------------------------------------------------------------------ */
/* Batched element pass (the CPU baseline form of mumps_sc STEP 2)            */
/* ------------------------------------------------------------------------ */
static int nvert_of(int etype) { return etype == ORC_HEXA ? 8 : (etype == ORC_TET ? 4 : 6); }

int orc_element_pass(int nelem, const int32_t *etype, const int32_t *norder,
                     const int32_t *nori_edge, const int32_t *nori_face,
                     const int32_t *bcflag, const double *xvert,
                     const double *kappa, int isol, int integration,
                     int stc_method, int nthreads,
                     const int64_t *elem_nnz, const int64_t *lcon_off,
                     const int64_t *schur_off, const int64_t *bub_off,
                     double *zastif, double *zbload, double *aschur,
                     double *bschur) {
  int bad = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel
  {
    double *aloc = (double *)malloc(sizeof(double) * ORC_MAXBRICKH * ORC_MAXBRICKH);
    double *bloc = (double *)malloc(sizeof(double) * ORC_MAXBRICKH);
    double *xnod = (double *)malloc(sizeof(double) * 3 * ORC_MAXBRICKH);
    double *aii = (double *)malloc(sizeof(double) * ORC_MAXBRICKH * ORC_MAXBRICKH);
    double *bi = (double *)malloc(sizeof(double) * ORC_MAXBRICKH);
    double *as = (double *)malloc(sizeof(double) * ORC_MAXBRICKH * ORC_MAXBRICKH);
    double *bs = (double *)malloc(sizeof(double) * ORC_MAXBRICKH);
    double *zs = (double *)malloc(sizeof(double) * ORC_MAXBRICKH * ORC_MAXBRICKH);
    double *zb = (double *)malloc(sizeof(double) * ORC_MAXBRICKH);
    int32_t nextract[ORC_MAXBRICKH], ndofm[32];
#pragma omp for schedule(dynamic)
    for (int e = 0; e < nelem; ++e) {
      int et = etype[e];
      const int32_t *no = &norder[19 * (size_t)e];
      int n = (et == ORC_HEXA) ? orc_nrdofH_hexa(no)
              : (et == ORC_TET) ? orc_nrdofH_tet(no) : orc_nrdofH_prism(no);
      int nb = orc_nrdofH_bubble(et, no);
      int ni = n - nb;
      int nv = nvert_of(et);
      for (int k = 0; k < n; ++k)
        for (int c = 0; c < 3; ++c)
          xnod[3 * k + c] = (k < nv) ? xvert[(size_t)e * 24 + 3 * k + c] : 0.0;
      int rc = orc_elem(et, no, &nori_edge[12 * (size_t)e], &nori_face[6 * (size_t)e], xnod,
                        kappa[e], isol, integration, 0, aloc, n, bloc);
      if (rc == 0 && nb > 0)
        rc = orc_stc_fwd(ni, nb, aloc, n, bloc, stc_method, aii, bi, as, bs);
      else if (rc == 0) {
        for (int j = 0; j < ni; ++j)
          for (int i = 0; i < ni; ++i) aii[i + (size_t)ni * j] = aloc[i + (size_t)n * j];
        for (int i = 0; i < ni; ++i) bi[i] = bloc[i];
      }
      if (rc != 0) {
#pragma omp critical
        { if (bad == 0 || e + 1 < bad) bad = e + 1; }
        continue;
      }
      int nrdofc = orc_celem_compress(et, no, &bcflag[26 * (size_t)e], aii, bi, NULL,
                                      nextract, zb, zs, ndofm);
      if (zastif) memcpy(&zastif[elem_nnz[e]], zs, sizeof(double) * (size_t)nrdofc * nrdofc);
      if (zbload) memcpy(&zbload[lcon_off[e]], zb, sizeof(double) * nrdofc);
      if (aschur && nb > 0) memcpy(&aschur[schur_off[e]], as, sizeof(double) * (size_t)nb * ni);
      if (bschur && nb > 0) memcpy(&bschur[bub_off[e]], bs, sizeof(double) * nb);
    }
    free(aloc); free(bloc); free(xnod); free(aii); free(bi);
    free(as); free(bs); free(zs); free(zb);
  }
  return bad;
}

/* ------------------------------------------------------------------------ */
/* element_error (src/element/util/compute_error.F90:226-360, H1 branch):    */
/* squared H1 error and norm with INTEGRATION=2 over-integration.            */
/* dof: element H1 dof in shape-function order (interface + bubbles).        */
/* ------------------------------------------------------------------------ */
int orc_element_error(int etype, const int32_t *norder, const int32_t *nori_edge,
                      const int32_t *nori_face, const double *xnod, const double *dof,
                      int isol, double *err2, double *norm2) {
  double xiloc[3 * ORC_MAX_NINT3 + 3 * 200], waloc[ORC_MAX_NINT3 + 200];
  /* set_3Dint is called without the face-order swap and INTEGRATION=2 */
  int32_t zero6[6] = {0, 0, 0, 0, 0, 0};
  int nint = quad_dispatch(etype, norder, zero6, 2, xiloc, waloc);
  if (nint <= 0) return -2;
  double *shap = (double *)malloc(sizeof(double) * ORC_MAXBRICKH);
  double *grad = (double *)malloc(sizeof(double) * 3 * ORC_MAXBRICKH);
  double e2 = 0.0, r2 = 0.0;
  for (int l = 0; l < nint; ++l) {
    int n = shape_dispatch(etype, &xiloc[3 * l], norder, nori_edge, nori_face, shap, grad);
    double X[3] = {0, 0, 0}, dxdxi[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double uh = 0.0, guh[3] = {0, 0, 0};
    for (int k = 0; k < n; ++k) {
      for (int c = 0; c < 3; ++c) X[c] += xnod[3 * k + c] * shap[k];
      for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) dxdxi[c + 3 * i] += xnod[3 * k + c] * grad[3 * k + i];
      uh += dof[k] * shap[k];
      for (int i = 0; i < 3; ++i) guh[i] += dof[k] * grad[3 * k + i];
    }
    double dxidx[9], rjac;
    orc_geom(dxdxi, dxidx, &rjac);
    double gx[3];
    for (int j = 0; j < 3; ++j)
      gx[j] = guh[0] * dxidx[0 + 3 * j] + guh[1] * dxidx[1 + 3 * j] + guh[2] * dxidx[2 + 3 * j];
    double u, gu[3];
    orc_exact(isol, X, &u, gu);
    double weight = waloc[l] * rjac;
    for (int j = 0; j < 3; ++j) {
      e2 += (gu[j] - gx[j]) * (gu[j] - gx[j]) * weight;
      r2 += gu[j] * gu[j] * weight;
    }
    e2 += (u - uh) * (u - uh) * weight;
    r2 += u * u * weight;
  }
  free(shap);
  free(grad);
  *err2 = e2;
  *norm2 = r2;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Jacobi families (Polynomials.F90:197-431, 553-646)                         */
/* ------------------------------------------------------------------------ */
#define JMAX 9

/* PolyJacobi (Polynomials.F90:197-268): shifted scaled Jacobi polynomials
 * P[a][i], rows a = 0..nord with alpha = minalpha + 2a, orders i = 0..nord-a
 * (the first subdiagonal is filled too, as in the reference). */
static void poly_jacobi(double x, double t, int nord, int minalpha, double P[JMAX][JMAX]) {
  for (int a = 0; a <= nord; ++a) P[a][0] = 1.0;
  double y = 0.0;
  if (nord >= 1) {
    y = 2.0 * x - t;
    for (int a = 0; a <= nord - 1; ++a) P[a][1] = y + (double)(minalpha + 2 * a) * x;
  }
  if (nord >= 2) {
    double tt = t * t;
    for (int a = 0; a <= nord - 2; ++a) {
      int al = minalpha + 2 * a;
      int aa = al * al;
      for (int i = 2; i <= nord - a; ++i) {
        int ai = 2 * i * (i + al) * (2 * i + al - 2);
        int bi = 2 * i + al - 1;
        int ci = (2 * i + al) * (2 * i + al - 2);
        int di = 2 * (i + al - 1) * (i - 1) * (2 * i + al);
        double v = (double)bi * ((double)ci * y + (double)aa * t) * P[a][i - 1] -
                   (double)di * tt * P[a][i - 2];
        P[a][i] = v / (double)ai;
      }
    }
  }
}

/* PolyIJacobi (Polynomials.F90:303-431): integrated Jacobi L[a][i], rows
 * a = 1..nord (alpha = minalpha + 2(a-1)), orders i = 1..nord-a+1; P[a][i-1]
 * the x-derivative (Jacobi), R[a][i-1] the t-derivative (idec == 0 only). */
static void poly_ijacobi(double x, double t, int nord, int minalpha, int idec,
                         double L[JMAX][JMAX], double P[JMAX][JMAX], double R[JMAX][JMAX]) {
  double pj[JMAX][JMAX];
  poly_jacobi(x, t, nord, minalpha, pj);
  /* ptemp(a, i) of the reference is row a-1 of PolyJacobi */
  for (int a = 1; a <= nord; ++a) {
    for (int i = 0; i <= nord - 1; ++i) P[a][i] = pj[a - 1][i];
    L[a][1] = x;
    if (!idec) R[a][0] = 0.0;
  }
  if (nord >= 2) {
    double tt = t * t;
    for (int a = 1; a <= nord - 1; ++a) {
      int al = minalpha + 2 * (a - 1);
      for (int i = 2; i <= nord - (a - 1); ++i) {
        int tia = i + i + al, tiam1 = tia - 1, tiam2 = tia - 2;
        double ai = (double)(i + al) / (double)(tiam1 * tia);
        double bi = (double)al / (double)(tiam2 * tia);
        double ci = ((double)i - 1.0) / (double)(tiam2 * tiam1);
        L[a][i] = ai * pj[a - 1][i] + bi * t * pj[a - 1][i - 1] - ci * tt * pj[a - 1][i - 2];
        if (!idec) {
          double r = -((double)(i - 1) * (pj[a - 1][i - 1] + t * pj[a - 1][i - 2]));
          R[a][i - 1] = r / (double)tiam2;
        }
      }
    }
  }
}

/* HomIJacobi (Polynomials.F90:604-646): homogenized integrated Jacobi of the
 * pair S = (s0, s1) with gradients DS[c][k]; HomL[a][i], DHomL[a][i][c]. */
static void hom_ijacobi(const double *S, const double DS[3][2], int nord, int minalpha,
                        int idec, double HomL[JMAX][JMAX], double DHomL[JMAX][JMAX][3]) {
  double hP[JMAX][JMAX], hR[JMAX][JMAX];
  if (idec) {
    poly_ijacobi(S[1], 1.0, nord, minalpha, 1, HomL, hP, hR);
    for (int a = 1; a <= nord; ++a)
      for (int i = 1; i <= nord - (a - 1); ++i)
        for (int c = 0; c < 3; ++c) DHomL[a][i][c] = hP[a][i - 1] * DS[c][1];
  } else {
    poly_ijacobi(S[1], S[0] + S[1], nord, minalpha, 0, HomL, hP, hR);
    double ds01[3];
    for (int c = 0; c < 3; ++c) ds01[c] = DS[c][0] + DS[c][1];
    for (int a = 1; a <= nord; ++a)
      for (int i = 1; i <= nord - (a - 1); ++i)
        for (int c = 0; c < 3; ++c)
          DHomL[a][i][c] = hP[a][i - 1] * DS[c][1] + hR[a][i - 1] * ds01[c];
  }
}

/* AncPhiTri (Ancillary.F90:397-442): triangle ancillary functions
 * phi[i][j] = phiE_i(s0,s1) * L^{2i}_j(s2; s0+s1+s2), i >= 2, j >= 1,
 * i + j <= nord.  S[k], DS[c][k] for k = 0..2. */
static void anc_phi_tri(const double *S, const double DS[3][3], int nord, int idec,
                        double phi[JMAX][JMAX], double dphi[JMAX][JMAX][3]) {
  double s01[2] = {S[0], S[1]}, ds01[3][2];
  for (int c = 0; c < 3; ++c) { ds01[c][0] = DS[c][0]; ds01[c][1] = DS[c][1]; }
  double phiE[16], dphiE[16][3];
  hom_ilegendre(s01, ds01, nord - 1, 0, phiE, dphiE);
  double sL[2] = {S[0] + S[1], S[2]}, dsL[3][2];
  for (int c = 0; c < 3; ++c) { dsL[c][0] = DS[c][0] + DS[c][1]; dsL[c][1] = DS[c][2]; }
  double hl[JMAX][JMAX], dhl[JMAX][JMAX][3];
  hom_ijacobi(sL, dsL, nord - 2, 4, idec, hl, dhl);
  /* homLal(i, j) of the reference is row i-1 of HomIJacobi */
  for (int nij = 3; nij <= nord; ++nij)
    for (int i = 2; i <= nij - 1; ++i) {
      int j = nij - i;
      phi[i][j] = phiE[i] * hl[i - 1][j];
      for (int c = 0; c < 3; ++c) dphi[i][j][c] = hl[i - 1][j] * dphiE[i][c] + phiE[i] * dhl[i - 1][j][c];
    }
}

/* OrientTri (Orient.F90:119-162): GS(k) = S(Or(nori, k)) */
static const int ORIENT_TRI[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 0}};

/* ------------------------------------------------------------------------ */
/* Tetrahedron H1 (Tetrahedron.F90:33-234; AffineTetrahedron,                */
/* AffineCoordinates.F90:74-89; BlendTetV / ProjectTetE / ProjectTetF,        */
/* BlendProject.F90:441-560).                                                 */
/* ------------------------------------------------------------------------ */
static const int TET_E[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
static const int TET_F[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};

static int tri_ndof(int p) { return p > 2 ? (p - 1) * (p - 2) / 2 : 0; }
static int tet_nbub(int p) { return p > 3 ? (p - 1) * (p - 2) * (p - 3) / 6 : 0; }

int orc_nrdofH_tet(const int32_t *norder) {
  int n = 4;
  for (int e = 0; e < 6; ++e) n += imax(norder[e] - 1, 0);
  for (int f = 0; f < 4; ++f) n += tri_ndof(norder[6 + f]);
  return n + tet_nbub(norder[10]);
}

/* set_3Dint_aux TETRA branch (set_3D_int.F90:305-323) with the Duffy rule of
 * init_gauss_quadrature (gauss_quadrature.F90:757-787): order = max order
 * + INTEGRATION capped at MAXP; (p+1) x (p+1) x (p+2) collapsed points. */
int orc_set_3D_int_tet(const int32_t *norder, int integration, double *xiloc,
                       double *waloc) {
  int nord = 0;
  for (int i = 0; i < 11; ++i) nord = imax(nord, norder[i]);
  nord = imin(nord + integration, ORC_MAXP);
  if (nord < 1) return -1;
  int np = nord;
  double xz[16], wz[16], xy[16], wy[16];
  orc_gauss1d(np + 2, xz, wz);
  orc_gauss1d(np + 1, xy, wy);
  int l = 0;
  for (int k = 0; k < np + 2; ++k) {
    double z = xz[k], wzk = wz[k];
    for (int j = 0; j < np + 1; ++j) {
      double y = xy[j], wyj = wy[j];
      for (int i = 0; i < np + 1; ++i) {
        double xx = xy[i], wx = wy[i];
        xiloc[3 * l + 0] = xx * (1.0 - y) * (1.0 - z);
        xiloc[3 * l + 1] = y * (1.0 - z);
        xiloc[3 * l + 2] = z;
        double omz = 1.0 - z;
        waloc[l] = wx * wyj * wzk * (omz * omz) * (1.0 - y);
        ++l;
      }
    }
  }
  return l;
}

int orc_shape3DH_tet(const double *xi, const int32_t *nord,
                     const int32_t *nori_edge, const int32_t *nori_face,
                     double *shap, double *grad) {
  double lam[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
  static const double DL[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  int m = 0;
  for (int v = 0; v < 4; ++v, ++m) {
    shap[m] = lam[v];
    for (int c = 0; c < 3; ++c) grad[3 * m + c] = DL[v][c];
  }
  /* edges: OrientE + AncPhiE (homogenized integrated Legendre, Idec false) */
  for (int e = 0; e < 6; ++e) {
    int p = nord[e];
    if (p - 1 <= 0) continue;
    int v0 = TET_E[e][0], v1 = TET_E[e][1];
    if (nori_edge[e] == 1) { int t = v0; v0 = v1; v1 = t; }
    double S[2] = {lam[v0], lam[v1]}, DS[3][2];
    for (int c = 0; c < 3; ++c) { DS[c][0] = DL[v0][c]; DS[c][1] = DL[v1][c]; }
    double phi[16], dphi[16][3];
    hom_ilegendre(S, DS, p, 0, phi, dphi);
    for (int i = 2; i <= p; ++i, ++m) {
      shap[m] = phi[i];
      for (int c = 0; c < 3; ++c) grad[3 * m + c] = dphi[i][c];
    }
  }
  /* faces: OrientTri + AncPhiTri */
  for (int f = 0; f < 4; ++f) {
    int p = nord[6 + f];
    if (tri_ndof(p) <= 0) continue;
    const int *o = ORIENT_TRI[nori_face[f]];
    double S[3], DS[3][3];
    for (int k = 0; k < 3; ++k) {
      int v = TET_F[f][o[k]];
      S[k] = lam[v];
      for (int c = 0; c < 3; ++c) DS[c][k] = DL[v][c];
    }
    double phi[JMAX][JMAX], dphi[JMAX][JMAX][3];
    anc_phi_tri(S, DS, p, 0, phi, dphi);
    for (int nij = 3; nij <= p; ++nij)
      for (int i = 2; i <= nij - 1; ++i, ++m) {
        int j = nij - i;
        shap[m] = phi[i][j];
        for (int c = 0; c < 3; ++c) grad[3 * m + c] = dphi[i][j][c];
      }
  }
  /* bubbles: AncPhiTri(lam0..2) x HomIJacobi((1-lam3, lam3), alpha = 2(i+j)) */
  int pb = nord[10];
  if (tet_nbub(pb) > 0) {
    double S[3] = {lam[0], lam[1], lam[2]}, DS[3][3];
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) DS[c][k] = DL[k][c];
    double phi[JMAX][JMAX], dphi[JMAX][JMAX][3];
    anc_phi_tri(S, DS, pb - 1, 0, phi, dphi);
    double Sz[2] = {1.0 - lam[3], lam[3]}, DSz[3][2];
    for (int c = 0; c < 3; ++c) { DSz[c][0] = -DL[3][c]; DSz[c][1] = DL[3][c]; }
    double hb[JMAX][JMAX], dhb[JMAX][JMAX][3];
    hom_ijacobi(Sz, DSz, pb - 3, 6, 1, hb, dhb);
    /* homLbet(nij, k) of the reference is row nij-2 of HomIJacobi */
    for (int nijk = 4; nijk <= pb; ++nijk)
      for (int nij = 3; nij <= nijk - 1; ++nij)
        for (int i = 2; i <= nij - 1; ++i, ++m) {
          int j = nij - i, k = nijk - nij;
          double hv = hb[nij - 2][k];
          shap[m] = phi[i][j] * hv;
          for (int c = 0; c < 3; ++c)
            grad[3 * m + c] = hv * dphi[i][j][c] + phi[i][j] * dhb[nij - 2][k][c];
        }
  }
  return m;
}


/* ------------------------------------------------------------------------ */
/* Triangle rules for the prism: Dunavant's symmetric rules of degree        */
/* 2,4,...,12 as tabulated in init_gauss_quadrature (gauss_quadrature.F90:  */
/* 130-270: barcoo = weight + barycentric triple per orbit, nnod = orbit     */
/* size), expanded into points as at gauss_quadrature.F90:663-700.  Only the */
/* sets NSELECT(1..MAXP) = 2,4,...,12 are needed.                            */
/* ------------------------------------------------------------------------ */
typedef struct { int set, size; double w, b1, b2, b3; } orc_orbit;
static const orc_orbit ORC_TRI_ORBITS[] = {
    {2, 3, 0.333333333333333, 0.666666666666667, 0.166666666666667, 0.166666666666667},
    {4, 3, 0.223381589678011, 0.10810301816807, 0.445948490915965, 0.445948490915965},
    {4, 3, 0.109951743655322, 0.816847572980459, 0.091576213509771, 0.091576213509771},
    {6, 3, 0.116786275726379, 0.501426509658179, 0.24928674517091, 0.24928674517091},
    {6, 3, 0.050844906370207, 0.873821971016996, 0.063089014491502, 0.063089014491502},
    {6, 6, 0.082851075618374, 0.053145049844817, 0.310352451033784, 0.636502499121399},
    {8, 1, 0.144315607677787, 0.333333333333333, 0.333333333333333, 0.333333333333333},
    {8, 3, 0.095091634267285, 0.081414823414554, 0.459292588292723, 0.459292588292723},
    {8, 3, 0.103217370534718, 0.65886138449648, 0.17056930775176, 0.17056930775176},
    {8, 3, 0.032458497623198, 0.898905543365938, 0.050547228317031, 0.050547228317031},
    {8, 6, 0.027230314174435, 0.008394777409958, 0.263112829634638, 0.728492392955404},
    {10, 1, 0.090817990382754, 0.333333333333333, 0.333333333333333, 0.333333333333333},
    {10, 3, 0.036725957756467, 0.028844733232685, 0.485577633383657, 0.485577633383657},
    {10, 3, 0.045321059435528, 0.781036849029926, 0.109481575485037, 0.109481575485037},
    {10, 6, 0.07275791684542, 0.14170721941488, 0.307939838764121, 0.550352941820999},
    {10, 6, 0.028327242531057, 0.025003534762686, 0.246672560639903, 0.728323904597411},
    {10, 6, 0.009421666963733, 0.009540815400299, 0.0668032510122, 0.9236559335875},
    {12, 3, 0.025731066440455, 0.02356522045239, 0.488217389773805, 0.488217389773805},
    {12, 3, 0.043692544538038, 0.120551215411079, 0.43972439229446, 0.43972439229446},
    {12, 3, 0.062858224217885, 0.457579229975768, 0.271210385012116, 0.271210385012116},
    {12, 3, 0.034796112930709, 0.744847708916828, 0.127576145541586, 0.127576145541586},
    {12, 3, 0.006166261051559, 0.957365299093579, 0.02131735045321, 0.02131735045321},
    {12, 6, 0.040371557766381, 0.115343494534698, 0.275713269685514, 0.608943235779788},
    {12, 6, 0.022356773202303, 0.022838332222257, 0.28132558098994, 0.695836086787803},
    {12, 6, 0.017316231108659, 0.02573405054833, 0.116251915907597, 0.858014033544073},
};
static const int ORC_NSELECT[7] = {0, 2, 4, 6, 8, 10, 12}; /* NSELECT(1:6) */

/* Points (barycentric, 3 per point) and weights (summing to 1) of set np. */
static int tri_rule(int np, double *bar, double *w) {
  int i = 0;
  for (size_t o = 0; o < sizeof(ORC_TRI_ORBITS) / sizeof(ORC_TRI_ORBITS[0]); ++o) {
    const orc_orbit *r = &ORC_TRI_ORBITS[o];
    if (r->set != np) continue;
    double x[6] = {r->b1, r->b2, r->b3, r->b1, r->b2, r->b3};
    for (int k = 0; k < 3; ++k) bar[3 * i + k] = x[k];
    w[i++] = r->w;
    if (r->size == 1) continue;
    for (int k = 0; k < 3; ++k) {
      bar[3 * i + k] = x[k + 1];
      bar[3 * (i + 1) + k] = x[k + 2];
    }
    w[i] = r->w;
    w[i + 1] = r->w;
    i += 2;
    if (r->size == 3) continue;
    for (int l = 1; l <= 3; ++l) {
      for (int k = 1; k <= 3; ++k) bar[3 * (i + l - 1) + (k - 1)] = x[3 + l - k - 1];
      w[i + l - 1] = r->w;
    }
    i += 3;
  }
  return i;
}

/* ------------------------------------------------------------------------ */
/* Prism H1 (Prism.F90:33-330; AffinePrism, AffineCoordinates.F90:91-110;    */
/* BlendPrisV / BlendProjectPrisME / QE / TF / ProjectPrisQF,                 */
/* BlendProject.F90:562-804; OrientQuad, Orient.F90:39-116; AncPhiQuad,       */
/* Ancillary.F90:171-206).  Norder(15): 6 mixed (horizontal) edges, 3 quad    */
/* (vertical) edges, 2 triangle faces, 3 quad faces (h*10+v), interior        */
/* (ph*10+pz).                                                                */
/* ------------------------------------------------------------------------ */
static const int PRIS_NUPAIR[3][2] = {{0, 1}, {1, 2}, {0, 2}}; /* ME 1-3 (4-6), QF 1-3 */

static void decod2i(int v, int *a, int *b) { *a = v / 10; *b = v % 10; }

int orc_nrdofH_prism(const int32_t *norder) {
  int n = 6;
  for (int e = 0; e < 9; ++e) n += imax(norder[e] - 1, 0);
  for (int f = 0; f < 2; ++f) n += tri_ndof(norder[9 + f]);
  for (int f = 0; f < 3; ++f) {
    int h, v;
    decod2i(norder[11 + f], &h, &v);
    n += imax(h - 1, 0) * imax(v - 1, 0);
  }
  int ph, pz;
  decod2i(norder[14], &ph, &pz);
  return n + tri_ndof(ph) * imax(pz - 1, 0);
}

/* set_3Dint_aux PRISM branch (set_3D_int.F90:264-300) on find_order_loc
 * orders (find_order.F90:88-94: quad faces swap (h,v) when NFAXES says so). */
int orc_set_3D_int_prism(const int32_t *norder, const int32_t *nori_face, int integration,
                         double *xiloc, double *waloc) {
  int32_t loc[19];
  for (int i = 0; i < 19; ++i) loc[i] = norder[i];
  static const int NFAXES3[8] = {0, 1, 0, 1, 1, 0, 1, 0};
  for (int j = 0; j < 3; ++j)
    if (nori_face && NFAXES3[nori_face[2 + j] & 7]) {
      int h, v;
      decod2i(norder[11 + j], &h, &v);
      loc[11 + j] = v * 10 + h;
    }
  int nordh = 0, nordz = 0;
  for (int i = 1; i <= 15; ++i) {
    if ((i >= 1 && i <= 6) || i == 10 || i == 11) nordh = imax(nordh, loc[i - 1]);
    else if (i >= 7 && i <= 9) nordz = imax(nordz, loc[i - 1]);
    else {
      int h, v;
      decod2i(loc[i - 1], &h, &v);
      nordh = imax(nordh, h);
      nordz = imax(nordz, v);
    }
  }
  nordh = imin(nordh + integration, ORC_MAXP);
  nordz = imin(nordz + integration, ORC_MAXP);
  if (nordh < 1 || nordz < 1) return -1;
  double bar[3 * 40], wt[40], xz[16], wz[16];
  int nintx = tri_rule(ORC_NSELECT[nordh], bar, wt);
  int nintz = nordz + 1;
  orc_gauss1d(nintz, xz, wz);
  int l = 0;
  for (int l2 = 0; l2 < nintz; ++l2)
    for (int l1 = 0; l1 < nintx; ++l1) {
      xiloc[3 * l + 0] = bar[3 * l1 + 1];
      xiloc[3 * l + 1] = bar[3 * l1 + 2];
      xiloc[3 * l + 2] = xz[l2];
      waloc[l] = wt[l1] / 2.0 * wz[l2];
      ++l;
    }
  return l;
}

int orc_shape3DH_prism(const double *xi, const int32_t *nord,
                       const int32_t *nori_edge, const int32_t *nori_face,
                       double *shap, double *grad) {
  const double Nu[3] = {1.0 - xi[0] - xi[1], xi[0], xi[1]};
  const double DNu[3][3] = {{-1.0, -1.0, 0.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}};
  const double Mu[2] = {1.0 - xi[2], xi[2]};
  const double DMu[2][3] = {{0.0, 0.0, -1.0}, {0.0, 0.0, 1.0}};
  int m = 0;
  /* vertices: Nu(v mod 3) * Mu(v / 3) */
  for (int v = 0; v < 6; ++v, ++m) {
    int a = v % 3, b = v / 3;
    shap[m] = Nu[a] * Mu[b];
    for (int c = 0; c < 3; ++c) grad[3 * m + c] = DNu[a][c] * Mu[b] + Nu[a] * DMu[b][c];
  }
  /* mixed edges: homogenized Legendre of the oriented Nu pair (Idec false) x Mu */
  for (int e = 0; e < 6; ++e) {
    int p = nord[e];
    if (p - 1 <= 0) continue;
    int a = PRIS_NUPAIR[e % 3][0], b = PRIS_NUPAIR[e % 3][1], mb = e / 3;
    if (nori_edge[e] == 1) { int t = a; a = b; b = t; }
    double S[2] = {Nu[a], Nu[b]}, DS[3][2];
    for (int c = 0; c < 3; ++c) { DS[c][0] = DNu[a][c]; DS[c][1] = DNu[b][c]; }
    double phi[16], dphi[16][3];
    hom_ilegendre(S, DS, p, 0, phi, dphi);
    for (int i = 2; i <= p; ++i, ++m) {
      shap[m] = phi[i] * Mu[mb];
      for (int c = 0; c < 3; ++c) grad[3 * m + c] = dphi[i][c] * Mu[mb] + phi[i] * DMu[mb][c];
    }
  }
  /* quad (vertical) edges: Legendre of the oriented Mu pair (Idec true) x Nu */
  for (int e = 0; e < 3; ++e) {
    int p = nord[6 + e];
    if (p - 1 <= 0) continue;
    int o0 = nori_edge[6 + e] == 1 ? 1 : 0, o1 = 1 - o0;
    double S[2] = {Mu[o0], Mu[o1]}, DS[3][2];
    for (int c = 0; c < 3; ++c) { DS[c][0] = DMu[o0][c]; DS[c][1] = DMu[o1][c]; }
    double phi[16], dphi[16][3];
    hom_ilegendre(S, DS, p, 1, phi, dphi);
    for (int i = 2; i <= p; ++i, ++m) {
      shap[m] = phi[i] * Nu[e];
      for (int c = 0; c < 3; ++c) grad[3 * m + c] = dphi[i][c] * Nu[e] + phi[i] * DNu[e][c];
    }
  }
  /* triangle faces: AncPhiTri of the oriented Nu triple (Idec true) x Mu */
  for (int f = 0; f < 2; ++f) {
    int p = nord[9 + f];
    if (tri_ndof(p) <= 0) continue;
    const int *o = ORIENT_TRI[nori_face[f]];
    double S[3], DS[3][3];
    for (int k = 0; k < 3; ++k) {
      S[k] = Nu[o[k]];
      for (int c = 0; c < 3; ++c) DS[c][k] = DNu[o[k]][c];
    }
    double phi[JMAX][JMAX], dphi[JMAX][JMAX][3];
    anc_phi_tri(S, DS, p, 1, phi, dphi);
    for (int nij = 3; nij <= p; ++nij)
      for (int i = 2; i <= nij - 1; ++i, ++m) {
        int j = nij - i;
        shap[m] = phi[i][j] * Mu[f];
        for (int c = 0; c < 3; ++c) grad[3 * m + c] = dphi[i][j][c] * Mu[f] + phi[i][j] * DMu[f][c];
      }
  }
  /* quad faces: OrientQuad of ((Nu pair; Idec false), (Mu pair; Idec true)), AncPhiQuad */
  for (int f = 0; f < 3; ++f) {
    int nf[2];
    decod2i(nord[11 + f], &nf[0], &nf[1]);
    if (nf[0] < 2 || nf[1] < 2) continue;
    /* ST(k, pair): pair 0 = Nu pair, pair 1 = Mu pair */
    double ST[2][2], DST[2][2][3];
    int idec[2] = {0, 1};
    int a = PRIS_NUPAIR[f][0], b = PRIS_NUPAIR[f][1];
    ST[0][0] = Nu[a]; ST[1][0] = Nu[b];
    ST[0][1] = Mu[0]; ST[1][1] = Mu[1];
    for (int c = 0; c < 3; ++c) {
      DST[0][0][c] = DNu[a][c]; DST[1][0][c] = DNu[b][c];
      DST[0][1][c] = DMu[0][c]; DST[1][1][c] = DMu[1][c];
    }
    const int *oq = ORQ[nori_face[2 + f] & 7];
    int pa1 = oq[0], pa2 = oq[1];
    double GS[2] = {ST[oq[2]][pa1], ST[oq[3]][pa1]}, GT[2] = {ST[oq[4]][pa2], ST[oq[5]][pa2]};
    double GDS[3][2], GDT[3][2];
    for (int c = 0; c < 3; ++c) {
      GDS[c][0] = DST[oq[2]][pa1][c]; GDS[c][1] = DST[oq[3]][pa1][c];
      GDT[c][0] = DST[oq[4]][pa2][c]; GDT[c][1] = DST[oq[5]][pa2][c];
    }
    double phs[16], dphs[16][3], pht[16], dpht[16][3];
    hom_ilegendre(GS, GDS, nf[0], idec[pa1], phs, dphs);
    hom_ilegendre(GT, GDT, nf[1], idec[pa2], pht, dpht);
    for (int j = 2; j <= nf[1]; ++j)
      for (int i = 2; i <= nf[0]; ++i, ++m) {
        shap[m] = phs[i] * pht[j];
        for (int c = 0; c < 3; ++c) grad[3 * m + c] = phs[i] * dpht[j][c] + pht[j] * dphs[i][c];
      }
  }
  /* bubbles: AncPhiTri(Nu; Idec true) x AncPhiE(Mu; Idec true) */
  int ph, pz;
  decod2i(nord[14], &ph, &pz);
  if (tri_ndof(ph) > 0 && pz >= 2) {
    double S[3] = {Nu[0], Nu[1], Nu[2]}, DS[3][3];
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) DS[c][k] = DNu[k][c];
    double phi[JMAX][JMAX], dphi[JMAX][JMAX][3];
    anc_phi_tri(S, DS, ph, 1, phi, dphi);
    double Sz[2] = {Mu[0], Mu[1]}, DSz[3][2];
    for (int c = 0; c < 3; ++c) { DSz[c][0] = DMu[0][c]; DSz[c][1] = DMu[1][c]; }
    double pe[16], dpe[16][3];
    hom_ilegendre(Sz, DSz, pz, 1, pe, dpe);
    for (int k = 2; k <= pz; ++k)
      for (int nij = 3; nij <= ph; ++nij)
        for (int i = 2; i <= nij - 1; ++i, ++m) {
          int j = nij - i;
          shap[m] = phi[i][j] * pe[k];
          for (int c = 0; c < 3; ++c) grad[3 * m + c] = dphi[i][j][c] * pe[k] + phi[i][j] * dpe[k][c];
        }
  }
  return m;
}

/* ------------------------------------------------------------------------ */
/* Constrained approximation (celem_systemI.F90:541-760)                      */
/* ------------------------------------------------------------------------ */
int orc_constrain(int ni, const double *aii, const double *bi, int ncoef, const int32_t *ck,
                  const int32_t *cl, const double *cv, int nmod, double *amod, double *bmod) {
  /* rows: ZBMOD(l) += BLOC(k) c, AAUX(l,:) += ALOC(k,:) c (loop over k, then
   * its connected modified dof); columns: ZAMOD(:,l) += AAUX(:,k) c */
  double *aux = (double *)calloc((size_t)nmod * (ni > 0 ? ni : 1), sizeof(double));
  if (!aux) return -1;
  for (int i = 0; i < nmod; ++i) bmod[i] = 0.0;
  for (size_t i = 0; i < (size_t)nmod * nmod; ++i) amod[i] = 0.0;
  for (int q = 0; q < ncoef; ++q) {
    const int k = ck[q], l = cl[q];
    if (k < 0 || k >= ni || l < 0 || l >= nmod) { free(aux); return -2; }
    bmod[l] = bmod[l] + bi[k] * cv[q];
    for (int j = 0; j < ni; ++j)
      aux[l + (size_t)nmod * j] = aux[l + (size_t)nmod * j] + aii[k + (size_t)ni * j] * cv[q];
  }
  for (int q = 0; q < ncoef; ++q) {
    const int k = ck[q], l = cl[q];
    for (int i = 0; i < nmod; ++i)
      amod[i + (size_t)nmod * l] = amod[i + (size_t)nmod * l] + aux[i + (size_t)nmod * k] * cv[q];
  }
  free(aux);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Dirichlet data by projection-based interpolation (update_Ddof.F90:70-250,  */
/* dhpvert.F90, edge/dhpedgeH.F90, face/dhpfaceH.F90) for a hexahedron whose  */
/* geometry block is the element itself (eta = xi, trilinear x(eta)).        */
/* ------------------------------------------------------------------------ */
static const int BRICK_E2V[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6},
                                     {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
static const int BRICK_F2V[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                    {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}};
static const int BRICK_F2E[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 9, 4, 8},
                                    {1, 10, 5, 9}, {2, 10, 6, 11}, {3, 11, 7, 8}};
static const double BRICK_XI[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                      {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

static void trilin(const double *xvert, const double *xi, double *x, double J[3][3]) {
  double Mu[2][3];
  for (int d = 0; d < 3; ++d) { Mu[0][d] = 1.0 - xi[d]; Mu[1][d] = xi[d]; }
  for (int i = 0; i < 3; ++i) {
    x[i] = 0.0;
    for (int j = 0; j < 3; ++j) J[i][j] = 0.0;
  }
  for (int v = 0; v < 8; ++v) {
    const int *s = HEXA_V[v];
    double b0 = Mu[s[0]][0], b1 = Mu[s[1]][1], b2 = Mu[s[2]][2];
    double g[3] = {(s[0] ? 1.0 : -1.0) * b1 * b2, b0 * (s[1] ? 1.0 : -1.0) * b2,
                   b0 * b1 * (s[2] ? 1.0 : -1.0)};
    for (int i = 0; i < 3; ++i) {
      x[i] += xvert[3 * v + i] * b0 * b1 * b2;
      for (int j = 0; j < 3; ++j) J[i][j] += xvert[3 * v + i] * g[j];
    }
  }
}

/* dgetrf + dgetrs on a small system (n <= 36), partial pivoting */
static int lu_solve(int n, double *A, double *b) {
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

int orc_dirichlet_hexa(const int32_t *norder, const int32_t *nori_edge, const int32_t *nori_face,
                       const double *xvert, const int32_t *bcflag, int isol, double *zd) {
  int32_t nd[32];
  orc_node_ndof(ORC_HEXA, norder, nd);
  int first[27];
  first[0] = 0;
  for (int i = 0; i < 26; ++i) first[i + 1] = first[i] + nd[i];
  for (int k = 0; k < first[26]; ++k) zd[k] = 0.0;
  double shap[ORC_MAXBRICKH], grad[3 * ORC_MAXBRICKH];
  /* vertices (dhpvert) */
  for (int v = 0; v < 8; ++v) {
    if (!bcflag[v]) continue;
    double u, gu[3];
    orc_exact(isol, &xvert[3 * v], &u, gu);
    zd[first[v]] = u;
  }
  /* edges (dhpedgeH): tangential H1-seminorm projection of u - u_vertex */
  for (int e = 0; e < 12; ++e) {
    const int n = nd[8 + e];
    if (!bcflag[8 + e] || n == 0) continue;
    int32_t no1[19];
    for (int i = 0; i < 12; ++i) no1[i] = 1;
    for (int i = 12; i < 18; ++i) no1[i] = 11;
    no1[18] = 111;
    no1[e] = norder[e];
    int nint = imin(norder[e] + 1, ORC_MAXP) + 1; /* set_1Dint, INTEGRATION = 1 */
    double xg[16], wg[16];
    orc_gauss1d(nint, xg, wg);
    double A[64], b[8];
    for (int i = 0; i < n * n; ++i) A[i] = 0.0;
    for (int i = 0; i < n; ++i) b[i] = 0.0;
    const double *x1 = BRICK_XI[BRICK_E2V[e][0]], *x2 = BRICK_XI[BRICK_E2V[e][1]];
    for (int l = 0; l < nint; ++l) {
      double xi[3], dxidt[3];
      for (int c = 0; c < 3; ++c) { dxidt[c] = x2[c] - x1[c]; xi[c] = x1[c] + xg[l] * dxidt[c]; }
      int nr = orc_shape3DH_hexa(xi, no1, nori_edge, nori_face, shap, grad);
      double bjac = sqrt(dxidt[0] * dxidt[0] + dxidt[1] * dxidt[1] + dxidt[2] * dxidt[2]);
      double rt[3] = {dxidt[0] / bjac, dxidt[1] / bjac, dxidt[2] / bjac};
      const double w = wg[l] * bjac;
      double x[3], J[3][3];
      trilin(xvert, xi, x, J);
      double u, gu[3];
      orc_exact(isol, x, &u, gu);
      double du[3];
      for (int i = 0; i < 3; ++i) du[i] = gu[0] * J[0][i] + gu[1] * J[1][i] + gu[2] * J[2][i];
      const int nlow = nr - n;
      for (int k = 0; k < nlow; ++k)
        for (int i = 0; i < 3; ++i) du[i] -= zd[k] * grad[3 * k + i];
      for (int j = 0; j < n; ++j) {
        const double *gj = &grad[3 * (nlow + j)];
        double pr = gj[0] * rt[0] + gj[1] * rt[1] + gj[2] * rt[2];
        double dv[3] = {pr * rt[0], pr * rt[1], pr * rt[2]};
        b[j] += (du[0] * dv[0] + du[1] * dv[1] + du[2] * dv[2]) * w;
        for (int i = 0; i < n; ++i) {
          const double *gi = &grad[3 * (nlow + i)];
          A[j + n * i] += (dv[0] * gi[0] + dv[1] * gi[1] + dv[2] * gi[2]) * w;
        }
      }
    }
    if (lu_solve(n, A, b)) return -1;
    for (int j = 0; j < n; ++j) zd[first[8 + e] + j] = b[j];
  }
  /* faces (dhpfaceH): tangential H1-seminorm projection of u - u_vertex - u_edges */
  for (int f = 0; f < 6; ++f) {
    const int n = nd[20 + f];
    if (!bcflag[20 + f] || n == 0) continue;
    int32_t no1[19];
    for (int i = 0; i < 12; ++i) no1[i] = norder[i];
    for (int i = 12; i < 18; ++i) no1[i] = 11;
    no1[18] = 111;
    no1[12 + f] = norder[12 + f];
    int hv[2];
    decod(norder[12 + f], 10, 2, hv);
    const int *fe = BRICK_F2E[f];
    int nx = imin(imax(imax(norder[fe[0]], norder[fe[2]]), hv[0]) + 1, ORC_MAXP) + 1;
    int ny = imin(imax(imax(norder[fe[1]], norder[fe[3]]), hv[1]) + 1, ORC_MAXP) + 1;
    double xa[16], wa[16], xb[16], wb[16];
    orc_gauss1d(nx, xa, wa);
    orc_gauss1d(ny, xb, wb);
    double *A = (double *)calloc((size_t)n * n, sizeof(double));
    double *b = (double *)calloc((size_t)n, sizeof(double));
    const double *v1 = BRICK_XI[BRICK_F2V[f][0]], *v2 = BRICK_XI[BRICK_F2V[f][1]],
                 *v3 = BRICK_XI[BRICK_F2V[f][3]];
    const double nsign = (f == 0 || f == 4 || f == 5) ? -1.0 : 1.0;
    for (int l2 = 0; l2 < ny; ++l2)
      for (int l1 = 0; l1 < nx; ++l1) {
        double xi[3], t1[3], t2[3];
        for (int c = 0; c < 3; ++c) {
          t1[c] = v2[c] - v1[c];
          t2[c] = v3[c] - v1[c];
          xi[c] = v1[c] + xa[l1] * t1[c] + xb[l2] * t2[c];
        }
        int nr = orc_shape3DH_hexa(xi, no1, nori_edge, nori_face, shap, grad);
        double rn[3] = {t1[1] * t2[2] - t1[2] * t2[1], t1[2] * t2[0] - t1[0] * t2[2],
                        t1[0] * t2[1] - t1[1] * t2[0]};
        double bjac = sqrt(rn[0] * rn[0] + rn[1] * rn[1] + rn[2] * rn[2]);
        for (int c = 0; c < 3; ++c) rn[c] = rn[c] * nsign / bjac;
        const double w = wa[l1] * wb[l2] * bjac;
        double x[3], J[3][3];
        trilin(xvert, xi, x, J);
        double u, gu[3];
        orc_exact(isol, x, &u, gu);
        double du[3];
        for (int i = 0; i < 3; ++i) du[i] = gu[0] * J[0][i] + gu[1] * J[1][i] + gu[2] * J[2][i];
        const int nlow = nr - n;
        for (int k = 0; k < nlow; ++k)
          for (int i = 0; i < 3; ++i) du[i] -= zd[k] * grad[3 * k + i];
        for (int j = 0; j < n; ++j) {
          const double *gj = &grad[3 * (nlow + j)];
          double pr = gj[0] * rn[0] + gj[1] * rn[1] + gj[2] * rn[2];
          double dv[3] = {gj[0] - pr * rn[0], gj[1] - pr * rn[1], gj[2] - pr * rn[2]};
          b[j] += (du[0] * dv[0] + du[1] * dv[1] + du[2] * dv[2]) * w;
          for (int i = 0; i < n; ++i) {
            const double *gi = &grad[3 * (nlow + i)];
            A[j + n * i] += (dv[0] * gi[0] + dv[1] * gi[1] + dv[2] * gi[2]) * w;
          }
        }
      }
    int rc = lu_solve(n, A, b);
    if (!rc)
      for (int j = 0; j < n; ++j) zd[first[20 + f] + j] = b[j];
    free(A);
    free(b);
    if (rc) return -1;
  }
  return first[26];
}

/* ------------------------------------------------------------------------ */
/* Geometry dof by projection-based interpolation of a geometry-block map     */
/* (update_gdof.F90:80-200, 404-435; hpvert.F90, hpedge.F90, hpface.F90,      */
/* hpmdle.F90) for one hexahedron.  The block map x(eta) and its Jacobian     */
/* come from gmap (the GMP routine hexa(No, eta, x, dxdeta) of the           */
/* reference); eta(xi) is trilinear in the element's vertex coordinates etav */
/* in the block (refgeom3D / brefgeom3D).  Projections are in eta: tangential */
/* derivative along edges, surface gradient on faces, full gradient in the   */
/* interior, each of what the lower-order dof leave.                          */
/* ------------------------------------------------------------------------ */
static void eta_map(const double *etav, const double *grad, double J[3][3], double Ji[3][3],
                    double *det) {
  /* detadxi(i, m) = sum_v etav(i, v) d phi_v / d xi_m over the 8 vertex functions */
  for (int i = 0; i < 3; ++i)
    for (int m = 0; m < 3; ++m) {
      double s = 0.0;
      for (int v = 0; v < 8; ++v) s += etav[3 * v + i] * grad[3 * v + m];
      J[i][m] = s;
    }
  double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  double d = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  *det = d;
  /* dxideta = inverse of detadxi */
  Ji[0][0] = c00 / d;
  Ji[1][0] = c01 / d;
  Ji[2][0] = c02 / d;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / d;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / d;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / d;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / d;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / d;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / d;
}

/* gradient in eta of function k: duHdeta(i) = sum_m gradH(m, k) dxideta(m, i) */
static void grad_eta(const double *grad, int k, double Ji[3][3], double *g) {
  for (int i = 0; i < 3; ++i)
    g[i] = grad[3 * k] * Ji[0][i] + grad[3 * k + 1] * Ji[1][i] + grad[3 * k + 2] * Ji[2][i];
}

/* LU with partial pivoting and three right-hand sides (b: n x 3, column-major
 * by component: b[c * n + j]) */
static int lu_solve3(int n, double *A, double *b) {
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
      double f = A[i + n * k] / A[k + n * k];
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

/* one projection point: add the point's contribution to A (n x n) and b
 * (n x 3).  kind 0: edge (rt = unit tangent in eta), 1: face (rn = unit
 * normal in eta), 2: interior.  Functions nlow.. nlow+n-1 are projected; the
 * first nlow carry the current xnod. */
static void gdof_point(int kind, const double *grad, double Ji[3][3], const double *rv,
                       const double *dxdeta, const double *xnod, int nlow, int n, double weight,
                       double *A, double *b) {
  double R[3][3];
  for (int c = 0; c < 3; ++c)
    for (int i = 0; i < 3; ++i) R[c][i] = dxdeta[3 * c + i];
  for (int k = 0; k < nlow; ++k) {
    double g[3];
    grad_eta(grad, k, Ji, g);
    for (int c = 0; c < 3; ++c)
      for (int i = 0; i < 3; ++i) R[c][i] -= xnod[3 * k + c] * g[i];
  }
  for (int j = 0; j < n; ++j) {
    double dv[3];
    grad_eta(grad, nlow + j, Ji, dv);
    if (kind == 0) {
      double pr = dv[0] * rv[0] + dv[1] * rv[1] + dv[2] * rv[2];
      for (int i = 0; i < 3; ++i) dv[i] = pr * rv[i];
    } else if (kind == 1) {
      double pr = dv[0] * rv[0] + dv[1] * rv[1] + dv[2] * rv[2];
      for (int i = 0; i < 3; ++i) dv[i] -= pr * rv[i];
    }
    for (int c = 0; c < 3; ++c)
      b[c * n + j] += (R[c][0] * dv[0] + R[c][1] * dv[1] + R[c][2] * dv[2]) * weight;
    for (int i = 0; i < n; ++i) {
      double du[3];
      grad_eta(grad, nlow + i, Ji, du);
      A[j + n * i] += (dv[0] * du[0] + dv[1] * du[1] + dv[2] * du[2]) * weight;
    }
  }
}

int orc_gdof_hexa(const int32_t *norder, const int32_t *nori_edge, const int32_t *nori_face,
                  const double *etav, int integration, orc_gmap_fn gmap, void *user, int linear,
                  double *xnod) {
  int32_t nd[32];
  orc_node_ndof(ORC_HEXA, norder, nd);
  int first[27];
  first[0] = 0;
  for (int i = 0; i < 26; ++i) first[i + 1] = first[i] + nd[i];
  /* the middle node's dof (node_ndof counts vertex..face nodes only) */
  const int nrdof = orc_nrdofH_hexa(norder);
  for (int k = 0; k < 3 * nrdof; ++k) xnod[k] = 0.0;
  double *shap = (double *)malloc(sizeof(double) * ORC_MAXBRICKH);
  double *grad = (double *)malloc(sizeof(double) * 3 * ORC_MAXBRICKH);
  double *A = (double *)malloc(sizeof(double) * ORC_MAXBRICKH * ORC_MAXBRICKH);
  double *b = (double *)malloc(sizeof(double) * 3 * ORC_MAXBRICKH);
  int rc = nrdof;
  double x[3], dxdeta[9];
  /* vertices (hpvert) */
  for (int v = 0; v < 8; ++v) {
    gmap(&etav[3 * v], x, dxdeta, user);
    for (int c = 0; c < 3; ++c) xnod[3 * v + c] = x[c];
  }
  if (linear) goto done;
  /* edges (hpedge): vertex functions + this edge's */
  for (int e = 0; e < 12; ++e) {
    const int n = nd[8 + e];
    if (n == 0) continue;
    int32_t no1[19];
    for (int i = 0; i < 12; ++i) no1[i] = 1;
    for (int i = 12; i < 18; ++i) no1[i] = 11;
    no1[18] = 111;
    no1[e] = norder[e];
    const int nint = imin(norder[e] + integration, ORC_MAXP) + 1; /* set_1Dint */
    double xg[16], wg[16];
    orc_gauss1d(nint, xg, wg);
    for (int i = 0; i < n * n; ++i) A[i] = 0.0;
    for (int i = 0; i < 3 * n; ++i) b[i] = 0.0;
    const double *x1 = BRICK_XI[BRICK_E2V[e][0]], *x2 = BRICK_XI[BRICK_E2V[e][1]];
    for (int l = 0; l < nint; ++l) {
      double xi[3], dxidt[3], J[3][3], Ji[3][3], det, eta[3] = {0, 0, 0};
      for (int c = 0; c < 3; ++c) { dxidt[c] = x2[c] - x1[c]; xi[c] = x1[c] + xg[l] * dxidt[c]; }
      const int nr = orc_shape3DH_hexa(xi, no1, nori_edge, nori_face, shap, grad);
      eta_map(etav, grad, J, Ji, &det);
      for (int v = 0; v < 8; ++v)
        for (int c = 0; c < 3; ++c) eta[c] += etav[3 * v + c] * shap[v];
      double detadt[3], bjac;
      for (int i = 0; i < 3; ++i) detadt[i] = J[i][0] * dxidt[0] + J[i][1] * dxidt[1] + J[i][2] * dxidt[2];
      bjac = sqrt(detadt[0] * detadt[0] + detadt[1] * detadt[1] + detadt[2] * detadt[2]);
      const double rt[3] = {detadt[0] / bjac, detadt[1] / bjac, detadt[2] / bjac};
      gmap(eta, x, dxdeta, user);
      /* the lower part: the element's vertex dof (the first nr - n functions) */
      gdof_point(0, grad, Ji, rt, dxdeta, xnod, nr - n, n, wg[l] * bjac, A, b);
    }
    if (lu_solve3(n, A, b)) { rc = -1; goto done; }
    for (int j = 0; j < n; ++j)
      for (int c = 0; c < 3; ++c) xnod[3 * (first[8 + e] + j) + c] = b[c * n + j];
  }
  /* faces (hpface): vertex and all edge functions + this face's */
  for (int f = 0; f < 6; ++f) {
    const int n = nd[20 + f];
    if (n == 0) continue;
    int32_t no1[19];
    for (int i = 0; i < 12; ++i) no1[i] = norder[i];
    for (int i = 12; i < 18; ++i) no1[i] = 11;
    no1[18] = 111;
    no1[12 + f] = norder[12 + f];
    int hv[2];
    decod(norder[12 + f], 10, 2, hv);
    const int *fe = BRICK_F2E[f];
    /* set_2Dint over face_order: per face axis the max of its edges and the face */
    const int nx = imin(imax(imax(norder[fe[0]], norder[fe[2]]), hv[0]) + integration, ORC_MAXP) + 1;
    const int ny = imin(imax(imax(norder[fe[1]], norder[fe[3]]), hv[1]) + integration, ORC_MAXP) + 1;
    double xa[16], wa[16], xb[16], wb[16];
    orc_gauss1d(nx, xa, wa);
    orc_gauss1d(ny, xb, wb);
    for (int i = 0; i < n * n; ++i) A[i] = 0.0;
    for (int i = 0; i < 3 * n; ++i) b[i] = 0.0;
    const double *v1 = BRICK_XI[BRICK_F2V[f][0]], *v2 = BRICK_XI[BRICK_F2V[f][1]],
                 *v3 = BRICK_XI[BRICK_F2V[f][3]];
    for (int l2 = 0; l2 < ny; ++l2)
      for (int l1 = 0; l1 < nx; ++l1) {
        double xi[3], t1[3], t2[3], J[3][3], Ji[3][3], det, eta[3] = {0, 0, 0};
        for (int c = 0; c < 3; ++c) {
          t1[c] = v2[c] - v1[c];
          t2[c] = v3[c] - v1[c];
          xi[c] = v1[c] + xa[l1] * t1[c] + xb[l2] * t2[c];
        }
        const int nr = orc_shape3DH_hexa(xi, no1, nori_edge, nori_face, shap, grad);
        eta_map(etav, grad, J, Ji, &det);
        for (int v = 0; v < 8; ++v)
          for (int c = 0; c < 3; ++c) eta[c] += etav[3 * v + c] * shap[v];
        double a1[3], a2[3];
        for (int i = 0; i < 3; ++i) {
          a1[i] = J[i][0] * t1[0] + J[i][1] * t1[1] + J[i][2] * t1[2];
          a2[i] = J[i][0] * t2[0] + J[i][1] * t2[1] + J[i][2] * t2[2];
        }
        double rn[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2],
                        a1[0] * a2[1] - a1[1] * a2[0]};
        const double bjac = sqrt(rn[0] * rn[0] + rn[1] * rn[1] + rn[2] * rn[2]);
        for (int c = 0; c < 3; ++c) rn[c] /= bjac; /* its sign is immaterial */
        gmap(eta, x, dxdeta, user);
        gdof_point(1, grad, Ji, rn, dxdeta, xnod, nr - n, n, wa[l1] * wb[l2] * bjac, A, b);
      }
    if (lu_solve3(n, A, b)) { rc = -1; goto done; }
    for (int j = 0; j < n; ++j)
      for (int c = 0; c < 3; ++c) xnod[3 * (first[20 + f] + j) + c] = b[c * n + j];
  }
  /* the middle node (hpmdle): every other function, the element's own rule */
  {
    const int n = nrdof - first[26];
    if (n > 0) {
      double *xq = (double *)malloc(sizeof(double) * 3 * ORC_MAXBRICKH);
      double *wq = (double *)malloc(sizeof(double) * ORC_MAXBRICKH);
      const int nint = orc_set_3D_int_hexa(norder, nori_face, integration, xq, wq);
      for (int i = 0; i < n * n; ++i) A[i] = 0.0;
      for (int i = 0; i < 3 * n; ++i) b[i] = 0.0;
      for (int l = 0; l < nint; ++l) {
        double J[3][3], Ji[3][3], det, eta[3] = {0, 0, 0};
        const int nr = orc_shape3DH_hexa(&xq[3 * l], norder, nori_edge, nori_face, shap, grad);
        eta_map(etav, grad, J, Ji, &det);
        for (int v = 0; v < 8; ++v)
          for (int c = 0; c < 3; ++c) eta[c] += etav[3 * v + c] * shap[v];
        gmap(eta, x, dxdeta, user);
        gdof_point(2, grad, Ji, NULL, dxdeta, xnod, nr - n, n, wq[l] * det, A, b);
      }
      free(xq);
      free(wq);
      if (lu_solve3(n, A, b)) { rc = -1; goto done; }
      for (int j = 0; j < n; ++j)
        for (int c = 0; c < 3; ++c) xnod[3 * (first[26] + j) + c] = b[c * n + j];
    }
  }
done:
  free(shap);
  free(grad);
  free(A);
  free(b);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Helpers shared with hp3d_oracle_dpg.c (hp3d_oracle_int.h)                  */
/* ------------------------------------------------------------------------ */
void orc_i_decod(int nick, int mod, int n, int *arr) { decod(nick, mod, n, arr); }
void orc_i_poly_legendre(double x, double t, int nord, double *p) { poly_legendre(x, t, nord, p); }
void orc_i_poly_ilegendre(double x, double t, int nord, int idec, double *L, double *P, double *R) {
  poly_ilegendre(x, t, nord, idec, L, P, R);
}
void orc_i_hom_ilegendre(const double *S, const double DS[3][2], int nord, int idec, double *homL,
                         double dhomL[][3]) {
  hom_ilegendre(S, DS, nord, idec, homL, dhomL);
}
const int (*orc_i_hexa_e(void))[5] { return HEXA_E; }
const int (*orc_i_hexa_f(void))[4] { return HEXA_F; }
const int (*orc_i_orq(void))[6] { return ORQ; }
