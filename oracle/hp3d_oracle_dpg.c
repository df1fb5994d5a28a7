/*
 * hp3d_oracle_dpg.c -- CPU FP64 restatement of the ultraweak DPG Maxwell
 * element of hp3D on hexahedra (problems/MAXWELL/ULTRAWEAK_DPG).
 *
 * TEST INFRASTRUCTURE ONLY (see hp3d_oracle.h).  Complex values are stored
 * as interleaved (re, im) doubles, the layout of Fortran complex(8).
 * Citations are to Oden-EAG/hp3d, paths relative to trunk/.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "hp3d_oracle.h"
#include "hp3d_oracle_int.h"

typedef double _Complex zdbl;

static int mx(int a, int b) { return a > b ? a : b; }

static void cross3(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

/* AffineHexahedron (AffineCoordinates.F90:56-72) */
static void affine_hexa(const double *xi, double Mu[2][3], double DMu[3][2][3]) {
  for (int d = 0; d < 3; ++d) {
    Mu[0][d] = 1.0 - xi[d];
    Mu[1][d] = xi[d];
    for (int c = 0; c < 3; ++c) DMu[c][0][d] = DMu[c][1][d] = 0.0;
    DMu[d][0][d] = -1.0;
    DMu[d][1][d] = 1.0;
  }
}

/* AncEE with Idec = .true. (Ancillary.F90:88-132): EE_i = P_i(S) DS(:,1),
 * i = 0..nord-1, curl zero.  HomLegendre (Polynomials.F90:455-465). */
static void anc_ee(const double *S, const double DS[3][2], int nord, double EE[][3]) {
  double P[16];
  orc_i_poly_legendre(S[1], S[0] + S[1], nord - 1, P);
  for (int i = 0; i < nord; ++i)
    for (int c = 0; c < 3; ++c) EE[i][c] = P[i] * DS[c][1];
}

int orc_nrdofE_hexa(const int32_t *norder) {
  int n = 0;
  for (int e = 0; e < 12; ++e) n += mx(norder[e], 0);
  for (int f = 0; f < 6; ++f) {
    int nf[2];
    orc_i_decod(norder[12 + f], 10, 2, nf);
    n += nf[0] * mx(nf[1] - 1, 0) + mx(nf[0] - 1, 0) * nf[1];
  }
  int nb[3];
  orc_i_decod(norder[18], 10, 3, nb);
  n += nb[0] * mx(nb[1] - 1, 0) * mx(nb[2] - 1, 0) + nb[1] * mx(nb[2] - 1, 0) * mx(nb[0] - 1, 0) +
       nb[2] * mx(nb[0] - 1, 0) * mx(nb[1] - 1, 0);
  return n;
}

int orc_shape3DE_hexa(const double *xi, const int32_t *nord, const int32_t *nori_edge,
                      const int32_t *nori_face, double *shapE, double *curlE) {
  const int(*HE)[5] = orc_i_hexa_e();
  const int(*HF)[4] = orc_i_hexa_f();
  const int(*OQ)[6] = orc_i_orq();
  double Mu[2][3], DMu[3][2][3];
  affine_hexa(xi, Mu, DMu);
  int m = 0;
  /* edges: ShapE = Mub1 Mub2 EE_i, CurlE = grad(Mub1 Mub2) x EE_i */
  for (int e = 0; e < 12; ++e) {
    int ne = nord[e];
    if (ne <= 0) continue;
    const int *t = HE[e];
    double mb1 = Mu[t[0]][t[1]], mb2 = Mu[t[2]][t[3]], dt[3];
    for (int c = 0; c < 3; ++c) dt[c] = mb1 * DMu[c][t[2]][t[3]] + DMu[c][t[0]][t[1]] * mb2;
    int ax = t[4], o0 = (nori_edge[e] == 1) ? 1 : 0, o1 = 1 - o0; /* OrientE */
    double GS[2] = {Mu[o0][ax], Mu[o1][ax]}, GDS[3][2];
    for (int c = 0; c < 3; ++c) {
      GDS[c][0] = DMu[c][o0][ax];
      GDS[c][1] = DMu[c][o1][ax];
    }
    double EE[16][3];
    anc_ee(GS, GDS, ne, EE);
    for (int i = 0; i < ne; ++i, ++m) {
      for (int c = 0; c < 3; ++c) shapE[3 * m + c] = mb1 * mb2 * EE[i][c];
      cross3(dt, EE[i], &curlE[3 * m]);
    }
  }
  /* faces: two families, E-type along one face axis times phi along the
   * other; ShapE = MubF EQuad, CurlE = MubF curl(EQuad) + grad(MubF) x EQuad */
  for (int f = 0; f < 6; ++f) {
    int nf[2];
    orc_i_decod(nord[12 + f], 10, 2, nf);
    const int *t = HF[f];
    double mbf = Mu[t[0]][t[1]], dmbf[3];
    for (int c = 0; c < 3; ++c) dmbf[c] = DMu[c][t[0]][t[1]];
    int axes[2] = {t[2], t[3]};
    const int *oq = OQ[nori_face[f] & 7]; /* OrientQuad */
    int pa[2] = {axes[oq[0]], axes[oq[1]]};
    double G[2][2], GD[2][3][2];
    for (int k = 0; k < 2; ++k) {
      G[k][0] = Mu[oq[2 + 2 * k]][pa[k]];
      G[k][1] = Mu[oq[3 + 2 * k]][pa[k]];
      for (int c = 0; c < 3; ++c) {
        GD[k][c][0] = DMu[c][oq[2 + 2 * k]][pa[k]];
        GD[k][c][1] = DMu[c][oq[3 + 2 * k]][pa[k]];
      }
    }
    for (int fam = 0; fam < 2; ++fam) {
      int a = fam, b = 1 - fam; /* (a,b) = (1,2) or (2,1) */
      if (nf[a] * (nf[b] - 1) <= 0) continue;
      double EE[16][3], ph[16], dph[16][3];
      anc_ee(G[a], GD[a], nf[a], EE);
      orc_i_hom_ilegendre(G[b], GD[b], nf[b], 1, ph, dph);
      /* outer loop over the index along face axis 2, inner along axis 1 */
      int n_out = (fam == 0) ? nf[b] - 1 : nf[a], n_in = (fam == 0) ? nf[a] : nf[b] - 1;
      for (int o = 0; o < n_out; ++o)
        for (int in = 0; in < n_in; ++in, ++m) {
          int i = (fam == 0) ? in : o;          /* E index 0.. */
          int j = (fam == 0) ? o + 2 : in + 2;  /* phi index 2.. */
          double eq[3], ceq[3], tmp[3];
          for (int c = 0; c < 3; ++c) eq[c] = EE[i][c] * ph[j];
          cross3(dph[j], EE[i], ceq);
          cross3(dmbf, eq, tmp);
          for (int c = 0; c < 3; ++c) {
            shapE[3 * m + c] = mbf * eq[c];
            curlE[3 * m + c] = mbf * ceq[c] + tmp[c];
          }
        }
    }
  }
  /* bubbles: E-type along axis a times phi along b and c; the loops run over
   * the z index (outer), y, x (inner) */
  int nb[3];
  orc_i_decod(nord[18], 10, 3, nb);
  for (int fam = 0; fam < 3; ++fam) {
    int a = fam, b = (fam + 1) % 3, c3 = (fam + 2) % 3;
    if (nb[a] * (nb[b] - 1) * (nb[c3] - 1) <= 0) continue;
    double S[3][2], DS[3][3][2];
    for (int d = 0; d < 3; ++d) {
      S[d][0] = Mu[0][d];
      S[d][1] = Mu[1][d];
      for (int c = 0; c < 3; ++c) {
        DS[d][c][0] = DMu[c][0][d];
        DS[d][c][1] = DMu[c][1][d];
      }
    }
    double EE[16][3], phb[16], dphb[16][3], phc[16], dphc[16][3];
    anc_ee(S[a], DS[a], nb[a], EE);
    orc_i_hom_ilegendre(S[b], DS[b], nb[b], 1, phb, dphb);
    orc_i_hom_ilegendre(S[c3], DS[c3], nb[c3], 1, phc, dphc);
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      lo[d] = (d == a) ? 0 : 2;
      hi[d] = (d == a) ? nb[d] - 1 : nb[d];
    }
    int idx[3];
    for (idx[2] = lo[2]; idx[2] <= hi[2]; ++idx[2])
      for (idx[1] = lo[1]; idx[1] <= hi[1]; ++idx[1])
        for (idx[0] = lo[0]; idx[0] <= hi[0]; ++idx[0], ++m) {
          int i = idx[a], j = idx[b], k = idx[c3];
          double eq[3], ceq[3], tmp[3];
          for (int c = 0; c < 3; ++c) eq[c] = EE[i][c] * phb[j];
          cross3(dphb[j], EE[i], ceq);
          cross3(dphc[k], eq, tmp);
          for (int c = 0; c < 3; ++c) {
            shapE[3 * m + c] = eq[c] * phc[k];
            curlE[3 * m + c] = phc[k] * ceq[c] + tmp[c];
          }
        }
  }
  return m;
}

/* shape3DQHexa (Hexahedron.F90:640-698) */
int orc_shape3DQ_hexa(const double *xi, const int32_t *nord, double *shapQ) {
  int nb[3];
  orc_i_decod(nord[18], 10, 3, nb);
  double P[3][16];
  for (int d = 0; d < 3; ++d) orc_i_poly_legendre(xi[d], 1.0, nb[d] - 1, P[d]);
  int m = 0;
  for (int k = 0; k < nb[2]; ++k)
    for (int j = 0; j < nb[1]; ++j)
      for (int i = 0; i < nb[0]; ++i) shapQ[m++] = P[0][i] * P[1][j] * P[2][k];
  return m;
}

/* shape1HH / shape1QQ (BrokenExactSequence.F90:45-108 -> Segment.F90:30-199):
 * vertex functions 1-x, x, then integrated Legendre phi_2..phi_n; Legendre
 * P_0..P_{n-1}. */
static int seg_h(double x, int n, double *h, double *dh) {
  h[0] = 1.0 - x; dh[0] = -1.0;
  h[1] = x;       dh[1] = 1.0;
  double L[16], P[16], R[16];
  orc_i_poly_ilegendre(x, 1.0, n, 1, L, P, R);
  int m = 2;
  for (int i = 2; i <= n; ++i, ++m) {
    h[m] = L[i];
    dh[m] = P[i - 1];
  }
  return m;
}
static int seg_q(double x, int n, double *q) {
  orc_i_poly_legendre(x, 1.0, n - 1, q);
  return n;
}

/* shape3EE -> shape3DEBrokenHexa (BrokenExactSequence.F90:481-532,
 * BrokenHexahedron.F90:139-258): tensor products of 1D H1 and L2 functions. */
int orc_shape3EE_hexa(const double *xi, int nordP, double *shapE, double *curlE) {
  int nb[3];
  orc_i_decod(nordP, 10, 3, nb);
  double h[3][16], dh[3][16], q[3][16];
  int nh[3], nq[3];
  for (int d = 0; d < 3; ++d) {
    nh[d] = seg_h(xi[d], nb[d], h[d], dh[d]);
    nq[d] = seg_q(xi[d], nb[d], q[d]);
  }
  int m = 0;
  for (int k = 0; k < nh[2]; ++k) /* x-directed */
    for (int j = 0; j < nh[1]; ++j)
      for (int i = 0; i < nq[0]; ++i, ++m) {
        double *s = &shapE[3 * m], *c = &curlE[3 * m];
        s[0] = q[0][i] * h[1][j] * h[2][k]; s[1] = 0.0; s[2] = 0.0;
        c[0] = 0.0;
        c[1] = q[0][i] * h[1][j] * dh[2][k];
        c[2] = -q[0][i] * dh[1][j] * h[2][k];
      }
  for (int k = 0; k < nh[2]; ++k) /* y-directed */
    for (int j = 0; j < nq[1]; ++j)
      for (int i = 0; i < nh[0]; ++i, ++m) {
        double *s = &shapE[3 * m], *c = &curlE[3 * m];
        s[0] = 0.0; s[1] = h[0][i] * q[1][j] * h[2][k]; s[2] = 0.0;
        c[0] = -h[0][i] * q[1][j] * dh[2][k];
        c[1] = 0.0;
        c[2] = dh[0][i] * q[1][j] * h[2][k];
      }
  for (int k = 0; k < nq[2]; ++k) /* z-directed */
    for (int j = 0; j < nh[1]; ++j)
      for (int i = 0; i < nh[0]; ++i, ++m) {
        double *s = &shapE[3 * m], *c = &curlE[3 * m];
        s[0] = 0.0; s[1] = 0.0; s[2] = h[0][i] * h[1][j] * q[2][k];
        c[0] = h[0][i] * dh[1][j] * q[2][k];
        c[1] = -dh[0][i] * h[1][j] * q[2][k];
        c[2] = 0.0;
      }
  return m;
}

/* face geometry of the brick (element_data.F90: BRICK_COORD, BRICK_FACE_TO_VERT,
 * BRICK_FACE_TO_EDGE, Nsign_param 616-660, face_param 554-611) */
static const double BRICK_COORD[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                         {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const int BRICK_F2V[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                    {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}};
static const int BRICK_F2E[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 9, 4, 8},
                                    {1, 10, 5, 9}, {2, 10, 6, 11}, {3, 11, 7, 8}};
static const int BRICK_NSIGN[6] = {-1, 1, 1, 1, -1, -1};
/* NFAXES(3, orientation): face axes swapped (element_data.F90:246-249) */
static const int NFAXES3[8] = {0, 1, 0, 1, 1, 0, 1, 0};

static void face_param(int f, const double *t, double *xi, double dxidt[3][2]) {
  const double *x1 = BRICK_COORD[BRICK_F2V[f][0]], *x2 = BRICK_COORD[BRICK_F2V[f][1]],
               *x3 = BRICK_COORD[BRICK_F2V[f][3]];
  for (int c = 0; c < 3; ++c) {
    dxidt[c][0] = x2[c] - x1[c];
    dxidt[c][1] = x3[c] - x1[c];
    xi[c] = x1[c] + t[0] * dxidt[c][0] + t[1] * dxidt[c][1];
  }
}

/* set_2D_int / set_2D_int_DPG for a quad face (set_2D_int.F90:72-149 ->
 * set_2Dint_aux 177-247): tensor Gauss rule of the face orders + INTEGRATION,
 * axes swapped for the orientation codes that swap them. */
int orc_set_2D_int_quad(const int32_t *norderf, int nori, int integration, int maxp,
                        double *tloc, double *wtloc) {
  int nxy[2];
  orc_i_decod(norderf[4], 10, 2, nxy);
  if (NFAXES3[nori & 7]) { int tmp = nxy[0]; nxy[0] = nxy[1]; nxy[1] = tmp; }
  int nx = mx(mx(norderf[0], norderf[2]), nxy[0]) + integration;
  int ny = mx(mx(norderf[1], norderf[3]), nxy[1]) + integration;
  if (nx > maxp) nx = maxp;
  if (ny > maxp) ny = maxp;
  double xa[16], wa[16], xb[16], wb[16];
  if (orc_gauss1d(nx + 1, xa, wa) || orc_gauss1d(ny + 1, xb, wb)) return -1;
  int l = 0;
  for (int l2 = 0; l2 <= ny; ++l2)
    for (int l1 = 0; l1 <= nx; ++l1, ++l) {
      tloc[2 * l] = xa[l1];
      tloc[2 * l + 1] = xb[l2];
      wtloc[l] = wa[l1] * wb[l2];
    }
  return l;
}

/* trilinear geometry from the 8 vertex functions (geom3D.F90:30-112 with
 * vertex-only geometry dof); bgeom3D (geom3D.F90:149-203) adds the face
 * tangents, the outward unit normal and the surface Jacobian. */
static int geom_hexa(const double *xvert, const double *xi, double *x, double *dxdxi,
                     double *dxidx, double *rjac) {
  double Mu[2][3], DMu[3][2][3];
  affine_hexa(xi, Mu, DMu);
  static const int V[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                              {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  for (int c = 0; c < 3; ++c) x[c] = 0.0;
  for (int k = 0; k < 9; ++k) dxdxi[k] = 0.0;
  for (int v = 0; v < 8; ++v) {
    double b0 = Mu[V[v][0]][0], b1 = Mu[V[v][1]][1], b2 = Mu[V[v][2]][2];
    double s = b0 * b1 * b2, g[3];
    for (int c = 0; c < 3; ++c)
      g[c] = b0 * b1 * DMu[c][V[v][2]][2] + b0 * DMu[c][V[v][1]][1] * b2 + DMu[c][V[v][0]][0] * b1 * b2;
    for (int i = 0; i < 3; ++i) {
      x[i] += xvert[3 * v + i] * s;
      for (int j = 0; j < 3; ++j) dxdxi[i + 3 * j] += xvert[3 * v + i] * g[j];
    }
  }
  return orc_geom(dxdxi, dxidx, rjac);
}

/* mfd_solutions (common/mfd_solutions.F90) cases 0-2 for the component
 * ICOMP_EXACT of E, exact (exact.F90: H = curl E / (-i omega mu)) and getf
 * (getf.F90: J = curl H - i omega epsilon E). */
static void mfd_scalar(int isol, double omega, const double *X, zdbl *p, zdbl gp[3], zdbl g2p[3][3]) {
  double x = X[0], y = X[1], z = X[2];
  *p = 0.0;
  for (int i = 0; i < 3; ++i) {
    gp[i] = 0.0;
    for (int j = 0; j < 3; ++j) g2p[i][j] = 0.0;
  }
  if (isol == 1) {
    double w = omega, sx = sin(w * x), sy = sin(w * y), sz = sin(w * z), cx = cos(w * x),
           cy = cos(w * y), cz = cos(w * z);
    zdbl c = 1.0 + 1.0 * I;
    *p = sx * sy * sz * c;
    gp[0] = w * cx * sy * sz * c; gp[1] = w * sx * cy * sz * c; gp[2] = w * sx * sy * cz * c;
    g2p[0][0] = g2p[1][1] = g2p[2][2] = -w * w * sx * sy * sz * c;
    g2p[0][1] = g2p[1][0] = w * w * cx * cy * sz * c;
    g2p[0][2] = g2p[2][0] = w * w * cx * sy * cz * c;
    g2p[1][2] = g2p[2][1] = w * w * sx * cy * cz * c;
  } else if (isol == 2) {
    zdbl cn = 100.0;
    *p = -cn * x * y * z * (x - 1.0) * (y - 1.0) * (z - 1.0);
    gp[0] = -cn * y * z * (2.0 * x - 1.0) * (y - 1.0) * (z - 1.0);
    gp[1] = -cn * x * z * (2.0 * y - 1.0) * (x - 1.0) * (z - 1.0);
    gp[2] = -cn * x * y * (2.0 * z - 1.0) * (x - 1.0) * (y - 1.0);
    g2p[0][0] = cn * y * z * (y - 1.0) * (z - 1.0) * (-2.0);
    g2p[1][1] = cn * x * z * (x - 1.0) * (z - 1.0) * (-2.0);
    g2p[2][2] = cn * x * y * (x - 1.0) * (y - 1.0) * (-2.0);
    g2p[0][1] = g2p[1][0] = -cn * z * (2.0 * x - 1.0) * (2.0 * y - 1.0) * (z - 1.0);
    g2p[0][2] = g2p[2][0] = -cn * y * (2.0 * x - 1.0) * (2.0 * z - 1.0) * (y - 1.0);
    g2p[1][2] = g2p[2][1] = -cn * x * (2.0 * y - 1.0) * (2.0 * z - 1.0) * (x - 1.0);
  }
}

void orc_maxw_exact(int isol, int icomp, double omega, double mu, double eps_re, double eps_im,
                    const double *X, double *E, double *H, double *J) {
  zdbl p, gp[3], g2p[3][3];
  mfd_scalar(isol, omega, X, &p, gp, g2p);
  int c = icomp - 1;
  zdbl e[3] = {0, 0, 0}, h[3], cc[3], j[3];
  e[c] = p;
  /* curl(p e_c) = grad p x e_c; curl curl(p e_c) = grad(d_c p) - lap(p) e_c */
  zdbl u[3] = {0, 0, 0};
  u[c] = 1.0;
  h[0] = gp[1] * u[2] - gp[2] * u[1];
  h[1] = gp[2] * u[0] - gp[0] * u[2];
  h[2] = gp[0] * u[1] - gp[1] * u[0];
  zdbl lap = g2p[0][0] + g2p[1][1] + g2p[2][2];
  for (int i = 0; i < 3; ++i) cc[i] = g2p[i][c] - (i == c ? lap : 0.0);
  zdbl fac = -I * omega * mu, epsz = eps_re + I * eps_im;
  for (int i = 0; i < 3; ++i) {
    h[i] /= fac;
    j[i] = cc[i] / fac - I * omega * epsz * e[i];
  }
  for (int i = 0; i < 3; ++i) {
    if (E) { E[2 * i] = creal(e[i]); E[2 * i + 1] = cimag(e[i]); }
    if (H) { H[2 * i] = creal(h[i]); H[2 * i + 1] = cimag(h[i]); }
    if (J) { J[2 * i] = creal(j[i]); J[2 * i + 1] = cimag(j[i]); }
  }
}

/* trial orders of the interface traces: no bubbles (norderi(19) = 111,
 * elem_maxwell.F90:215-217) */
static void trace_orders(const int32_t *norder, int32_t *norderi) {
  memcpy(norderi, norder, 19 * sizeof(int32_t));
  norderi[18] = 111;
}

int orc_dpg_sizes(const int32_t *norder, int nord_add, int32_t *sizes) {
  int32_t ni[19];
  trace_orders(norder, ni);
  int nb[3];
  orc_i_decod(norder[18], 10, 3, nb);
  int ee = orc_nrdofE_hexa(ni), nq = nb[0] * nb[1] * nb[2];
  int nordP = norder[18] + nord_add * 111, pb[3];
  orc_i_decod(nordP, 10, 3, pb);
  int test = pb[0] * (pb[1] + 1) * (pb[2] + 1) + pb[1] * (pb[2] + 1) * (pb[0] + 1) +
             pb[2] * (pb[0] + 1) * (pb[1] + 1);
  sizes[0] = ee;          /* NrdofEi */
  sizes[1] = nq;          /* NrdofQ */
  sizes[2] = test;        /* NrdofEE */
  sizes[3] = 2 * test;    /* NrTest */
  sizes[4] = 2 * ee + 6 * nq; /* NrTrial */
  return sizes[4];
}

/* packed upper index of (i, j), i <= j, 0-based (ij_upper_to_packed) */
static size_t pku(int i, int j) { return (size_t)i + (size_t)j * (j + 1) / 2; }

int orc_dpg_maxwell_elem(const int32_t *norder, const int32_t *nori_edge, const int32_t *nori_face,
                         const double *xvert, double eps_re, double eps_im, int32_t imp_mask,
                         const orc_maxw_params *prm, double *zaloc_out, double *zbloc_out) {
  int32_t sz[5], norderi[19];
  orc_dpg_sizes(norder, prm->nord_add, sz);
  trace_orders(norder, norderi);
  const int nEi = sz[0], nQ = sz[1], nEE = sz[2], nT = sz[3], nR = sz[4];
  const int nordP = norder[18] + prm->nord_add * 111;
  const zdbl epsz = eps_re + I * eps_im;
  const zdbl za = I * prm->omega * prm->epsilon * epsz; /* i omega epsilon eps */
  const zdbl zc1 = I * prm->omega * prm->mu;
  const double afac = prm->alpha; /* GRAPH_NORM */
  zdbl *gram = (zdbl *)calloc(pku(nT - 1, nT - 1) + 1, sizeof(zdbl));
  zdbl *S = (zdbl *)calloc((size_t)nT * (nR + 1), sizeof(zdbl)); /* stiff_ALL, col-major */
  double *shapEE = (double *)malloc(sizeof(double) * 3 * nEE);
  double *curlEE = (double *)malloc(sizeof(double) * 3 * nEE);
  double *shapF = (double *)malloc(sizeof(double) * 3 * nEE);
  double *curlF = (double *)malloc(sizeof(double) * 3 * nEE);
  double *shapE = (double *)malloc(sizeof(double) * 3 * (nEi + 1));
  double *curlE = (double *)malloc(sizeof(double) * 3 * (nEi + 1));
  double *shapFi = (double *)malloc(sizeof(double) * 3 * (nEi + 1));
  double shapQ[512];
  int rc = 0;
#define SEL(row, col) S[(size_t)(row) + (size_t)nT * (col)]
  /* ---- element integrals (elem_maxwell.F90:224-427) ---- */
  double xiloc[3 * 600], waloc[600];
  int nint = orc_set_3D_int_hexa(norder, nori_face, prm->nord_add, xiloc, waloc);
  for (int l = 0; l < nint && !rc; ++l) {
    const double *xi = &xiloc[3 * l];
    double x[3], dxdxi[9], dxidx[9], rjac;
    if (geom_hexa(xvert, xi, x, dxdxi, dxidx, &rjac)) { rc = -1; break; }
    orc_shape3DQ_hexa(xi, norder, shapQ);
    orc_shape3EE_hexa(xi, nordP, shapEE, curlEE);
    const double weight = rjac * waloc[l];
    double J6[6];
    orc_maxw_exact(prm->isol, prm->icomp, prm->omega, prm->mu, prm->epsilon * eps_re,
                   prm->epsilon * eps_im, x, NULL, NULL, J6);
    zdbl zJ[3] = {J6[0] + I * J6[1], J6[2] + I * J6[3], J6[4] + I * J6[5]};
    if (prm->isol == 0) zJ[0] = zJ[1] = zJ[2] = 0.0;
    /* pullbacks */
    for (int k = 0; k < nEE; ++k)
      for (int c = 0; c < 3; ++c) {
        double sf = 0.0, cf = 0.0;
        for (int i = 0; i < 3; ++i) {
          sf += dxidx[i + 3 * c] * shapEE[3 * k + i];
          cf += dxdxi[c + 3 * i] * curlEE[3 * k + i];
        }
        shapF[3 * k + c] = sf;
        curlF[3 * k + c] = cf / rjac;
      }
    for (int k1 = 0; k1 < nEE; ++k1) {
      const double *F = &shapF[3 * k1], *CF = &curlF[3 * k1];
      zdbl eTF[3]; /* epsTfldF = conj(za) F */
      for (int c = 0; c < 3; ++c) eTF[c] = conj(za) * F[c];
      /* load: (J, F) */
      SEL(2 * k1, nR) += (F[0] * zJ[0] + F[1] * zJ[1] + F[2] * zJ[2]) * weight;
      /* stiffness with the L2 trial fields */
      for (int k2 = 0; k2 < nQ; ++k2) {
        const int m = 2 * nEi + 6 * k2;
        const double fE = shapQ[k2] / rjac;
        for (int c = 0; c < 3; ++c) {
          SEL(2 * k1, m + c) -= fE * conj(eTF[c]) * weight;
          SEL(2 * k1, m + 3 + c) += fE * CF[c] * weight;
          SEL(2 * k1 + 1, m + c) += fE * CF[c] * weight;
          SEL(2 * k1 + 1, m + 3 + c) += zc1 * fE * F[c] * weight;
        }
      }
      /* Gram of the scaled adjoint graph norm (upper triangle) */
      for (int k2 = k1; k2 < nEE; ++k2) {
        const double *E = &shapF[3 * k2], *CE = &curlF[3 * k2];
        zdbl eTE[3], ecE[3];
        for (int c = 0; c < 3; ++c) {
          eTE[c] = conj(za) * E[c];
          ecE[c] = za * CE[c];
        }
        double FF = F[0] * E[0] + F[1] * E[1] + F[2] * E[2];
        double CC = CF[0] * CE[0] + CF[1] * CE[1] + CF[2] * CE[2];
        zdbl zaux = conj(eTF[0]) * eTE[0] + conj(eTF[1]) * eTE[1] + conj(eTF[2]) * eTE[2];
        gram[pku(2 * k1, 2 * k2)] += (zaux + afac * FF + CC) * weight;
        zdbl zcux = cabs(zc1) * cabs(zc1) * FF;
        gram[pku(2 * k1 + 1, 2 * k2 + 1)] += (zcux + afac * FF + CC) * weight;
        zaux = -(F[0] * ecE[0] + F[1] * ecE[1] + F[2] * ecE[2]);
        zcux = conj(zc1) * (CF[0] * E[0] + CF[1] * E[1] + CF[2] * E[2]);
        gram[pku(2 * k1, 2 * k2 + 1)] += (zaux + zcux) * weight;
        if (k1 != k2) {
          zaux = -(CF[0] * eTE[0] + CF[1] * eTE[1] + CF[2] * eTE[2]);
          zcux = zc1 * (F[0] * CE[0] + F[1] * CE[1] + F[2] * CE[2]);
          gram[pku(2 * k1 + 1, 2 * k2)] += (zaux + zcux) * weight;
        }
      }
    }
  }
  /* ---- boundary integrals with the traces (elem_maxwell.F90:440-556) ---- */
  for (int f = 0; f < 6 && !rc; ++f) {
    int32_t nordf[5];
    for (int i = 0; i < 4; ++i) nordf[i] = norder[BRICK_F2E[f][i]];
    nordf[4] = norder[12 + f];
    double tl[2 * 100], wt[100];
    int nf = orc_set_2D_int_quad(nordf, nori_face[f], prm->nord_add, ORC_MAXP + 1, tl, wt);
    for (int l = 0; l < nf; ++l) {
      double xi[3], dxidt[3][2], x[3], dxdxi[9], dxidx[9], rjac;
      face_param(f, &tl[2 * l], xi, dxidt);
      orc_shape3EE_hexa(xi, nordP, shapEE, curlEE);
      orc_shape3DE_hexa(xi, norderi, nori_edge, nori_face, shapE, curlE);
      if (geom_hexa(xvert, xi, x, dxdxi, dxidx, &rjac)) { rc = -1; break; }
      double t1[3], t2[3], rn[3];
      for (int i = 0; i < 3; ++i) {
        t1[i] = t2[i] = 0.0;
        for (int j = 0; j < 3; ++j) {
          t1[i] += dxdxi[i + 3 * j] * dxidt[j][0];
          t2[i] += dxdxi[i + 3 * j] * dxidt[j][1];
        }
      }
      cross3(t1, t2, rn);
      double bjac = sqrt(rn[0] * rn[0] + rn[1] * rn[1] + rn[2] * rn[2]);
      for (int i = 0; i < 3; ++i) rn[i] = rn[i] * BRICK_NSIGN[f] / bjac;
      const double weight = bjac * wt[l];
      for (int k = 0; k < nEE; ++k)
        for (int c = 0; c < 3; ++c) {
          double s = 0.0;
          for (int i = 0; i < 3; ++i) s += dxidx[i + 3 * c] * shapEE[3 * k + i];
          shapF[3 * k + c] = s;
        }
      for (int k = 0; k < nEi; ++k)
        for (int c = 0; c < 3; ++c) {
          double s = 0.0;
          for (int i = 0; i < 3; ++i) s += dxidx[i + 3 * c] * shapE[3 * k + i];
          shapFi[3 * k + c] = s;
        }
      for (int k1 = 0; k1 < nEE; ++k1) {
        const double *E1 = &shapF[3 * k1];
        for (int k2 = 0; k2 < nEi; ++k2) {
          double nxE[3];
          cross3(rn, &shapFi[3 * k2], nxE);
          double v = (E1[0] * nxE[0] + E1[1] * nxE[1] + E1[2] * nxE[2]) * weight;
          SEL(2 * k1, 2 * k2 + 1) += v; /* <n x H, F> */
          SEL(2 * k1 + 1, 2 * k2) += v; /* <n x E, G> */
        }
      }
    }
  }
  /* ---- DPG system (elem_maxwell.F90:560-639): G = U^H U (ZPPTRF),
   *      U^H X = [B|l] (ZTPTRS), X^H X (ZHERK) ---- */
  for (int j = 0; j < nT && !rc; ++j) {
    for (int i = 0; i < j; ++i) { /* solve U^H u = g(0:j-1, j) */
      zdbl t = gram[pku(i, j)];
      for (int k = 0; k < i; ++k) t -= conj(gram[pku(k, i)]) * gram[pku(k, j)];
      gram[pku(i, j)] = t / creal(gram[pku(i, i)]);
    }
    double ajj = creal(gram[pku(j, j)]);
    for (int k = 0; k < j; ++k) ajj -= creal(conj(gram[pku(k, j)]) * gram[pku(k, j)]);
    if (!(ajj > 0.0)) { rc = -2; break; }
    gram[pku(j, j)] = sqrt(ajj);
  }
  if (!rc)
    for (int col = 0; col <= nR; ++col) {
      zdbl *x = &S[(size_t)nT * col];
      for (int i = 0; i < nT; ++i) {
        zdbl t = x[i];
        for (int k = 0; k < i; ++k) t -= conj(gram[pku(k, i)]) * x[k];
        x[i] = t / creal(gram[pku(i, i)]);
      }
    }
  if (!rc) {
    const int n1 = nR + 1;
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i <= j; ++i) {
        zdbl s = 0.0;
        const zdbl *xi_ = &S[(size_t)nT * i], *xj = &S[(size_t)nT * j];
        for (int k = 0; k < nT; ++k) s += conj(xi_[k]) * xj[k];
        if (j < nR) {
          zaloc_out[2 * ((size_t)i + (size_t)nR * j)] = creal(s);
          zaloc_out[2 * ((size_t)i + (size_t)nR * j) + 1] = cimag(s);
          zaloc_out[2 * ((size_t)j + (size_t)nR * i)] = creal(s);
          zaloc_out[2 * ((size_t)j + (size_t)nR * i) + 1] = -cimag(s);
        } else if (i < nR) { /* the (load, load) entry is not an output */
          zbloc_out[2 * i] = creal(s);
          zbloc_out[2 * i + 1] = cimag(s);
        }
      }
  }
  /* ---- impedance penalty (elem_maxwell.F90:664-876, IBCFLAG = 2) ---- */
  if (!rc && prm->ibcflag == 2 && imp_mask) {
    const double gam = prm->gamma;
    for (int f = 0; f < 6; ++f) {
      if (!((imp_mask >> f) & 1)) continue;
      int32_t nordf[5];
      for (int i = 0; i < 4; ++i) nordf[i] = norder[BRICK_F2E[f][i]];
      nordf[4] = norder[12 + f];
      double tl[2 * 100], wt[100];
      int nf = orc_set_2D_int_quad(nordf, nori_face[f], 0, ORC_MAXP, tl, wt);
      for (int l = 0; l < nf; ++l) {
        double xi[3], dxidt[3][2], x[3], dxdxi[9], dxidx[9], rjac;
        face_param(f, &tl[2 * l], xi, dxidt);
        orc_shape3DE_hexa(xi, norderi, nori_edge, nori_face, shapE, curlE);
        geom_hexa(xvert, xi, x, dxdxi, dxidx, &rjac);
        double t1[3], t2[3], rn[3];
        for (int i = 0; i < 3; ++i) {
          t1[i] = t2[i] = 0.0;
          for (int j = 0; j < 3; ++j) {
            t1[i] += dxdxi[i + 3 * j] * dxidt[j][0];
            t2[i] += dxdxi[i + 3 * j] * dxidt[j][1];
          }
        }
        cross3(t1, t2, rn);
        double bjac = sqrt(rn[0] * rn[0] + rn[1] * rn[1] + rn[2] * rn[2]);
        for (int i = 0; i < 3; ++i) rn[i] = rn[i] * BRICK_NSIGN[f] / bjac;
        const double weight = bjac * wt[l];
        for (int k = 0; k < nEi; ++k)
          for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int i = 0; i < 3; ++i) s += shapE[3 * k + i] * dxidx[i + 3 * c];
            shapFi[3 * k + c] = s;
          }
        for (int k1 = 0; k1 < nEi; ++k1) {
          double nF[3], nnF[3];
          cross3(rn, &shapFi[3 * k1], nF);
          cross3(rn, nF, nnF);
          for (int k2 = 0; k2 < nEi; ++k2) {
            double nE[3], nnE[3];
            cross3(rn, &shapFi[3 * k2], nE);
            cross3(rn, nE, nnE);
            double a = (nnF[0] * nnE[0] + nnF[1] * nnE[1] + nnF[2] * nnE[2]) * gam * gam * weight;
            double b = -(nnF[0] * nE[0] + nnF[1] * nE[1] + nnF[2] * nE[2]) * gam * weight;
            double c2 = -(nF[0] * nnE[0] + nF[1] * nnE[1] + nF[2] * nnE[2]) * gam * weight;
            double d = (nF[0] * nE[0] + nF[1] * nE[1] + nF[2] * nE[2]) * weight;
            zaloc_out[2 * ((size_t)(2 * k1) + (size_t)nR * (2 * k2))] += a;
            zaloc_out[2 * ((size_t)(2 * k1) + (size_t)nR * (2 * k2 + 1))] += b;
            zaloc_out[2 * ((size_t)(2 * k1 + 1) + (size_t)nR * (2 * k2))] += c2;
            zaloc_out[2 * ((size_t)(2 * k1 + 1) + (size_t)nR * (2 * k2 + 1))] += d;
          }
        }
      }
    }
  }
#undef SEL
  free(gram); free(S); free(shapEE); free(curlEE); free(shapF); free(curlF);
  free(shapE); free(curlE); free(shapFi);
  return rc ? rc : nR;
}

/* stc_fwd_herm (stc.F90:338-416) for a complex Hermitian element matrix:
 * interface dof first.  aii (ni x ni), aschur (nb x ni), all complex
 * interleaved, column-major. */
int orc_stc_fwd_z(int ni, int nb, const double *a_, int lda, const double *b_, double *aii_,
                  double *bi_, double *aschur_, double *bschur_) {
  const zdbl *a = (const zdbl *)a_, *b = (const zdbl *)b_;
  zdbl *aii = (zdbl *)aii_, *bi = (zdbl *)bi_, *aschur = (zdbl *)aschur_, *bschur = (zdbl *)bschur_;
  zdbl *abb = (zdbl *)malloc(sizeof(zdbl) * (size_t)nb * nb);
  zdbl *aib = (zdbl *)malloc(sizeof(zdbl) * (size_t)ni * nb);
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
  /* Abb = U^H U */
  for (int j = 0; j < nb && !rc; ++j) {
    double s = creal(abb[j + (size_t)nb * j]);
    for (int k = 0; k < j; ++k) s -= creal(conj(abb[k + (size_t)nb * j]) * abb[k + (size_t)nb * j]);
    if (!(s > 0.0)) { rc = -1; break; }
    double ujj = sqrt(s);
    abb[j + (size_t)nb * j] = ujj;
    for (int i = j + 1; i < nb; ++i) {
      zdbl t = abb[j + (size_t)nb * i];
      for (int k = 0; k < j; ++k) t -= conj(abb[k + (size_t)nb * j]) * abb[k + (size_t)nb * i];
      abb[j + (size_t)nb * i] = t / ujj;
    }
  }
  if (!rc)
    for (int c = -1; c < ni; ++c) {
      zdbl *x = (c < 0) ? bschur : &aschur[(size_t)nb * c];
      for (int k = 0; k < nb; ++k) { /* U^H y = x */
        zdbl t = x[k];
        for (int i = 0; i < k; ++i) t -= conj(abb[i + (size_t)nb * k]) * x[i];
        x[k] = t / creal(abb[k + (size_t)nb * k]);
      }
      for (int k = nb - 1; k >= 0; --k) { /* U z = y */
        zdbl t = x[k];
        for (int i = k + 1; i < nb; ++i) t -= abb[k + (size_t)nb * i] * x[i];
        x[k] = t / creal(abb[k + (size_t)nb * k]);
      }
    }
  if (!rc) {
    for (int i = 0; i < ni; ++i) {
      zdbl s = 0.0;
      for (int k = 0; k < nb; ++k) s += aib[i + (size_t)ni * k] * bschur[k];
      bi[i] -= s;
    }
    for (int j = 0; j < ni; ++j)
      for (int i = 0; i < ni; ++i) {
        zdbl s = 0.0;
        for (int k = 0; k < nb; ++k) s += aib[i + (size_t)ni * k] * aschur[k + (size_t)nb * j];
        aii[i + (size_t)ni * j] -= s;
      }
  }
  free(abb);
  free(aib);
  return rc;
}

/* H(curl) shape functions per element node (vertices, edges, faces:
 * ndof_nod, element_data.F90:808-884, E branch) */
int orc_node_nshapeE(const int32_t *norder, int32_t *nsh) {
  for (int v = 0; v < 8; ++v) nsh[v] = 0;
  for (int e = 0; e < 12; ++e) nsh[8 + e] = mx(norder[e], 0);
  for (int f = 0; f < 6; ++f) {
    int nf[2];
    orc_i_decod(norder[12 + f], 10, 2, nf);
    nsh[20 + f] = nf[0] * mx(nf[1] - 1, 0) + mx(nf[0] - 1, 0) * nf[1];
  }
  return 26;
}

/* celem_systemI H(curl) branch (celem_systemI.F90:353-420) with the two
 * components (E, H traces) of the EHtrc attribute, then the Dirichlet lift
 * and compression (800-845).  bcflag per node: bit 0 = E component known
 * (Dirichlet), bit 1 = H component known.  Complex interleaved arrays. */
int orc_celem_compress_z(const int32_t *norder, const int32_t *bcflag, const double *aii_,
                         const double *bi_, const double *zdofd_, int32_t *nextract,
                         double *zbload_, double *zastif_, int32_t *ndofm) {
  const zdbl *aii = (const zdbl *)aii_, *bi = (const zdbl *)bi_, *zdofd = (const zdbl *)zdofd_;
  zdbl *zbload = (zdbl *)zbload_, *zastif = (zdbl *)zastif_;
  int32_t ns[26];
  orc_node_nshapeE(norder, ns);
  int first[26], ni = 0;
  for (int i = 0; i < 26; ++i) { first[i] = ni; ni += 2 * ns[i]; }
  int k = 0;
  for (int i = 25; i >= 0; --i) {
    int kold = k;
    for (int j = 0; j < ns[i]; ++j)
      for (int comp = 0; comp < 2; ++comp)
        if (!((bcflag[i] >> comp) & 1)) nextract[k++] = first[i] + 2 * j + comp;
    ndofm[i] = k - kold;
  }
  int nc = k;
  zdbl *zb = (zdbl *)malloc(sizeof(zdbl) * (ni > 0 ? ni : 1));
  for (int i = 0; i < ni; ++i) zb[i] = bi[i];
  if (zdofd)
    for (int i2 = 0; i2 < 26; ++i2)
      for (int j = 0; j < ns[i2]; ++j)
        for (int comp = 0; comp < 2; ++comp) {
          if (!((bcflag[i2] >> comp) & 1)) continue;
          int k2 = first[i2] + 2 * j + comp;
          for (int k1 = 0; k1 < ni; ++k1) zb[k1] -= aii[k1 + (size_t)ni * k2] * zdofd[k2];
        }
  for (int l1 = 0; l1 < nc; ++l1) {
    zbload[l1] = zb[nextract[l1]];
    for (int l2 = 0; l2 < nc; ++l2)
      zastif[(size_t)l1 * nc + l2] = aii[nextract[l1] + (size_t)ni * nextract[l2]];
  }
  free(zb);
  return nc;
}

/* The whole DPG element pass over a batch (OpenMP over elements):
 * elem_maxwell -> stc_fwd_herm -> celem compression.  Outputs at the given
 * offsets (complex counts); NULL skips an output. */
int orc_dpg_pass(int nelem, const int32_t *norder, const int32_t *nori_edge,
                 const int32_t *nori_face, const int32_t *bcflag, const int32_t *imp_mask,
                 const double *xvert, const double *eps, const orc_maxw_params *prm, int nthreads,
                 const int64_t *elem_nnz, const int64_t *lcon_off, const int64_t *schur_off,
                 const int64_t *bub_off, double *zastif, double *zbload, double *aschur,
                 double *bschur) {
  int bad = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int e = 0; e < nelem; ++e) {
    const int32_t *no = &norder[(size_t)19 * e];
    int32_t sz[5];
    orc_dpg_sizes(no, prm->nord_add, sz);
    const int nR = sz[4], ni = 2 * sz[0], nb = 6 * sz[1];
    double *zal = (double *)malloc(sizeof(double) * 2 * (size_t)nR * nR);
    double *zbl = (double *)malloc(sizeof(double) * 2 * nR);
    double *aii = (double *)malloc(sizeof(double) * 2 * (size_t)ni * ni);
    double *bi = (double *)malloc(sizeof(double) * 2 * ni);
    double *as = (double *)malloc(sizeof(double) * 2 * ((size_t)nb * ni + 1));
    double *bs = (double *)malloc(sizeof(double) * 2 * (nb + 1));
    double *za = (double *)malloc(sizeof(double) * 2 * (size_t)ni * ni);
    double *zb = (double *)malloc(sizeof(double) * 2 * ni);
    int32_t nx[1024], ndm[26];
    int rc = orc_dpg_maxwell_elem(no, &nori_edge[(size_t)12 * e], &nori_face[(size_t)6 * e],
                                  &xvert[(size_t)24 * e], eps[2 * e], eps[2 * e + 1],
                                  imp_mask ? imp_mask[e] : 0, prm, zal, zbl);
    if (rc > 0) rc = orc_stc_fwd_z(ni, nb, zal, nR, zbl, aii, bi, as, bs);
    if (rc == 0) {
      int nc = orc_celem_compress_z(no, &bcflag[(size_t)26 * e], aii, bi, NULL, nx, zb, za, ndm);
      if (zastif) memcpy(&zastif[2 * elem_nnz[e]], za, sizeof(double) * 2 * (size_t)nc * nc);
      if (zbload) memcpy(&zbload[2 * lcon_off[e]], zb, sizeof(double) * 2 * nc);
      if (aschur) memcpy(&aschur[2 * schur_off[e]], as, sizeof(double) * 2 * (size_t)nb * ni);
      if (bschur) memcpy(&bschur[2 * bub_off[e]], bs, sizeof(double) * 2 * nb);
    } else {
#ifdef _OPENMP
#pragma omp critical
#endif
      if (!bad || e + 1 < bad) bad = e + 1;
    }
    free(zal); free(zbl); free(aii); free(bi); free(as); free(bs); free(za); free(zb);
  }
  return bad;
}
