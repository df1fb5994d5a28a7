/*
 * hp3d_oracle_int.h -- helpers shared between the oracle's source files.
 * TEST INFRASTRUCTURE ONLY (see hp3d_oracle.h).
 */
#ifndef HP3D_ORACLE_INT_H
#define HP3D_ORACLE_INT_H

/* decod (encod_decod.F90): digits of a MODORDER code */
void orc_i_decod(int nick, int mod, int n, int *arr);
/* PolyLegendre (Polynomials.F90:34-80) */
void orc_i_poly_legendre(double x, double t, int nord, double *p);
/* PolyILegendre (Polynomials.F90:113-160) */
void orc_i_poly_ilegendre(double x, double t, int nord, int idec, double *L, double *P, double *R);
/* HomILegendre (Polynomials.F90:494-530) */
void orc_i_hom_ilegendre(const double *S, const double DS[3][2], int nord, int idec, double *homL,
                         double dhomL[][3]);
/* BlendProjectHexaE / BlendProjectHexaF / OrientQuad tables (see hp3d_oracle.c) */
const int (*orc_i_hexa_e(void))[5];
const int (*orc_i_hexa_f(void))[4];
const int (*orc_i_orq(void))[6];

#endif
