/*
 * abi_client.c -- a plain C caller of the element pass, compiled by gcc
 * against include/hp3dg.h (no C++, no Python), the way a Fortran host's
 * ISO_C_BINDING interface binds the library.
 *
 *   abi_client layout
 *       prints "struct field offset size" for every field of the public
 *       structs (and "struct - sizeof -") so that a test can pin the layouts
 *       the other bindings (ctypes, the Fortran bind(C) types) assume.
 *   abi_client run <in> <out> [precision]
 *       <in>: int32 n_elem, int32 n_nodes_global, n_elem hp3dg_elem_desc,
 *             n_elem x 24 doubles of vertex coordinates, n_elem kappa.
 *       Fills hp3dg_opts field by field, calls hp3dg_batch_begin /
 *       hp3dg_batch_submit / hp3dg_batch_run / hp3dg_batch_sync /
 *       hp3dg_batch_download, then per element hp3dg_get_condensed and
 *       hp3dg_get_schur, and hp3dg_index_map, and writes to <out>:
 *       int64 nrdof, int64 lcon_total, int32 lcon[lcon_total], then per
 *       element int32 nrdofc, int32 nb, int32 ni, zbload[nrdofc],
 *       zastif[nrdofc^2], aschur[nb*ni], bschur[nb] (doubles).
 * Exit status 0 on success, 2 on a usage or file error, 3 on a library error
 * (its message on stderr).
 */
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hp3dg.h"

#define FIELD(S, F) printf(#S " " #F " %zu %zu\n", offsetof(S, F), sizeof(((S *)0)->F))
#define SIZE(S) printf(#S " - %zu -\n", sizeof(S))

static int layout(void) {
  FIELD(hp3dg_opts, precision);
  FIELD(hp3dg_opts, integration);
  FIELD(hp3dg_opts, isol);
  FIELD(hp3dg_opts, keep_elem);
  FIELD(hp3dg_opts, timing);
  FIELD(hp3dg_opts, device);
  FIELD(hp3dg_opts, ozaki_radix);
  FIELD(hp3dg_opts, ozaki_digits);
  FIELD(hp3dg_opts, stc_method);
  FIELD(hp3dg_opts, launch_mode);
  FIELD(hp3dg_opts, schur_fp64);
  FIELD(hp3dg_opts, download_chunks);
  FIELD(hp3dg_opts, fault_inject);
  FIELD(hp3dg_opts, tune);
  FIELD(hp3dg_opts, reserved);
  SIZE(hp3dg_opts);
  FIELD(hp3dg_elem_desc, etype);
  FIELD(hp3dg_elem_desc, mdle);
  FIELD(hp3dg_elem_desc, norder);
  FIELD(hp3dg_elem_desc, nori_edge);
  FIELD(hp3dg_elem_desc, nori_face);
  FIELD(hp3dg_elem_desc, nodes);
  FIELD(hp3dg_elem_desc, bcflag);
  SIZE(hp3dg_elem_desc);
  FIELD(hp3dg_constraints, n);
  FIELD(hp3dg_constraints, iel);
  FIELD(hp3dg_constraints, node_off);
  FIELD(hp3dg_constraints, nodm);
  FIELD(hp3dg_constraints, ndof);
  FIELD(hp3dg_constraints, bcflag);
  FIELD(hp3dg_constraints, coef_off);
  FIELD(hp3dg_constraints, coef_k);
  FIELD(hp3dg_constraints, coef_l);
  FIELD(hp3dg_constraints, coef_v);
  FIELD(hp3dg_constraints, zdofd);
  SIZE(hp3dg_constraints);
  FIELD(hp3dg_dpg_opts, omega);
  FIELD(hp3dg_dpg_opts, mu);
  FIELD(hp3dg_dpg_opts, epsilon);
  FIELD(hp3dg_dpg_opts, gamma);
  FIELD(hp3dg_dpg_opts, alpha);
  FIELD(hp3dg_dpg_opts, ibcflag);
  FIELD(hp3dg_dpg_opts, nord_add);
  FIELD(hp3dg_dpg_opts, isol);
  FIELD(hp3dg_dpg_opts, icomp);
  FIELD(hp3dg_dpg_opts, device);
  FIELD(hp3dg_dpg_opts, timing);
  FIELD(hp3dg_dpg_opts, keep_elem);
  FIELD(hp3dg_dpg_opts, precision);
  FIELD(hp3dg_dpg_opts, reserved);
  SIZE(hp3dg_dpg_opts);
  return 0;
}

static int fail(const char *what, int rc) {
  fprintf(stderr, "%s: %d (%s)\n", what, rc, hp3dg_strerror(rc));
  return 3;
}

static int run(const char *in, const char *out, int precision) {
  FILE *f = fopen(in, "rb");
  if (!f) return 2;
  int32_t hdr[2];
  if (fread(hdr, sizeof(int32_t), 2, f) != 2) return 2;
  const int32_t nel = hdr[0], nnodes = hdr[1];
  hp3dg_elem_desc *desc = (hp3dg_elem_desc *)calloc((size_t)nel, sizeof(hp3dg_elem_desc));
  double *xvert = (double *)calloc((size_t)nel * 24, sizeof(double));
  double *kappa = (double *)calloc((size_t)nel, sizeof(double));
  if (!desc || !xvert || !kappa) return 2;
  if (fread(desc, sizeof(hp3dg_elem_desc), (size_t)nel, f) != (size_t)nel ||
      fread(xvert, sizeof(double), (size_t)nel * 24, f) != (size_t)nel * 24 ||
      fread(kappa, sizeof(double), (size_t)nel, f) != (size_t)nel)
    return 2;
  fclose(f);

  hp3dg_opts o;
  memset(&o, 0, sizeof o);
  o.precision = precision;
  o.integration = 1;
  o.isol = 10;
  o.keep_elem = 0;
  o.timing = 0;
  o.device = 0;
  o.ozaki_radix = 0;
  o.ozaki_digits = 0;
  o.stc_method = 0;
  o.launch_mode = 0;
  o.schur_fp64 = 0;
  o.download_chunks = 1;
  o.fault_inject = 0;
  hp3dg_ctx *ctx = NULL;
  int rc = hp3dg_batch_begin(&o, &ctx);
  if (rc) return fail("hp3dg_batch_begin", rc);
  if ((rc = hp3dg_batch_submit(ctx, nel, desc, xvert, kappa, NULL, nnodes)))
    return fail("hp3dg_batch_submit", rc);
  if ((rc = hp3dg_batch_run(ctx))) return fail("hp3dg_batch_run", rc);
  if ((rc = hp3dg_batch_sync(ctx))) return fail("hp3dg_batch_sync", rc);
  if ((rc = hp3dg_batch_download(ctx))) return fail("hp3dg_batch_download", rc);

  int64_t nnz = 0, lcon_total = 0, schur_total = 0, bub_total = 0, nrdof = 0;
  if ((rc = hp3dg_output_sizes(ctx, &nnz, &lcon_total, &schur_total, &bub_total)))
    return fail("hp3dg_output_sizes", rc);
  int32_t *lcon = (int32_t *)calloc((size_t)lcon_total + 1, sizeof(int32_t));
  if (!lcon) return 2;
  if ((rc = hp3dg_index_map(ctx, NULL, NULL, NULL, lcon, &nrdof)))
    return fail("hp3dg_index_map", rc);

  FILE *g = fopen(out, "wb");
  if (!g) return 2;
  fwrite(&nrdof, sizeof nrdof, 1, g);
  fwrite(&lcon_total, sizeof lcon_total, 1, g);
  fwrite(lcon, sizeof(int32_t), (size_t)lcon_total, g);
  for (int32_t e = 0; e < nel; ++e) {
    int32_t nrdofc = 0, nb = 0, ni = 0;
    /* sizes first (NULL buffers), then the data */
    if ((rc = hp3dg_get_condensed(ctx, e, NULL, NULL, &nrdofc)))
      return fail("hp3dg_get_condensed (size)", rc);
    if ((rc = hp3dg_get_schur(ctx, e, NULL, NULL, &nb, &ni)))
      return fail("hp3dg_get_schur (size)", rc);
    double *zb = (double *)calloc((size_t)nrdofc + 1, sizeof(double));
    double *zs = (double *)calloc((size_t)nrdofc * nrdofc + 1, sizeof(double));
    double *as = (double *)calloc((size_t)nb * ni + 1, sizeof(double));
    double *bs = (double *)calloc((size_t)nb + 1, sizeof(double));
    if (!zb || !zs || !as || !bs) return 2;
    if ((rc = hp3dg_get_condensed(ctx, e, zb, zs, &nrdofc))) return fail("hp3dg_get_condensed", rc);
    if ((rc = hp3dg_get_schur(ctx, e, as, bs, &nb, &ni))) return fail("hp3dg_get_schur", rc);
    fwrite(&nrdofc, sizeof nrdofc, 1, g);
    fwrite(&nb, sizeof nb, 1, g);
    fwrite(&ni, sizeof ni, 1, g);
    fwrite(zb, sizeof(double), (size_t)nrdofc, g);
    fwrite(zs, sizeof(double), (size_t)nrdofc * nrdofc, g);
    fwrite(as, sizeof(double), (size_t)nb * ni, g);
    fwrite(bs, sizeof(double), (size_t)nb, g);
    free(zb); free(zs); free(as); free(bs);
  }
  fclose(g);
  hp3dg_batch_end(ctx);
  free(lcon); free(desc); free(xvert); free(kappa);
  return 0;
}

int main(int argc, char **argv) {
  if (argc >= 2 && strcmp(argv[1], "layout") == 0) return layout();
  if (argc >= 4 && strcmp(argv[1], "run") == 0)
    return run(argv[2], argv[3], argc >= 5 ? atoi(argv[4]) : HP3DG_FP64);
  fprintf(stderr, "usage: abi_client layout | run <in> <out> [precision]\n");
  return 2;
}
