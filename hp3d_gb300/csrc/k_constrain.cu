// k_constrain.cu -- constrained approximation of the condensed element
// systems (hanging nodes): celem_systemI.F90:541-760 (ZBMOD = C^T b,
// ZAMOD = C^T A C with logic's coefficients), then the Dirichlet lift and the
// compression over the modified element nodes (celem_systemI.F90:800-845).
//
// A batch with constrained elements compresses every element first into a
// work layout (constrained elements: all ni interface dof, no lift); this
// kernel then writes the final outputs: a copy for the other elements, the
// transform for the constrained ones.  The coefficients arrive as gather
// lists per modified dof l: (k, c) pairs in the reference's loop order, so
// both passes accumulate in the same order as the two loops of
// celem_systemI.
#include "hp3dg_kernels.h"

namespace hp3dg {

namespace {

constexpr int CS_THREADS = 256;

__global__ void __launch_bounds__(CS_THREADS) k_constrain(ConstrainArgs a) {
  const int e = blockIdx.x;
  const int tid = threadIdx.x;
  const int j = a.cidx[e];
  const int64_t lo = a.lcon_off[e];
  const int nc = (int)(a.lcon_off[e + 1] - lo);
  double* Z = a.zastif + a.elem_nnz[e];
  double* zb = a.zbload + lo;
  const double* Sw = a.zwork + a.welem_nnz[e];
  const double* bw = a.bwork + a.wlcon_off[e];
  if (j < 0) {  // unconstrained: the work block is the final block
    for (int64_t x = tid; x < (int64_t)nc * nc; x += CS_THREADS) Z[x] = Sw[x];
    for (int x = tid; x < nc; x += CS_THREADS) zb[x] = bw[x];
    return;
  }
  const int ni = (int)(a.wlcon_off[e + 1] - a.wlcon_off[e]);  // S is ni x ni, row-major
  const int nmod = a.nmod[j];
  const int* gp = a.gptr + a.gptr_off[j];  // nmod + 1 row pointers
  const int* gk = a.gk;
  const double* gv = a.gv;
  double* aux = a.aux + a.aux_off[j];      // nmod x ni, row-major
  // rows: AUX(l, :) = sum_{(k,c) in G(l)} c S(k, :)
  for (int64_t x = tid; x < (int64_t)nmod * ni; x += CS_THREADS) {
    const int l = (int)(x / ni), k2 = (int)(x % ni);
    double s = 0.0;
    for (int q = gp[l]; q < gp[l + 1]; ++q) s += Sw[(int64_t)gk[q] * ni + k2] * gv[q];
    aux[x] = s;
  }
  __syncthreads();
  const int* nx = a.cnextract + lo;
  const uint8_t* dir = a.mdir + a.mdof_off[j];
  const double* zd = a.mzd ? a.mzd + a.mdof_off[j] : nullptr;
  // columns: ZAMOD(l1, l2) = sum_{(k,c) in G(l2)} c AUX(l1, k), compressed
  for (int64_t x = tid; x < (int64_t)nc * nc; x += CS_THREADS) {
    const int l1 = nx[x / nc], l2 = nx[x % nc];
    double s = 0.0;
    for (int q = gp[l2]; q < gp[l2 + 1]; ++q) s += aux[(int64_t)l1 * ni + gk[q]] * gv[q];
    Z[x] = s;
  }
  // load: ZBMOD(l) = sum c b(k), then the lift by the known modified dof
  for (int r = tid; r < nc; r += CS_THREADS) {
    const int l1 = nx[r];
    double v = 0.0;
    for (int q = gp[l1]; q < gp[l1 + 1]; ++q) v += bw[gk[q]] * gv[q];
    if (zd)
      for (int l2 = 0; l2 < nmod; ++l2) {
        if (!dir[l2]) continue;
        double s = 0.0;
        for (int q = gp[l2]; q < gp[l2 + 1]; ++q) s += aux[(int64_t)l1 * ni + gk[q]] * gv[q];
        v -= s * zd[l2];
      }
    zb[r] = v;
  }
}

}  // namespace

void launch_constrain(int nel, const ConstrainArgs& a, cudaStream_t st) {
  if (nel <= 0) return;
  k_constrain<<<nel, CS_THREADS, 0, st>>>(a);
}

}  // namespace hp3dg
