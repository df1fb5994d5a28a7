// api_dpg.cu -- C-ABI host runtime of the ultraweak DPG Maxwell pass
// (include/hp3dg.h, hp3dg_dpg_*).
//
// The host side does what elem.F90 / celem_systemI.F90 do around the
// element routine: the sizes of the spaces (elem.F90:78-103), the DPG
// quadrature rules (set_3D_int_DPG, set_2D_int_DPG; the impedance penalty's
// set_2D_int), the extraction vector of the EHtrc unknowns with their
// Dirichlet components (celem_systemI.F90:353-420) and the element's trace
// orientation map; every number of the element pass is computed on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/hp3dg.h"
#include "hp3dg_dpg.cuh"
#include "hp3dg_kernels.h"

using namespace hp3dg;

struct hp3dg_dpg_ctx {
  hp3dg_dpg_opts opts{};
  int device = 0;
  cudaStream_t stream = nullptr;
  bool submitted = false, ran = false, downloaded = false, tables = false;
  int nel = 0, nnodes = 0;
  DpgDims d{};
  DpgPhys ph{};
  std::vector<int64_t> lcon_off, elem_nnz, schur_off, bub_off;
  int32_t last_bad = -1;
  int64_t launches = 0;    // kernels launched by the last run
  std::vector<hp3dg_elem_desc> desc_prev;  // descriptors of the current batch
  std::vector<void*> dev;  // every device allocation of the batch
  double *d_xiV = nullptr, *d_wV = nullptr, *d_xiF = nullptr, *d_wF = nullptr, *d_xiI = nullptr,
         *d_wI = nullptr;
  DpgTables t{};
  DpgWork w{};
  double *d_xvert = nullptr, *d_eps = nullptr;
  int *d_imp = nullptr, *d_nextract = nullptr, *d_nodes = nullptr, *d_ndofm = nullptr;
  uint32_t* d_perm = nullptr;
  int64_t *d_lcon_off = nullptr, *d_elem_nnz = nullptr, *d_schur_off = nullptr,
          *d_bub_off = nullptr;
  double *d_zastif = nullptr, *d_zbload = nullptr, *d_aschur = nullptr, *d_bschur = nullptr,
         *d_zkeep = nullptr;
  int *d_first = nullptr, *d_cnt = nullptr, *d_nfirst = nullptr, *d_lcon = nullptr;
  int64_t *d_scan = nullptr, *d_blk = nullptr, *d_total = nullptr;
  int* d_flags = nullptr;
  double *h_zastif = nullptr, *h_zbload = nullptr, *h_aschur = nullptr, *h_bschur = nullptr,
         *h_zkeep = nullptr;
  int *h_lcon = nullptr, *h_nfirst = nullptr;
  int64_t h_nrdof = 0;
  cudaEvent_t ev[5] = {};
  float times[5] = {0, 0, 0, 0, 0};
};

namespace {

#define CK(x)                                      \
  do {                                             \
    if ((x) != cudaSuccess) return HP3DG_ERR_CUDA; \
  } while (0)

template <class T>
T* dalloc(hp3dg_dpg_ctx* c, size_t n, int* err) {
  void* p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
    *err = HP3DG_ERR_ALLOC;
    return nullptr;
  }
  c->dev.push_back(p);
  return (T*)p;
}

void free_batch(hp3dg_dpg_ctx* c) {
  for (void* p : c->dev) cudaFree(p);
  c->dev.clear();
  void* h[] = {c->h_zastif, c->h_zbload, c->h_aschur, c->h_bschur, c->h_zkeep, c->h_lcon,
               c->h_nfirst};
  for (void* p : h)
    if (p) cudaFreeHost(p);
  c->h_zastif = c->h_zbload = c->h_aschur = c->h_bschur = c->h_zkeep = nullptr;
  c->h_lcon = c->h_nfirst = nullptr;
  c->submitted = c->ran = c->downloaded = c->tables = false;
}

// brick faces (element_data.F90: BRICK_COORD, BRICK_FACE_TO_VERT, Nsign_param)
const double BRICK_COORD[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
const int BRICK_F2V[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                             {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}};
const double BRICK_NSIGN[6] = {-1, 1, 1, 1, -1, -1};
constexpr int MAXPP = MAXP + 1;  // MAXP + MAXNORD_ADD (parametersDPG.F90)

// tensor rule of n points per axis on a face (set_2Dint_aux, quad branch)
void face_points(const DpgDims& d, int n, std::vector<double>& xi, std::vector<double>& w) {
  double x[16], wx[16];
  gauss_rule01(n, x, wx);
  for (int f = 0; f < 6; ++f)
    for (int l2 = 0; l2 < n; ++l2)
      for (int l1 = 0; l1 < n; ++l1) {
        for (int c = 0; c < 3; ++c)
          xi.push_back(BRICK_COORD[BRICK_F2V[f][0]][c] + x[l1] * d.dxidt[f][c][0] +
                       x[l2] * d.dxidt[f][c][1]);
        w.push_back(wx[l1] * wx[l2]);
      }
}

}  // namespace

extern "C" {

int hp3dg_dpg_begin(const hp3dg_dpg_opts* opts, hp3dg_dpg_ctx** out) {
  if (!opts || !out) return HP3DG_ERR_ARG;
  if (opts->nord_add < 1 || opts->ibcflag < 0 || opts->ibcflag > 2 || opts->ibcflag == 1 ||
      opts->isol < 0 || opts->isol > 2 || opts->icomp < 1 || opts->icomp > 3 ||
      !(opts->omega > 0.0) || !(opts->mu > 0.0) ||
      (opts->precision != HP3DG_FP64 && opts->precision != HP3DG_MIXED))
    return HP3DG_ERR_ARG;
  auto* c = new hp3dg_dpg_ctx;
  c->opts = *opts;
  c->device = opts->device;
  if (cudaSetDevice(c->device) != cudaSuccess) { delete c; return HP3DG_ERR_CUDA; }
  if (opts->precision == HP3DG_MIXED) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess) { delete c; return HP3DG_ERR_CUDA; }
    if (prop.major != 10) { delete c; return HP3DG_ERR_UNSUPPORTED; }  // tcgen05 needs sm_10x
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return HP3DG_ERR_CUDA;
  }
  for (auto& e : c->ev) cudaEventCreate(&e);
  c->ph = DpgPhys{opts->omega, opts->mu, opts->epsilon, opts->gamma, opts->alpha,
                  opts->ibcflag, opts->isol, opts->icomp};
  *out = c;
  return HP3DG_OK;
}

int hp3dg_dpg_submit(hp3dg_dpg_ctx* c, int32_t nel, const hp3dg_elem_desc* desc,
                     const double* xvert, const double* eps, int32_t nnodes) {
  if (!c || nel < 0 || (nel > 0 && (!desc || !xvert || !eps)) || nnodes < 0) return HP3DG_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  // the same mesh again (new vertices or permittivities): keep the device
  // buffers, the digit tables and the pinned results; upload the two inputs
  if (c->submitted && nel > 0 && nel == c->nel && nnodes == c->nnodes &&
      c->desc_prev.size() == (size_t)nel &&
      memcmp(c->desc_prev.data(), desc, sizeof(hp3dg_elem_desc) * (size_t)nel) == 0) {
    CK(cudaMemcpyAsync(c->d_xvert, xvert, sizeof(double) * 24 * (size_t)nel,
                       cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_eps, eps, sizeof(double) * 2 * (size_t)nel, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->ran = c->downloaded = false;
    return HP3DG_OK;
  }
  free_batch(c);
  c->desc_prev.clear();
  c->nel = nel;
  c->nnodes = nnodes;
  if (nel == 0) { c->submitted = true; return HP3DG_OK; }
  // one isotropic order for the batch (elem.F90 sizes)
  const int p = desc[0].norder[0];
  if (p < 1 || p > DPG_MAXP || p + c->opts.nord_add > MAXP) return HP3DG_ERR_BAD_ORDER;
  for (int e = 0; e < nel; ++e) {
    const hp3dg_elem_desc& d = desc[e];
    if (d.etype != HP3DG_HEXA) return HP3DG_ERR_UNSUPPORTED;
    for (int i = 0; i < 12; ++i)
      if (d.norder[i] != p) return HP3DG_ERR_BAD_ORDER;
    for (int i = 12; i < 18; ++i)
      if (d.norder[i] != 11 * p) return HP3DG_ERR_BAD_ORDER;
    if (d.norder[18] != 111 * p) return HP3DG_ERR_BAD_ORDER;
    for (int i = 0; i < 26; ++i)
      if (d.nodes[i] < 0 || d.nodes[i] >= nnodes) return HP3DG_ERR_ARG;
    for (int i = 0; i < 12; ++i)
      if (d.nori_edge[i] < 0 || d.nori_edge[i] > 1) return HP3DG_ERR_ARG;
    for (int i = 0; i < 6; ++i)
      if (d.nori_face[i] < 0 || d.nori_face[i] > 7) return HP3DG_ERR_ARG;
  }
  DpgDims& d = c->d;
  d.p = p;
  d.q = p + c->opts.nord_add;
  d.nEE = dpg_nEE(d.q);
  d.nEi = dpg_nEi(p);
  d.nQ = dpg_nQ(p);
  d.nr = 2 * d.nEi + 6 * d.nQ;
  for (int f = 0; f < 6; ++f) {
    for (int cc = 0; cc < 3; ++cc) {
      const double* x1 = BRICK_COORD[BRICK_F2V[f][0]];
      d.dxidt[f][cc][0] = BRICK_COORD[BRICK_F2V[f][1]][cc] - x1[cc];
      d.dxidt[f][cc][1] = BRICK_COORD[BRICK_F2V[f][3]][cc] - x1[cc];
    }
    d.nsign[f] = BRICK_NSIGN[f];
  }
  // quadrature: volume and faces with INTEGRATION = NORD_ADD (MAXPP cap),
  // impedance faces with INTEGRATION = 0 (MAXP cap)
  const int nv1 = std::min(p + c->opts.nord_add, MAXPP) + 1;
  const int ni1 = std::min(p, MAXP) + 1;
  std::vector<double> xiV, wV, xiF, wF, xiI, wI;
  {
    double x[16], wx[16];
    gauss_rule01(nv1, x, wx);
    for (int l3 = 0; l3 < nv1; ++l3)
      for (int l2 = 0; l2 < nv1; ++l2)
        for (int l1 = 0; l1 < nv1; ++l1) {
          xiV.push_back(x[l1]); xiV.push_back(x[l2]); xiV.push_back(x[l3]);
          wV.push_back(wx[l1] * wx[l2] * wx[l3]);
        }
  }
  face_points(d, nv1, xiF, wF);
  face_points(d, ni1, xiI, wI);
  d.nv = (int)wV.size();
  d.nfp = nv1 * nv1;
  d.nip = ni1 * ni1;
  // per element: trace orientation map, extraction, impedance faces, offsets
  const int ni = 2 * d.nEi, nq = 6 * d.nQ;
  std::vector<uint32_t> perm((size_t)nel * d.nEi);
  std::vector<int> nextract, imp(nel), ndofm((size_t)nel * 26), nodes((size_t)nel * 26);
  std::vector<double> xv((size_t)nel * 24), ep(2 * (size_t)nel);
  c->lcon_off.assign(nel + 1, 0);
  c->elem_nnz.assign(nel + 1, 0);
  c->schur_off.assign(nel + 1, 0);
  c->bub_off.assign(nel + 1, 0);
  int nsh[26], first[26];
  for (int i = 0; i < 26; ++i) nsh[i] = i < 8 ? 0 : (i < 20 ? p : 2 * p * (p - 1));
  for (int i = 0, f = 0; i < 26; ++i) { first[i] = f; f += 2 * nsh[i]; }
  for (int e = 0; e < nel; ++e) {
    const hp3dg_elem_desc& de = desc[e];
    dpg_trace_perm(p, de.nori_edge, de.nori_face, &perm[(size_t)e * d.nEi]);
    int k = 0;
    for (int i = 25; i >= 0; --i) {
      int cnt = 0;
      for (int j = 0; j < nsh[i]; ++j)
        for (int comp = 0; comp < 2; ++comp)
          if (!((de.bcflag[i] >> comp) & 1)) {
            nextract.push_back(first[i] + 2 * j + comp);
            ++cnt;
          }
      ndofm[(size_t)e * 26 + i] = cnt;
      k += cnt;
    }
    imp[e] = 0;
    for (int f = 0; f < 6; ++f)
      if (de.bcflag[20 + f] & 4) imp[e] |= 1 << f;
    for (int i = 0; i < 26; ++i) nodes[(size_t)e * 26 + i] = de.nodes[i];
    for (int i = 0; i < 24; ++i) xv[(size_t)e * 24 + i] = xvert[(size_t)e * 24 + i];
    ep[2 * e] = eps[2 * e];
    ep[2 * e + 1] = eps[2 * e + 1];
    c->lcon_off[e + 1] = c->lcon_off[e] + k;
    c->elem_nnz[e + 1] = c->elem_nnz[e] + (int64_t)k * k;
    c->schur_off[e + 1] = c->schur_off[e] + (int64_t)nq * ni;
    c->bub_off[e + 1] = c->bub_off[e] + nq;
  }
  int err = 0;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (!err && cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
      err = HP3DG_ERR_CUDA;
  };
  c->d_xiV = dalloc<double>(c, xiV.size(), &err);
  c->d_wV = dalloc<double>(c, wV.size(), &err);
  c->d_xiF = dalloc<double>(c, xiF.size(), &err);
  c->d_wF = dalloc<double>(c, wF.size(), &err);
  c->d_xiI = dalloc<double>(c, xiI.size(), &err);
  c->d_wI = dalloc<double>(c, wI.size(), &err);
  const size_t t3 = 3 * (size_t)d.nEE;
  c->t.vs = dalloc<double>(c, d.nv * t3, &err);
  c->t.vc = dalloc<double>(c, d.nv * t3, &err);
  c->t.vq = dalloc<double>(c, (size_t)d.nv * d.nQ, &err);
  c->t.fs = dalloc<double>(c, 6 * d.nfp * t3, &err);
  c->t.fscratch = dalloc<double>(c, 6 * d.nfp * t3, &err);
  c->t.ft = dalloc<double>(c, 6 * (size_t)d.nfp * 3 * d.nEi, &err);
  c->t.it = dalloc<double>(c, 6 * (size_t)d.nip * 3 * d.nEi, &err);
  DpgWork& w = c->w;
  const size_t ne = nel, nt = 2 * (size_t)d.nEE, n1 = d.nr + 1;
  w.gV = dalloc<double>(c, ne * d.nv * DPG_GV, &err);
  w.gF = dalloc<double>(c, ne * 6 * d.nfp * 9, &err);
  w.gI = dalloc<double>(c, ne * 6 * d.nip * 36, &err);
  w.MFF = dalloc<double>(c, ne * d.nEE * d.nEE, &err);
  w.MCC = dalloc<double>(c, ne * d.nEE * d.nEE, &err);
  w.MFC = dalloc<double>(c, (size_t)d.nEE * d.nEE, &err);
  w.P = dalloc<double>(c, ne * d.nEE * 3 * d.nQ, &err);
  w.R = dalloc<double>(c, ne * d.nEE * 3 * d.nQ, &err);
  w.T = dalloc<double>(c, ne * d.nEE * d.nEi, &err);
  w.load = dalloc<double>(c, ne * 2 * d.nEE, &err);
  w.G = w.S = w.Z = w.M = w.W = w.Y = nullptr;
  c->d_zkeep = c->opts.keep_elem ? dalloc<double>(c, ne * 2 * n1 * n1, &err) : nullptr;
  w.tc = c->opts.precision == HP3DG_MIXED;
  if (w.tc) {
    // augmented matrix (nt + n1)^2, inverse diagonal blocks, ASchur workspace
    const size_t na = nt + n1, nq = 6 * (size_t)d.nQ;
    w.M = dalloc<double>(c, ne * 2 * na * na, &err);
    w.W = dalloc<double>(c, ne * 2 * 4096 * (size_t)dpg_aug_wslots((int)nt, (int)nq), &err);
    w.Y = dalloc<double>(c, ne * 2 * nq * (n1 - nq), &err);
    w.tb.a = dalloc<uint8_t>(c, ne * dpg_tc_a_bytes((int)na), &err);
    w.tb.b = dalloc<uint8_t>(c, ne * dpg_tc_b_bytes((int)na), &err);
    w.tb.ea = dalloc<int>(c, ne * dpg_tc_ex_slots((int)na), &err);
    w.tb.eb = dalloc<int>(c, ne * dpg_tc_ex_slots((int)na), &err);
    if (ozaki_plan(d.nv, d.nEE, 7, 7, &w.gplan)) err = HP3DG_ERR_ARG;
    for (int which = 0; which < 2 && !err; ++which) {
      w.gmdig[which] = (uint16_t*)dalloc<uint8_t>(c, ozaki_m_bytes(w.gplan), &err);
      w.gmscale[which] = dalloc<double>(c, w.gplan.ncols, &err);
      w.gddig[which] = (uint16_t*)dalloc<uint8_t>(c, ozaki_d_bytes(w.gplan, (int)ne), &err);
      w.gdscale[which] = dalloc<double>(c, (ne + 127) / 128 * 128, &err);
      w.gD[which] = dalloc<double>(c, ne * 6 * d.nv, &err);
    }
    const int kPR = 3 * d.nv, kT = 9 * 6 * d.nfp;
    if (ozaki_plan_dense(kPR, d.nEE * d.nQ, 7, 7, &w.bplan[0]) ||
        ozaki_plan_dense(kPR, d.nEE * d.nQ, 7, 7, &w.bplan[1]) ||
        ozaki_plan_dense(kT, d.nEE * d.nEi, 7, 7, &w.bplan[2]))
      err = HP3DG_ERR_ARG;
    size_t mdense = 0, dbytes = 0;
    for (int which = 0; which < 3 && !err; ++which) {
      w.bmdig[which] = (uint16_t*)dalloc<uint8_t>(c, ozaki_m_bytes(w.bplan[which]), &err);
      w.bmscale[which] = dalloc<double>(c, w.bplan[which].ncols, &err);
      mdense = std::max(mdense, (size_t)w.bplan[which].kreal * w.bplan[which].nreal);
      dbytes = std::max(dbytes, ozaki_d_bytes(w.bplan[which], which < 2 ? 3 * (int)ne : (int)ne));
    }
    w.bddig = (uint16_t*)dalloc<uint8_t>(c, dbytes, &err);
    w.bdscale = dalloc<double>(c, (3 * ne + 127) / 128 * 128, &err);
    w.bDP = dalloc<double>(c, 3 * ne * kPR, &err);
    w.bDR = dalloc<double>(c, 3 * ne * kPR, &err);
    w.bMd = dalloc<double>(c, mdense, &err);
  } else {
    w.G = dalloc<double>(c, ne * 2 * nt * nt, &err);
    w.S = dalloc<double>(c, ne * 2 * nt * n1, &err);
    w.Z = dalloc<double>(c, ne * 2 * n1 * n1, &err);
  }
  c->d_xvert = dalloc<double>(c, xv.size(), &err);
  c->d_eps = dalloc<double>(c, ep.size(), &err);
  c->d_imp = dalloc<int>(c, ne, &err);
  c->d_perm = dalloc<uint32_t>(c, perm.size(), &err);
  c->d_nextract = dalloc<int>(c, nextract.size(), &err);
  c->d_nodes = dalloc<int>(c, nodes.size(), &err);
  c->d_ndofm = dalloc<int>(c, ndofm.size(), &err);
  c->d_lcon_off = dalloc<int64_t>(c, ne + 1, &err);
  c->d_elem_nnz = dalloc<int64_t>(c, ne + 1, &err);
  c->d_schur_off = dalloc<int64_t>(c, ne + 1, &err);
  c->d_bub_off = dalloc<int64_t>(c, ne + 1, &err);
  c->d_zastif = dalloc<double>(c, 2 * (size_t)c->elem_nnz[nel], &err);
  c->d_zbload = dalloc<double>(c, 2 * (size_t)c->lcon_off[nel], &err);
  c->d_aschur = dalloc<double>(c, 2 * (size_t)c->schur_off[nel], &err);
  c->d_bschur = dalloc<double>(c, 2 * (size_t)c->bub_off[nel], &err);
  const size_t ns = ne * 26;
  c->d_first = dalloc<int>(c, nnodes, &err);
  c->d_cnt = dalloc<int>(c, ns, &err);
  c->d_scan = dalloc<int64_t>(c, ns, &err);
  c->d_blk = dalloc<int64_t>(c, (ns + 1023) / 1024 + 1, &err);
  c->d_total = dalloc<int64_t>(c, 1, &err);
  c->d_nfirst = dalloc<int>(c, nnodes, &err);
  c->d_lcon = dalloc<int>(c, c->lcon_off[nel], &err);
  c->d_flags = dalloc<int>(c, 4, &err);
  if (err) { free_batch(c); return err; }
  up(c->d_xiV, xiV.data(), xiV.size() * 8);
  up(c->d_wV, wV.data(), wV.size() * 8);
  up(c->d_xiF, xiF.data(), xiF.size() * 8);
  up(c->d_wF, wF.data(), wF.size() * 8);
  up(c->d_xiI, xiI.data(), xiI.size() * 8);
  up(c->d_wI, wI.data(), wI.size() * 8);
  up(c->d_xvert, xv.data(), xv.size() * 8);
  up(c->d_eps, ep.data(), ep.size() * 8);
  up(c->d_imp, imp.data(), imp.size() * 4);
  up(c->d_perm, perm.data(), perm.size() * 4);
  up(c->d_nextract, nextract.data(), nextract.size() * 4);
  up(c->d_nodes, nodes.data(), nodes.size() * 4);
  up(c->d_ndofm, ndofm.data(), ndofm.size() * 4);
  up(c->d_lcon_off, c->lcon_off.data(), (ne + 1) * 8);
  up(c->d_elem_nnz, c->elem_nnz.data(), (ne + 1) * 8);
  up(c->d_schur_off, c->schur_off.data(), (ne + 1) * 8);
  up(c->d_bub_off, c->bub_off.data(), (ne + 1) * 8);
  if (!err && cudaStreamSynchronize(c->stream) != cudaSuccess) err = HP3DG_ERR_CUDA;
  if (err) { free_batch(c); return err; }
  w.xiV = c->d_xiV; w.wV = c->d_wV; w.xiF = c->d_xiF; w.wF = c->d_wF;
  w.xiI = c->d_xiI; w.wI = c->d_wI;
  c->desc_prev.assign(desc, desc + nel);
  c->submitted = true;
  return HP3DG_OK;
}

int hp3dg_dpg_run(hp3dg_dpg_ctx* c) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  if (c->nel == 0) { c->ran = true; return HP3DG_OK; }
  if (!c->tables) {
    launch_dpg_tables(c->d, c->d_xiV, c->d_wV, c->d_xiF, c->d_xiI, c->t, c->w.MFC, st);
    if (c->w.tc && launch_dpg_gram_tables(c->d, c->t, c->w, st)) return HP3DG_ERR_CUDA;
    c->tables = true;
  }
  CK(cudaMemsetAsync(c->d_flags, 0x7f, 4 * sizeof(int), st));
  cudaEventRecord(c->ev[0], st);
  c->launches = 0;
  bool fail = false;
  auto stage = [&](int s) {
    const int k = launch_dpg_stage(s, c->nel, c->d, c->ph, c->t, c->w, c->d_xvert, c->d_eps,
                                   c->d_imp, c->d_perm, c->d_nextract, c->d_lcon_off,
                                   c->d_elem_nnz, c->d_schur_off, c->d_bub_off, c->d_zastif,
                                   c->d_zbload, c->d_aschur, c->d_bschur,
                                   c->w.tc ? c->d_zkeep : nullptr, c->d_flags, st);
    if (k < 0) fail = true;
    else c->launches += k;
  };
  stage(0);
  cudaEventRecord(c->ev[1], st);
  stage(1);
  if (c->d_zkeep && !c->w.tc) {
    const size_t n1 = c->d.nr + 1;
    CK(cudaMemcpyAsync(c->d_zkeep, c->w.Z, (size_t)c->nel * 2 * n1 * n1 * 8,
                       cudaMemcpyDeviceToDevice, st));
  }
  cudaEventRecord(c->ev[2], st);
  stage(2);
  cudaEventRecord(c->ev[3], st);
  launch_index_maps(c->nel, 26, c->nnodes, c->d_nodes, c->d_ndofm, c->d_lcon_off, c->d_first,
                    c->d_cnt, c->d_scan, c->d_blk, c->d_total, c->d_nfirst, c->d_lcon, st);
  c->launches += 7;
  cudaEventRecord(c->ev[4], st);
  if (fail) return HP3DG_ERR_CUDA;
  CK(cudaPeekAtLastError());
  c->ran = true;
  c->downloaded = false;
  return HP3DG_OK;
}

int hp3dg_dpg_sync(hp3dg_dpg_ctx* c) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->ran) return HP3DG_ERR_STATE;
  cudaSetDevice(c->device);
  CK(cudaStreamSynchronize(c->stream));
  if (c->nel == 0) return HP3DG_OK;
  int fl[4];
  CK(cudaMemcpy(fl, c->d_flags, sizeof(fl), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&c->times[i], c->ev[i], c->ev[i + 1]);
  cudaEventElapsedTime(&c->times[4], c->ev[0], c->ev[4]);
  const int NONE = 0x7f7f7f7f;
  c->last_bad = -1;
  // a timeout leaves the later stages reading unfinished data: reported first
  if (fl[0] != NONE) { c->last_bad = fl[0]; return HP3DG_ERR_NEG_JACOBIAN; }
  if (fl[2] != NONE) return HP3DG_ERR_TIMEOUT;  // a bounded wait of a tensor-core kernel gave up
  if (fl[1] != NONE) { c->last_bad = fl[1]; return HP3DG_ERR_NOT_SPD; }
  return HP3DG_OK;
}

int hp3dg_dpg_download(hp3dg_dpg_ctx* c) {
  int rc = hp3dg_dpg_sync(c);
  if (rc != HP3DG_OK) return rc;
  if (c->nel == 0) { c->downloaded = true; return HP3DG_OK; }
  const int nel = c->nel;
  auto hal = [](void** p, size_t bytes) {
    if (*p) return true;
    return cudaMallocHost(p, bytes ? bytes : 8) == cudaSuccess;
  };
  const size_t n1 = c->d.nr + 1;
  if (!hal((void**)&c->h_zastif, 16 * c->elem_nnz[nel]) ||
      !hal((void**)&c->h_zbload, 16 * c->lcon_off[nel]) ||
      !hal((void**)&c->h_aschur, 16 * c->schur_off[nel]) ||
      !hal((void**)&c->h_bschur, 16 * c->bub_off[nel]) ||
      !hal((void**)&c->h_lcon, 4 * c->lcon_off[nel]) ||
      !hal((void**)&c->h_nfirst, 4 * (size_t)c->nnodes) ||
      (c->d_zkeep && !hal((void**)&c->h_zkeep, 16 * n1 * n1 * nel)))
    return HP3DG_ERR_ALLOC;
  cudaStream_t st = c->stream;
  CK(cudaMemcpyAsync(c->h_zastif, c->d_zastif, 16 * c->elem_nnz[nel], cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_zbload, c->d_zbload, 16 * c->lcon_off[nel], cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_aschur, c->d_aschur, 16 * c->schur_off[nel], cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_bschur, c->d_bschur, 16 * c->bub_off[nel], cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_lcon, c->d_lcon, 4 * c->lcon_off[nel], cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_nfirst, c->d_nfirst, 4 * (size_t)c->nnodes, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&c->h_nrdof, c->d_total, 8, cudaMemcpyDeviceToHost, st));
  if (c->d_zkeep)
    CK(cudaMemcpyAsync(c->h_zkeep, c->d_zkeep, 16 * n1 * n1 * nel, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  c->downloaded = true;
  return HP3DG_OK;
}

int hp3dg_dpg_sizes(const hp3dg_dpg_ctx* c, int32_t* ntrial, int32_t* ni, int32_t* nb) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  if (ntrial) *ntrial = c->d.nr;
  if (ni) *ni = 2 * c->d.nEi;
  if (nb) *nb = 6 * c->d.nQ;
  return HP3DG_OK;
}

int hp3dg_dpg_get_elem(const hp3dg_dpg_ctx* c, int32_t iel, double* zaloc, int32_t ld,
                       double* zbloc) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->downloaded || !c->h_zkeep) return HP3DG_ERR_STATE;
  if (iel < 0 || iel >= c->nel) return HP3DG_ERR_ARG;
  const int n = c->d.nr;
  const size_t n1 = n + 1;
  if (zaloc && ld < n) return HP3DG_ERR_ARG;
  const double* z = c->h_zkeep + 2 * n1 * n1 * iel;
  for (int j = 0; j < n; ++j) {
    if (zaloc) std::memcpy(zaloc + 2 * (size_t)ld * j, z + 2 * n1 * j, 16 * (size_t)n);
  }
  if (zbloc) std::memcpy(zbloc, z + 2 * n1 * n, 16 * (size_t)n);
  return HP3DG_OK;
}

int hp3dg_dpg_get_condensed(const hp3dg_dpg_ctx* c, int32_t iel, double* zbload,
                            double* zastif, int32_t* nrdofc) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->downloaded) return HP3DG_ERR_STATE;
  if (iel < 0 || iel >= c->nel) return HP3DG_ERR_ARG;
  const int64_t lo = c->lcon_off[iel], nc = c->lcon_off[iel + 1] - lo;
  if (nrdofc) *nrdofc = (int32_t)nc;
  if (zbload) std::memcpy(zbload, c->h_zbload + 2 * lo, 16 * nc);
  if (zastif) std::memcpy(zastif, c->h_zastif + 2 * c->elem_nnz[iel], 16 * nc * nc);
  return HP3DG_OK;
}

int hp3dg_dpg_get_schur(const hp3dg_dpg_ctx* c, int32_t iel, double* aschur, double* bschur,
                        int32_t* nb, int32_t* ni) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->downloaded) return HP3DG_ERR_STATE;
  if (iel < 0 || iel >= c->nel) return HP3DG_ERR_ARG;
  const int b = 6 * c->d.nQ, i = 2 * c->d.nEi;
  if (nb) *nb = b;
  if (ni) *ni = i;
  if (aschur) std::memcpy(aschur, c->h_aschur + 2 * c->schur_off[iel], 16 * (size_t)b * i);
  if (bschur) std::memcpy(bschur, c->h_bschur + 2 * c->bub_off[iel], 16 * (size_t)b);
  return HP3DG_OK;
}

int hp3dg_dpg_index_map(const hp3dg_dpg_ctx* c, int32_t* nfirst, int64_t* elem_nnz,
                        int64_t* lcon_off, int32_t* lcon, int64_t* nrdof) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->downloaded) return HP3DG_ERR_STATE;
  const int nel = c->nel;
  if (nfirst) std::memcpy(nfirst, c->h_nfirst, 4 * (size_t)c->nnodes);
  if (elem_nnz) std::memcpy(elem_nnz, c->elem_nnz.data(), 8 * (size_t)(nel + 1));
  if (lcon_off) std::memcpy(lcon_off, c->lcon_off.data(), 8 * (size_t)(nel + 1));
  if (lcon) std::memcpy(lcon, c->h_lcon, 4 * (size_t)c->lcon_off[nel]);
  if (nrdof) *nrdof = c->h_nrdof;
  return HP3DG_OK;
}

int hp3dg_dpg_phase_times(const hp3dg_dpg_ctx* c, float* ms, int32_t n) {
  if (!c || !ms) return HP3DG_ERR_ARG;
  for (int i = 0; i < n && i < 5; ++i) ms[i] = c->times[i];
  return HP3DG_OK;
}

int32_t hp3dg_dpg_last_bad_element(const hp3dg_dpg_ctx* c) { return c ? c->last_bad : -1; }

int hp3dg_dpg_pass_stats(const hp3dg_dpg_ctx* c, int64_t* kernels) {
  if (!c || !kernels) return HP3DG_ERR_ARG;
  if (!c->ran) return HP3DG_ERR_STATE;
  *kernels = c->launches;
  return HP3DG_OK;
}

void hp3dg_dpg_end(hp3dg_dpg_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_batch(c);
  for (auto& e : c->ev) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
}

}  // extern "C"
