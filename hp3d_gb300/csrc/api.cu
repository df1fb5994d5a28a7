// api.cu -- host runtime behind the C ABI (include/hp3dg.h).
//
// Owns the device buffers of one batch, groups elements into bins (type +
// local order tuple, find_order_loc), builds the per-bin reference tables
// once, and launches the pass on one stream.  The descriptor bookkeeping of
// mumps_sc STEP 1 (solver/omp_mumps/mumps_sc.F90:102-188: dof counts,
// elem_nnz offsets) and of celem_systemI's extraction vector
// (constrs/celem_systemI.F90:290-350: NEXTRACT, nodes in reverse order,
// Dirichlet dof skipped) happens here at submit time; everything numerical
// happens on the GPU.
#include "../../include/hp3dg.h"
#include "hp3dg_internal.cuh"
#include "hp3dg_kernels.h"
#include "hp3dg_simplex.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

using namespace hp3dg;

namespace {

// 1D Gauss-Legendre tables of the reference (gauss_quadrature.F90:518-660,
// rescaled to [0,1] as at 749-750); the same rounded decimal values.
const double GX[10][10] = {
    {0.0},
    {-.577350269189626, .577350269189626},
    {-.774596669241483, .000000000000000, .774596669241483},
    {-.861136311594053, -.339981043584856, .339981043584856, .861136311594053},
    {-.906179845938664, -.538469310105683, .000000000000000, .538469310105683, .906179845938664},
    {-.932469514203152, -.661209386466265, -.238619186083197, .238619186083197, .661209386466265,
     .932469514203152},
    {-.949107912342759, -.741531185599394, -.405845151377397, .000000000000000, .405845151377397,
     .741531185599394, .949107912342759},
    {-.960289856497536, -.796666477413627, -.525532409916329, -.183434642495650, .183434642495650,
     .525532409916329, .796666477413627, .960289856497536},
    {-.968160239507626, -.836031107326636, -.613371432700590, -.324253423403809, .000000000000000,
     .324253423403809, .613371432700590, .836031107326636, .968160239507626},
    {-.9739065285171717200779640, -.8650633666889845107320967, -.6794095682990244062343274,
     -.4333953941292471907992659, -.1488743389816312108848260, .1488743389816312108848260,
     .4333953941292471907992659, .6794095682990244062343274, .8650633666889845107320967,
     .9739065285171717200779640}};
const double GW[10][10] = {
    {2.000000000000000},
    {1.000000000000000, 1.000000000000000},
    {.555555555555556, .888888888888889, .555555555555556},
    {.347854845137454, .652145154862546, .652145154862546, .347854845137454},
    {.236926885056189, .478628670499366, .568888888888889, .478628670499366, .236926885056189},
    {.171324492379170, .360761573048139, .467913934572691, .467913934572691, .360761573048139,
     .171324492379170},
    {.129484966168870, .279705391489277, .381830050505119, .417959183673469, .381830050505119,
     .279705391489277, .129484966168870},
    {.101228536290376, .222381034453374, .313706645877887, .362683783378362, .362683783378362,
     .313706645877887, .222381034453374, .101228536290376},
    {.081274388361574, .180648160694857, .260610696402935, .312347077040003, .330239355001260,
     .312347077040003, .260610696402935, .180648160694857, .081274388361574},
    {.0666713443086881375935688, .1494513491505805931457763, .2190863625159820439955349,
     .2692667193099963550912269, .2955242247147528701738930, .2955242247147528701738930,
     .2692667193099963550912269, .2190863625159820439955349, .1494513491505805931457763,
     .0666713443086881375935688}};

}  // namespace

// the rule with n points on [0,1] (gauss_quadrature.F90:749-750)
int hp3dg::gauss_rule01(int n, double* x, double* w) {
  if (n < 1 || n > 10) return -1;
  for (int i = 0; i < n; ++i) {
    x[i] = 0.5 * (1.0 + GX[n - 1][i]);
    w[i] = 0.5 * GW[n - 1][i];
  }
  return n;
}

namespace {

// set_3Dint_aux BRICK branch (set_3D_int.F90:155-245) on local orders.
int hexa_quadrature(const int* nl, int integration, std::vector<double>& xi,
                    std::vector<double>& w) {
  int nx = 0, ny = 0, nz = 0;
  auto mx = [](int& a, int b) { a = std::max(a, b); };
  for (int i = 1; i <= 19; ++i) {
    int h, v, x, y, z;
    switch (i) {
      case 1: case 3: case 5: case 7: mx(nx, nl[i - 1]); break;
      case 2: case 4: case 6: case 8: mx(ny, nl[i - 1]); break;
      case 9: case 10: case 11: case 12: mx(nz, nl[i - 1]); break;
      case 13: case 14: decod2(nl[i - 1], h, v); mx(nx, h); mx(ny, v); break;
      case 15: case 17: decod2(nl[i - 1], h, v); mx(nx, h); mx(nz, v); break;
      case 16: case 18: decod2(nl[i - 1], h, v); mx(ny, h); mx(nz, v); break;
      case 19: decod3(nl[i - 1], x, y, z); mx(nx, x); mx(ny, y); mx(nz, z); break;
    }
  }
  nx = std::min(nx + integration, MAXP) + 1;
  ny = std::min(ny + integration, MAXP) + 1;
  nz = std::min(nz + integration, MAXP) + 1;
  xi.clear(); w.clear();
  for (int l3 = 0; l3 < nz; ++l3)
    for (int l2 = 0; l2 < ny; ++l2)
      for (int l1 = 0; l1 < nx; ++l1) {
        xi.push_back(0.5 * (1.0 + GX[nx - 1][l1]));
        xi.push_back(0.5 * (1.0 + GX[ny - 1][l2]));
        xi.push_back(0.5 * (1.0 + GX[nz - 1][l3]));
        w.push_back((0.5 * GW[nx - 1][l1]) * (0.5 * GW[ny - 1][l2]) * (0.5 * GW[nz - 1][l3]));
      }
  return (int)w.size();
}

// set_3Dint_aux TETRA branch (set_3D_int.F90:305-323): order p = max order
// + INTEGRATION (capped at MAXP), Duffy-collapsed Gauss rule of
// init_gauss_quadrature (gauss_quadrature.F90:757-787): p+1 points in x and
// y, p+2 in z, xi = (x(1-y)(1-z), y(1-z), z), w = wx wy wz (1-z)^2 (1-y).
int tet_quadrature(int pm, int integration, std::vector<double>& xi, std::vector<double>& w) {
  int np = std::min(pm + integration, MAXP);
  xi.clear(); w.clear();
  for (int k = 0; k < np + 2; ++k) {
    double z = 0.5 * (1.0 + GX[np + 1][k]), wz = 0.5 * GW[np + 1][k];
    for (int j = 0; j < np + 1; ++j) {
      double y = 0.5 * (1.0 + GX[np][j]), wy = 0.5 * GW[np][j];
      for (int i = 0; i < np + 1; ++i) {
        double x = 0.5 * (1.0 + GX[np][i]), wx = 0.5 * GW[np][i];
        xi.push_back(x * (1.0 - y) * (1.0 - z));
        xi.push_back(y * (1.0 - z));
        xi.push_back(z);
        w.push_back(wx * wy * wz * ((1.0 - z) * (1.0 - z)) * (1.0 - y));
      }
    }
  }
  return (int)w.size();
}

// Triangle rules of the prism: Dunavant's symmetric rules of degree 2..12 in
// the 15-digit form of init_gauss_quadrature (gauss_quadrature.F90:130-270:
// per orbit a weight, a barycentric triple and the orbit size 1, 3 or 6),
// expanded into points in the order of gauss_quadrature.F90:663-700.
struct TriOrbit { int degree, size; double w, b[3]; };
const TriOrbit TRI_ORBITS[] = {
    {2, 3, 0.333333333333333, {0.666666666666667, 0.166666666666667, 0.166666666666667}},
    {4, 3, 0.223381589678011, {0.10810301816807, 0.445948490915965, 0.445948490915965}},
    {4, 3, 0.109951743655322, {0.816847572980459, 0.091576213509771, 0.091576213509771}},
    {6, 3, 0.116786275726379, {0.501426509658179, 0.24928674517091, 0.24928674517091}},
    {6, 3, 0.050844906370207, {0.873821971016996, 0.063089014491502, 0.063089014491502}},
    {6, 6, 0.082851075618374, {0.053145049844817, 0.310352451033784, 0.636502499121399}},
    {8, 1, 0.144315607677787, {0.333333333333333, 0.333333333333333, 0.333333333333333}},
    {8, 3, 0.095091634267285, {0.081414823414554, 0.459292588292723, 0.459292588292723}},
    {8, 3, 0.103217370534718, {0.65886138449648, 0.17056930775176, 0.17056930775176}},
    {8, 3, 0.032458497623198, {0.898905543365938, 0.050547228317031, 0.050547228317031}},
    {8, 6, 0.027230314174435, {0.008394777409958, 0.263112829634638, 0.728492392955404}},
    {10, 1, 0.090817990382754, {0.333333333333333, 0.333333333333333, 0.333333333333333}},
    {10, 3, 0.036725957756467, {0.028844733232685, 0.485577633383657, 0.485577633383657}},
    {10, 3, 0.045321059435528, {0.781036849029926, 0.109481575485037, 0.109481575485037}},
    {10, 6, 0.07275791684542, {0.14170721941488, 0.307939838764121, 0.550352941820999}},
    {10, 6, 0.028327242531057, {0.025003534762686, 0.246672560639903, 0.728323904597411}},
    {10, 6, 0.009421666963733, {0.009540815400299, 0.0668032510122, 0.9236559335875}},
    {12, 3, 0.025731066440455, {0.02356522045239, 0.488217389773805, 0.488217389773805}},
    {12, 3, 0.043692544538038, {0.120551215411079, 0.43972439229446, 0.43972439229446}},
    {12, 3, 0.062858224217885, {0.457579229975768, 0.271210385012116, 0.271210385012116}},
    {12, 3, 0.034796112930709, {0.744847708916828, 0.127576145541586, 0.127576145541586}},
    {12, 3, 0.006166261051559, {0.957365299093579, 0.02131735045321, 0.02131735045321}},
    {12, 6, 0.040371557766381, {0.115343494534698, 0.275713269685514, 0.608943235779788}},
    {12, 6, 0.022356773202303, {0.022838332222257, 0.28132558098994, 0.695836086787803}},
    {12, 6, 0.017316231108659, {0.02573405054833, 0.116251915907597, 0.858014033544073}},
};

int tri_rule(int degree, std::vector<double>& bar, std::vector<double>& w) {
  bar.clear(); w.clear();
  for (const TriOrbit& r : TRI_ORBITS) {
    if (r.degree != degree) continue;
    const double x[6] = {r.b[0], r.b[1], r.b[2], r.b[0], r.b[1], r.b[2]};
    const int rot = r.size == 1 ? 1 : 3;
    for (int q = 0; q < rot; ++q) {  // identity, then the two cyclic shifts
      for (int k = 0; k < 3; ++k) bar.push_back(x[k + q]);
      w.push_back(r.w);
    }
    if (r.size == 6)
      for (int l = 1; l <= 3; ++l) {  // the three reflections
        for (int k = 1; k <= 3; ++k) bar.push_back(x[3 + l - k - 1]);
        w.push_back(r.w);
      }
  }
  return (int)w.size();
}

// set_3Dint_aux PRISM branch (set_3D_int.F90:264-300) on the bin orders
// (horizontal ph, vertical pz): the triangle rule NSELECT(ph) = degree 2ph
// times Gauss with pz+1 points; xi = (bar2, bar3, z), w = w_tri/2 * w_z.
int prism_quadrature(int ph, int pz, int integration, std::vector<double>& xi,
                     std::vector<double>& w) {
  int nh = std::min(ph + integration, MAXP), nz = std::min(pz + integration, MAXP) + 1;
  std::vector<double> bar, wt;
  int nt = tri_rule(2 * nh, bar, wt);
  xi.clear(); w.clear();
  for (int l2 = 0; l2 < nz; ++l2)
    for (int l1 = 0; l1 < nt; ++l1) {
      xi.push_back(bar[3 * l1 + 1]);
      xi.push_back(bar[3 * l1 + 2]);
      xi.push_back(0.5 * (1.0 + GX[nz - 1][l2]));
      w.push_back(wt[l1] / 2.0 * (0.5 * GW[nz - 1][l2]));
    }
  return (int)w.size();
}

// ---- per element type (element_data.F90 node tables, ndof_nod 808-884) ----
int type_nvert(int t) { return t == HP3DG_HEXA ? 8 : (t == HP3DG_PRISM ? 6 : 4); }
int type_nnode(int t) { return t == HP3DG_HEXA ? 26 : (t == HP3DG_PRISM ? 20 : 14); }

// dof per vertex / edge / face node in element node order; returns node count
int node_ndof(int t, const int* no, int* nd) {
  if (t == HP3DG_PRISM) {
    for (int v = 0; v < 6; ++v) nd[v] = 1;
    for (int e = 0; e < 9; ++e) nd[6 + e] = no[e] > 1 ? no[e] - 1 : 0;
    for (int f = 0; f < 2; ++f) nd[15 + f] = tri_ndof(no[9 + f]);
    for (int f = 0; f < 3; ++f) {
      int h, v; decod2(no[11 + f], h, v);
      nd[17 + f] = (h > 1 && v > 1) ? (h - 1) * (v - 1) : 0;
    }
    return 20;
  }
  if (t == HP3DG_TET) {
    for (int v = 0; v < 4; ++v) nd[v] = 1;
    for (int e = 0; e < 6; ++e) nd[4 + e] = no[e] > 1 ? no[e] - 1 : 0;
    for (int f = 0; f < 4; ++f) nd[10 + f] = tri_ndof(no[6 + f]);
    return 14;
  }
  for (int v = 0; v < 8; ++v) nd[v] = 1;
  for (int q = 0; q < 12; ++q) nd[8 + q] = no[q] - 1;
  for (int f = 0; f < 6; ++f) { int h, v; decod2(no[12 + f], h, v); nd[20 + f] = (h - 1) * (v - 1); }
  return 26;
}
int elem_nbub(int t, const int* no) {
  return t == HP3DG_TET ? tet_nbub(no[10]) : (t == HP3DG_PRISM ? prism_nbub(no) : hexa_nbub(no));
}
int elem_ndof(int t, const int* no) {
  return t == HP3DG_TET ? tet_ndof(no) : (t == HP3DG_PRISM ? prism_ndof(no) : hexa_ndof(no));
}

// descriptor checks (CheckOrder / the reference's order and orientation ranges)
int validate_desc(const hp3dg_elem_desc& d, int nnodes) {
  if (d.etype == HP3DG_HEXA) {
    for (int i = 0; i < 12; ++i)
      if (d.norder[i] < 1 || d.norder[i] > MAXP || (d.nori_edge[i] & ~1)) return HP3DG_ERR_BAD_ORDER;
    for (int f = 0; f < 6; ++f) {
      int h, v; decod2(d.norder[12 + f], h, v);
      if (h < 1 || h > MAXP || v < 1 || v > MAXP || d.nori_face[f] < 0 || d.nori_face[f] > 7)
        return HP3DG_ERR_BAD_ORDER;
    }
    int x, y, z; decod3(d.norder[18], x, y, z);
    if (x < 1 || x > MAXP || y < 1 || y > MAXP || z < 1 || z > MAXP || d.norder[18] > 999)
      return HP3DG_ERR_BAD_ORDER;
  } else if (d.etype == HP3DG_TET) {
    for (int i = 0; i < 11; ++i)
      if (d.norder[i] < 1 || d.norder[i] > MAXP) return HP3DG_ERR_BAD_ORDER;
    for (int e = 0; e < 6; ++e)
      if (d.nori_edge[e] & ~1) return HP3DG_ERR_BAD_ORDER;
    for (int f = 0; f < 4; ++f)
      if (d.nori_face[f] < 0 || d.nori_face[f] > 5) return HP3DG_ERR_BAD_ORDER;
  } else if (d.etype == HP3DG_PRISM) {
    for (int i = 0; i < 11; ++i)
      if (d.norder[i] < 1 || d.norder[i] > MAXP) return HP3DG_ERR_BAD_ORDER;
    for (int i = 11; i < 15; ++i) {
      int h, v; decod2(d.norder[i], h, v);
      if (h < 1 || h > MAXP || v < 1 || v > MAXP || d.norder[i] > 99) return HP3DG_ERR_BAD_ORDER;
    }
    for (int e = 0; e < 9; ++e)
      if (d.nori_edge[e] & ~1) return HP3DG_ERR_BAD_ORDER;
    for (int f = 0; f < 2; ++f)
      if (d.nori_face[f] < 0 || d.nori_face[f] > 5) return HP3DG_ERR_BAD_ORDER;
    for (int f = 2; f < 5; ++f)
      if (d.nori_face[f] < 0 || d.nori_face[f] > 7) return HP3DG_ERR_BAD_ORDER;
  } else {
    return HP3DG_ERR_BAD_ORDER;
  }
  for (int i = 0; i < type_nnode(d.etype); ++i)
    if (d.nodes[i] < 0 || d.nodes[i] >= nnodes) return HP3DG_ERR_ARG;
  return HP3DG_OK;
}

// Bin of an element: hexa by its per-axis maximum local orders; tet by its
// maximum order and the orientation class of each triangle face.  full =
// the bin element's orders, fo = the face orientations of the bin tables.
void bin_key(const hp3dg_elem_desc& d, std::vector<int>& key, int* full, int* fo) {
  for (int i = 0; i < 19; ++i) full[i] = 0;
  for (int f = 0; f < 6; ++f) fo[f] = 0;
  if (d.etype == HP3DG_PRISM) {
    prism_bin_orders(d.norder, d.nori_face, full);
    for (int f = 0; f < 2; ++f) fo[f] = tri_class(d.nori_face[f]);
    key = {HP3DG_PRISM, full[14], fo[0], fo[1]};
    return;
  }
  if (d.etype == HP3DG_TET) {
    int pm = 0;
    for (int i = 0; i < 11; ++i) pm = std::max(pm, (int)d.norder[i]);
    for (int i = 0; i < 11; ++i) full[i] = pm;
    for (int f = 0; f < 4; ++f) fo[f] = tri_class(d.nori_face[f]);
    key = {HP3DG_TET, pm, fo[0], fo[1], fo[2], fo[3]};
    return;
  }
  int loc[19];
  hexa_order_loc(d.norder, d.nori_face, loc);
  hexa_bin_orders(loc, full);
  key.assign(full, full + 19);
  key.insert(key.begin(), HP3DG_HEXA);
}

int bin_quadrature(int t, const int* full, int integration, std::vector<double>& xi,
                   std::vector<double>& w) {
  if (t == HP3DG_TET) return tet_quadrature(full[0], integration, xi, w);
  if (t == HP3DG_PRISM) return prism_quadrature(full[14] / 10, full[14] % 10, integration, xi, w);
  return hexa_quadrature(full, integration, xi, w);
}

// testing (hp3dg_opts.fault_inject = 2): the submit running on this thread
// makes every device allocation fail
thread_local bool tl_alloc_fault = false;
struct AllocFaultScope {
  explicit AllocFaultScope(bool on) { tl_alloc_fault = on; }
  ~AllocFaultScope() { tl_alloc_fault = false; }
};

template <class T>
T* dalloc(size_t count, int* err) {
  if (count == 0) count = 1;
  if (tl_alloc_fault) { *err = HP3DG_ERR_ALLOC; return nullptr; }
  void* p = nullptr;
  if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) { *err = HP3DG_ERR_ALLOC; return nullptr; }
  return (T*)p;
}

struct Bin {
  int etype = HP3DG_HEXA, nvert = 8;
  int nord_loc[19];  // full (bin) orders: per-axis maxima of the member elements' local orders
  int face_nori[6] = {0, 0, 0, 0, 0, 0};  // face orientations of the tables (tet: class)
  int n = 0, nb = 0, ni = 0, nint = 0;
  std::vector<int> elems;
  std::vector<double> xi, wq;
  bool tables = false;
  int* d_elist = nullptr;
  double *d_xi = nullptr, *d_wq = nullptr, *d_shap = nullptr, *d_grad = nullptr;
  double *d_D = nullptr, *d_F = nullptr, *d_b0 = nullptr, *d_PK = nullptr, *d_S = nullptr;
  double* d_Yg = nullptr;  // global Y slab for bins whose Y does not fit in shared memory
  uint32_t* d_perm = nullptr;
  uint8_t* d_dmask = nullptr;
  // error-evaluation tables (INTEGRATION = 2 rule)
  bool etable = false;
  int nint_err = 0;
  std::vector<double> xi_err, wq_err;
  double *d_xi_err = nullptr, *d_wq_err = nullptr, *d_shap_err = nullptr, *d_grad_err = nullptr;
  // mixed precision
  bool mtable = false;
  OzakiPlan plan{};
  uint16_t *d_mdig = nullptr, *d_ddig = nullptr;
  double *d_mscale = nullptr, *d_dscale = nullptr;
  // condensation with every product on tensor cores (mixed, nb <= 64)
  bool cond_tc = false;
  CondTcBufs ctb{};
  // tuning-table variant (0 = built-in rules)
  int tune_cond = 0, tune_grp = 0;
  bool tuned = false;
  // tensor-core Schur update (mixed): Y digits, column exponents, condensed load
  bool tc_schur = false;
  TcFactorOut tco{};
  uint8_t* d_ydig = nullptr;
  int* d_yexp = nullptr;
  double* d_bi = nullptr;
};

}  // namespace

struct hp3dg_ctx {
  hp3dg_opts opts{};
  int device = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  int nel = 0, nnodes = 0;
  bool submitted = false, ran = false, downloaded = false;
  int last_bad = -1;
  std::vector<int> n_e, nb_e, ni_e, bin_of, pos_in_bin, etype_e;
  std::vector<int64_t> elem_nnz, lcon_off, schur_off, bub_off, zd_off;
  std::vector<int> nextract;
  std::vector<Bin> bins;
  StageGroup sg;  // grouped launches of the per-element stage kernels (bins or chunks)
  CondGroup cg;   // grouped launches of the fused condensation (its bins or chunks)
  std::vector<int> cg_index;  // stage-group unit -> condensation segment, or -1
  bool have_zdofd = false;
  // device inputs
  int *d_norder = nullptr, *d_nori_e = nullptr, *d_nori_f = nullptr, *d_nodes = nullptr,
      *d_ndofm = nullptr, *d_nextract = nullptr, *d_n_e = nullptr, *d_ni_e = nullptr,
      *d_nb_e = nullptr;
  double *d_xvert = nullptr, *d_kappa = nullptr, *d_zdofd = nullptr;
  int64_t *d_elem_nnz = nullptr, *d_lcon_off = nullptr, *d_schur_off = nullptr,
          *d_bub_off = nullptr, *d_zd_off = nullptr;
  // outputs
  double *d_zastif = nullptr, *d_zbload = nullptr, *d_aschur = nullptr, *d_bschur = nullptr;
  int *d_lcon = nullptr, *d_nfirst = nullptr;
  // index-map scratch
  int *d_first = nullptr, *d_cnt = nullptr;
  int64_t *d_scan = nullptr, *d_blk = nullptr, *d_total = nullptr;
  int* d_flags = nullptr;  // [0] bad Jacobian element, [1] non-SPD element, [2] mixed flag
  // host results
  double *h_zastif = nullptr, *h_zbload = nullptr, *h_aschur = nullptr, *h_bschur = nullptr,
         *h_PK = nullptr, *h_b0 = nullptr;
  int *h_lcon = nullptr, *h_nfirst = nullptr;
  int64_t h_nrdof = 0;
  size_t pk_total = 0, b0_total = 0;
  std::vector<int64_t> pk_off, b0_off;  // per element, into h_PK / h_b0 when keep_elem
  // after the solve
  std::vector<int64_t> dof_off;
  int64_t *d_dof_off = nullptr;
  double *d_dofs = nullptr, *d_xglob = nullptr, *h_dofs = nullptr;
  double *d_err2 = nullptr, *d_nrm2 = nullptr, *d_djdk = nullptr, *d_djdx = nullptr;
  bool have_dofs = false;
  cudaEvent_t ev[8] = {};
  float times[6] = {0, 0, 0, 0, 0, 0};
  cudaGraphExec_t graph = nullptr;  // the captured pass; rebuilt after every new structure
  int64_t graph_kernels = -1;        // kernel nodes of the captured pass
  // pipelined download: the pass in element chunks, each recording an event
  int nchunk = 1;
  int chunk_lo[9] = {0};            // chunk boundaries (element positions of the single bin)
  cudaEvent_t chunk_ev[8] = {};
  cudaStream_t copy_stream = nullptr;
  bool chunked_run = false;
  // a batch of several bins runs them on parallel branches: the bins are
  // spread over NBRANCH streams forked from the library stream
  static constexpr int NBRANCH = 4;
  cudaStream_t branch[NBRANCH] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[NBRANCH] = {};
  std::vector<hp3dg_elem_desc> last_desc;  // descriptors of the current batch
  double* d_xnod = nullptr;  // isoparametric geometry dof (hp3dg_batch_set_geometry)
  bool iso = false;
  // constrained approximation: the compression writes a work layout (every
  // element; constrained elements with all their interface dof), which
  // k_constrain turns into the final outputs.  Without constraints the work
  // pointers alias the final ones.
  bool constrained = false;
  int node_stride = 26;  // node slots per element of the index maps
  int* d_wnextract = nullptr;
  int64_t *d_wlcon_off = nullptr, *d_welem_nnz = nullptr;
  double *d_zwork = nullptr, *d_bwork = nullptr;
  ConstrainArgs cargs{};
  std::vector<void*> cbufs;  // allocations of the constraint data
};

namespace {

void free_bin(Bin& b) {
  cudaFree(b.d_elist); cudaFree(b.d_xi); cudaFree(b.d_wq); cudaFree(b.d_shap); cudaFree(b.d_grad);
  cudaFree(b.d_D); cudaFree(b.d_F); cudaFree(b.d_b0); cudaFree(b.d_PK); cudaFree(b.d_S);
  cudaFree(b.d_Yg);
  cudaFree(b.d_perm); cudaFree(b.d_dmask); cudaFree(b.d_mdig); cudaFree(b.d_ddig);
  cudaFree(b.d_mscale); cudaFree(b.d_dscale);
  cudaFree(b.d_xi_err); cudaFree(b.d_wq_err); cudaFree(b.d_shap_err); cudaFree(b.d_grad_err);
  cudaFree(b.d_ydig); cudaFree(b.d_yexp); cudaFree(b.d_bi);
  cudaFree(b.ctb.kbd); cudaFree(b.ctb.lid); cudaFree(b.ctb.ltd);
  cudaFree(b.ctb.ekb); cudaFree(b.ctb.eli); cudaFree(b.ctb.elt); cudaFree(b.ctb.bi);
  b = Bin();
}

void free_batch(hp3dg_ctx* c) {
  for (void* p : c->cbufs) cudaFree(p);
  c->cbufs.clear();
  c->sg = StageGroup{};
  c->cg = CondGroup{};
  c->cg_index.clear();
  if (c->constrained) {
    c->d_wnextract = nullptr;
    c->d_wlcon_off = c->d_welem_nnz = nullptr;
    c->d_zwork = c->d_bwork = nullptr;
  }
  c->constrained = false;
  c->node_stride = 26;
  c->cargs = ConstrainArgs{};
  if (c->graph) cudaGraphExecDestroy(c->graph);
  c->graph = nullptr;
  c->graph_kernels = -1;
  for (auto& b : c->bins) free_bin(b);
  c->bins.clear();
  void* dev[] = {c->d_norder, c->d_nori_e, c->d_nori_f, c->d_nodes, c->d_ndofm, c->d_nextract,
                 c->d_n_e, c->d_ni_e, c->d_nb_e,
                 c->d_xvert, c->d_kappa, c->d_zdofd, c->d_elem_nnz, c->d_lcon_off,
                 c->d_schur_off, c->d_bub_off, c->d_zd_off, c->d_zastif, c->d_zbload,
                 c->d_aschur, c->d_bschur, c->d_lcon, c->d_nfirst, c->d_first, c->d_cnt,
                 c->d_scan, c->d_blk, c->d_total, c->d_dof_off, c->d_dofs, c->d_xglob,
                 c->d_err2, c->d_nrm2, c->d_djdk, c->d_djdx, c->d_xnod};
  for (void* p : dev) cudaFree(p);
  c->d_xnod = nullptr;
  c->iso = false;
  cudaFreeHost(c->h_dofs);
  c->h_dofs = nullptr;
  c->d_dof_off = nullptr; c->d_dofs = c->d_xglob = nullptr;
  c->d_err2 = c->d_nrm2 = c->d_djdk = c->d_djdx = nullptr;
  c->have_dofs = false;
  void* host[] = {c->h_zastif, c->h_zbload, c->h_aschur, c->h_bschur, c->h_lcon, c->h_nfirst,
                  c->h_PK, c->h_b0};
  for (void* p : host) cudaFreeHost(p);
  c->d_norder = c->d_nori_e = c->d_nori_f = c->d_nodes = c->d_ndofm = c->d_nextract = nullptr;
  c->d_n_e = c->d_ni_e = c->d_nb_e = nullptr;
  c->d_xvert = c->d_kappa = c->d_zdofd = nullptr;
  c->d_elem_nnz = c->d_lcon_off = c->d_schur_off = c->d_bub_off = c->d_zd_off = nullptr;
  c->d_zastif = c->d_zbload = c->d_aschur = c->d_bschur = nullptr;
  c->d_lcon = c->d_nfirst = c->d_first = c->d_cnt = nullptr;
  c->d_scan = c->d_blk = c->d_total = nullptr;
  c->h_zastif = c->h_zbload = c->h_aschur = c->h_bschur = c->h_PK = c->h_b0 = nullptr;
  c->h_lcon = c->h_nfirst = nullptr;
  c->submitted = c->ran = c->downloaded = false;
}

#define CK(x)                                  \
  do {                                         \
    if ((x) != cudaSuccess) return HP3DG_ERR_CUDA; \
  } while (0)

}  // namespace

namespace {

// Segment tables of the grouped stage launches (device arrays freed with the
// batch): one segment per bin, or for a batch of one bin that runs in element
// chunks one per chunk.  Every vertex-geometry pass launches its stage-0
// kernels through these tables, so an element's arithmetic is the same
// whatever batch it is in.
int build_stage_group(hp3dg_ctx* c) {
  c->sg = StageGroup{};
  if (c->bins.empty()) return HP3DG_OK;
  const bool mixed = c->opts.precision == HP3DG_MIXED;
  std::vector<StageSeg> segs;
  std::vector<int> pel{0}, pgeo{0}, pdsc{0}, psl{0};
  int max_nint = 0;
  auto add = [&](Bin& B, int j0, int j1) {
    StageSeg g{};
    const int nel = j1 - j0;
    g.etype = B.etype;
    g.nvert = B.nvert;
    g.n = B.n;
    g.nint = B.nint;
    g.nel = nel;
    for (int i = 0; i < 19; ++i) g.full[i] = B.nord_loc[i];
    g.elist = B.d_elist + j0;
    g.wq = B.d_wq;
    g.shap = B.d_shap;
    g.grad = B.d_grad;
    g.D = B.d_D + (size_t)j0 * B.nint * 6;
    g.F = B.d_F + (size_t)j0 * B.nint;
    g.b0 = B.d_b0 + (size_t)j0 * B.n;
    g.perm = B.d_perm + (size_t)j0 * B.n;
    const int neb = (nel + 63) / 64;
    if (mixed) {
      g.K = 6 * B.nint;
      g.nk = B.plan.kdim / 16;
      g.radix = B.plan.radix;
      g.digits = B.plan.digits;
      // D digit tiles of 64 elements; a chunk starts at a multiple of 128
      g.ddig = (uint16_t*)((uint8_t*)B.d_ddig + (size_t)(j0 / 128) * ozaki_d_bytes(B.plan, 128));
      g.dscale = B.d_dscale + j0;
    }
    segs.push_back(g);
    pel.push_back(pel.back() + nel);
    pgeo.push_back(pgeo.back() + nel * ((B.nint + 127) / 128));
    pdsc.push_back(pdsc.back() + neb * 64);
    psl.push_back(psl.back() + (mixed ? g.nk * neb : 0));
    max_nint = std::max(max_nint, B.nint);
  };
  if (c->bins.size() == 1 && c->nchunk > 1)
    for (int k = 0; k < c->nchunk; ++k) add(c->bins[0], c->chunk_lo[k], c->chunk_lo[k + 1]);
  else
    for (Bin& B : c->bins) add(B, 0, (int)B.elems.size());
  int err = 0;
  StageGroup& G = c->sg;
  G.segs = dalloc<StageSeg>(segs.size(), &err);
  G.pre_el = dalloc<int>(pel.size(), &err);
  G.pre_geom = dalloc<int>(pgeo.size(), &err);
  G.pre_dsc = dalloc<int>(pdsc.size(), &err);
  G.pre_slice = dalloc<int>(psl.size(), &err);
  for (void* p : {(void*)G.segs, (void*)G.pre_el, (void*)G.pre_geom, (void*)G.pre_dsc,
                  (void*)G.pre_slice})
    if (p) c->cbufs.push_back(p);
  if (err) { c->sg = StageGroup{}; return err; }
  CK(cudaMemcpy(G.segs, segs.data(), segs.size() * sizeof(StageSeg), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(G.pre_el, pel.data(), pel.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(G.pre_geom, pgeo.data(), pgeo.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(G.pre_dsc, pdsc.data(), pdsc.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(G.pre_slice, psl.data(), psl.size() * 4, cudaMemcpyHostToDevice));
  G.nseg = (int)segs.size();
  G.h_pre.clear();
  for (auto* v : {&pel, &pgeo, &pdsc, &psl}) G.h_pre.insert(G.h_pre.end(), v->begin(), v->end());
  G.max_nint = max_nint;
  // the fused condensation's segments: the same units, where the bin uses it
  std::vector<CondSegIn> cin;
  c->cg_index.assign(G.nseg, -1);
  // (multi-bin batches: bins without bubbles follow, condensed by the
  // compression kernel alone)
  auto cadd = [&](int unit, Bin& B, int j0, int j1, bool plain) {
    if (plain ? B.nb != 0 : !B.cond_tc) return;
    const size_t nsu = (size_t)B.ni * (B.ni + 1) / 2, npk = (size_t)B.n * (B.n + 1) / 2;
    CondSegIn q;
    q.nfull = B.n; q.nif = B.ni; q.nbf = B.nb; q.nel = j1 - j0;
    q.elist = B.d_elist + j0;
    q.PK = B.d_PK + (size_t)j0 * npk;
    q.b0 = B.d_b0 + (size_t)j0 * B.n;
    q.perm = B.d_perm + (size_t)j0 * B.n;
    q.W = B.d_S + (size_t)j0 * nsu;
    q.dmask = B.d_dmask + (size_t)j0 * B.ni;
    CondTcBufs t = B.ctb;
    if (plain) {
      q.t = CondTcBufs{};
      c->cg_index[unit] = (int)cin.size();
      cin.push_back(q);
      return;
    }
    t.kbd += (size_t)j0 * t.bytes_a;
    t.lid += (size_t)j0 * t.bytes_b;
    t.ltd += (size_t)j0 * t.bytes_b;
    t.ekb += (size_t)j0 * t.nr;
    t.eli += (size_t)j0 * t.nbr;
    t.elt += (size_t)j0 * t.nbr;
    t.bi += (size_t)j0 * B.ni;
    q.t = t;
    c->cg_index[unit] = (int)cin.size();
    cin.push_back(q);
  };
  if (c->bins.size() == 1 && c->nchunk > 1) {
    for (int k = 0; k < c->nchunk; ++k)
      cadd(k, c->bins[0], c->chunk_lo[k], c->chunk_lo[k + 1], false);
  } else {
    for (size_t b = 0; b < c->bins.size(); ++b)
      cadd((int)b, c->bins[b], 0, (int)c->bins[b].elems.size(), false);
    if (c->bins.size() > 1)
      for (size_t b = 0; b < c->bins.size(); ++b)
        cadd((int)b, c->bins[b], 0, (int)c->bins[b].elems.size(), true);
  }
  if (!cin.empty()) {
    const int rc = cond_tc_group_build(cin, &c->cg, &c->cbufs);
    if (rc == -1) return HP3DG_ERR_ALLOC;
    if (rc) return HP3DG_ERR_UNSUPPORTED;
  }
  return HP3DG_OK;
}

}  // namespace

extern "C" {

const char* hp3dg_strerror(int s) {
  switch (s) {
    case HP3DG_OK: return "ok";
    case HP3DG_ERR_NEG_JACOBIAN: return "negative Jacobian at a quadrature point";
    case HP3DG_ERR_NOT_SPD: return "bubble block is not positive definite";
    case HP3DG_ERR_BAD_ORDER: return "order outside 1..MAXP or unsupported element type";
    case HP3DG_ERR_ALLOC: return "allocation failed";
    case HP3DG_ERR_CUDA: return "CUDA call failed";
    case HP3DG_ERR_TIMEOUT: return "bounded device wait gave up";
    case HP3DG_ERR_ARG: return "invalid argument";
    case HP3DG_ERR_STATE: return "call out of order";
    case HP3DG_ERR_UNSUPPORTED: return "unsupported on this device or configuration";
    default: return "unknown status";
  }
}

int hp3dg_batch_begin(const hp3dg_opts* opts, hp3dg_ctx** out) {
  if (!out) return HP3DG_ERR_ARG;
  *out = nullptr;
  hp3dg_ctx* c = new hp3dg_ctx();
  if (opts) c->opts = *opts;
  else c->opts.isol = 10;
  if (c->opts.precision != HP3DG_FP64 && c->opts.precision != HP3DG_MIXED) { delete c; return HP3DG_ERR_ARG; }
  if (c->opts.integration < 0 || c->opts.integration > MAXP) { delete c; return HP3DG_ERR_ARG; }
  if (c->opts.download_chunks < 0 || c->opts.download_chunks > 8) { delete c; return HP3DG_ERR_ARG; }
  c->device = c->opts.device;
  if (cudaSetDevice(c->device) != cudaSuccess) { delete c; return HP3DG_ERR_CUDA; }
  if (c->opts.precision == HP3DG_MIXED) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, c->device) != cudaSuccess) { delete c; return HP3DG_ERR_CUDA; }
    if (p.major != 10) { delete c; return HP3DG_ERR_UNSUPPORTED; }  // tcgen05 needs sm_10x
  }
  if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) { delete c; return HP3DG_ERR_CUDA; }
  c->stream = c->own;
  for (auto& e : c->ev) cudaEventCreate(&e);
  for (auto& e : c->chunk_ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return HP3DG_ERR_CUDA;
  }
  cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming);
  for (int b = 0; b < hp3dg_ctx::NBRANCH; ++b) {
    cudaEventCreateWithFlags(&c->join_ev[b], cudaEventDisableTiming);
    if (cudaStreamCreateWithFlags(&c->branch[b], cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return HP3DG_ERR_CUDA;
    }
  }
  if (cudaMalloc(&c->d_flags, 4 * sizeof(int)) != cudaSuccess) { delete c; return HP3DG_ERR_ALLOC; }
  *out = c;
  return HP3DG_OK;
}

int hp3dg_set_stream(hp3dg_ctx* c, void* stream) {
  if (!c) return HP3DG_ERR_ARG;
  c->stream = stream ? (cudaStream_t)stream : c->own;
  return HP3DG_OK;
}

int hp3dg_batch_submit(hp3dg_ctx* c, int32_t nel, const hp3dg_elem_desc* desc,
                       const double* xvert, const double* kappa, const double* zdofd,
                       int32_t nnodes) {
  return hp3dg_batch_submit_constrained(c, nel, desc, xvert, kappa, zdofd, nnodes, nullptr);
}

int hp3dg_batch_submit_constrained(hp3dg_ctx* c, int32_t nel, const hp3dg_elem_desc* desc,
                                   const double* xvert, const double* kappa,
                                   const double* zdofd, int32_t nnodes,
                                   const hp3dg_constraints* cons) {
  if (!c || nel < 0 || (nel > 0 && (!desc || !xvert)) || nnodes < 0) return HP3DG_ERR_ARG;
  if (cons && cons->n == 0) cons = nullptr;
  cudaSetDevice(c->device);
  // Resubmit of the same mesh (identical descriptors, node count and
  // Dirichlet layout) with new geometry / coefficients / Dirichlet values:
  // keep every buffer, the bin tables, the tensor-core operand digits, the
  // captured graph and the pinned host buffers; upload the numeric inputs.
  if (!cons && !c->constrained && c->submitted && nel == c->nel && nnodes == c->nnodes &&
      (zdofd != nullptr) == c->have_zdofd &&
      nel > 0 && c->last_desc.size() == (size_t)nel &&
      std::memcmp(c->last_desc.data(), desc, sizeof(hp3dg_elem_desc) * (size_t)nel) == 0) {
    cudaStream_t st = c->stream;
    CK(cudaMemcpyAsync(c->d_xvert, xvert, (size_t)nel * 24 * 8, cudaMemcpyHostToDevice, st));
    if (kappa) {
      CK(cudaMemcpyAsync(c->d_kappa, kappa, (size_t)nel * 8, cudaMemcpyHostToDevice, st));
    } else {
      std::vector<double> one(nel, 1.0);
      CK(cudaMemcpyAsync(c->d_kappa, one.data(), (size_t)nel * 8, cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
    }
    if (zdofd) CK(cudaMemcpyAsync(c->d_zdofd, zdofd, c->zd_off[nel] * 8, cudaMemcpyHostToDevice, st));
    if (c->iso) {  // back to the vertex geometry; the captured pass read the geometry dof
      c->iso = false;
      if (c->graph) cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
      c->graph_kernels = -1;
    }
    c->ran = c->downloaded = c->have_dofs = false;
    return HP3DG_OK;
  }
  AllocFaultScope fault_scope(c->opts.fault_inject == 2);
  free_batch(c);
  c->last_desc.clear();
  c->nel = nel;
  c->nnodes = nnodes;
  c->n_e.assign(nel, 0); c->nb_e.assign(nel, 0); c->ni_e.assign(nel, 0);
  c->bin_of.assign(nel, 0); c->pos_in_bin.assign(nel, 0); c->etype_e.assign(nel, 0);
  c->elem_nnz.assign(nel + 1, 0); c->lcon_off.assign(nel + 1, 0);
  c->schur_off.assign(nel + 1, 0); c->bub_off.assign(nel + 1, 0); c->zd_off.assign(nel + 1, 0);
  c->nextract.clear();
  std::vector<int> norder((size_t)nel * 19), nori_e((size_t)nel * 12), nori_f((size_t)nel * 6),
      nodes((size_t)nel * 26), ndofm((size_t)nel * 26);
  std::map<std::vector<int>, int> binmap;
  c->last_bad = -1;
  for (int e = 0; e < nel; ++e) {
    const hp3dg_elem_desc& d = desc[e];
    int vr = validate_desc(d, nnodes);
    if (vr != HP3DG_OK) { c->last_bad = e; return vr; }
    const int t = d.etype;
    c->etype_e[e] = t;
    std::copy(d.norder, d.norder + 19, &norder[19 * (size_t)e]);
    std::copy(d.nori_edge, d.nori_edge + 12, &nori_e[12 * (size_t)e]);
    std::copy(d.nori_face, d.nori_face + 6, &nori_f[6 * (size_t)e]);
    const int nn = type_nnode(t);
    // slots beyond the type's node count are padding (-1: skipped by the index maps)
    for (int i = 0; i < 26; ++i) nodes[26 * (size_t)e + i] = i < nn ? d.nodes[i] : -1;
    std::vector<int> key;
    int full[19], fo[6];
    bin_key(d, key, full, fo);
    auto it = binmap.find(key);
    int b;
    if (it == binmap.end()) {
      b = (int)c->bins.size();
      binmap[key] = b;
      c->bins.emplace_back();
      Bin& B = c->bins.back();
      B.etype = t;
      B.nvert = type_nvert(t);
      std::copy(full, full + 19, B.nord_loc);
      std::copy(fo, fo + 6, B.face_nori);
      B.n = elem_ndof(t, full);
      B.nb = elem_nbub(t, full);
      B.ni = B.n - B.nb;
      B.nint = bin_quadrature(t, full, c->opts.integration, B.xi, B.wq);
      if (condense_smem_small(B.ni, B.nb) > 227 * 1024) { c->last_bad = e; free_batch(c); return HP3DG_ERR_UNSUPPORTED; }
    } else {
      b = it->second;
    }
    c->bin_of[e] = b;
    c->pos_in_bin[e] = (int)c->bins[b].elems.size();
    c->bins[b].elems.push_back(e);
    // per-node dof counts (ndof_nod) in element node order, Dirichlet skipped
    int nd[26];
    node_ndof(t, d.norder, nd);
    int first[26], ni = 0;
    for (int i = 0; i < nn; ++i) { first[i] = ni; ni += nd[i]; }
    int nrdofc = 0;
    for (int i = 25; i >= 0; --i) {
      int act = (i >= nn || d.bcflag[i]) ? 0 : nd[i];
      ndofm[26 * (size_t)e + i] = act;
      for (int q = 0; q < act; ++q) c->nextract.push_back(first[i] + q);
      nrdofc += act;
    }
    c->nb_e[e] = elem_nbub(t, d.norder); c->ni_e[e] = ni; c->n_e[e] = ni + c->nb_e[e];
    c->elem_nnz[e + 1] = c->elem_nnz[e] + (int64_t)nrdofc * nrdofc;
    c->lcon_off[e + 1] = c->lcon_off[e] + nrdofc;
    c->schur_off[e + 1] = c->schur_off[e] + (int64_t)c->nb_e[e] * ni;
    c->bub_off[e + 1] = c->bub_off[e] + c->nb_e[e];
    c->zd_off[e + 1] = c->zd_off[e] + ni;
  }
  c->dof_off.assign(nel + 1, 0);
  for (int e = 0; e < nel; ++e) c->dof_off[e + 1] = c->dof_off[e] + c->n_e[e];
  // ---- constrained approximation ----
  std::vector<int> wnextract, cidx, cnmod, cgptr, cgk;
  std::vector<int64_t> wlcon_off, welem_nnz, cgptr_off, caux_off, cmdof_off;
  std::vector<double> cgv, cmzd;
  std::vector<uint8_t> cmdir;
  if (cons) {
    const int nc_el = cons->n;
    if (!cons->iel || !cons->node_off || !cons->nodm || !cons->ndof || !cons->bcflag ||
        !cons->coef_off || !cons->coef_k || !cons->coef_l || !cons->coef_v || nc_el < 0)
      { free_batch(c); return HP3DG_ERR_ARG; }
    cidx.assign(nel, -1);
    int stride = 26;
    for (int j = 0; j < nc_el; ++j) {
      const int e = cons->iel[j];
      if (e < 0 || e >= nel || (j > 0 && e <= cons->iel[j - 1])) { free_batch(c); return HP3DG_ERR_ARG; }
      cidx[e] = j;
      const int64_t nn = cons->node_off[j + 1] - cons->node_off[j];
      if (nn <= 0 || nn > 4096) { free_batch(c); return HP3DG_ERR_ARG; }
      stride = std::max(stride, (int)nn);
    }
    // final extraction, offsets and index-map node lists
    std::vector<int> nodes2((size_t)nel * stride, -1), ndofm2((size_t)nel * stride, 0);
    std::vector<int> fnext;
    std::vector<int64_t> flcon(nel + 1, 0), fnnz(nel + 1, 0);
    wlcon_off.assign(nel + 1, 0);
    welem_nnz.assign(nel + 1, 0);
    cgptr_off.assign(nc_el, 0);
    caux_off.assign(nc_el + 1, 0);
    cmdof_off.assign(nc_el + 1, 0);
    cnmod.assign(nc_el, 0);
    int64_t pos = 0;  // running position in c->nextract (conforming extraction)
    for (int e = 0; e < nel; ++e) {
      const int j = cidx[e];
      const int ni = c->ni_e[e];
      const int nconf = (int)(c->lcon_off[e + 1] - c->lcon_off[e]);
      int nrdofc;
      if (j < 0) {
        for (int i = 0; i < 26; ++i) {
          nodes2[(size_t)e * stride + i] = nodes[(size_t)e * 26 + i];
          ndofm2[(size_t)e * stride + i] = ndofm[(size_t)e * 26 + i];
        }
        for (int q = 0; q < nconf; ++q) {
          fnext.push_back(c->nextract[pos + q]);
          wnextract.push_back(c->nextract[pos + q]);
        }
        nrdofc = nconf;
        wlcon_off[e + 1] = wlcon_off[e] + nrdofc;
        welem_nnz[e + 1] = welem_nnz[e] + (int64_t)nrdofc * nrdofc;
      } else {
        const int64_t n0 = cons->node_off[j], nn = cons->node_off[j + 1] - n0;
        std::vector<int> mfirst(nn + 1, 0);
        for (int64_t i = 0; i < nn; ++i) {
          const int g = cons->nodm[n0 + i], nd = cons->ndof[n0 + i];
          if (g < 0 || g >= nnodes || nd < 0) { free_batch(c); return HP3DG_ERR_ARG; }
          mfirst[i + 1] = mfirst[i] + nd;
          nodes2[(size_t)e * stride + i] = g;
          ndofm2[(size_t)e * stride + i] = cons->bcflag[n0 + i] ? 0 : nd;
        }
        const int nmod = mfirst[nn];
        cnmod[j] = nmod;
        nrdofc = 0;
        for (int64_t i = nn - 1; i >= 0; --i)
          if (!cons->bcflag[n0 + i])
            for (int q = 0; q < cons->ndof[n0 + i]; ++q) { fnext.push_back(mfirst[i] + q); ++nrdofc; }
        for (int q = 0; q < ni; ++q) wnextract.push_back(q);
        wlcon_off[e + 1] = wlcon_off[e] + ni;
        welem_nnz[e + 1] = welem_nnz[e] + (int64_t)ni * ni;
        // gather lists by modified dof, stable in the given (reference) order
        const int64_t c0 = cons->coef_off[j], c1 = cons->coef_off[j + 1];
        std::vector<int> cnt(nmod + 1, 0);
        for (int64_t q = c0; q < c1; ++q) {
          const int k = cons->coef_k[q], l = cons->coef_l[q];
          if (k < 0 || k >= ni || l < 0 || l >= nmod) { free_batch(c); return HP3DG_ERR_ARG; }
          ++cnt[l + 1];
        }
        for (int l = 0; l < nmod; ++l) cnt[l + 1] += cnt[l];
        cgptr_off[j] = (int64_t)cgptr.size();
        const int base = (int)cgk.size();
        for (int l = 0; l <= nmod; ++l) cgptr.push_back(base + cnt[l]);
        cgk.resize(base + (c1 - c0));
        cgv.resize(base + (c1 - c0));
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int64_t q = c0; q < c1; ++q) {
          const int l = cons->coef_l[q];
          cgk[base + fill[l]] = cons->coef_k[q];
          cgv[base + fill[l]] = cons->coef_v[q];
          ++fill[l];
        }
        caux_off[j + 1] = caux_off[j] + (int64_t)nmod * ni;
        cmdof_off[j + 1] = cmdof_off[j] + nmod;
        for (int64_t i = 0; i < nn; ++i)
          for (int q = 0; q < cons->ndof[n0 + i]; ++q) {
            cmdir.push_back(cons->bcflag[n0 + i] ? 1 : 0);
            cmzd.push_back(cons->zdofd ? cons->zdofd[cmdof_off[j] + mfirst[i] + q] : 0.0);
          }
      }
      pos += nconf;
      flcon[e + 1] = flcon[e] + nrdofc;
      fnnz[e + 1] = fnnz[e] + (int64_t)nrdofc * nrdofc;
    }
    c->nextract.swap(fnext);
    c->lcon_off.swap(flcon);
    c->elem_nnz.swap(fnnz);
    nodes.swap(nodes2);
    ndofm.swap(ndofm2);
    c->node_stride = stride;
    c->constrained = true;
  }
  int err = 0;
  // ---- device inputs ----
  c->d_norder = dalloc<int>(norder.size(), &err);
  c->d_nori_e = dalloc<int>(nori_e.size(), &err);
  c->d_nori_f = dalloc<int>(nori_f.size(), &err);
  c->d_nodes = dalloc<int>(nodes.size(), &err);
  c->d_ndofm = dalloc<int>(ndofm.size(), &err);
  c->d_nextract = dalloc<int>(c->nextract.size(), &err);
  c->d_xvert = dalloc<double>((size_t)nel * 24, &err);
  c->d_kappa = dalloc<double>(nel, &err);
  c->d_elem_nnz = dalloc<int64_t>(nel + 1, &err);
  c->d_lcon_off = dalloc<int64_t>(nel + 1, &err);
  c->d_schur_off = dalloc<int64_t>(nel + 1, &err);
  c->d_bub_off = dalloc<int64_t>(nel + 1, &err);
  c->d_zd_off = dalloc<int64_t>(nel + 1, &err);
  c->d_dof_off = dalloc<int64_t>(nel + 1, &err);
  c->d_n_e = dalloc<int>(nel, &err);
  c->d_ni_e = dalloc<int>(nel, &err);
  c->d_nb_e = dalloc<int>(nel, &err);
  c->have_zdofd = zdofd != nullptr;
  if (zdofd) c->d_zdofd = dalloc<double>(c->zd_off[nel], &err);
  // ---- outputs ----
  c->d_zastif = dalloc<double>(c->elem_nnz[nel], &err);
  c->d_zbload = dalloc<double>(c->lcon_off[nel], &err);
  c->d_aschur = dalloc<double>(c->schur_off[nel], &err);
  c->d_bschur = dalloc<double>(c->bub_off[nel], &err);
  c->d_lcon = dalloc<int>(c->lcon_off[nel], &err);
  c->d_nfirst = dalloc<int>(nnodes, &err);
  int64_t ns = (int64_t)nel * c->node_stride;
  c->d_first = dalloc<int>(nnodes, &err);
  c->d_cnt = dalloc<int>(ns, &err);
  c->d_scan = dalloc<int64_t>(ns, &err);
  c->d_blk = dalloc<int64_t>((ns + 1023) / 1024 + 1, &err);
  c->d_total = dalloc<int64_t>(1, &err);
  if (err) { free_batch(c); return err; }
  cudaStream_t st = c->stream;
  CK(cudaMemcpyAsync(c->d_norder, norder.data(), norder.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_nori_e, nori_e.data(), nori_e.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_nori_f, nori_f.data(), nori_f.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_nodes, nodes.data(), nodes.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_ndofm, ndofm.data(), ndofm.size() * 4, cudaMemcpyHostToDevice, st));
  if (!c->nextract.empty())
    CK(cudaMemcpyAsync(c->d_nextract, c->nextract.data(), c->nextract.size() * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_xvert, xvert, (size_t)nel * 24 * 8, cudaMemcpyHostToDevice, st));
  if (kappa) {
    CK(cudaMemcpyAsync(c->d_kappa, kappa, (size_t)nel * 8, cudaMemcpyHostToDevice, st));
  } else {
    std::vector<double> one(nel, 1.0);
    CK(cudaMemcpyAsync(c->d_kappa, one.data(), (size_t)nel * 8, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
  }
  CK(cudaMemcpyAsync(c->d_elem_nnz, c->elem_nnz.data(), (nel + 1) * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_lcon_off, c->lcon_off.data(), (nel + 1) * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_schur_off, c->schur_off.data(), (nel + 1) * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_bub_off, c->bub_off.data(), (nel + 1) * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_zd_off, c->zd_off.data(), (nel + 1) * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->d_dof_off, c->dof_off.data(), (nel + 1) * 8, cudaMemcpyHostToDevice, st));
  if (nel > 0) {
    CK(cudaMemcpyAsync(c->d_n_e, c->n_e.data(), (size_t)nel * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->d_ni_e, c->ni_e.data(), (size_t)nel * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->d_nb_e, c->nb_e.data(), (size_t)nel * 4, cudaMemcpyHostToDevice, st));
  }
  if (zdofd)
    CK(cudaMemcpyAsync(c->d_zdofd, zdofd, c->zd_off[nel] * 8, cudaMemcpyHostToDevice, st));
  // ---- work layout and constraint data ----
  if (!c->constrained) {
    c->d_wnextract = c->d_nextract;
    c->d_wlcon_off = c->d_lcon_off;
    c->d_welem_nnz = c->d_elem_nnz;
    c->d_zwork = c->d_zastif;
    c->d_bwork = c->d_zbload;
  } else {
    auto calloc_ = [&](size_t bytes) -> void* {
      void* p = nullptr;
      if (cudaMalloc(&p, bytes ? bytes : 8) != cudaSuccess) { err = HP3DG_ERR_ALLOC; return nullptr; }
      c->cbufs.push_back(p);
      return p;
    };
    auto upc = [&](void* dst, const void* src, size_t bytes) {
      if (!err && bytes && cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
        err = HP3DG_ERR_CUDA;
    };
    const int nc_el = cons->n;
    c->d_wnextract = (int*)calloc_(wnextract.size() * 4);
    c->d_wlcon_off = (int64_t*)calloc_((nel + 1) * 8);
    c->d_welem_nnz = (int64_t*)calloc_((nel + 1) * 8);
    c->d_zwork = (double*)calloc_(welem_nnz[nel] * 8);
    c->d_bwork = (double*)calloc_(wlcon_off[nel] * 8);
    ConstrainArgs& a = c->cargs;
    int* d_cidx = (int*)calloc_((size_t)nel * 4);
    int* d_nmod = (int*)calloc_((size_t)nc_el * 4);
    int64_t* d_gptr_off = (int64_t*)calloc_((size_t)nc_el * 8);
    int* d_gptr = (int*)calloc_(cgptr.size() * 4);
    int* d_gk = (int*)calloc_(cgk.size() * 4);
    double* d_gv = (double*)calloc_(cgv.size() * 8);
    int64_t* d_aux_off = (int64_t*)calloc_((size_t)(nc_el + 1) * 8);
    double* d_aux = (double*)calloc_(caux_off[nc_el] * 8);
    int64_t* d_mdof_off = (int64_t*)calloc_((size_t)(nc_el + 1) * 8);
    uint8_t* d_mdir = (uint8_t*)calloc_(cmdir.size());
    double* d_mzd = cons->zdofd ? (double*)calloc_(cmzd.size() * 8) : nullptr;
    if (err) { free_batch(c); return err; }
    upc(c->d_wnextract, wnextract.data(), wnextract.size() * 4);
    upc(c->d_wlcon_off, wlcon_off.data(), (nel + 1) * 8);
    upc(c->d_welem_nnz, welem_nnz.data(), (nel + 1) * 8);
    upc(d_cidx, cidx.data(), (size_t)nel * 4);
    upc(d_nmod, cnmod.data(), (size_t)nc_el * 4);
    upc(d_gptr_off, cgptr_off.data(), (size_t)nc_el * 8);
    upc(d_gptr, cgptr.data(), cgptr.size() * 4);
    upc(d_gk, cgk.data(), cgk.size() * 4);
    upc(d_gv, cgv.data(), cgv.size() * 8);
    upc(d_aux_off, caux_off.data(), (size_t)(nc_el + 1) * 8);
    upc(d_mdof_off, cmdof_off.data(), (size_t)(nc_el + 1) * 8);
    upc(d_mdir, cmdir.data(), cmdir.size());
    if (d_mzd) upc(d_mzd, cmzd.data(), cmzd.size() * 8);
    if (!err && cudaStreamSynchronize(st) != cudaSuccess) err = HP3DG_ERR_CUDA;
    if (err) { free_batch(c); return err; }
    a.cidx = d_cidx;
    a.lcon_off = c->d_lcon_off; a.elem_nnz = c->d_elem_nnz;
    a.zastif = c->d_zastif; a.zbload = c->d_zbload;
    a.wlcon_off = c->d_wlcon_off; a.welem_nnz = c->d_welem_nnz;
    a.zwork = c->d_zwork; a.bwork = c->d_bwork;
    a.nmod = d_nmod; a.gptr_off = d_gptr_off; a.gptr = d_gptr; a.gk = d_gk; a.gv = d_gv;
    a.aux_off = d_aux_off; a.aux = d_aux;
    a.cnextract = c->d_nextract;
    a.mdof_off = d_mdof_off; a.mdir = d_mdir; a.mzd = d_mzd;
  }
  // ---- per-bin buffers ----
  for (auto& B : c->bins) {
    size_t ne = B.elems.size();
    B.d_elist = dalloc<int>(ne, &err);
    B.d_xi = dalloc<double>(B.xi.size(), &err);
    B.d_wq = dalloc<double>(B.wq.size(), &err);
    B.d_shap = dalloc<double>((size_t)B.nint * B.n, &err);
    B.d_grad = dalloc<double>((size_t)B.nint * 3 * B.n, &err);
    B.d_D = dalloc<double>(ne * B.nint * 6, &err);
    B.d_F = dalloc<double>(ne * B.nint, &err);
    B.d_b0 = dalloc<double>(ne * B.n, &err);
    B.d_PK = dalloc<double>(ne * ((size_t)B.n * (B.n + 1) / 2), &err);
    B.d_S = dalloc<double>(ne * ((size_t)B.ni * (B.ni + 1) / 2), &err);
    B.d_perm = dalloc<uint32_t>(ne * B.n, &err);
    B.d_dmask = dalloc<uint8_t>(ne * B.ni, &err);
    if (condense_smem(B.ni, B.nb) > 227 * 1024)
      B.d_Yg = dalloc<double>(ne * (size_t)B.nb * (B.ni + 1), &err);
    if (err) { free_batch(c); return err; }
    CK(cudaMemcpyAsync(B.d_elist, B.elems.data(), ne * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B.d_xi, B.xi.data(), B.xi.size() * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B.d_wq, B.wq.data(), B.wq.size() * 8, cudaMemcpyHostToDevice, st));
    if (zdofd) {
      std::vector<uint8_t> dm(ne * B.ni, 0);  // element ni <= bin ni
      for (size_t j = 0; j < ne; ++j) {
        const hp3dg_elem_desc& d = desc[B.elems[j]];
        int nd[26];
        int nn = node_ndof(d.etype, d.norder, nd), k = 0;
        for (int i = 0; i < nn; ++i)
          for (int q = 0; q < nd[i]; ++q)
            dm[j * B.ni + k++] = (d.bcflag[i] && !(c->constrained && cidx[B.elems[j]] >= 0)) ? 1 : 0;
      }
      CK(cudaMemcpyAsync(B.d_dmask, dm.data(), dm.size(), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
    }
    if (c->opts.precision == HP3DG_MIXED) {
      int rc = ozaki_plan(B.nint, B.n, c->opts.ozaki_radix, c->opts.ozaki_digits, &B.plan);
      if (rc) { free_batch(c); return HP3DG_ERR_UNSUPPORTED; }
      B.d_ddig = (uint16_t*)dalloc<uint8_t>(ozaki_d_bytes(B.plan, (int)ne), &err);
      B.d_dscale = dalloc<double>(ne + 128, &err);
      // the tuning table's variant for this bin (cond, raster group); a
      // variant the bin cannot use falls back to the built-in rule
      TuneRec tr;
      if (c->opts.tune == 0 && tune_lookup(B.etype, B.n, B.nb, B.nint, HP3DG_MIXED, &tr)) {
        B.tune_cond = tr.cond;
        B.tune_grp = tr.grp;
        B.tuned = true;
      }
      const bool ok_cond_tc = !c->opts.schur_fp64 && !B.d_Yg &&
                              cond_tc_supported(B.ni, B.nb, COND_TC_DIGITS);
      const bool ok_tc_schur = !c->opts.schur_fp64 && !B.d_Yg &&
                               schur_tc_supported(B.ni, B.nb, B.plan.digits);
      int cond = B.tune_cond;
      if ((cond == 1 && !ok_cond_tc) || (cond == 2 && !ok_tc_schur)) cond = 0;
      // the condensation products have K = nb <= 64: radix 8, 6 digits keep
      // every level sum exact (below 2^23) with 21 digit pairs
      B.cond_tc = ok_cond_tc && (cond == 0 || cond == 1);
      if (B.cond_tc) {
        CondTcBufs& t = B.ctb;
        cond_tc_make_out(B.ni, B.nb, COND_TC_RADIX, COND_TC_DIGITS, t);
        t.kbd = dalloc<uint8_t>(ne * t.bytes_a, &err);
        t.lid = dalloc<uint8_t>(ne * t.bytes_b, &err);
        t.ltd = dalloc<uint8_t>(ne * t.bytes_b, &err);
        t.ekb = dalloc<int>(ne * (size_t)t.nr, &err);
        t.eli = dalloc<int>(ne * (size_t)t.nbr, &err);
        t.elt = dalloc<int>(ne * (size_t)t.nbr, &err);
        t.bi = dalloc<double>(ne * (size_t)B.ni, &err);
      }
      B.tc_schur = !B.cond_tc && ok_tc_schur && (cond == 0 || cond == 2);
      if (B.tc_schur) {
        TcFactorOut& t = B.tco;
        t.nr = schur_tc_rows(B.ni);
        t.nkb = schur_tc_kblocks(B.nb);
        t.digits = B.plan.digits;
        t.radix = B.plan.radix;
        t.ebytes = schur_tc_elem_bytes(B.ni, B.nb, B.plan.digits);
        B.d_ydig = dalloc<uint8_t>(ne * t.ebytes, &err);
        B.d_yexp = dalloc<int>(ne * (size_t)t.nr, &err);
        B.d_bi = dalloc<double>(ne * (size_t)B.ni, &err);
        t.ydig = B.d_ydig; t.yexp = B.d_yexp; t.bi = B.d_bi;
      }
      if (err) { free_batch(c); return err; }
    }
  }
  CK(cudaStreamSynchronize(st));
  c->last_desc.assign(desc, desc + nel);
  // pipelined download: chunks of the single bin at 128-element boundaries
  c->nchunk = 1;
  c->chunk_lo[0] = 0;
  c->chunk_lo[1] = nel;
  const int want = std::min(std::max((int)c->opts.download_chunks, 1), 8);
  if (want > 1 && c->bins.size() == 1 && nel >= 256 && !c->opts.keep_elem && !c->constrained) {
    const int cs = (nel + want - 1) / want;
    const int step = (cs + 127) / 128 * 128;
    int k = 0;
    for (int lo = 0; lo < nel && k < 8; lo += step) c->chunk_lo[k++] = lo;
    c->nchunk = k;
    c->chunk_lo[k] = nel;
  }
  if (int rc = build_stage_group(c)) { free_batch(c); return rc; }
  c->submitted = true;
  return HP3DG_OK;
}

}  // extern "C"

namespace {

// Marks a phase boundary for hp3dg_phase_times.  Inside a stream capture the
// record must be an external event node so that the replayed graph records it.
void mark(hp3dg_ctx* c, int i, cudaStream_t st, bool capturing) {
  if (!c->opts.timing) return;
  if (capturing) cudaEventRecordWithFlags(c->ev[i], st, cudaEventRecordExternal);
  else cudaEventRecord(c->ev[i], st);
}

// One stage of the pass for positions [j0, j1) of bin B (every per-bin
// buffer is indexed by the position in the bin, so a range is the same
// launches on offset base pointers; j0 is a multiple of 128, the block of the
// D digit tiles).  stage 0: orientation map, geometry, load, digit slicing;
// 1: contraction; 2: condensation and compression.
int enqueue_range(hp3dg_ctx* c, Bin& B, int j0, int j1, int stage, cudaStream_t st) {
  const int ne = j1 - j0;
  if (ne <= 0) return HP3DG_OK;
  const size_t npk = (size_t)B.n * (B.n + 1) / 2, nsu = (size_t)B.ni * (B.ni + 1) / 2;
  const int* el = B.d_elist + j0;
  uint32_t* perm = B.d_perm + (size_t)j0 * B.n;
  double* D = B.d_D + (size_t)j0 * B.nint * 6;
  double* F = B.d_F + (size_t)j0 * B.nint;
  double* b0 = B.d_b0 + (size_t)j0 * B.n;
  double* PK = B.d_PK + (size_t)j0 * npk;
  double* S = B.d_S + (size_t)j0 * nsu;
  uint8_t* dm = B.d_dmask + (size_t)j0 * B.ni;
  const double* zd = c->have_zdofd ? c->d_zdofd : nullptr;
  const bool mixed = c->opts.precision == HP3DG_MIXED;
  const size_t dblk = mixed ? ozaki_d_bytes(B.plan, 128) : 0;  // D digits of 128 elements
  uint16_t* ddig = mixed ? (uint16_t*)((uint8_t*)B.d_ddig + (size_t)(j0 / 128) * dblk) : nullptr;
  double* dscale = mixed ? B.d_dscale + j0 : nullptr;
  if (stage == 0 && !c->iso) {
    // the segment of this range in the stage group: bin b, or chunk k of a
    // chunked one-bin batch
    int k = 0;
    if (c->bins.size() == 1 && c->nchunk > 1) {
      while (k < c->nchunk && c->chunk_lo[k] != j0) ++k;
    } else {
      k = (int)(&B - c->bins.data());
    }
    if (k >= c->sg.nseg) return HP3DG_ERR_STATE;
    launch_stage0_grouped(c->sg, k, k + 1, c->d_norder, c->d_nori_e, c->d_nori_f, c->d_xvert,
                          c->d_kappa, c->opts.isol, c->d_flags, st);
    if (mixed && launch_slice_d_grouped(c->sg, k, k + 1, st)) return HP3DG_ERR_CUDA;
    return HP3DG_OK;
  }
  if (stage == 0) {
    launch_orient(B.etype, ne, el, c->d_norder, c->d_nori_e, c->d_nori_f, B.nord_loc, B.n, perm, st);
    launch_geom(ne, B.nvert, el, B.nint, B.n, B.d_wq, B.d_shap, B.d_grad, c->d_xvert, c->d_kappa,
                c->opts.isol, D, F, c->d_flags, st, c->iso ? c->d_xnod : nullptr, c->d_dof_off,
                perm);
    launch_load_hexa(ne, B.nint, B.n, B.d_shap, F, b0, st);
    if (mixed) launch_ozaki_slice_d(B.plan, ne, B.nint, D, ddig, dscale, st);
    return HP3DG_OK;
  }
  if (stage == 1) {
    if (mixed) {
      if (launch_ozaki_gemm(B.plan, ne, B.n, ddig, dscale, B.d_mdig, B.d_mscale, PK, c->d_flags + 2,
                            st, c->opts.fault_inject == 1 ? 1 : 0, B.tune_grp))
        return HP3DG_ERR_CUDA;
    } else {
      launch_contract_fp64(ne, B.nint, B.n, B.ni, B.nb, B.d_grad, D, PK, st);
    }
    return HP3DG_OK;
  }
  if (B.cond_tc) {
    // Cholesky + explicit inverse in FP64; Y, W = Y^T Y and ASchur on tensor
    // cores; then S = K_ii - W and the compression, through the condensation
    // group's segment of this bin or chunk
    int k = 0;
    if (c->bins.size() == 1 && c->nchunk > 1) {
      while (k < c->nchunk && c->chunk_lo[k] != j0) ++k;
    } else {
      k = (int)(&B - c->bins.data());
    }
    const int cgk = k < (int)c->cg_index.size() ? c->cg_index[k] : -1;
    if (cgk < 0) return HP3DG_ERR_STATE;
    if (launch_cond_tc_group(c->cg, cgk, cgk + 1, c->d_ni_e, c->d_nb_e, c->d_schur_off,
                             c->d_bub_off, c->d_aschur, c->d_bschur, c->d_flags + 1,
                             c->d_flags + 2, st))
      return HP3DG_ERR_CUDA;
    launch_compress_group(c->cg, cgk, cgk + 1, c->d_ni_e, c->d_wnextract, c->d_wlcon_off,
                          c->d_welem_nnz, c->d_zd_off, zd, c->d_zwork, c->d_bwork, st);
    return HP3DG_OK;
  }
  TcFactorOut tco = B.tco;
  if (B.tc_schur) {
    tco.ydig += (size_t)j0 * tco.ebytes;
    tco.yexp += (size_t)j0 * tco.nr;
    tco.bi += (size_t)j0 * B.ni;
  }
  double* Yg = B.d_Yg ? B.d_Yg + (size_t)j0 * B.nb * (B.ni + 1) : nullptr;
  if (launch_condense(ne, B.n, B.ni, B.nb, el, c->d_ni_e, c->d_nb_e, PK, b0, perm, c->d_wnextract,
                      c->d_wlcon_off, c->d_welem_nnz, c->d_schur_off, c->d_bub_off, c->d_zd_off, zd,
                      dm, S, c->d_zwork, c->d_bwork, c->d_aschur, c->d_bschur, Yg,
                      c->d_flags + 1, st, B.tc_schur ? &tco : nullptr))
    return HP3DG_ERR_CUDA;
  if (B.tc_schur) {
    // S = K_ii - Y^T Y on tensor cores, then the compression
    if (launch_schur_tc(ne, B.n, B.ni, B.nb, tco.radix, tco.digits, tco.ydig, tco.yexp, el,
                        c->d_ni_e, S, c->d_flags + 2, st))
      return HP3DG_ERR_CUDA;
    launch_compress(ne, B.n, B.ni, B.nb, el, c->d_ni_e, PK, perm, S, tco.bi, c->d_wnextract,
                    c->d_wlcon_off, c->d_welem_nnz, c->d_zd_off, zd, dm, c->d_zwork, c->d_bwork,
                    st);
  }
  return HP3DG_OK;
}

// The per-run work of the pass, enqueued on st: flags reset, the three stages
// over every bin (stage-major, with the phase timers between them) or, for a
// pipelined download, all stages chunk by chunk with an event after each
// chunk; then the global index maps.  Bin tables are built beforehand.
int enqueue_pass(hp3dg_ctx* c, cudaStream_t st, bool capturing) {
  if (cudaMemsetAsync(c->d_flags, 0x7f, 4 * sizeof(int), st) != cudaSuccess) return HP3DG_ERR_CUDA;
  if (c->nchunk > 1) {
    Bin& B = c->bins[0];
    for (int k = 0; k < c->nchunk; ++k) {
      for (int stage = 0; stage < 3; ++stage) {
        int rc = enqueue_range(c, B, c->chunk_lo[k], c->chunk_lo[k + 1], stage, st);
        if (rc) return rc;
      }
      if (capturing) cudaEventRecordWithFlags(c->chunk_ev[k], st, cudaEventRecordExternal);
      else cudaEventRecord(c->chunk_ev[k], st);
    }
    mark(c, 2, st, capturing);
    mark(c, 3, st, capturing);
    mark(c, 4, st, capturing);
  } else if (c->bins.size() == 1) {
    for (int stage = 0; stage < 3; ++stage) {
      int rc = enqueue_range(c, c->bins[0], 0, (int)c->bins[0].elems.size(), stage, st);
      if (rc) return rc;
      mark(c, 2 + stage, st, capturing);
    }
  } else {
    // bins on parallel branches (largest estimated work first, each to the
    // least loaded branch); a captured graph keeps the branches as
    // independent paths, so small bins' kernels run side by side
    const int nb = (int)c->bins.size();
    std::vector<int> order(nb);
    std::vector<double> work(nb);
    for (int b = 0; b < nb; ++b) {
      order[b] = b;
      const Bin& B = c->bins[b];
      work[b] = (double)B.elems.size() * B.nint * B.n * (double)B.n + 1e6;
    }
    std::sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
    double load[hp3dg_ctx::NBRANCH] = {0};
    std::vector<int> owner(nb);
    for (int b : order) {
      int k = 0;
      for (int j = 1; j < hp3dg_ctx::NBRANCH; ++j)
        if (load[j] < load[k]) k = j;
      owner[b] = k;
      load[k] += work[b];
    }
    auto fork = [&]() -> bool {
      if (cudaEventRecord(c->fork_ev, st) != cudaSuccess) return false;
      for (int k = 0; k < hp3dg_ctx::NBRANCH; ++k)
        if (cudaStreamWaitEvent(c->branch[k], c->fork_ev, 0) != cudaSuccess) return false;
      return true;
    };
    auto join = [&]() -> bool {
      for (int k = 0; k < hp3dg_ctx::NBRANCH; ++k) {
        if (cudaEventRecord(c->join_ev[k], c->branch[k]) != cudaSuccess) return false;
        if (cudaStreamWaitEvent(st, c->join_ev[k], 0) != cudaSuccess) return false;
      }
      return true;
    };
    const bool mixed = c->opts.precision == HP3DG_MIXED;
    // Stage 0 (orientation maps, geometry, loads, digit slicing) of every
    // bin in one launch per kernel over the segment tables (vertex geometry);
    // in mixed precision the contractions of all bins as one persistent
    // launch over their joint tile space; the rest per bin on the branches.
    const bool grouped0 = c->sg.nseg == (int)c->bins.size() && !c->iso;
    if (grouped0) {
      launch_stage0_grouped(c->sg, 0, c->sg.nseg, c->d_norder, c->d_nori_e, c->d_nori_f,
                            c->d_xvert, c->d_kappa, c->opts.isol, c->d_flags, st);
      if (mixed && launch_slice_d_grouped(c->sg, 0, c->sg.nseg, st)) return HP3DG_ERR_CUDA;
    } else {
      if (!fork()) return HP3DG_ERR_CUDA;
      for (int b : order) {
        Bin& B = c->bins[b];
        int rc = enqueue_range(c, B, 0, (int)B.elems.size(), 0, c->branch[owner[b]]);
        if (rc) return rc;
      }
      if (!join()) return HP3DG_ERR_CUDA;
    }
    if (mixed) {
      std::vector<OzakiGemmItem> items;
      for (int b : order) {
        Bin& B = c->bins[b];
        items.push_back({&B.plan, (int)B.elems.size(), B.n * (B.n + 1) / 2, B.d_ddig, B.d_dscale,
                         B.d_mdig, B.d_mscale, B.d_PK, B.tune_grp});
      }
      if (launch_ozaki_gemm_group(items.data(), (int)items.size(), c->d_flags + 2, st,
                                  c->opts.fault_inject == 1 ? 1 : 0))
        return HP3DG_ERR_CUDA;
    }
    if (!fork()) return HP3DG_ERR_CUDA;
    // the condensation of every bin in the condensation group (the
    // tensor-core path, and bins without bubbles): one launch per kernel, on
    // the main stream beside the branches that condense the other bins (in
    // FP64 after them, once every bin's contraction is done)
    const bool grouped2 = c->cg.nseg > 0;
    auto cond_group = [&]() -> int {
      const double* zd = c->have_zdofd ? c->d_zdofd : nullptr;
      if (launch_cond_tc_group(c->cg, 0, c->cg.ntc, c->d_ni_e, c->d_nb_e, c->d_schur_off,
                               c->d_bub_off, c->d_aschur, c->d_bschur, c->d_flags + 1,
                               c->d_flags + 2, st))
        return HP3DG_ERR_CUDA;
      launch_compress_group(c->cg, 0, c->cg.nseg, c->d_ni_e, c->d_wnextract, c->d_wlcon_off,
                            c->d_welem_nnz, c->d_zd_off, zd, c->d_zwork, c->d_bwork, st);
      return HP3DG_OK;
    };
    if (grouped2 && mixed && cond_group()) return HP3DG_ERR_CUDA;
    for (int b : order)
      for (int stage = mixed ? 2 : 1; stage < 3; ++stage) {
        Bin& B = c->bins[b];
        if (grouped2 && stage == 2 && c->cg_index[b] >= 0) continue;
        int rc = enqueue_range(c, B, 0, (int)B.elems.size(), stage, c->branch[owner[b]]);
        if (rc) return rc;
      }
    if (!join()) return HP3DG_ERR_CUDA;
    if (grouped2 && !mixed && cond_group()) return HP3DG_ERR_CUDA;
    // the per-stage timers are not meaningful across branches
    mark(c, 2, st, capturing);
    mark(c, 3, st, capturing);
    mark(c, 4, st, capturing);
  }
  if (c->constrained) launch_constrain(c->nel, c->cargs, st);
  launch_index_maps(c->nel, c->node_stride, c->nnodes, c->d_nodes, c->d_ndofm, c->d_lcon_off,
                    c->d_first, c->d_cnt, c->d_scan, c->d_blk, c->d_total, c->d_nfirst, c->d_lcon,
                    st);
  mark(c, 5, st, capturing);
  return cudaPeekAtLastError() == cudaSuccess ? HP3DG_OK : HP3DG_ERR_CUDA;
}

}  // namespace

extern "C" {

int hp3dg_batch_run(hp3dg_ctx* c) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  int err = 0;
  mark(c, 0, st, false);
  // tables (once per bin; they stay resident across runs)
  for (auto& B : c->bins) {
    if (!B.tables) {
      launch_tables(B.etype, B.nord_loc, B.face_nori, B.nint, B.n, B.d_xi, B.d_shap, B.d_grad, st);
      B.tables = true;
    }
    if (c->opts.precision == HP3DG_MIXED && !B.mtable) {
      B.d_mdig = (uint16_t*)dalloc<uint8_t>(ozaki_m_bytes(B.plan), &err);
      B.d_mscale = dalloc<double>(B.plan.ncols, &err);
      double* work = dalloc<double>((size_t)B.plan.kdim * 64, &err);
      if (err) { cudaFree(work); return err; }
      int rc = launch_ozaki_build_m(B.plan, B.nint, B.n, B.ni, B.nb, B.d_grad, B.d_mdig,
                                    B.d_mscale, work, st);
      cudaStreamSynchronize(st);
      cudaFree(work);
      if (rc) return HP3DG_ERR_CUDA;
      B.mtable = true;
    }
  }
  mark(c, 1, st, false);
  if (c->opts.launch_mode == 1) {
    int rc = enqueue_pass(c, st, false);
    if (rc) return rc;
  } else {
    if (!c->graph) {
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
      int rc = enqueue_pass(c, st, true);
      cudaError_t ce = cudaStreamEndCapture(st, &g);
      if (rc || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc ? rc : HP3DG_ERR_CUDA;
      }
      size_t nn = 0;
      c->graph_kernels = 0;
      if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn) {
        std::vector<cudaGraphNode_t> nodes(nn);
        if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
          for (size_t i = 0; i < nn; ++i) {
            cudaGraphNodeType ty;
            if (cudaGraphNodeGetType(nodes[i], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
              ++c->graph_kernels;
          }
      }
      ce = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) { c->graph = nullptr; return HP3DG_ERR_CUDA; }
    }
    CK(cudaGraphLaunch(c->graph, st));
  }
  c->ran = true;
  c->downloaded = false;
  c->chunked_run = c->nchunk > 1;
  return HP3DG_OK;
}

int hp3dg_batch_sync(hp3dg_ctx* c) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->ran) return HP3DG_ERR_STATE;
  cudaSetDevice(c->device);
  CK(cudaStreamSynchronize(c->stream));
  int fl[4];
  CK(cudaMemcpy(fl, c->d_flags, sizeof(fl), cudaMemcpyDeviceToHost));
  if (c->opts.timing) {
    for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&c->times[i], c->ev[i], c->ev[i + 1]);
    cudaEventElapsedTime(&c->times[5], c->ev[0], c->ev[5]);
  }
  const int NONE = 0x7f7f7f7f;
  c->last_bad = -1;
  // a bad Jacobian is an input error found before the products; a timeout of
  // a tensor-core kernel leaves the later stages reading unfinished data, so
  // it is reported before what those stages flagged
  if (fl[0] != NONE) { c->last_bad = fl[0]; return HP3DG_ERR_NEG_JACOBIAN; }
  if (fl[2] != NONE) return HP3DG_ERR_TIMEOUT;  // a bounded wait of the tensor-core kernel gave up
  if (fl[1] != NONE) { c->last_bad = fl[1]; return HP3DG_ERR_NOT_SPD; }
  return HP3DG_OK;
}

int hp3dg_batch_download(hp3dg_ctx* c) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->ran) return HP3DG_ERR_STATE;
  cudaSetDevice(c->device);
  int nel = c->nel;
  auto hal = [](void** p, size_t bytes) {
    if (*p) return true;
    return cudaMallocHost(p, bytes ? bytes : 8) == cudaSuccess;
  };
  if (!hal((void**)&c->h_zastif, c->elem_nnz[nel] * 8) || !hal((void**)&c->h_zbload, c->lcon_off[nel] * 8) ||
      !hal((void**)&c->h_aschur, c->schur_off[nel] * 8) || !hal((void**)&c->h_bschur, c->bub_off[nel] * 8) ||
      !hal((void**)&c->h_lcon, c->lcon_off[nel] * 4) || !hal((void**)&c->h_nfirst, (size_t)c->nnodes * 4))
    return HP3DG_ERR_ALLOC;
  cudaStream_t st = c->stream;
  if (c->chunked_run) {
    // each chunk's outputs (contiguous in element order) as soon as its event
    // fires, on the copy stream, while the pass continues on st
    cudaStream_t cs = c->copy_stream;
    for (int k = 0; k < c->nchunk; ++k) {
      const int e0 = c->chunk_lo[k], e1 = c->chunk_lo[k + 1];
      CK(cudaStreamWaitEvent(cs, c->chunk_ev[k], 0));
      CK(cudaMemcpyAsync(c->h_zastif + c->elem_nnz[e0], c->d_zastif + c->elem_nnz[e0],
                         (c->elem_nnz[e1] - c->elem_nnz[e0]) * 8, cudaMemcpyDeviceToHost, cs));
      CK(cudaMemcpyAsync(c->h_zbload + c->lcon_off[e0], c->d_zbload + c->lcon_off[e0],
                         (c->lcon_off[e1] - c->lcon_off[e0]) * 8, cudaMemcpyDeviceToHost, cs));
      CK(cudaMemcpyAsync(c->h_aschur + c->schur_off[e0], c->d_aschur + c->schur_off[e0],
                         (c->schur_off[e1] - c->schur_off[e0]) * 8, cudaMemcpyDeviceToHost, cs));
      CK(cudaMemcpyAsync(c->h_bschur + c->bub_off[e0], c->d_bschur + c->bub_off[e0],
                         (c->bub_off[e1] - c->bub_off[e0]) * 8, cudaMemcpyDeviceToHost, cs));
    }
    // the index maps come last in the pass
    int rc = hp3dg_batch_sync(c);
    if (rc != HP3DG_OK) { cudaStreamSynchronize(cs); return rc; }
    CK(cudaMemcpyAsync(c->h_lcon, c->d_lcon, c->lcon_off[nel] * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(c->h_nfirst, c->d_nfirst, (size_t)c->nnodes * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&c->h_nrdof, c->d_total, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(cs));
    CK(cudaStreamSynchronize(st));
    c->downloaded = true;
    return HP3DG_OK;
  }
  int rc = hp3dg_batch_sync(c);
  if (rc != HP3DG_OK) return rc;
  CK(cudaMemcpyAsync(c->h_zastif, c->d_zastif, c->elem_nnz[nel] * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_zbload, c->d_zbload, c->lcon_off[nel] * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_aschur, c->d_aschur, c->schur_off[nel] * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_bschur, c->d_bschur, c->bub_off[nel] * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_lcon, c->d_lcon, c->lcon_off[nel] * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(c->h_nfirst, c->d_nfirst, (size_t)c->nnodes * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&c->h_nrdof, c->d_total, 8, cudaMemcpyDeviceToHost, st));
  if (c->opts.keep_elem) {
    c->pk_off.assign(nel, 0); c->b0_off.assign(nel, 0);
    size_t pk = 0, b0 = 0;
    for (auto& B : c->bins) { pk += B.elems.size() * ((size_t)B.n * (B.n + 1) / 2); b0 += B.elems.size() * B.n; }
    if (!hal((void**)&c->h_PK, pk * 8) || !hal((void**)&c->h_b0, b0 * 8)) return HP3DG_ERR_ALLOC;
    size_t po = 0, bo = 0;
    for (auto& B : c->bins) {
      size_t ne = B.elems.size(), pe = (size_t)B.n * (B.n + 1) / 2;
      CK(cudaMemcpyAsync(c->h_PK + po, B.d_PK, ne * pe * 8, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(c->h_b0 + bo, B.d_b0, ne * B.n * 8, cudaMemcpyDeviceToHost, st));
      for (size_t j = 0; j < ne; ++j) { c->pk_off[B.elems[j]] = po + j * pe; c->b0_off[B.elems[j]] = bo + j * B.n; }
      po += ne * pe; bo += ne * B.n;
    }
  }
  CK(cudaStreamSynchronize(st));
  c->downloaded = true;
  return HP3DG_OK;
}

int hp3dg_get_elem(const hp3dg_ctx* c, int32_t iel, double* aloc, int32_t ld, double* bloc) {
  if (!c || !aloc || !bloc) return HP3DG_ERR_ARG;
  if (!c->downloaded || !c->opts.keep_elem) return HP3DG_ERR_STATE;
  if (iel < 0 || iel >= c->nel) return HP3DG_ERR_ARG;
  int n = c->n_e[iel];
  if (ld < n) return HP3DG_ERR_ARG;
  const Bin& B = c->bins[c->bin_of[iel]];
  const int ni = B.ni, nb = B.nb;  // the packed matrix is the bin element's
  // dof map of this element (same map the device uses)
  int no[19], oe[12], of[6];
  // descriptors are not kept on the host; recompute the map from device copies
  cudaMemcpy(no, c->d_norder + 19 * (size_t)iel, sizeof(no), cudaMemcpyDeviceToHost);
  cudaMemcpy(oe, c->d_nori_e + 12 * (size_t)iel, sizeof(oe), cudaMemcpyDeviceToHost);
  cudaMemcpy(of, c->d_nori_f + 6 * (size_t)iel, sizeof(of), cudaMemcpyDeviceToHost);
  const double* PK = c->h_PK + c->pk_off[iel];
  const double* b0 = c->h_b0 + c->b0_off[iel];
  auto dmap = [&](int a) {
    if (B.etype == HP3DG_TET) return tet_dof_map(a, no, oe, of, B.nord_loc[0]);
    if (B.etype == HP3DG_PRISM) return prism_dof_map(a, no, oe, of, B.nord_loc);
    return hexa_dof_map(a, no, oe, of, B.nord_loc);
  };
  for (int a = 0; a < n; ++a) {
    uint32_t ma = dmap(a);
    int ra = (int)(ma & 0x7fffffffu);
    bloc[a] = (ma & 0x80000000u) ? -b0[ra] : b0[ra];
    for (int b = 0; b < n; ++b) {
      uint32_t mb = dmap(b);
      int rb = (int)(mb & 0x7fffffffu);
      double v = PK[pk_index(ra, rb, ni, nb)];
      aloc[(size_t)b * ld + a] = ((ma ^ mb) & 0x80000000u) ? -v : v;
    }
  }
  return HP3DG_OK;
}

int hp3dg_get_condensed(const hp3dg_ctx* c, int32_t iel, double* zbload, double* zastif,
                        int32_t* nrdofc) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->downloaded) return HP3DG_ERR_STATE;
  if (iel < 0 || iel >= c->nel) return HP3DG_ERR_ARG;
  int64_t nc = c->lcon_off[iel + 1] - c->lcon_off[iel];
  if (nrdofc) *nrdofc = (int32_t)nc;
  if (zbload) std::memcpy(zbload, c->h_zbload + c->lcon_off[iel], nc * 8);
  if (zastif) std::memcpy(zastif, c->h_zastif + c->elem_nnz[iel], nc * nc * 8);
  return HP3DG_OK;
}

int hp3dg_get_schur(const hp3dg_ctx* c, int32_t iel, double* aschur, double* bschur,
                    int32_t* nb, int32_t* ni) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->downloaded) return HP3DG_ERR_STATE;
  if (iel < 0 || iel >= c->nel) return HP3DG_ERR_ARG;
  if (nb) *nb = c->nb_e[iel];
  if (ni) *ni = c->ni_e[iel];
  if (aschur) std::memcpy(aschur, c->h_aschur + c->schur_off[iel], (c->schur_off[iel + 1] - c->schur_off[iel]) * 8);
  if (bschur) std::memcpy(bschur, c->h_bschur + c->bub_off[iel], (c->bub_off[iel + 1] - c->bub_off[iel]) * 8);
  return HP3DG_OK;
}

int hp3dg_index_map(const hp3dg_ctx* c, int32_t* nfirst_dof, int64_t* elem_nnz,
                    int64_t* lcon_off, int32_t* lcon, int64_t* nrdof) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->downloaded) return HP3DG_ERR_STATE;
  if (nfirst_dof) std::memcpy(nfirst_dof, c->h_nfirst, (size_t)c->nnodes * 4);
  if (elem_nnz) std::memcpy(elem_nnz, c->elem_nnz.data(), (c->nel + 1) * 8);
  if (lcon_off) std::memcpy(lcon_off, c->lcon_off.data(), (c->nel + 1) * 8);
  if (lcon) std::memcpy(lcon, c->h_lcon, c->lcon_off[c->nel] * 4);
  if (nrdof) *nrdof = c->h_nrdof;
  return HP3DG_OK;
}

int hp3dg_batch_set_geometry(hp3dg_ctx* c, const double* xnod) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  CK(cudaStreamSynchronize(st));
  const int64_t ndof = c->nel > 0 ? c->dof_off[c->nel] : 0;
  if (xnod && ndof > 0) {
    if (!c->d_xnod && cudaMalloc(&c->d_xnod, (size_t)ndof * 3 * sizeof(double)) != cudaSuccess) {
      c->d_xnod = nullptr;
      return HP3DG_ERR_ALLOC;
    }
    CK(cudaMemcpyAsync(c->d_xnod, xnod, (size_t)ndof * 3 * sizeof(double), cudaMemcpyHostToDevice,
                       st));
    CK(cudaStreamSynchronize(st));
  }
  // the geometry kernel is part of the captured pass: capture again
  if (c->graph) cudaGraphExecDestroy(c->graph);
  c->graph = nullptr;
  c->graph_kernels = -1;
  c->iso = xnod != nullptr && ndof > 0;
  c->ran = c->downloaded = c->have_dofs = false;
  return HP3DG_OK;
}

int hp3dg_backsub(hp3dg_ctx* c, const double* x_global) {
  if (!c || !x_global) return HP3DG_ERR_ARG;
  if (!c->ran) return HP3DG_ERR_STATE;
  if (c->constrained) return HP3DG_ERR_UNSUPPORTED;
  cudaSetDevice(c->device);
  int rc = hp3dg_batch_sync(c);
  if (rc != HP3DG_OK) return rc;
  cudaStream_t st = c->stream;
  int err = 0;
  // nrdof is known after the index maps ran
  int64_t nrdof = 0;
  CK(cudaMemcpy(&nrdof, c->d_total, 8, cudaMemcpyDeviceToHost));
  if (!c->d_xglob) c->d_xglob = dalloc<double>(nrdof > 0 ? nrdof : 1, &err);
  if (!c->d_dofs) c->d_dofs = dalloc<double>(c->dof_off[c->nel], &err);
  if (err) return err;
  if (!c->h_dofs && cudaMallocHost((void**)&c->h_dofs, c->dof_off[c->nel] * 8 + 8) != cudaSuccess)
    return HP3DG_ERR_ALLOC;
  CK(cudaMemcpyAsync(c->d_xglob, x_global, nrdof * 8, cudaMemcpyHostToDevice, st));
  for (auto& B : c->bins)
    launch_backsub((int)B.elems.size(), B.ni, B.d_elist, c->d_ni_e, c->d_nb_e, c->d_nextract,
                   c->d_lcon_off, c->d_lcon, c->d_xglob, c->d_zd_off,
                   c->have_zdofd ? c->d_zdofd : nullptr, c->d_schur_off, c->d_bub_off,
                   c->d_aschur, c->d_bschur, c->d_dof_off, c->d_dofs, st);
  CK(cudaMemcpyAsync(c->h_dofs, c->d_dofs, c->dof_off[c->nel] * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (cudaPeekAtLastError() != cudaSuccess) return HP3DG_ERR_CUDA;
  c->have_dofs = true;
  return HP3DG_OK;
}

int hp3dg_get_dofs(const hp3dg_ctx* c, int32_t iel, double* dof, int32_t* n) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->have_dofs) return HP3DG_ERR_STATE;
  if (iel < 0 || iel >= c->nel) return HP3DG_ERR_ARG;
  if (n) *n = c->n_e[iel];
  if (dof) std::memcpy(dof, c->h_dofs + c->dof_off[iel], c->n_e[iel] * 8);
  return HP3DG_OK;
}

int hp3dg_element_error(hp3dg_ctx* c, int32_t isol, double* err2, double* nrm2) {
  if (c && c->iso) return HP3DG_ERR_UNSUPPORTED;  // vertex geometry only
  if (!c || !err2 || !nrm2) return HP3DG_ERR_ARG;
  if (!c->have_dofs) return HP3DG_ERR_STATE;
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  int err = 0;
  if (!c->d_err2) c->d_err2 = dalloc<double>(c->nel, &err);
  if (!c->d_nrm2) c->d_nrm2 = dalloc<double>(c->nel, &err);
  if (err) return err;
  for (auto& B : c->bins) {
    if (!B.etable) {
      B.nint_err = bin_quadrature(B.etype, B.nord_loc, 2, B.xi_err, B.wq_err);
      B.d_xi_err = dalloc<double>(B.xi_err.size(), &err);
      B.d_wq_err = dalloc<double>(B.wq_err.size(), &err);
      B.d_shap_err = dalloc<double>((size_t)B.nint_err * B.n, &err);
      B.d_grad_err = dalloc<double>((size_t)B.nint_err * 3 * B.n, &err);
      if (err) return err;
      CK(cudaMemcpyAsync(B.d_xi_err, B.xi_err.data(), B.xi_err.size() * 8, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(B.d_wq_err, B.wq_err.data(), B.wq_err.size() * 8, cudaMemcpyHostToDevice, st));
      launch_tables(B.etype, B.nord_loc, B.face_nori, B.nint_err, B.n, B.d_xi_err, B.d_shap_err,
                    B.d_grad_err, st);
      CK(cudaStreamSynchronize(st));
      B.etable = true;
    }
    launch_element_error((int)B.elems.size(), B.nvert, B.nint_err, B.n, isol, B.d_elist, c->d_n_e, B.d_wq_err,
                         B.d_shap_err, B.d_grad_err, c->d_xvert, B.d_perm, c->d_dof_off, c->d_dofs,
                         c->d_err2, c->d_nrm2, st);
  }
  CK(cudaMemcpyAsync(err2, c->d_err2, (size_t)c->nel * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(nrm2, c->d_nrm2, (size_t)c->nel * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return cudaPeekAtLastError() == cudaSuccess ? HP3DG_OK : HP3DG_ERR_CUDA;
}

int hp3dg_adjoint(hp3dg_ctx* c, const double* dofs, double* djdkappa, double* djdx) {
  if (c && c->iso) return HP3DG_ERR_UNSUPPORTED;  // vertex geometry only
  if (!c || !djdkappa || !djdx) return HP3DG_ERR_ARG;
  if (!c->ran) return HP3DG_ERR_STATE;
  if (c->constrained) return HP3DG_ERR_UNSUPPORTED;
  if (!dofs && !c->have_dofs) return HP3DG_ERR_STATE;
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  int err = 0;
  if (!c->d_dofs) c->d_dofs = dalloc<double>(c->dof_off[c->nel], &err);
  if (!c->d_djdk) c->d_djdk = dalloc<double>(c->nel, &err);
  if (!c->d_djdx) c->d_djdx = dalloc<double>((size_t)c->nel * 24, &err);
  if (err) return err;
  if (dofs) CK(cudaMemcpyAsync(c->d_dofs, dofs, c->dof_off[c->nel] * 8, cudaMemcpyHostToDevice, st));
  for (auto& B : c->bins)
    launch_adjoint((int)B.elems.size(), B.nvert, B.nint, B.n, c->opts.isol, B.d_elist, c->d_n_e, B.d_wq, B.d_shap,
                   B.d_grad, c->d_xvert, c->d_kappa, B.d_perm, c->d_dof_off, c->d_dofs, c->d_djdk,
                   c->d_djdx, st);
  CK(cudaMemcpyAsync(djdkappa, c->d_djdk, (size_t)c->nel * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(djdx, c->d_djdx, (size_t)c->nel * 24 * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return cudaPeekAtLastError() == cudaSuccess ? HP3DG_OK : HP3DG_ERR_CUDA;
}

int hp3dg_output_sizes(const hp3dg_ctx* c, int64_t* nnz, int64_t* lcon, int64_t* schur,
                       int64_t* bub) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  if (nnz) *nnz = c->elem_nnz[c->nel];
  if (lcon) *lcon = c->lcon_off[c->nel];
  if (schur) *schur = c->schur_off[c->nel];
  if (bub) *bub = c->bub_off[c->nel];
  return HP3DG_OK;
}

int hp3dg_device_outputs(const hp3dg_ctx* c, const double** zastif, const double** zbload,
                         const double** aschur, const double** bschur, const int32_t** lcon) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  if (zastif) *zastif = c->d_zastif;
  if (zbload) *zbload = c->d_zbload;
  if (aschur) *aschur = c->d_aschur;
  if (bschur) *bschur = c->d_bschur;
  if (lcon) *lcon = c->d_lcon;
  return HP3DG_OK;
}

int hp3dg_phase_times(const hp3dg_ctx* c, float* ms, int32_t n) {
  if (!c || !ms || n < 0) return HP3DG_ERR_ARG;
  for (int i = 0; i < n && i < 6; ++i) ms[i] = c->times[i];
  return HP3DG_OK;
}

int hp3dg_mixed_config(const hp3dg_ctx* c, int32_t* radix, int32_t* digits, int32_t* pairs) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted || c->opts.precision != HP3DG_MIXED || c->bins.empty()) return HP3DG_ERR_STATE;
  const OzakiPlan& p = c->bins[0].plan;
  if (radix) *radix = p.radix;
  if (digits) *digits = p.digits;
  if (pairs) *pairs = ozaki_pairs(p);
  return HP3DG_OK;
}

int hp3dg_bin_info(const hp3dg_ctx* c, int32_t* nbins, int32_t b, int32_t* info,
                   int32_t* bin_of) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  if (nbins) *nbins = (int32_t)c->bins.size();
  if (info) {
    if (b < 0 || b >= (int)c->bins.size()) return HP3DG_ERR_ARG;
    const Bin& B = c->bins[b];
    info[0] = B.etype; info[1] = B.n; info[2] = B.nb; info[3] = B.nint;
    info[4] = (int32_t)B.elems.size();
    info[5] = B.cond_tc ? 1 : (B.tc_schur ? 2 : 3);
    info[6] = B.tune_grp;
    info[7] = B.tuned ? 1 : 0;
  }
  if (bin_of)
    for (int e = 0; e < c->nel; ++e) bin_of[e] = c->bin_of[e];
  return HP3DG_OK;
}

int hp3dg_pass_stats(const hp3dg_ctx* c, int64_t* kernels, double* contraction_flops) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  if (kernels) *kernels = c->graph ? c->graph_kernels : -1;
  if (contraction_flops) {
    double f = 0.0;
    for (const auto& B : c->bins) {
      const double ne = (double)B.elems.size(), n = B.n, nint = B.nint;
      if (c->opts.precision == HP3DG_MIXED)
        f += ne * ozaki_pairs(B.plan) * 2.0 * (6.0 * nint) * (n * (n + 1) / 2);
      else
        f += ne * n * (n + 1) * 3.0 * nint;
    }
    *contraction_flops = f;
  }
  return HP3DG_OK;
}

int hp3dg_dirichlet_dofs(hp3dg_ctx* c, int32_t isol, double* zdofd, int64_t* n) {
  if (c && c->iso) return HP3DG_ERR_UNSUPPORTED;  // vertex geometry only
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  const int nel = c->nel;
  if (n) *n = nel > 0 ? c->zd_off[nel] : 0;
  if (!zdofd || nel == 0) return HP3DG_OK;
  if ((int)c->last_desc.size() != nel) return HP3DG_ERR_STATE;
  for (int e = 0; e < nel; ++e)
    if (c->etype_e[e] != HP3DG_HEXA) return HP3DG_ERR_UNSUPPORTED;
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  std::vector<int> bc((size_t)nel * 26);
  for (int e = 0; e < nel; ++e)
    for (int i = 0; i < 26; ++i) bc[(size_t)e * 26 + i] = c->last_desc[e].bcflag[i] ? 1 : 0;
  std::vector<double> gx(16 * 11, 0.0), gw(16 * 11, 0.0);
  for (int m = 1; m <= 10; ++m) gauss_rule01(m, &gx[16 * m], &gw[16 * m]);
  int *d_bc = nullptr, *d_bad = nullptr;
  double *d_gx = nullptr, *d_gw = nullptr, *d_work = nullptr, *d_zd = nullptr;
  int rc = HP3DG_OK;
  const size_t nz = c->zd_off[nel];
  if (cudaMalloc(&d_bc, bc.size() * 4) != cudaSuccess || cudaMalloc(&d_bad, 4) != cudaSuccess ||
      cudaMalloc(&d_gx, gx.size() * 8) != cudaSuccess || cudaMalloc(&d_gw, gw.size() * 8) != cudaSuccess ||
      cudaMalloc(&d_work, dirichlet_work_doubles(nel) * 8) != cudaSuccess ||
      cudaMalloc(&d_zd, nz * 8) != cudaSuccess)
    rc = HP3DG_ERR_ALLOC;
  int badv = 0x7f7f7f7f;
  if (rc == HP3DG_OK &&
      (cudaMemcpyAsync(d_bc, bc.data(), bc.size() * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
       cudaMemcpyAsync(d_gx, gx.data(), gx.size() * 8, cudaMemcpyHostToDevice, st) != cudaSuccess ||
       cudaMemcpyAsync(d_gw, gw.data(), gw.size() * 8, cudaMemcpyHostToDevice, st) != cudaSuccess ||
       cudaMemcpyAsync(d_bad, &badv, 4, cudaMemcpyHostToDevice, st) != cudaSuccess))
    rc = HP3DG_ERR_CUDA;
  if (rc == HP3DG_OK) {
    launch_dirichlet(nel, c->d_norder, c->d_nori_e, c->d_nori_f, d_bc, c->d_xvert, c->d_zd_off,
                     d_gx, d_gw, isol, d_work, d_zd, d_bad, st);
    if (cudaMemcpyAsync(zdofd, d_zd, nz * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&badv, d_bad, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = HP3DG_ERR_CUDA;
    else if (badv != 0x7f7f7f7f) {
      c->last_bad = badv;
      rc = HP3DG_ERR_NOT_SPD;
    }
  }
  cudaFree(d_bc); cudaFree(d_bad); cudaFree(d_gx); cudaFree(d_gw); cudaFree(d_work); cudaFree(d_zd);
  return rc;
}

}  // extern "C"

namespace {

// hexahedron reference vertices, edge and face vertex lists (element_data.F90)
const double HBRICK_XI[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
const int HBRICK_E2V[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6},
                               {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int HBRICK_F2V[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                              {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}};
const int HBRICK_F2E[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 9, 4, 8},
                              {1, 10, 5, 9}, {2, 10, 6, 11}, {3, 11, 7, 8}};

void hexa_node_counts(const int* nord, int* first) {
  first[0] = 0;
  for (int i = 0; i < 27; ++i) {
    int n;
    if (i < 8) n = 1;
    else if (i < 20) n = std::max(nord[i - 8] - 1, 0);
    else if (i < 26) { int a, b; decod2(nord[12 + i - 20], a, b); n = std::max(a - 1, 0) * std::max(b - 1, 0); }
    else { int x, y, z; decod3(nord[18], x, y, z); n = std::max(x - 1, 0) * std::max(y - 1, 0) * std::max(z - 1, 0); }
    first[i + 1] = first[i] + n;
  }
}

// The projection points of every element (hexahedra): per element its 8
// vertices, then per edge, face and the interior with dof the points of
// set_1Dint / set_2Dint (face_order) / set_3Dint at INTEGRATION = integration
// (xi and the rule's weight: 4 doubles per point), and per element the start
// of each node's points (28 entries, the last one its end).  nmax: the
// largest node dof count.
int gdof_points_build(const hp3dg_ctx* c, std::vector<double>& pts, std::vector<int64_t>& node_pt,
                      int* nmax) {
  const int nel = c->nel, I = c->opts.integration;
  if ((int)c->last_desc.size() != nel) return HP3DG_ERR_STATE;
  pts.clear();
  node_pt.assign((size_t)nel * 28, 0);
  *nmax = 1;
  double gx[16], gw[16], hx[16], hw[16];
  for (int e = 0; e < nel; ++e) {
    const hp3dg_elem_desc& d = c->last_desc[e];
    if (d.etype != HP3DG_HEXA) return HP3DG_ERR_UNSUPPORTED;
    int first[28];
    hexa_node_counts(d.norder, first);
    int64_t* np = &node_pt[(size_t)e * 28];
    auto put = [&](const double* xi, double w) {
      pts.push_back(xi[0]); pts.push_back(xi[1]); pts.push_back(xi[2]); pts.push_back(w);
    };
    for (int v = 0; v < 8; ++v) {
      np[v] = (int64_t)pts.size() / 4;
      put(HBRICK_XI[v], 1.0);
    }
    for (int id = 0; id < 12; ++id) {
      np[8 + id] = (int64_t)pts.size() / 4;
      if (first[9 + id] == first[8 + id]) continue;
      *nmax = std::max(*nmax, first[9 + id] - first[8 + id]);
      const int nint = std::min(d.norder[id] + I, MAXP) + 1;
      gauss_rule01(nint, gx, gw);
      const double *x1 = HBRICK_XI[HBRICK_E2V[id][0]], *x2 = HBRICK_XI[HBRICK_E2V[id][1]];
      for (int l = 0; l < nint; ++l) {
        double xi[3];
        for (int q = 0; q < 3; ++q) xi[q] = x1[q] + gx[l] * (x2[q] - x1[q]);
        put(xi, gw[l]);
      }
    }
    for (int id = 0; id < 6; ++id) {
      np[20 + id] = (int64_t)pts.size() / 4;
      if (first[21 + id] == first[20 + id]) continue;
      *nmax = std::max(*nmax, first[21 + id] - first[20 + id]);
      int h, v;
      decod2(d.norder[12 + id], h, v);
      const int* fe = HBRICK_F2E[id];
      const int nx = std::min(std::max(std::max(d.norder[fe[0]], d.norder[fe[2]]), h) + I, MAXP) + 1;
      const int ny = std::min(std::max(std::max(d.norder[fe[1]], d.norder[fe[3]]), v) + I, MAXP) + 1;
      gauss_rule01(nx, gx, gw);
      gauss_rule01(ny, hx, hw);
      const double *v1 = HBRICK_XI[HBRICK_F2V[id][0]], *v2 = HBRICK_XI[HBRICK_F2V[id][1]],
                   *v3 = HBRICK_XI[HBRICK_F2V[id][3]];
      for (int l2 = 0; l2 < ny; ++l2)
        for (int l1 = 0; l1 < nx; ++l1) {
          double xi[3];
          for (int q = 0; q < 3; ++q)
            xi[q] = v1[q] + gx[l1] * (v2[q] - v1[q]) + hx[l2] * (v3[q] - v1[q]);
          put(xi, gw[l1] * hw[l2]);
        }
    }
    np[26] = (int64_t)pts.size() / 4;
    if (first[27] > first[26]) {
      *nmax = std::max(*nmax, first[27] - first[26]);
      int loc[19];
      hexa_order_loc(d.norder, d.nori_face, loc);
      std::vector<double> xq, wq;
      hexa_quadrature(loc, I, xq, wq);
      for (size_t l = 0; l < wq.size(); ++l) put(&xq[3 * l], wq[l]);
    }
    np[27] = (int64_t)pts.size() / 4;
  }
  return HP3DG_OK;
}

// eta(xi): trilinear in the element's vertex coordinates in the block
void eta_trilinear(const double* ev, const double* xi, double* eta) {
  for (int q = 0; q < 3; ++q) eta[q] = 0.0;
  for (int v = 0; v < 8; ++v) {
    double b = 1.0;
    for (int a = 0; a < 3; ++a) b *= HBRICK_XI[v][a] > 0.5 ? xi[a] : 1.0 - xi[a];
    for (int q = 0; q < 3; ++q) eta[q] += ev[3 * v + q] * b;
  }
}

}  // namespace

extern "C" {

int hp3dg_gdof_points(hp3dg_ctx* c, const double* etav, double* eta, int64_t* npts) {
  if (!c) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  std::vector<double> pts;
  std::vector<int64_t> node_pt;
  int nmax = 0;
  const int rc = gdof_points_build(c, pts, node_pt, &nmax);
  if (rc != HP3DG_OK) return rc;
  const int64_t n = (int64_t)pts.size() / 4;
  if (npts) *npts = n;
  if (eta) {
    if (!etav) return HP3DG_ERR_ARG;
    for (int e = 0; e < c->nel; ++e)
      for (int64_t l = node_pt[(size_t)e * 28]; l < node_pt[(size_t)e * 28 + 27]; ++l)
        eta_trilinear(etav + (size_t)24 * e, &pts[4 * l], eta + 3 * l);
  }
  return HP3DG_OK;
}

int hp3dg_update_gdof(hp3dg_ctx* c, const double* etav, const double* x, const double* dxdeta,
                      const int32_t* linear, double* xnod, int32_t apply) {
  if (!c || !etav || !x || !dxdeta) return HP3DG_ERR_ARG;
  if (!c->submitted) return HP3DG_ERR_STATE;
  const int nel = c->nel;
  if (nel == 0) return HP3DG_OK;
  std::vector<double> pts;
  std::vector<int64_t> node_pt;
  int nmax = 0;
  int rc = gdof_points_build(c, pts, node_pt, &nmax);
  if (rc != HP3DG_OK) return rc;
  const int64_t npts = (int64_t)pts.size() / 4;
  // each node takes the values of the first element containing it
  std::vector<int> src((size_t)nel * 26, -1);
  {
    std::map<int, int> firstv;
    for (int e = 0; e < nel; ++e)
      for (int i = 0; i < 26; ++i) {
        const int nod = c->last_desc[e].nodes[i];
        auto it = firstv.find(nod);
        if (it == firstv.end()) firstv[nod] = e * 26 + i;
        else src[(size_t)e * 26 + i] = it->second;
      }
  }
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  const int64_t ndof = c->dof_off[nel];
  const int64_t wstride = (int64_t)gdof_work_doubles(nmax);
  int chunk = (int)std::min<int64_t>(nel, std::max<int64_t>(64, (256LL << 20) / (8 * wstride)));
  double *d_etav = nullptr, *d_pts = nullptr, *d_x = nullptr, *d_j = nullptr, *d_xn = nullptr,
         *d_work = nullptr;
  int64_t* d_np = nullptr;
  int *d_src = nullptr, *d_lin = nullptr, *d_bad = nullptr;
  int err = 0;
  d_etav = dalloc<double>((size_t)nel * 24, &err);
  d_pts = dalloc<double>(pts.size(), &err);
  d_x = dalloc<double>((size_t)npts * 3, &err);
  d_j = dalloc<double>((size_t)npts * 9, &err);
  d_xn = dalloc<double>((size_t)ndof * 3, &err);
  d_work = dalloc<double>((size_t)chunk * wstride, &err);
  d_np = dalloc<int64_t>(node_pt.size(), &err);
  d_src = dalloc<int>(src.size(), &err);
  d_lin = linear ? dalloc<int>(nel, &err) : nullptr;
  d_bad = dalloc<int>(1, &err);
  rc = err;
  int badv = 0x7f7f7f7f;
  if (rc == HP3DG_OK &&
      (cudaMemcpyAsync(d_etav, etav, (size_t)nel * 24 * 8, cudaMemcpyHostToDevice, st) ||
       cudaMemcpyAsync(d_pts, pts.data(), pts.size() * 8, cudaMemcpyHostToDevice, st) ||
       cudaMemcpyAsync(d_x, x, (size_t)npts * 3 * 8, cudaMemcpyHostToDevice, st) ||
       cudaMemcpyAsync(d_j, dxdeta, (size_t)npts * 9 * 8, cudaMemcpyHostToDevice, st) ||
       cudaMemcpyAsync(d_np, node_pt.data(), node_pt.size() * 8, cudaMemcpyHostToDevice, st) ||
       cudaMemcpyAsync(d_src, src.data(), src.size() * 4, cudaMemcpyHostToDevice, st) ||
       (linear && cudaMemcpyAsync(d_lin, linear, (size_t)nel * 4, cudaMemcpyHostToDevice, st)) ||
       cudaMemcpyAsync(d_bad, &badv, 4, cudaMemcpyHostToDevice, st)))
    rc = HP3DG_ERR_CUDA;
  if (rc == HP3DG_OK &&
      launch_gdof(nel, c->d_norder, c->d_nori_e, c->d_nori_f, d_etav, d_np, d_pts, d_x, d_j,
                  d_lin, d_src, c->d_dof_off, d_xn, d_work, wstride, chunk, d_bad, st))
    rc = HP3DG_ERR_CUDA;
  if (rc == HP3DG_OK &&
      ((xnod && cudaMemcpyAsync(xnod, d_xn, (size_t)ndof * 3 * 8, cudaMemcpyDeviceToHost, st)) ||
       cudaMemcpyAsync(&badv, d_bad, 4, cudaMemcpyDeviceToHost, st) ||
       cudaStreamSynchronize(st)))
    rc = HP3DG_ERR_CUDA;
  if (rc == HP3DG_OK && badv != 0x7f7f7f7f) {
    c->last_bad = badv;
    rc = HP3DG_ERR_NOT_SPD;
  }
  if (rc == HP3DG_OK && apply) {
    // the projected dof become the pass's isoparametric geometry
    if (c->d_xnod) cudaFree(c->d_xnod);
    c->d_xnod = d_xn;
    d_xn = nullptr;
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_kernels = -1;
    c->iso = true;
    c->ran = c->downloaded = c->have_dofs = false;
  }
  cudaFree(d_etav); cudaFree(d_pts); cudaFree(d_x); cudaFree(d_j); cudaFree(d_xn);
  cudaFree(d_work); cudaFree(d_np); cudaFree(d_src); cudaFree(d_lin); cudaFree(d_bad);
  return rc;
}

int32_t hp3dg_last_bad_element(const hp3dg_ctx* c) { return c ? c->last_bad : -1; }

void hp3dg_batch_end(hp3dg_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_batch(c);
  cudaFree(c->d_flags);
  for (auto& e : c->ev) cudaEventDestroy(e);
  for (auto& e : c->chunk_ev) cudaEventDestroy(e);
  cudaStreamDestroy(c->copy_stream);
  cudaEventDestroy(c->fork_ev);
  for (int b = 0; b < hp3dg_ctx::NBRANCH; ++b) {
    cudaEventDestroy(c->join_ev[b]);
    cudaStreamDestroy(c->branch[b]);
  }
  cudaStreamDestroy(c->own);
  delete c;
}

}  // extern "C"
