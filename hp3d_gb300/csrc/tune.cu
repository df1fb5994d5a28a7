// Tuning table of the element pass: per-bin kernel variants chosen by an
// offline sweep on the target GPU (hp3d_gb300/autotune.py), stored as JSON and
// read at submit.  The reference schedules its element loop dynamically
// (solver/omp_mumps/mumps_sc.F90:253-255, !$OMP DO SCHEDULE(DYNAMIC)) and
// picks a quadrature rule per element type (quadrature/set_3D_int.F90:155-388);
// here the (type, order) bins are fixed at submit, so the choice of kernel
// variant per bin is made once, from measured times, before the pass is
// captured.
//
// File format (the subset of JSON this reader accepts: objects, arrays,
// numbers, strings, true/false/null):
//   {"version": 1, "device": "...",
//    "launch": {"nstage": 5},
//    "bins": [{"etype": 1, "n": 216, "nb": 64, "nint": 343, "precision": 1,
//              "cond": 1, "grp": 13, ...}, ...]}
// Keys a record does not use (timings, notes) are skipped.  cond: 0 = the
// built-in rule, 1 = fused tensor-core condensation, 2 = FP64 factor with the
// tensor-core Schur update, 3 = FP64 throughout; grp: column blocks per raster
// group of the contraction (0 = built-in rule); nstage: ring stages of the
// contraction's operand pipeline (0 = as many as fit).
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hp3dg.h"
#include "hp3dg_kernels.h"

namespace hp3dg {
namespace {

struct Json {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  double num = 0.0;
  std::string str;
  std::vector<Json> items;                         // ARR
  std::vector<std::pair<std::string, Json>> keys;  // OBJ
  const Json* get(const char* k) const {
    for (const auto& kv : keys)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
};

struct Parser {
  const char* p;
  const char* end;
  int depth = 0;
  void ws() {
    while (p < end && isspace((unsigned char)*p)) ++p;
  }
  bool lit(const char* s) {
    const size_t n = strlen(s);
    if ((size_t)(end - p) < n || strncmp(p, s, n) != 0) return false;
    p += n;
    return true;
  }
  bool string(std::string& out) {
    if (p >= end || *p != '"') return false;
    ++p;
    while (p < end && *p != '"') {
      if (*p == '\\') {
        if (++p >= end) return false;
        const char c = *p;
        out.push_back(c == 'n' ? '\n' : c == 't' ? '\t' : c);  // \uXXXX is not used here
      } else {
        out.push_back(*p);
      }
      ++p;
    }
    if (p >= end) return false;
    ++p;
    return true;
  }
  bool value(Json& v) {
    ws();
    if (p >= end || ++depth > 32) return false;
    bool ok = true;
    if (*p == '{') {
      v.kind = Json::OBJ;
      ++p;
      ws();
      if (p < end && *p == '}') {
        ++p;
      } else {
        while (ok) {
          ws();
          std::string k;
          Json x;
          ok = string(k);
          ws();
          ok = ok && p < end && *p == ':';
          if (ok) ++p;
          ok = ok && value(x);
          if (ok) v.keys.emplace_back(std::move(k), std::move(x));
          ws();
          if (ok && p < end && *p == ',') { ++p; continue; }
          ok = ok && p < end && *p == '}';
          if (ok) ++p;
          break;
        }
      }
    } else if (*p == '[') {
      v.kind = Json::ARR;
      ++p;
      ws();
      if (p < end && *p == ']') {
        ++p;
      } else {
        while (ok) {
          Json x;
          ok = value(x);
          if (ok) v.items.push_back(std::move(x));
          ws();
          if (ok && p < end && *p == ',') { ++p; continue; }
          ok = ok && p < end && *p == ']';
          if (ok) ++p;
          break;
        }
      }
    } else if (*p == '"') {
      v.kind = Json::STR;
      ok = string(v.str);
    } else if (lit("true")) {
      v.kind = Json::BOOL; v.num = 1;
    } else if (lit("false")) {
      v.kind = Json::BOOL; v.num = 0;
    } else if (lit("null")) {
      v.kind = Json::NUL;
    } else {
      char* q = nullptr;
      std::string tok;
      while (p < end && (isdigit((unsigned char)*p) || strchr("+-.eE", *p))) tok.push_back(*p++);
      v.kind = Json::NUM;
      v.num = strtod(tok.c_str(), &q);
      ok = !tok.empty() && q && *q == '\0';
    }
    --depth;
    return ok;
  }
};

struct TuneTable {
  bool loaded = false;
  int nstage = 0;
  std::vector<TuneRec> recs;
};

std::mutex g_mu;
TuneTable g_tab;
bool g_env_tried = false;

int as_int(const Json* v, int dflt) {
  return (v && (v->kind == Json::NUM || v->kind == Json::BOOL)) ? (int)v->num : dflt;
}

// parse a table; returns HP3DG_OK or HP3DG_ERR_ARG (malformed, or a record
// without its key fields or with a value out of range)
int parse_table(const std::string& text, TuneTable* t) {
  Json root;
  Parser ps{text.data(), text.data() + text.size()};
  if (!ps.value(root) || root.kind != Json::OBJ) return HP3DG_ERR_ARG;
  ps.ws();
  if (ps.p != ps.end) return HP3DG_ERR_ARG;
  TuneTable out;
  out.loaded = true;
  if (const Json* l = root.get("launch")) {
    if (l->kind != Json::OBJ) return HP3DG_ERR_ARG;
    out.nstage = as_int(l->get("nstage"), 0);
    if (out.nstage < 0 || out.nstage > 16) return HP3DG_ERR_ARG;
  }
  const Json* bins = root.get("bins");
  if (bins && bins->kind != Json::ARR) return HP3DG_ERR_ARG;
  if (bins)
    for (const Json& b : bins->items) {
      if (b.kind != Json::OBJ) return HP3DG_ERR_ARG;
      TuneRec r;
      r.etype = as_int(b.get("etype"), -1);
      r.n = as_int(b.get("n"), -1);
      r.nb = as_int(b.get("nb"), -1);
      r.nint = as_int(b.get("nint"), -1);
      r.precision = as_int(b.get("precision"), -1);
      r.cond = as_int(b.get("cond"), 0);
      r.grp = as_int(b.get("grp"), 0);
      if (r.etype < HP3DG_HEXA || r.etype > HP3DG_TET || r.n <= 0 || r.nb < 0 || r.nint <= 0 ||
          (r.precision != HP3DG_FP64 && r.precision != HP3DG_MIXED) || r.cond < 0 ||
          r.cond > 3 || r.grp < 0)
        return HP3DG_ERR_ARG;
      out.recs.push_back(r);
    }
  *t = std::move(out);
  return HP3DG_OK;
}

int load_file(const char* path, TuneTable* t) {
  FILE* f = fopen(path, "rb");
  if (!f) return HP3DG_ERR_ARG;
  std::string text;
  char buf[4096];
  size_t k;
  while ((k = fread(buf, 1, sizeof(buf), f)) > 0) {
    text.append(buf, k);
    if (text.size() > (64u << 20)) { fclose(f); return HP3DG_ERR_ARG; }
  }
  fclose(f);
  return parse_table(text, t);
}

}  // namespace

// The table entry of a bin, if any (the process-wide table; the file named
// by HP3DG_TUNE_FILE is read on first use when no table was loaded).
bool tune_lookup(int etype, int n, int nb, int nint, int precision, TuneRec* out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_tab.loaded && !g_env_tried) {
    g_env_tried = true;
    const char* env = getenv("HP3DG_TUNE_FILE");
    TuneTable t;
    if (env && *env && load_file(env, &t) == HP3DG_OK) g_tab = std::move(t);
  }
  for (const TuneRec& r : g_tab.recs)
    if (r.etype == etype && r.n == n && r.nb == nb && r.nint == nint && r.precision == precision) {
      *out = r;
      return true;
    }
  return false;
}

int tune_nstage() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_tab.nstage;
}

}  // namespace hp3dg

extern "C" {

int hp3dg_tune_load(const char* path, int32_t* nrec) {
  using namespace hp3dg;
  TuneTable t;
  if (path) {
    const int rc = load_file(path, &t);
    if (rc != HP3DG_OK) return rc;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  g_tab = std::move(t);
  g_env_tried = true;  // an explicit load (or clear) takes precedence over the variable
  if (nrec) *nrec = (int32_t)g_tab.recs.size();
  return HP3DG_OK;
}

int hp3dg_tune_lookup(int32_t etype, int32_t n, int32_t nb, int32_t nint, int32_t precision,
                      int32_t* cond, int32_t* grp, int32_t* nstage) {
  hp3dg::TuneRec r;
  const bool hit = hp3dg::tune_lookup(etype, n, nb, nint, precision, &r);
  if (cond) *cond = hit ? r.cond : 0;
  if (grp) *grp = hit ? r.grp : 0;
  if (nstage) *nstage = hp3dg::tune_nstage();
  return hit ? HP3DG_OK : HP3DG_ERR_ARG;
}

}  // extern "C"
