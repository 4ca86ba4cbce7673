// extern "C" entry points of include/ccx.h.  Every entry point catches all C++
// exceptions, stores the message for ccx_last_error() and returns a status code.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <chrono>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "ccx.h"
#include "checkpoint.hpp"
#include "engine.hpp"
#include "layout.hpp"

struct ccx_layout {
  std::shared_ptr<ccx::Layout> L;
};
struct ccx_engine {
  std::shared_ptr<const ccx::Layout> L;
  std::unique_ptr<ccx::IEngine> E;
};
struct ccx_learner {
  std::unique_ptr<ccx::ILearner> M;
};

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

template <typename F>
int guard(F &&f) {
  try {
    f();
    return CCX_OK;
  } catch (const ccx::EngineError &e) {
    return fail(e.code, e.what());
  } catch (const std::bad_alloc &) {
    return fail(CCX_ENOMEM, "host allocation failed");
  } catch (const std::invalid_argument &e) {
    return fail(CCX_EINVAL, e.what());
  } catch (const std::exception &e) {
    return fail(CCX_EINVAL, e.what());
  } catch (...) {
    return fail(CCX_EINVAL, "unknown error");
  }
}

const ccx::ChannelFamily *family(const ccx::Layout &L, int kind) {
  switch (kind) {
    case CCX_CH_HHHH: return &L.fam[1];
    case CCX_CH_HHHP: return &L.fam[2];
    case CCX_CH_HHPP: return &L.fam[3];
    case CCX_CH_HPHP: return &L.fam[4];
    case CCX_CH_HPPP: return &L.fam[5];
    case CCX_CH_PH_PHHP: return &L.ph[1];
    case CCX_CH_PH_HPHP: return &L.ph[2];
    case CCX_CH_PH_HPPH: return &L.ph[3];
    default: return nullptr;
  }
}

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

// list-directed read of comma / blank separated fields
std::vector<std::string> fields(const std::string &line) {
  std::vector<std::string> out;
  std::string cur;
  for (char c : line) {
    if (c == ',' || std::isspace((unsigned char)c)) {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
    } else {
      cur.push_back(c);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

double to_d(const std::string &s, const char *what) {
  std::string t = s;
  for (char &c : t)
    if (c == 'd' || c == 'D') c = 'e';
  char *end = nullptr;
  const double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str() || *end) throw std::invalid_argument(std::string("ccm_in: bad number for ") + what + ": '" + s + "'");
  return v;
}
int to_i(const std::string &s, const char *what) {
  const double v = to_d(s, what);
  if (v != (double)(long)v) throw std::invalid_argument(std::string("ccm_in: expected an integer for ") + what);
  return (int)v;
}
bool to_l(const std::string &s) {
  std::string t;
  for (char c : s) t.push_back((char)std::toupper((unsigned char)c));
  if (!t.empty() && t[0] == '.') t = t.substr(1);
  return !t.empty() && t[0] == 'T';
}
std::string lower(std::string s) {
  for (char &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

}  // namespace

namespace ccx {
void set_last_error(const std::string &msg) { g_err = msg; }
}  // namespace ccx

extern "C" {

const char *ccx_last_error(void) { return g_err.c_str(); }

// Each value line of ccm_in follows one comment line (read(5,*);read(5,*) ...).
int ccx_deck_parse(const char *text, ccx_deck *out) {
  if (!text || !out) return fail(CCX_EINVAL, "null argument");
  return guard([&] {
    std::vector<std::string> lines;
    {
      std::istringstream is(text);
      std::string l;
      while (std::getline(is, l)) lines.push_back(l);
    }
    ccx_deck d;
    std::memset(&d, 0, sizeof d);
    d.potential = CCX_POT_MINNESOTA;
    d.lec_seed = 20261203ULL;
    d.mode = CCX_MODE_REFERENCE;
    d.diis_dim = 8;
    d.tol = 1e-6;
    d.max_iter = 100;
    d.precision = CCX_PREC_FP64;
    auto value = [&](int k) -> std::vector<std::string> {
      const size_t idx = 2 * (size_t)k + 1;
      if (idx >= lines.size()) throw std::invalid_argument("ccm_in: missing value line " + std::to_string(k + 1));
      return fields(lines[idx]);
    };
    auto need = [&](const std::vector<std::string> &f, size_t n, int k) {
      if (f.size() < n) throw std::invalid_argument("ccm_in: value line " + std::to_string(k + 1) + " has too few fields");
    };
    auto f = value(0); need(f, 2, 0);
    d.chiral_order = to_i(f[0], "chiral order");
    d.lambda = to_d(f[1], "cutoff");
    f = value(1); need(f, 2, 1);
    d.cE = to_d(f[0], "cE");
    d.cD = to_d(f[1], "cD");
    f = value(2); need(f, 1, 2);
    d.A = to_i(f[0], "number of particles");
    f = value(3); need(f, 2, 3);
    {
      const std::string m = lower(f[0]), t = lower(f[1]);
      if (m != "pnm" && m != "snm") throw std::invalid_argument("ccm_in: matter type must be pnm or snm");
      if (t != "density" && t != "kfermi") throw std::invalid_argument("ccm_in: input type must be density or kfermi");
      d.snm = m == "snm";
      d.input_is_kfermi = t == "kfermi";
    }
    f = value(4); need(f, 1, 4);
    std::snprintf(d.bc, sizeof d.bc, "%s", f[0].c_str());
    f = value(5); need(f, 3, 5);
    d.dens_or_kf = to_d(f[0], "density");
    d.ntwist = to_i(f[1], "ntwist");
    d.nmax = to_i(f[2], "nmax");
    d.my_twists = f.size() > 3 ? to_i(f[3], "my_twists") : 1;
    f = value(6); need(f, 1, 6);
    std::snprintf(d.cc_approx, sizeof d.cc_approx, "%s", f[0].c_str());
    f = value(7); need(f, 2, 7);
    d.tnf_switch = to_l(f[0]);
    d.tnf_approx = to_i(f[1], "3nf approximation");
    f = value(8); need(f, 2, 8);
    d.cutoff_3nf = to_d(f[0], "3nf cutoff");
    d.nexp_3nf = to_i(f[1], "3nf exponent");
    // extension block: "key = value" lines after the ninth value line
    for (size_t i = 18; i < lines.size(); ++i) {
      const std::string l = trim(lines[i]);
      if (l.empty() || l[0] == '!' || l[0] == '#') continue;
      const size_t eq = l.find('=');
      if (eq == std::string::npos) throw std::invalid_argument("ccm_in extension: expected key = value: " + l);
      const std::string k = lower(trim(l.substr(0, eq))), v = trim(l.substr(eq + 1));
      if (k == "potential") {
        const std::string p = lower(v);
        if (p == "minnesota") d.potential = CCX_POT_MINNESOTA;
        else if (p == "chiral_like" || p == "chiral-like") d.potential = CCX_POT_CHIRAL_LIKE;
        else throw std::invalid_argument("ccm_in extension: unknown potential " + v);
      } else if (k == "lec_seed") d.lec_seed = (uint64_t)std::strtoull(v.c_str(), nullptr, 10);
      else if (k == "mode") {
        const std::string m = lower(v);
        if (m == "reference") d.mode = CCX_MODE_REFERENCE;
        else if (m == "standard") d.mode = CCX_MODE_STANDARD;
        else throw std::invalid_argument("ccm_in extension: unknown mode " + v);
      } else if (k == "diis_dim") d.diis_dim = to_i(v, "diis_dim");
      else if (k == "tol") d.tol = to_d(v, "tol");
      else if (k == "max_iter") d.max_iter = to_i(v, "max_iter");
      else if (k == "precision") {
        const std::string m = lower(v);
        if (m == "fp64") d.precision = CCX_PREC_FP64;
        else if (m == "mixed") d.precision = CCX_PREC_MIXED;
        else throw std::invalid_argument("ccm_in extension: unknown precision " + v);
      } else if (k == "theta") {
        auto t = fields(v);
        if (t.size() != 3) throw std::invalid_argument("ccm_in extension: theta needs three values");
        for (int q = 0; q < 3; ++q) d.theta[q] = to_d(t[q], "theta");
      } else {
        throw std::invalid_argument("ccm_in extension: unknown key " + k);
      }
    }
    if (d.A <= 0) throw std::invalid_argument("ccm_in: number of particles must be positive");
    if (d.nmax < 0) throw std::invalid_argument("ccm_in: nmax must be >= 0");
    if (!(d.dens_or_kf > 0)) throw std::invalid_argument("ccm_in: density/kF must be positive");
    *out = d;
  });
}

int ccx_layout_from_basis(const ccx_basis_params *p, ccx_layout **out) {
  if (!p || !out) return fail(CCX_EINVAL, "null argument");
  return guard([&] {
    auto L = std::make_shared<ccx::Layout>();
    L->b = ccx::build_basis(p->nmax, p->A, p->snm != 0, p->density, p->theta);
    ccx::build_layout(*L);
    *out = new ccx_layout{L};
  });
}

int ccx_layout_from_orbits(const ccx_orbits *o, ccx_layout **out) {
  if (!o || !out || !o->nx || !o->ny || !o->nz || !o->sz || !o->tz || !o->kx || !o->ky || !o->kz)
    return fail(CCX_EINVAL, "null argument");
  return guard([&] {
    if (o->n_states <= 0 || o->n_holes <= 0 || o->n_holes > o->n_states) throw std::invalid_argument("bad state counts");
    auto L = std::make_shared<ccx::Layout>();
    ccx::Basis &B = L->b;
    const int n = o->n_states;
    B.ns = n;
    B.A = o->n_holes;
    B.nx.assign(o->nx, o->nx + n); B.ny.assign(o->ny, o->ny + n); B.nz.assign(o->nz, o->nz + n);
    B.sz.assign(o->sz, o->sz + n); B.tz.assign(o->tz, o->tz + n);
    B.kx.assign(o->kx, o->kx + n); B.ky.assign(o->ky, o->ky + n); B.kz.assign(o->kz, o->kz + n);
    if (o->e) B.e.assign(o->e, o->e + n);
    else B.e.assign(n, 0.0);
    B.L = o->box_length;
    B.tzmin = 1;
    B.tzmax = 1;
    for (int i = 0; i < n; ++i) {
      if (B.sz[i] != -1 && B.sz[i] != 1) throw std::invalid_argument("sz must be -1 or +1");
      if (B.tz[i] != -1 && B.tz[i] != 1) throw std::invalid_argument("tz must be -1 or +1");
      B.tzmin = std::min(B.tzmin, B.tz[i]);
    }
    ccx::build_layout(*L);
    *out = new ccx_layout{L};
  });
}

int ccx_layout_destroy(ccx_layout *l) {
  delete l;
  return CCX_OK;
}

int ccx_layout_orbits(const ccx_layout *l, ccx_orbits *out) {
  if (!l || !out) return fail(CCX_EINVAL, "null argument");
  const ccx::Basis &B = l->L->b;
  out->n_states = B.ns;
  out->n_holes = B.A;
  out->nx = B.nx.data(); out->ny = B.ny.data(); out->nz = B.nz.data();
  out->sz = B.sz.data(); out->tz = B.tz.data();
  out->kx = B.kx.data(); out->ky = B.ky.data(); out->kz = B.kz.data();
  out->e = B.e.data();
  out->box_length = B.L;
  return CCX_OK;
}

int ccx_layout_counts(const ccx_layout *l, int64_t counts[8]) {
  if (!l || !counts) return fail(CCX_EINVAL, "null argument");
  const ccx::Layout &L = *l->L;
  counts[0] = L.fam[3].count();
  counts[1] = L.fam[1].count();
  counts[2] = L.fam[2].count();
  counts[3] = L.fam[4].count();
  counts[4] = L.ph[1].count();
  counts[5] = L.ph[2].count();
  counts[6] = L.ph[3].count();
  counts[7] = L.n_amps;
  return CCX_OK;
}

int ccx_layout_channel(const ccx_layout *l, int32_t kind, int32_t ch, int32_t qn[4], int32_t *n1, int32_t *n2) {
  if (!l) return fail(CCX_EINVAL, "null layout");
  const ccx::ChannelFamily *F = family(*l->L, kind);
  if (!F) return fail(CCX_EINVAL, "unknown channel kind");
  if (ch < 0 || ch >= F->count()) return fail(CCX_EINVAL, "channel index out of range");
  if (qn)
    for (int i = 0; i < 4; ++i) qn[i] = F->qn[ch][i];
  if (n1) *n1 = F->side1[ch].size();
  if (n2) *n2 = F->side2[ch].size();
  return CCX_OK;
}

int ccx_layout_pairs(const ccx_layout *l, int32_t kind, int32_t ch, int32_t *s1, int32_t *s2) {
  if (!l) return fail(CCX_EINVAL, "null layout");
  const ccx::ChannelFamily *F = family(*l->L, kind);
  if (!F) return fail(CCX_EINVAL, "unknown channel kind");
  if (ch < 0 || ch >= F->count()) return fail(CCX_EINVAL, "channel index out of range");
  auto put = [](const ccx::PairList &p, int32_t *o) {
    if (!o) return;
    for (int i = 0; i < p.size(); ++i) { o[2 * i] = p.p[i]; o[2 * i + 1] = p.q[i]; }
  };
  put(F->side1[ch], s1);
  put(F->side2[ch], s2);
  return CCX_OK;
}

int ccx_layout_hash(const ccx_layout *l, uint64_t *h) {
  if (!l || !h) return fail(CCX_EINVAL, "null argument");
  *h = l->L->hash();
  return CCX_OK;
}

int ccx_t2_checkpoint_write(const ccx_layout *l, const char *path, const double *t2) {
  if (!l || !path || !t2) return fail(CCX_EINVAL, "null argument");
  return guard([&] { ccx::write_t2_checkpoint(*l->L, path, t2); });
}
int ccx_t2_checkpoint_read(const ccx_layout *l, const char *path, int32_t flags, double *t2) {
  if (!l || !path || !t2) return fail(CCX_EINVAL, "null argument");
  if (flags & ~CCX_CKPT_ANY_TWIST) return fail(CCX_EINVAL, "unknown checkpoint flags");
  return guard([&] { ccx::read_t2_checkpoint(*l->L, path, (flags & CCX_CKPT_ANY_TWIST) != 0, t2); });
}

int ccx_engine_create(const ccx_layout *l, const ccx_engine_options *opt, ccx_engine **out) {
  if (!l || !out) return fail(CCX_EINVAL, "null argument");
  return guard([&] {
    const int dev = opt ? opt->device : 0;
    const bool cplx = opt ? opt->scalar == CCX_SCALAR_COMPLEX : true;
    auto e = std::make_unique<ccx_engine>();
    e->L = l->L;
    e->E = ccx::make_engine(l->L, dev, cplx);
    *out = e.release();
  });
}

int ccx_engine_destroy(ccx_engine *e) {
  return guard([&] { delete e; });
}

#define ENGINE_CALL(e, body)                                   \
  if (!(e)) return fail(CCX_EINVAL, "null engine");            \
  return guard([&] { body; })

int ccx_engine_memory(const ccx_engine *e, int64_t *bytes) {
  if (!bytes) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, *bytes = e->E->device_bytes());
}
int ccx_set_triples_precision(ccx_engine *e, int32_t precision) {
  ENGINE_CALL(e, e->E->set_triples_precision(precision));
}
int ccx_engine_diis_fallbacks(const ccx_engine *e, int64_t *n) {
  if (!n) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, *n = e->E->diis_fallbacks());
}
int ccx_engine_launches(const ccx_engine *e, int64_t *n) {
  if (!n) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, *n = e->E->launches());
}
int ccx_engine_iter_log(const ccx_engine *e, int32_t capacity, ccx_iter_record *records, int32_t *n) {
  if (!n || capacity < 0 || (capacity > 0 && !records)) return fail(CCX_EINVAL, "null argument or negative capacity");
  ENGINE_CALL(e, {
    const std::vector<ccx::IterRecord> &log = e->E->iter_log();
    *n = (int32_t)log.size();
    const size_t m = std::min(log.size(), (size_t)capacity);
    for (size_t i = 0; i < m; ++i) {
      const ccx::IterRecord &s = log[i];
      ccx_iter_record &d = records[i];
      d.iteration = s.iteration;
      d.kind = s.kind;
      d.energy[0] = s.e[0];
      d.energy[1] = s.e[1];
      d.de = s.de;
      d.res_norm = s.res_norm;
      d.ms = s.ms;
      for (int k = 0; k < 9; ++k) d.term_ms[k] = s.term_ms[k];
    }
  });
}
int ccx_engine_set_profiling(ccx_engine *e, int32_t on) { ENGINE_CALL(e, e->E->set_profiling(on != 0)); }
int ccx_engine_timers(const ccx_engine *e, double ms[10]) {
  if (!ms) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, e->E->timers(ms));
}
int ccx_engine_autotune(ccx_engine *e, int32_t shapes[4], double ms[8]) {
  if (!shapes || !ms) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, {
    int s[4];
    e->E->autotune(s, ms);
    for (int k = 0; k < 4; ++k) shapes[k] = s[k];
  });
}
int ccx_engine_autotune_tc(ccx_engine *e, int32_t precision, int32_t merged[3], double ms[6]) {
  if (!merged || !ms) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, {
    int m[3];
    e->E->autotune_tc(precision, m, ms);
    for (int k = 0; k < 3; ++k) merged[k] = m[k];
  });
}
int ccx_ccd_iter_batch(ccx_engine *const *engines, int32_t n, const ccx_iter_opts *opt, ccx_iter_result *res,
                       double *seconds) {
  if (!engines || !opt || !res || n < 1) return fail(CCX_EINVAL, "bad batch arguments");
  for (int32_t i = 0; i < n; ++i)
    if (!engines[i]) return fail(CCX_EINVAL, "null engine in the batch");
  return guard([&] {
    ccx::IterOpts o;
    o.mode = opt->mode;
    o.precision = opt->precision;
    o.max_iter = opt->max_iter;
    o.tol = opt->tol;
    o.diis_dim = opt->diis_dim;
    o.defect_period = opt->defect_period;
    o.verbose = opt->verbose;
    o.rebase = opt->rebase;
    o.rebase_drop = opt->rebase_drop;
    std::vector<ccx::IterResult> rr(n);
    std::vector<ccx::IEngine *> act;
    for (int32_t i = 0; i < n; ++i) {
      engines[i]->E->set_timing(false);
      engines[i]->E->std_begin(o, rr[i]);
      if (!engines[i]->E->std_done()) act.push_back(engines[i]->E.get());
    }
    const auto t0 = std::chrono::steady_clock::now();
    // lockstep: every engine's launches go to its own stream, so the GPU overlaps the
    // engines; one host synchronisation per step for the whole batch
    while (!act.empty()) {
      for (auto *e : act) {
        e->std_launch_residual();
        e->std_launch_update();
        e->std_launch_dots();
      }
      for (auto *e : act) e->sync();
      std::vector<ccx::IEngine *> next;
      for (auto *e : act)
        if (!e->std_after_update()) {
          e->std_after_dots();
          if (!e->std_done()) next.push_back(e);
        }
      act.swap(next);
    }
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (int32_t i = 0; i < n; ++i) {
      ccx_iter_result &x = res[i];
      x.iterations = rr[i].iterations;
      x.converged = rr[i].converged;
      x.e_mbpt2[0] = rr[i].e_mbpt2[0];
      x.e_mbpt2[1] = rr[i].e_mbpt2[1];
      x.e_ccd[0] = rr[i].e_ccd[0];
      x.e_ccd[1] = rr[i].e_ccd[1];
      x.res_norm = rr[i].res_norm;
      x.seconds = dt;
      x.fp64_sweeps = rr[i].fp64_sweeps;
      x.mixed_iterations = rr[i].mixed_iterations;
    }
    if (seconds) *seconds = dt;
  });
}
int ccx_learner_create(int32_t device, uint64_t seed, ccx_learner **out) {
  if (!out) return fail(CCX_EINVAL, "null argument");
  *out = nullptr;
  return guard([&] {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) throw ccx::EngineError(CCX_ENOGPU, "no CUDA device");
    auto *l = new ccx_learner;
    try {
      l->M = ccx::make_learner(device, seed);
    } catch (...) {
      delete l;
      throw;
    }
    *out = l;
  });
}
int ccx_learner_destroy(ccx_learner *l) {
  delete l;
  return CCX_OK;
}
#define LEARNER_CALL(l, body)                                  \
  if (!(l)) return fail(CCX_EINVAL, "null learner");           \
  return guard([&] { body; })
static ccx::MLView ml_view_of(ccx_engine *e, bool need_t) {
  ccx::MLView v;
  if (!e->E->ml_view(v, need_t)) throw ccx::EngineError(CCX_EINVAL, "the learned warm start needs a real engine");
  return v;
}
int ccx_learner_add_solution(ccx_learner *l, ccx_engine *e) {
  if (!e) return fail(CCX_EINVAL, "null engine");
  LEARNER_CALL(l, l->M->add_solution(ml_view_of(e, true), 1));
}
int ccx_learner_add_solution_sampled(ccx_learner *l, ccx_engine *e, int32_t stride) {
  if (!e || stride < 1) return fail(CCX_EINVAL, "null engine or stride < 1");
  LEARNER_CALL(l, l->M->add_solution(ml_view_of(e, true), stride));
}
int ccx_learner_set_prior(ccx_learner *l, ccx_engine *target, int32_t n, ccx_engine *const *engines,
                          const double *weights) {
  if (!target || n < 0 || (n > 0 && (!engines || !weights))) return fail(CCX_EINVAL, "bad prior arguments");
  for (int32_t i = 0; i < n; ++i)
    if (!engines[i]) return fail(CCX_EINVAL, "null engine in the prior");
  LEARNER_CALL(l, {
    std::vector<ccx::MLView> vs;
    for (int32_t i = 0; i < n; ++i) vs.push_back(ml_view_of(engines[i], true));
    l->M->set_prior(ml_view_of(target, false), vs.data(), weights, n);
  });
}
int ccx_learner_clear(ccx_learner *l) { LEARNER_CALL(l, l->M->clear()); }
int ccx_learner_samples(const ccx_learner *l, int64_t *n) {
  if (!n) return fail(CCX_EINVAL, "null argument");
  LEARNER_CALL(l, *n = l->M->samples());
}
int ccx_learner_train(ccx_learner *l, int32_t steps, int32_t batch, double lr, uint64_t seed, double *loss) {
  LEARNER_CALL(l, {
    const double v = l->M->train(steps, batch, lr, seed);
    if (loss) *loss = v;
  });
}
int ccx_init_learned(ccx_engine *e, ccx_learner *l) {
  if (!e) return fail(CCX_EINVAL, "null engine");
  LEARNER_CALL(l, {
    l->M->warm_start(ml_view_of(e, false));
    e->E->mark_t_set();
  });
}
int ccx_learner_get_params(const ccx_learner *l, float *p) {
  if (!p) return fail(CCX_EINVAL, "null argument");
  LEARNER_CALL(l, l->M->get_params(p));
}
int ccx_learner_set_params(ccx_learner *l, const float *p) {
  if (!p) return fail(CCX_EINVAL, "null argument");
  LEARNER_CALL(l, l->M->set_params(p));
}
int ccx_learner_loss_grad(ccx_learner *l, const float *X, const float *y, int32_t n, double *loss, float *grad) {
  if (!X || !y || !loss || !grad || n <= 0) return fail(CCX_EINVAL, "bad arguments");
  LEARNER_CALL(l, l->M->loss_grad(X, y, n, loss, grad));
}
int ccx_learner_infer(ccx_learner *l, const float *X, int32_t n, float *out, int32_t tensor_cores) {
  if (!X || !out || n <= 0) return fail(CCX_EINVAL, "bad arguments");
  LEARNER_CALL(l, l->M->infer(X, n, out, tensor_cores));
}
int ccx_engine_kernel_timers(const ccx_engine *e, double ms[16], int64_t launches[16]) {
  if (!ms || !launches) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, e->E->kernel_timers(ms, launches));
}
int ccx_set_fock(ccx_engine *e, const double *fock, const double e0[2]) {
  if (!fock) return fail(CCX_EINVAL, "null Fock matrix");
  ENGINE_CALL(e, e->E->set_fock(fock, e0));
}
int ccx_set_vblocks(ccx_engine *e, int32_t kind, int32_t n, const int32_t *chs, const double *const *v) {
  if (n < 0 || (n > 0 && (!chs || !v))) return fail(CCX_EINVAL, "null block list");
  for (int32_t i = 0; i < n; ++i)
    if (!v[i]) return fail(CCX_EINVAL, "null V block in the list");
  ENGINE_CALL(e, e->E->set_vblocks(kind, n, chs, v));
}
int ccx_set_vblock(ccx_engine *e, int32_t kind, int32_t ch, const double *v) {
  ENGINE_CALL(e, e->E->set_vblock(kind, ch, v));
}
int ccx_generate_interaction(ccx_engine *e, const ccx_potential *pot) {
  if (!pot) return fail(CCX_EINVAL, "null potential");
  ENGINE_CALL(e, {
    if (pot->kind != CCX_POT_MINNESOTA && pot->kind != CCX_POT_CHIRAL_LIKE) throw std::invalid_argument("unknown potential kind");
    ccx::PotentialSpec p;
    p.kind = pot->kind;
    p.lec_seed = pot->lec_seed;
    p.f32_literals = pot->f32_literals;
    e->E->generate(p);
  });
}
int ccx_get_e0(ccx_engine *e, double e0[2]) {
  if (!e0) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, e->E->get_e0(e0));
}
int ccx_get_vblock(ccx_engine *e, int32_t kind, int32_t ch, double *v) { ENGINE_CALL(e, e->E->get_vblock(kind, ch, v)); }
int ccx_get_fock(ccx_engine *e, double *f) {
  if (!f) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, e->E->get_fock(f));
}
int ccx_engine_stream(const ccx_engine *e, void **stream) {
  if (!stream) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, *stream = e->E->stream());
}
int ccx_device_fp64_peak(int32_t device, double *tflops) {
  if (!tflops) return fail(CCX_EINVAL, "null argument");
  return guard([&] {
    const double v = ccx::fp64_peak(device);
    if (v <= 0) throw ccx::EngineError(CCX_ECUDA, "FP64 probe failed (no GPU?)");
    *tflops = v;
  });
}
int ccx_selftest_tc_gemm(int32_t device, int32_t kind, int32_t nprob, const int32_t *M, const int32_t *N,
                         const int32_t *K, int32_t use_alo, uint64_t seed, double *max_rel_err, double *ms) {
  if (!M || !N || !K || !max_rel_err || !ms || nprob <= 0 || kind < 0 || kind > 2)
    return fail(CCX_EINVAL, "bad selftest arguments");
  return guard([&] { ccx::tc_selftest(device, kind, nprob, M, N, K, use_alo, seed, max_rel_err, ms); });
}
int ccx_host_alloc(int64_t bytes, void **ptr) {
  if (!ptr || bytes <= 0) return fail(CCX_EINVAL, "bad host allocation arguments");
  *ptr = nullptr;
  const cudaError_t e = cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocPortable | cudaHostAllocMapped);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    return fail(CCX_ENOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
  }
  return CCX_OK;
}
int ccx_host_free(void *ptr) {
  if (!ptr) return CCX_OK;
  const cudaError_t e = cudaFreeHost(ptr);
  return e == cudaSuccess ? CCX_OK : fail(CCX_ECUDA, std::string("cudaFreeHost: ") + cudaGetErrorString(e));
}
int ccx_selftest_tc_wait(int32_t device, int64_t wait_cycles, int32_t *kernel_error) {
  if (!kernel_error || wait_cycles <= 0) return fail(CCX_EINVAL, "bad selftest arguments");
  return guard([&] {
    // two BF16x3 problems, 384 x 96 x 640 and 200 x 48 x 300, through the persistent kernel
    const int32_t M[2] = {384, 200}, N[2] = {96, 48}, K[2] = {640, 300};
    double rel = 0.0, ms = 0.0;
    int err = 0;
    ccx::tc_selftest(device, 0, 2, M, N, K, 1, 7, &rel, &ms, wait_cycles, &err);
    *kernel_error = err;
    if (err == 0 && !(rel < 2e-4)) throw ccx::EngineError(CCX_ENUMERIC, "tensor-core self-test product is wrong");
  });
}
int ccx_setup_t_amplitudes(ccx_engine *e) { ENGINE_CALL(e, e->E->mp2()); }
int ccx_set_t2(ccx_engine *e, int32_t ch, const double *t) {
  if (!t) return fail(CCX_EINVAL, "null T2 block");
  ENGINE_CALL(e, e->E->set_t2(ch, t));
}
int ccx_get_t2(ccx_engine *e, int32_t ch, double *t) {
  if (!t) return fail(CCX_EINVAL, "null T2 block");
  ENGINE_CALL(e, e->E->get_t2(ch, t));
}
int ccx_get_t2_eqn(ccx_engine *e, int32_t ch, double *r) {
  if (!r) return fail(CCX_EINVAL, "null block");
  ENGINE_CALL(e, e->E->get_r2(ch, r));
}
int ccx_set_t2_all(ccx_engine *e, const double *t) {
  if (!t) return fail(CCX_EINVAL, "null T2");
  ENGINE_CALL(e, e->E->set_t2_all(t));
}
int ccx_get_t2_all(ccx_engine *e, double *t) {
  if (!t) return fail(CCX_EINVAL, "null T2");
  ENGINE_CALL(e, e->E->get_t2_all(t));
}
int ccx_get_denominators(ccx_engine *e, double *d2ij, double *d2ab) {
  if (!d2ij || !d2ab) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, e->E->get_denominators(d2ij, d2ab));
}
int ccx_t2_intermediate(ccx_engine *e) { ENGINE_CALL(e, e->E->t2_intermediate()); }
int ccx_diis_setup(ccx_engine *e, int32_t subspace, int32_t step) { ENGINE_CALL(e, e->E->diis_setup(subspace, step)); }
int ccx_diis_t1t2(ccx_engine *e, int32_t *count) {
  if (!count) return fail(CCX_EINVAL, "null count");
  ENGINE_CALL(e, {
    int c = *count;
    e->E->diis_t1t2(&c);
    *count = c;
  });
}
int ccx_ccd_energy(ccx_engine *e, double ener[2]) {
  if (!ener) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, e->E->energy(ener));
}
int ccx_residual_norm(ccx_engine *e, double *norm) {
  if (!norm) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, *norm = e->E->residual_norm());
}
int ccx_engine_prepare(ccx_engine *e, const ccx_iter_opts *opt) {
  if (!opt) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, {
    ccx::IterOpts o;
    o.mode = opt->mode;
    o.precision = opt->precision;
    o.max_iter = opt->max_iter;
    o.tol = opt->tol;
    o.diis_dim = opt->diis_dim;
    o.defect_period = opt->defect_period;
    o.rebase = opt->rebase;
    o.rebase_drop = opt->rebase_drop;
    o.verbose = opt->verbose;
    e->E->prepare(o);
  });
}
int ccx_ccd_iter(ccx_engine *e, const ccx_iter_opts *opt, ccx_iter_result *res) {
  if (!opt || !res) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, {
    if (opt->max_iter < 1) throw std::invalid_argument("max_iter must be >= 1");
    if (!(opt->tol > 0)) throw std::invalid_argument("tol must be positive");
    ccx::IterOpts o;
    o.mode = opt->mode;
    o.precision = opt->precision;
    o.max_iter = opt->max_iter;
    o.tol = opt->tol;
    o.diis_dim = opt->diis_dim;
    o.defect_period = opt->defect_period;
    o.rebase = opt->rebase;
    o.rebase_drop = opt->rebase_drop;
    o.verbose = opt->verbose;
    ccx::IterResult r;
    e->E->ccd_iter(o, r);
    res->iterations = r.iterations;
    res->converged = r.converged;
    res->e_mbpt2[0] = r.e_mbpt2[0];
    res->e_mbpt2[1] = r.e_mbpt2[1];
    res->e_ccd[0] = r.e_ccd[0];
    res->e_ccd[1] = r.e_ccd[1];
    res->res_norm = r.res_norm;
    res->seconds = r.seconds;
    res->fp64_sweeps = r.fp64_sweeps;
    res->mixed_iterations = r.mixed_iterations;
  });
}
int ccx_pert_triples(ccx_engine *e, double et[2]) {
  if (!et) return fail(CCX_EINVAL, "null argument");
  ENGINE_CALL(e, e->E->triples(et));
}

}  // extern "C"
