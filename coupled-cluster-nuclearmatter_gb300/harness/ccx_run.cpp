// ccx_run: a host program that drives the C ABI (include/ccx.h) the way the reference's
// Fortran driver drives its solver, so that the boundary can be exercised where no
// Fortran compiler exists.
//
//   ccm_main.f90:31-32, 893-1197   read ccm_in, build the basis    -> ccx_deck_parse,
//                                                                     ccx_layout_from_basis
//   ccm_iter.f90:819-1311          the vnn_* blocks (host arrays)  -> ccx_set_fock,
//                                                                     ccx_set_vblock per channel
//   ccm_iter.f90:2329-2368         setup_t_amplitudes (MP2)        -> ccx_setup_t_amplitudes
//   ccm_iter.f90:20-96             ccd_iter: t2_intermediate,      -> ccx_t2_intermediate,
//                                  diis_t1t2, ccd_energy_save,        ccx_diis_t1t2,
//                                  |dE| < 1e-6                        ccx_ccd_energy
//   ccm_triples.f90:528-735        pert_triples2                   -> ccx_pert_triples
//
// "--blocks host" hands the interaction over as the Fortran shim would: every block is
// held in a host array in the reference's layout and passed with ccx_set_vblock (the
// arrays are exported from a device-generated helper engine, since the synthetic
// potentials are generated on the device).  "--loop solver" runs ccx_ccd_iter instead
// of the reference loop.  Output is one "key value..." line per result; "--json" adds
// one JSON line per iteration and a final result record (the values of the (8f12.5)
// line ccm_main.f90:338-339 writes).
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ccx.h"

namespace {

struct Args {
  std::string deck, load, save, blocks = "generated", loop, mode, precision, rebase = "digits", pot;
  int nmax = -1, A = -1, snm = -1, device = 0, max_iter = -1, diis = 8, scalar = -1;
  double density = -1.0, theta[3] = {0, 0, 0}, tol = -1.0;
  bool triples = false, layout_only = false, has_theta = false, f64_literals = false, json = false;
};

[[noreturn]] void usage(const char *msg) {
  if (msg) std::fprintf(stderr, "ccx_run: %s\n", msg);
  std::fprintf(stderr,
               "usage: ccx_run [--deck ccm_in | --nmax N --A A --density RHO [--snm] [--theta X Y Z]]\n"
               "               [--potential minnesota|chiral_like] [--real|--complex] [--blocks generated|host]\n"
               "               [--loop shim|solver] [--mode reference|standard] [--precision fp64|bf16x3|tf32x3]\n"
               "               [--rebase fp64|digits] [--tol T] [--max-iter N] [--diis N] [--triples]\n"
               "               [--load FILE] [--save FILE] [--device D] [--layout-only] [--f64-literals]\n"
               "               [--json]\n");
  std::exit(2);
}

// a failed ABI call: its status and message, and the status as the exit code
void check(int rc, const char *what) {
  if (rc == CCX_OK) return;
  std::fprintf(stderr, "ccx_run: %s failed with status %d: %s\n", what, rc, ccx_last_error());
  std::exit(rc);
}

Args parse(int argc, char **argv) {
  Args a;
  for (int i = 1; i < argc; ++i) {
    const std::string k = argv[i];
    auto val = [&](const char *name) -> const char * {
      if (i + 1 >= argc) usage((std::string("missing value of ") + name).c_str());
      return argv[++i];
    };
    auto num = [&](const char *name) {
      const char *s = val(name);
      char *end = nullptr;
      errno = 0;
      const double v = std::strtod(s, &end);
      if (errno || end == s || *end) usage((std::string("bad number for ") + name).c_str());
      return v;
    };
    if (k == "--deck") a.deck = val("--deck");
    else if (k == "--nmax") a.nmax = (int)num("--nmax");
    else if (k == "--A") a.A = (int)num("--A");
    else if (k == "--density") a.density = num("--density");
    else if (k == "--snm") a.snm = 1;
    else if (k == "--theta") {
      for (double &t : a.theta) t = num("--theta");
      a.has_theta = true;
    } else if (k == "--potential") a.pot = val("--potential");
    else if (k == "--real") a.scalar = CCX_SCALAR_REAL;
    else if (k == "--complex") a.scalar = CCX_SCALAR_COMPLEX;
    else if (k == "--blocks") a.blocks = val("--blocks");
    else if (k == "--loop") a.loop = val("--loop");
    else if (k == "--mode") a.mode = val("--mode");
    else if (k == "--precision") a.precision = val("--precision");
    else if (k == "--rebase") a.rebase = val("--rebase");
    else if (k == "--tol") a.tol = num("--tol");
    else if (k == "--max-iter") a.max_iter = (int)num("--max-iter");
    else if (k == "--diis") a.diis = (int)num("--diis");
    else if (k == "--triples") a.triples = true;
    else if (k == "--load") a.load = val("--load");
    else if (k == "--save") a.save = val("--save");
    else if (k == "--device") a.device = (int)num("--device");
    else if (k == "--layout-only") a.layout_only = true;
    else if (k == "--f64-literals") a.f64_literals = true;
    else if (k == "--json") a.json = true;
    else if (k == "-h" || k == "--help") usage(nullptr);
    else usage(("unknown option " + k).c_str());
  }
  if (a.blocks != "generated" && a.blocks != "host") usage("--blocks is generated or host");
  return a;
}

std::string read_file(const std::string &path) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) {
    std::fprintf(stderr, "ccx_run: cannot open %s: %s\n", path.c_str(), std::strerror(errno));
    std::exit(CCX_EINVAL);
  }
  std::string s;
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, n);
  std::fclose(f);
  return s;
}

// a JSON number: shortest round-trip form; NaN and Inf (which JSON lacks) as null
std::string jnum(double v) {
  if (!std::isfinite(v)) return "null";
  char b[32];
  std::snprintf(b, sizeof b, "%.17g", v);
  return b;
}

const char *kIterKind[] = {"reference", "fp64", "mixed"};
const char *kTermName[] = {"tph_gather", "i9_i7", "i6", "i4", "ring", "r_init", "ladders", "update", "diis"};

// one iteration of the solve as a JSON line: the energy per nucleon, its change, the
// residual norm (null where the loop has none) and the times
void json_iteration(const ccx_iter_record &r, double e0, int A, bool has_norm) {
  std::string s = "{\"record\": \"iteration\", \"iteration\": " + std::to_string(r.iteration) + ", \"kind\": \"" +
                  kIterKind[r.kind] + "\", \"e_ccd\": [" + jnum(r.energy[0]) + ", " + jnum(r.energy[1]) +
                  "], \"e_per_a\": " + jnum((e0 + r.energy[0]) / A) + ", \"de\": " + jnum(r.de) +
                  ", \"res_norm\": " + (has_norm ? jnum(r.res_norm) : std::string("null")) +
                  ", \"ms\": " + jnum(r.ms);
  bool timed = false;
  for (double t : r.term_ms) timed = timed || t != 0.0;
  if (timed) {
    s += ", \"term_ms\": {";
    for (int k = 0; k < 9; ++k) s += std::string(k ? ", " : "") + "\"" + kTermName[k] + "\": " + jnum(r.term_ms[k]);
    s += "}";
  }
  std::printf("%s}\n", s.c_str());
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// every V block of a generated engine `from`, handed to `to` one channel at a time from
// host arrays in the reference's layout, as the Fortran shim passes vnn_*(ch)%val
void hand_over_blocks(ccx_layout *L, ccx_engine *from, ccx_engine *to, int n_states) {
  std::vector<double> fock((size_t)2 * n_states * n_states);
  double e0[2];
  check(ccx_get_fock(from, fock.data()), "ccx_get_fock");
  check(ccx_get_e0(from, e0), "ccx_get_e0");
  check(ccx_set_fock(to, fock.data(), e0), "ccx_set_fock");
  int64_t counts[8];
  check(ccx_layout_counts(L, counts), "ccx_layout_counts");
  struct Fam {
    int32_t kind, chkind;
    int64_t n;
    bool square_pp;
  };
  const Fam fams[] = {{CCX_CH_HHPP, CCX_CH_HHPP, counts[0], false},
                      {CCX_V_PPPP, CCX_CH_HHPP, counts[0], true},
                      {CCX_CH_HHHH, CCX_CH_HHHH, counts[1], false},
                      {CCX_CH_HPHP, CCX_CH_HPHP, counts[3], false}};
  std::vector<double> v;
  for (const Fam &f : fams)
    for (int32_t ch = 0; ch < (int32_t)f.n; ++ch) {
      int32_t qn[4], n1 = 0, n2 = 0;
      check(ccx_layout_channel(L, f.chkind, ch, qn, &n1, &n2), "ccx_layout_channel");
      const int64_t rows = f.square_pp ? n2 : n1, cols = (f.kind == CCX_CH_HHHH || f.kind == CCX_CH_HPHP) ? n1 : n2;
      if (rows * cols == 0) continue;
      v.assign((size_t)2 * rows * cols, 0.0);
      check(ccx_get_vblock(from, f.kind, ch, v.data()), "ccx_get_vblock");
      check(ccx_set_vblock(to, f.kind, ch, v.data()), "ccx_set_vblock");
    }
}

}  // namespace

int main(int argc, char **argv) {
  Args a = parse(argc, argv);
  ccx_deck d{};
  bool have_deck = false;
  if (!a.deck.empty()) {
    check(ccx_deck_parse(read_file(a.deck).c_str(), &d), "ccx_deck_parse");
    have_deck = true;
  }
  // the basis: the deck's values (density, or kfermi as ccm_main.f90:930-945 converts
  // it), with command-line values taking precedence
  ccx_basis_params bp{};
  bp.nmax = a.nmax >= 0 ? a.nmax : (have_deck ? d.nmax : -1);
  bp.A = a.A >= 0 ? a.A : (have_deck ? d.A : -1);
  bp.snm = a.snm >= 0 ? a.snm : (have_deck ? d.snm : 0);
  double rho = a.density;
  if (rho < 0 && have_deck) {
    const double pi = 3.14159265358979323846;
    rho = d.input_is_kfermi ? (d.snm ? 2.0 : 1.0) * d.dens_or_kf * d.dens_or_kf * d.dens_or_kf / 3.0 / (pi * pi)
                            : d.dens_or_kf;
  }
  bp.density = rho;
  for (int k = 0; k < 3; ++k) bp.theta[k] = a.has_theta ? a.theta[k] : (have_deck ? d.theta[k] : 0.0);
  if (bp.nmax < 0 || bp.A <= 0 || bp.density <= 0) usage("give a deck, or --nmax, --A and --density");

  ccx_layout *L = nullptr;
  check(ccx_layout_from_basis(&bp, &L), "ccx_layout_from_basis");
  int64_t c[8];
  uint64_t hash = 0;
  check(ccx_layout_counts(L, c), "ccx_layout_counts");
  check(ccx_layout_hash(L, &hash), "ccx_layout_hash");
  ccx_orbits orb{};
  check(ccx_layout_orbits(L, &orb), "ccx_layout_orbits");
  std::printf("layout states %d holes %d box_fm %.10g hhpp %lld hhhh %lld hhhp %lld hphp %lld ph %lld amps %lld "
              "hash %016llx\n",
              orb.n_states, orb.n_holes, orb.box_length, (long long)c[0], (long long)c[1], (long long)c[2],
              (long long)c[3], (long long)c[4], (long long)c[7], (unsigned long long)hash);
  std::fflush(stdout);
  if (a.layout_only) {
    ccx_layout_destroy(L);
    return 0;
  }

  // the interaction and the engine
  const std::string pot = !a.pot.empty() ? a.pot
                          : (have_deck && d.potential == CCX_POT_CHIRAL_LIKE) ? "chiral_like"
                                                                              : "minnesota";
  if (pot != "minnesota" && pot != "chiral_like") usage("--potential is minnesota or chiral_like");
  ccx_potential p{};
  p.kind = pot == "chiral_like" ? CCX_POT_CHIRAL_LIKE : CCX_POT_MINNESOTA;
  p.lec_seed = have_deck ? d.lec_seed : 20261203ull;
  // the reference writes the Minnesota constants and the nucleon mass as default-real
  // (4-byte) literals; --f64-literals keeps them in double precision
  p.f32_literals = a.f64_literals ? 0 : 1;
  ccx_engine_options eo{};
  eo.device = a.device;
  eo.scalar = a.scalar >= 0 ? a.scalar : (p.kind == CCX_POT_CHIRAL_LIKE ? CCX_SCALAR_COMPLEX : CCX_SCALAR_REAL);
  ccx_engine *E = nullptr;
  check(ccx_engine_create(L, &eo, &E), "ccx_engine_create");
  if (a.blocks == "host") {
    ccx_engine *G = nullptr;
    check(ccx_engine_create(L, &eo, &G), "ccx_engine_create");
    check(ccx_generate_interaction(G, &p), "ccx_generate_interaction");
    hand_over_blocks(L, G, E, orb.n_states);
    check(ccx_engine_destroy(G), "ccx_engine_destroy");
  } else {
    check(ccx_generate_interaction(E, &p), "ccx_generate_interaction");
  }
  double e0[2];
  check(ccx_get_e0(E, e0), "ccx_get_e0");
  std::printf("e0 %.17g %.17g\n", e0[0], e0[1]);

  // the amplitudes: MP2, or a checkpoint of this lattice
  std::vector<double> t2((size_t)2 * c[7]);
  if (!a.load.empty()) {
    check(ccx_t2_checkpoint_read(L, a.load.c_str(), 0, t2.data()), "ccx_t2_checkpoint_read");
    check(ccx_set_t2_all(E, t2.data()), "ccx_set_t2_all");
  } else {
    check(ccx_setup_t_amplitudes(E), "ccx_setup_t_amplitudes");
  }

  const std::string mode = !a.mode.empty() ? a.mode
                           : (have_deck && d.mode == CCX_MODE_STANDARD) ? "standard"
                                                                       : "reference";
  if (mode != "reference" && mode != "standard") usage("--mode is reference or standard");
  const std::string loop = !a.loop.empty() ? a.loop : (mode == "reference" ? "shim" : "solver");
  if (loop != "shim" && loop != "solver") usage("--loop is shim or solver");
  if (loop == "shim" && mode != "reference") usage("the reference loop (--loop shim) runs the reference mode");
  const double tol = a.tol > 0 ? a.tol : (have_deck ? d.tol : (mode == "reference" ? 1e-6 : 1e-10));
  const int max_iter = a.max_iter > 0 ? a.max_iter : (have_deck ? d.max_iter : 100);

  double ener1[2], ener2[2] = {0, 0};
  check(ccx_ccd_energy(E, ener1), "ccx_ccd_energy");
  std::printf("e_mbpt2 %.17g %.17g\n", ener1[0], ener1[1]);
  const double e_mbpt2 = ener1[0];
  const double t0 = now();
  int iterations = 0;
  double e_ccd[2];
  if (loop == "shim") {
    // ccd_iter (ccm_iter.f90:20-96): subspace 6, DIIS every 6, stop on |dE| <= tol
    check(ccx_diis_setup(E, 6, 6), "ccx_diis_setup");
    int32_t count = 0;
    double dener = 4.0, tprev = now();
    for (int it = 1; it <= max_iter && std::fabs(dener) > tol; ++it) {
      check(ccx_t2_intermediate(E), "ccx_t2_intermediate");
      ++count;
      check(ccx_diis_t1t2(E, &count), "ccx_diis_t1t2");
      check(ccx_ccd_energy(E, ener2), "ccx_ccd_energy");
      dener = ener2[0] - ener1[0];
      ener1[0] = ener2[0];
      ener1[1] = ener2[1];
      iterations = it;
      std::printf("iter %d e_ccd %.17g de %.3e\n", it, ener2[0], dener);
      if (a.json) {
        ccx_iter_record rec{};
        rec.iteration = it;
        rec.kind = CCX_ITER_REFERENCE;
        rec.energy[0] = ener2[0];
        rec.energy[1] = ener2[1];
        rec.de = dener;
        const double t = now();
        rec.ms = 1e3 * (t - tprev);
        tprev = t;
        json_iteration(rec, e0[0], bp.A, false);
      }
    }
    e_ccd[0] = ener1[0];
    e_ccd[1] = ener1[1];
  } else {
    ccx_iter_opts o{};
    o.mode = mode == "standard" ? CCX_MODE_STANDARD : CCX_MODE_REFERENCE;
    if (a.precision.empty()) o.precision = have_deck ? d.precision : CCX_PREC_FP64;
    else if (a.precision == "fp64") o.precision = CCX_PREC_FP64;
    else if (a.precision == "bf16x3") o.precision = CCX_PREC_MIXED;
    else if (a.precision == "tf32x3") o.precision = CCX_PREC_MIXED_TF32;
    else usage("--precision is fp64, bf16x3 or tf32x3");
    o.max_iter = max_iter;
    o.tol = tol;
    o.diis_dim = a.diis;
    o.rebase = a.rebase == "fp64" ? CCX_REBASE_FP64 : CCX_REBASE_DIGITS;
    ccx_iter_result r{};
    check(ccx_ccd_iter(E, &o, &r), "ccx_ccd_iter");
    iterations = r.iterations;
    e_ccd[0] = r.e_ccd[0];
    e_ccd[1] = r.e_ccd[1];
    std::printf("converged %d res_norm %.3e fp64_sweeps %d mixed_iterations %d\n", r.converged, r.res_norm,
                r.fp64_sweeps, r.mixed_iterations);
    if (a.json) {
      int32_t n = 0;
      check(ccx_engine_iter_log(E, 0, nullptr, &n), "ccx_engine_iter_log");
      std::vector<ccx_iter_record> log((size_t)n);
      if (n > 0) check(ccx_engine_iter_log(E, n, log.data(), &n), "ccx_engine_iter_log");
      for (const ccx_iter_record &rec : log) json_iteration(rec, e0[0], bp.A, true);
    }
  }
  const double secs = now() - t0;
  std::printf("e_ccd %.17g %.17g\n", e_ccd[0], e_ccd[1]);
  std::printf("e_per_a %.17g\n", (e0[0] + e_ccd[0]) / bp.A);
  std::printf("iterations %d seconds %.6f\n", iterations, secs);
  const bool triples = a.triples || (have_deck && std::strcmp(d.cc_approx, "CCD(T)") == 0);
  double et[2] = {0, 0};
  if (triples) {
    check(ccx_pert_triples(E, et), "ccx_pert_triples");
    std::printf("e_triples %.17g %.17g\n", et[0], et[1]);
  }
  if (a.json) {
    // ccm_main.f90:338-339: cE, cD, kf, density, and per nucleon E0, MBPT2 = E0 + the MP2
    // correlation energy, E_CCD = E0 + the CCD correlation energy, and E_CCD + E(T)
    // (null where (T) was not computed); kf from the density as ccm_main.f90:930-945
    const double pi = 3.14159265358979323846;
    const double kf = std::cbrt(3.0 * pi * pi * bp.density / (bp.snm ? 2.0 : 1.0));
    const double A = bp.A;
    std::printf("{\"record\": \"result\", \"cE\": %s, \"cD\": %s, \"kf\": %s, \"density\": %s, \"e0_per_a\": %s, "
                "\"mbpt2_per_a\": %s, \"eccd_per_a\": %s, \"eccdt_per_a\": %s, \"iterations\": %d}\n",
                jnum(have_deck ? d.cE : 0.0).c_str(), jnum(have_deck ? d.cD : 0.0).c_str(), jnum(kf).c_str(),
                jnum(bp.density).c_str(), jnum(e0[0] / A).c_str(), jnum((e0[0] + e_mbpt2) / A).c_str(),
                jnum((e0[0] + e_ccd[0]) / A).c_str(),
                triples ? jnum((e0[0] + e_ccd[0] + et[0]) / A).c_str() : "null", iterations);
  }
  if (!a.save.empty()) {
    check(ccx_get_t2_all(E, t2.data()), "ccx_get_t2_all");
    check(ccx_t2_checkpoint_write(L, a.save.c_str(), t2.data()), "ccx_t2_checkpoint_write");
    std::printf("saved %s\n", a.save.c_str());
  }
  check(ccx_engine_destroy(E), "ccx_engine_destroy");
  check(ccx_layout_destroy(L), "ccx_layout_destroy");
  return 0;
}
