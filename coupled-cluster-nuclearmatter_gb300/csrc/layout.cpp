// Host-side basis and channel layout (see layout.hpp).
#include "layout.hpp"

#include <cmath>
#include <cstdio>
#include <sstream>
#include <stdexcept>

namespace ccx {

namespace {

// Constants of the reference's constants module (ccm_modules.f90:91-95).  p_mass
// is a default-real literal there, so its value is the 4-byte rounding of 939.565.
constexpr double kPi = 3.14159265358979;
constexpr double kHbarc = 197.326968;
const double kPMass = (double)939.565f;

// Index sort with the exact step sequence of the reference's `index` routine
// (ccm_main.f90:2654-2732): straight insertion below 7 elements, otherwise a
// median-of-three partition with an explicit stack.  Ties in |k|^2 are frequent
// on the lattice, and the holes are the first A sorted states, so the tie order
// decides the layout; any other sort would give a different (valid) basis order.
// a[1..n] keys, perm[1..n] receives the sorted positions.
void index_sort(int n, const std::vector<double> &a, std::vector<int> &perm) {
  perm.assign(n + 1, 0);
  for (int j = 1; j <= n; ++j) perm[j] = j;
  std::vector<int> stack(2 * 64 + 2, 0);
  int top = 0, lo = 1, hi = n;
  auto key = [&](int pos) { return a[perm[pos]]; };
  while (true) {
    if (hi - lo < 7) {
      for (int j = lo + 1; j <= hi; ++j) {
        const int cur = perm[j];
        const double v = a[cur];
        int i = j - 1;
        while (i >= 1 && key(i) > v) {
          perm[i + 1] = perm[i];
          --i;
        }
        perm[i + 1] = cur;
      }
      if (top == 0) return;
      hi = stack[top];
      lo = stack[top - 1];
      top -= 2;
      continue;
    }
    const int mid = (lo + hi) / 2;
    std::swap(perm[mid], perm[lo + 1]);
    if (key(lo + 1) > key(hi)) std::swap(perm[lo + 1], perm[hi]);
    if (key(lo) > key(hi)) std::swap(perm[lo], perm[hi]);
    if (key(lo + 1) > key(lo)) std::swap(perm[lo + 1], perm[lo]);
    int i = lo + 1, j = hi;
    const int pivot = perm[lo];
    const double pv = a[pivot];
    while (true) {
      do ++i; while (key(i) < pv);
      do --j; while (key(j) > pv);
      if (j < i) break;
      std::swap(perm[i], perm[j]);
    }
    perm[lo] = perm[j];
    perm[j] = pivot;
    top += 2;
    if (top >= (int)stack.size()) throw std::runtime_error("basis sort: stack overflow");
    if (hi - i + 1 >= j - lo) {
      stack[top] = hi;
      stack[top - 1] = i;
      hi = j - 1;
    } else {
      stack[top] = j - 1;
      stack[top - 1] = lo;
      lo = i;
    }
  }
}

}  // namespace

int32_t Basis::orbitof(int32_t x, int32_t y, int32_t z, int32_t s, int32_t t) const {
  if (x < -nkmax[0] || x > nkmax[0] || y < -nkmax[1] || y > nkmax[1] || z < -nkmax[2] || z > nkmax[2])
    return -1;
  if (t < tzmin || t > tzmax) return -1;
  const int32_t ey = 2 * nkmax[1] + 1, ez = 2 * nkmax[2] + 1;
  size_t idx = ((((size_t)(x + nkmax[0]) * ey + (y + nkmax[1])) * ez + (z + nkmax[2])) * 2 + (s > 0)) * 2 + (t > 0);
  return orbit_of[idx];
}

Basis build_basis(int32_t nmax, int32_t A, bool snm, double density, const double theta[3]) {
  if (nmax < 0 || A <= 0 || !(density > 0.0)) throw std::invalid_argument("basis: bad nmax/A/density");
  Basis B;
  B.A = A;
  B.tzmin = snm ? -1 : 1;
  B.tzmax = 1;
  // lx = (real(below_ef)/dens)**(1/3), ccm_main.f90:943
  B.L = std::pow((double)(float)A / density, 1.0 / 3.0);
  const int nk = 2 * nmax + 1;
  // spin/isospin multiplicity ((szmax-szmin+2)*(tzmax-tzmin+2))/4, ccm_main.f90:1135
  const int g = (4 * (B.tzmax - B.tzmin + 2)) / 4;
  B.ns = g * nk * nk * nk;
  if (A > B.ns) throw std::invalid_argument("basis: more particles than states");
  // k-mesh: theta/L, then (-2 pi i + theta)/L, (+2 pi i + theta)/L, ccm_main.f90:1036-1047
  std::vector<double> mesh[3];
  for (int d = 0; d < 3; ++d) {
    mesh[d].resize(nk);
    mesh[d][0] = theta[d] / B.L;
    for (int i = 1; i <= nmax; ++i) {
      mesh[d][2 * i - 1] = (2.0 * (double)(-i) * kPi + theta[d]) / B.L;
      mesh[d][2 * i] = (2.0 * (double)i * kPi + theta[d]) / B.L;
    }
  }
  const int npt = nk * nk * nk;
  std::vector<double> k2(npt + 1, 0.0);
  {
    int ii = 0;
    for (int i = 0; i < nk; ++i)
      for (int j = 0; j < nk; ++j)
        for (int k = 0; k < nk; ++k) {
          const double x = mesh[0][i] * mesh[0][i], y = mesh[1][j] * mesh[1][j], z = mesh[2][k] * mesh[2][k];
          k2[++ii] = (x + y) + z;
        }
  }
  std::vector<int> sorted;
  index_sort(npt, k2, sorted);
  std::vector<int> rank(npt + 1, 0);
  for (int r = 1; r <= npt; ++r) rank[sorted[r]] = r;

  B.nx.assign(B.ns, 0); B.ny.assign(B.ns, 0); B.nz.assign(B.ns, 0);
  B.sz.assign(B.ns, 0); B.tz.assign(B.ns, 0);
  B.kx.assign(B.ns, 0.0); B.ky.assign(B.ns, 0.0); B.kz.assign(B.ns, 0.0); B.e.assign(B.ns, 0.0);
  const int tzstep = (B.tzmax - B.tzmin + 2) / 2;
  int ii = 0;
  for (int i = 0; i < nk; ++i)
    for (int j = 0; j < nk; ++j)
      for (int k = 0; k < nk; ++k) {
        ++ii;
        const int r = rank[ii];
        int is = 0;
        for (int s = -1; s <= 1; s += 2) {
          ++is;
          int it = 0;
          for (int t = B.tzmin; t <= B.tzmax; t += tzstep) {
            ++it;
            const int o = g * (r - 1) + 2 * (it - 1) + is - 1;
            B.kx[o] = mesh[0][i];
            B.ky[o] = mesh[1][j];
            B.kz[o] = mesh[2][k];
            B.nx[o] = (int32_t)std::lround(((mesh[0][i] * B.L - theta[0]) / 2.0) / kPi);
            B.ny[o] = (int32_t)std::lround(((mesh[1][j] * B.L - theta[1]) / 2.0) / kPi);
            B.nz[o] = (int32_t)std::lround(((mesh[2][k] * B.L - theta[2]) / 2.0) / kPi);
            B.sz[o] = s;
            B.tz[o] = t;
            const double kk = (B.kx[o] * B.kx[o] + B.ky[o] * B.ky[o]) + B.kz[o] * B.kz[o];
            B.e[o] = kk * (kHbarc * kHbarc) / kPMass / 2.0;
          }
        }
      }
  return B;
}

namespace {

void fill_orbit_of(Basis &B) {
  for (int d = 0; d < 3; ++d) B.nkmax[d] = 0;
  for (int i = 0; i < B.ns; ++i) {
    B.nkmax[0] = std::max(B.nkmax[0], B.nx[i]);
    B.nkmax[1] = std::max(B.nkmax[1], B.ny[i]);
    B.nkmax[2] = std::max(B.nkmax[2], B.nz[i]);
  }
  const size_t n = (size_t)(2 * B.nkmax[0] + 1) * (2 * B.nkmax[1] + 1) * (2 * B.nkmax[2] + 1) * 4;
  B.orbit_of.assign(n, -1);
  const int32_t ey = 2 * B.nkmax[1] + 1, ez = 2 * B.nkmax[2] + 1;
  for (int i = 0; i < B.ns; ++i) {
    if (B.nx[i] < -B.nkmax[0] || B.ny[i] < -B.nkmax[1] || B.nz[i] < -B.nkmax[2])
      throw std::invalid_argument("basis: lattice not symmetric about 0");
    size_t idx = ((((size_t)(B.nx[i] + B.nkmax[0]) * ey + (B.ny[i] + B.nkmax[1])) * ez + (B.nz[i] + B.nkmax[2])) * 2 +
                  (B.sz[i] > 0)) * 2 + (B.tz[i] > 0);
    B.orbit_of[idx] = i;
  }
}

// Channel enumeration shared by the pair-sum (sign=+1) and particle-hole
// (sign=-1) families: the bounding box of n_p +/- n_q over all orbital pairs.
void pair_box(const Basis &B, int sign, int32_t lo[3], int32_t hi[3]) {
  for (int d = 0; d < 3; ++d) { lo[d] = 1 << 30; hi[d] = -(1 << 30); }
  int32_t mn[3] = {1 << 30, 1 << 30, 1 << 30}, mx[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
  for (int i = 0; i < B.ns; ++i) {
    const int32_t v[3] = {B.nx[i], B.ny[i], B.nz[i]};
    for (int d = 0; d < 3; ++d) { mn[d] = std::min(mn[d], v[d]); mx[d] = std::max(mx[d], v[d]); }
  }
  for (int d = 0; d < 3; ++d) {
    if (sign > 0) { lo[d] = 2 * mn[d]; hi[d] = 2 * mx[d]; }
    else { lo[d] = mn[d] - mx[d]; hi[d] = mx[d] - mn[d]; }
  }
}

template <typename F>
void for_each_key(const ChannelGrid &g, F f) {
  for (int tz = -1; tz <= 1; ++tz)
    for (int x = g.lo[0]; x <= g.hi[0]; ++x)
      for (int y = g.lo[1]; y <= g.hi[1]; ++y)
        for (int z = g.lo[2]; z <= g.hi[2]; ++z) f(tz, x, y, z);
}

}  // namespace

int32_t Layout::chan3_of_pair(int32_t p, int32_t q) const {
  const int tz = (b.tz[p] + b.tz[q]) / 2;
  return grid[3].get(tz, b.nx[p] + b.nx[q], b.ny[p] + b.ny[q], b.nz[p] + b.nz[q]) - 1;
}

void build_layout(Layout &L) {
  Basis &B = L.b;
  fill_orbit_of(B);
  const int ns = B.ns, A = B.A;
  // ---- pair-sum channels: ccm_iter.f90:199-603 ----
  int32_t lo[3], hi[3];
  pair_box(B, +1, lo, hi);
  ChannelGrid cnt[4];
  for (int k = 1; k <= 3; ++k) cnt[k].init(lo, hi);
  for (int k = 1; k <= 6; ++k) L.grid[k].init(lo, hi);
  for (int a = 0; a < ns; ++a)
    for (int c = 0; c < ns; ++c) {
      const size_t g = cnt[1].index((B.tz[a] + B.tz[c]) / 2, B.nx[a] + B.nx[c], B.ny[a] + B.ny[c], B.nz[a] + B.nz[c]);
      const int kind = (a < A && c < A) ? 1 : (a < A && c >= A) ? 2 : (a >= A && c >= A) ? 3 : 0;
      if (kind) cnt[kind].id[g]++;
    }
  for_each_key(L.grid[1], [&](int tz, int x, int y, int z) {
    const size_t g = cnt[1].index(tz, x, y, z);
    const int32_t nh = cnt[1].id[g], nhp = cnt[2].id[g], npp = cnt[3].id[g];
    auto add = [&](int kind, int32_t n1, int32_t n2) {
      L.grid[kind].id[g] = L.fam[kind].count() + 1;
      L.fam[kind].qn.push_back({tz, x, y, z});
      L.fam[kind].side1.emplace_back();
      L.fam[kind].side2.emplace_back();
      L.fam[kind].side1.back().p.reserve(n1);
      L.fam[kind].side2.back().p.reserve(n2);
    };
    if (nh) add(1, nh, 0);
    if (nh && nhp) add(2, nh, nhp);
    if (nh && npp) add(3, nh, npp);
    if (nhp) add(4, nhp, 0);
    if (nh && npp) add(6, npp, 0);
  });
  // hppp channels of setup_vnn_hppp_block (ccm_iter.f90:1407-1445): hp and pp pairs
  for_each_key(L.grid[1], [&](int tz, int x, int y, int z) {
    const size_t g = cnt[1].index(tz, x, y, z);
    if (cnt[2].id[g] && cnt[3].id[g]) {
      L.grid[5].id[g] = L.fam[5].count() + 1;
      L.fam[5].qn.push_back({tz, x, y, z});
      L.fam[5].side1.emplace_back();
      L.fam[5].side2.emplace_back();
    }
  });
  const size_t nn = (size_t)ns * ns;
  L.hh_hhpp.assign(nn, 0); L.pp_hhpp.assign(nn, 0); L.hh_hhhh.assign(nn, 0);
  L.hp_hphp.assign(nn, 0); L.hh_hhhp.assign(nn, 0); L.hp_hhhp.assign(nn, 0);
  L.hp_hppp.assign(nn, 0); L.pp_hppp.assign(nn, 0);
  auto key_of = [&](int p, int q, int kind) {
    return L.grid[kind].get((B.tz[p] + B.tz[q]) / 2, B.nx[p] + B.nx[q], B.ny[p] + B.ny[q], B.nz[p] + B.nz[q]);
  };
  // hole-hole pairs, a outer / b inner over the holes (ccm_iter.f90:415-481)
  for (int p = 0; p < A; ++p)
    for (int q = 0; q < A; ++q) {
      if (int c = key_of(p, q, 1)) { L.fam[1].side1[c - 1].push(p, q); L.hh_hhhh[(size_t)p * ns + q] = L.fam[1].side1[c - 1].size(); }
      if (int c = key_of(p, q, 2)) { L.fam[2].side1[c - 1].push(p, q); L.hh_hhhp[(size_t)p * ns + q] = L.fam[2].side1[c - 1].size(); }
      if (int c = key_of(p, q, 3)) { L.fam[3].side1[c - 1].push(p, q); L.hh_hhpp[(size_t)p * ns + q] = L.fam[3].side1[c - 1].size(); }
    }
  // hole-particle pairs (ccm_iter.f90:486-550)
  for (int p = 0; p < A; ++p)
    for (int q = A; q < ns; ++q) {
      if (int c = key_of(p, q, 2)) { L.fam[2].side2[c - 1].push(p, q); L.hp_hhhp[(size_t)p * ns + q] = L.fam[2].side2[c - 1].size(); }
      if (int c = key_of(p, q, 4)) { L.fam[4].side1[c - 1].push(p, q); L.hp_hphp[(size_t)p * ns + q] = L.fam[4].side1[c - 1].size(); }
      if (int c = key_of(p, q, 5)) { L.fam[5].side1[c - 1].push(p, q); L.hp_hppp[(size_t)p * ns + q] = L.fam[5].side1[c - 1].size(); }
    }
  // particle-particle pairs (ccm_iter.f90:556-603); the pppp list equals the hhpp one
  for (int p = A; p < ns; ++p)
    for (int q = A; q < ns; ++q) {
      if (int c = key_of(p, q, 3)) {
        L.fam[3].side2[c - 1].push(p, q);
        L.pp_hhpp[(size_t)p * ns + q] = L.fam[3].side2[c - 1].size();
        L.fam[6].side1[key_of(p, q, 6) - 1].push(p, q);
      }
      if (int c = key_of(p, q, 5)) { L.fam[5].side2[c - 1].push(p, q); L.pp_hppp[(size_t)p * ns + q] = L.fam[5].side2[c - 1].size(); }
    }
  // ---- particle-hole channels keyed by n_p - n_q (ccm_iter.f90:1840-2105) ----
  pair_box(B, -1, lo, hi);
  ChannelGrid c1, c2;
  c1.init(lo, hi);
  c2.init(lo, hi);
  for (int k = 1; k <= 3; ++k) L.phgrid[k].init(lo, hi);
  for (int a = 0; a < ns; ++a)
    for (int c = 0; c < ns; ++c) {
      const size_t g = c1.index((B.tz[a] - B.tz[c]) / 2, B.nx[a] - B.nx[c], B.ny[a] - B.ny[c], B.nz[a] - B.nz[c]);
      if (a < A && c >= A) c1.id[g]++;
      if (a >= A && c < A) c2.id[g]++;
    }
  for_each_key(L.phgrid[1], [&](int tz, int x, int y, int z) {
    const size_t g = c1.index(tz, x, y, z);
    auto add = [&](int kind) {
      L.phgrid[kind].id[g] = L.ph[kind].count() + 1;
      L.ph[kind].qn.push_back({tz, x, y, z});
      L.ph[kind].side1.emplace_back();
      L.ph[kind].side2.emplace_back();
    };
    if (c2.id[g] && c1.id[g]) add(1);
    if (c1.id[g]) add(2);
    if (c1.id[g] && c2.id[g]) add(3);
  });
  L.ph_ph_phhp.assign(nn, 0);
  L.hp_ph_phhp.assign(nn, 0);
  auto dkey = [&](int p, int q, int kind) {
    return L.phgrid[kind].get((B.tz[p] - B.tz[q]) / 2, B.nx[p] - B.nx[q], B.ny[p] - B.ny[q], B.nz[p] - B.nz[q]);
  };
  for (int p = 0; p < A; ++p)
    for (int q = A; q < ns; ++q) {
      if (int c = dkey(p, q, 1)) { L.ph[1].side2[c - 1].push(p, q); L.hp_ph_phhp[(size_t)p * ns + q] = L.ph[1].side2[c - 1].size(); }
      if (int c = dkey(p, q, 2)) L.ph[2].side1[c - 1].push(p, q);
      if (int c = dkey(p, q, 3)) L.ph[3].side1[c - 1].push(p, q);
    }
  for (int p = A; p < ns; ++p)
    for (int q = 0; q < A; ++q) {
      if (int c = dkey(p, q, 1)) { L.ph[1].side1[c - 1].push(p, q); L.ph_ph_phhp[(size_t)p * ns + q] = L.ph[1].side1[c - 1].size(); }
      if (int c = dkey(p, q, 3)) L.ph[3].side2[c - 1].push(p, q);
    }

  // ---- packed tables for the device ----
  const int nc = L.fam[3].count();
  L.pk.assign(nc, PackedChannel());
  int64_t toff = 0, aoff = 0;
  for (int c = 0; c < nc; ++c) {
    PackedChannel &P = L.pk[c];
    const PairList &hh = L.fam[3].side1[c], &pp = L.fam[3].side2[c];
    P.n_hh = hh.size();
    P.n_pp = pp.size();
    P.hh_packed.assign(P.n_hh, 0);
    P.pp_packed.assign(P.n_pp, 0);
    for (int r = 0; r < P.n_hh; ++r)
      if (hh.p[r] < hh.q[r]) { P.hh_of_packed.push_back(r); P.hh_packed[r] = ++P.H; }
    for (int r = 0; r < P.n_pp; ++r)
      if (pp.p[r] < pp.q[r]) { P.pp_of_packed.push_back(r); P.pp_packed[r] = ++P.P; }
    // the swapped pair (q,p) sits in the same channel; its packed slot carries a minus sign
    for (int r = 0; r < P.n_hh; ++r)
      if (hh.p[r] > hh.q[r]) P.hh_packed[r] = -P.hh_packed[L.hh_hhpp[(size_t)hh.q[r] * ns + hh.p[r]] - 1];
    for (int r = 0; r < P.n_pp; ++r)
      if (pp.p[r] > pp.q[r]) P.pp_packed[r] = -P.pp_packed[L.pp_hhpp[(size_t)pp.q[r] * ns + pp.p[r]] - 1];
    P.t_off = toff;
    P.amp_off = aoff;
    toff += (int64_t)P.P * P.H;
    aoff += (int64_t)P.n_pp * P.n_hh;
    const auto &q = L.fam[3].qn[c];
    P.hhhh = L.grid[1].get(q[0], q[1], q[2], q[3]) - 1;
  }
  L.n_amps = aoff;
  L.n_tpacked = toff;
}

uint64_t Layout::hash() const {
  uint64_t h = 1469598103934665603ULL;
  auto mix = [&](const void *p, size_t n) {
    const unsigned char *c = (const unsigned char *)p;
    for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ULL; }
  };
  mix(&b.ns, sizeof b.ns);
  mix(&b.A, sizeof b.A);
  mix(b.nx.data(), b.ns * 4); mix(b.ny.data(), b.ns * 4); mix(b.nz.data(), b.ns * 4);
  mix(b.sz.data(), b.ns * 4); mix(b.tz.data(), b.ns * 4);
  for (int k : {1, 2, 3, 4}) {
    for (int c = 0; c < fam[k].count(); ++c) {
      mix(fam[k].qn[c].data(), 16);
      for (const PairList *l : {&fam[k].side1[c], &fam[k].side2[c]}) {
        mix(l->p.data(), l->p.size() * 4);
        mix(l->q.data(), l->q.size() * 4);
      }
    }
  }
  for (int k : {1, 2, 3}) {
    for (int c = 0; c < ph[k].count(); ++c) {
      mix(ph[k].qn[c].data(), 16);
      for (const PairList *l : {&ph[k].side1[c], &ph[k].side2[c]}) {
        mix(l->p.data(), l->p.size() * 4);
        mix(l->q.data(), l->q.size() * 4);
      }
    }
  }
  return h;
}

std::string describe(const Layout &L) {
  std::ostringstream s;
  s << "states " << L.b.ns << " holes " << L.b.A << " L " << L.b.L << " hhpp " << L.fam[3].count() << " amps "
    << L.n_amps << " packed " << L.n_tpacked << " ph " << L.ph[1].count();
  return s.str();
}

}  // namespace ccx
