// Host-side basis and channel layout of the CCD engine.
//
// Reproduces the reference's single-particle order (setup_sp_data,
// deltafull-CCMkspace/ccm_main.f90:1003-1197) and its two-body channel tables
// (setup_channel_structures, ccm_iter.f90:175-812; setup_ph_channel_structures,
// ccm_iter.f90:1816-2105) so that T2 and V blocks passed across the C ABI have the
// reference's exact shapes and element order.  On top of that it derives the
// packed (a<b, i<j) tables the GPU kernels work on.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace ccx {

struct PairList {
  std::vector<int32_t> p, q;  // 0-based orbitals
  int32_t size() const { return (int32_t)p.size(); }
  void push(int32_t a, int32_t b) { p.push_back(a); q.push_back(b); }
};

// A family of two-body channels keyed by (tz, N) in reference enumeration order.
struct ChannelFamily {
  std::vector<std::array<int32_t, 4>> qn;  // tz, Nx, Ny, Nz
  std::vector<PairList> side1, side2;
  int32_t count() const { return (int32_t)qn.size(); }
};

// Dense (tz, N) -> 1-based channel id grid over a bounding box.
struct ChannelGrid {
  int32_t lo[3] = {0, 0, 0}, hi[3] = {-1, -1, -1}, ext[3] = {0, 0, 0};
  std::vector<int32_t> id;  // 3 tz values x box
  void init(const int32_t *l, const int32_t *h) {
    for (int d = 0; d < 3; d++) { lo[d] = l[d]; hi[d] = h[d]; ext[d] = h[d] - l[d] + 1; }
    id.assign((size_t)3 * ext[0] * ext[1] * ext[2], 0);
  }
  bool inside(int32_t tz, int32_t x, int32_t y, int32_t z) const {
    return tz >= -1 && tz <= 1 && x >= lo[0] && x <= hi[0] && y >= lo[1] && y <= hi[1] && z >= lo[2] &&
           z <= hi[2];
  }
  size_t index(int32_t tz, int32_t x, int32_t y, int32_t z) const {
    return (((size_t)(tz + 1) * ext[0] + (x - lo[0])) * ext[1] + (y - lo[1])) * ext[2] + (z - lo[2]);
  }
  int32_t get(int32_t tz, int32_t x, int32_t y, int32_t z) const {
    return inside(tz, x, y, z) ? id[index(tz, x, y, z)] : 0;
  }
};

struct Basis {
  int32_t ns = 0, A = 0;
  int32_t tzmin = 1, tzmax = 1;
  std::vector<int32_t> nx, ny, nz, sz, tz;
  std::vector<double> kx, ky, kz, e;
  double L = 0.0;
  int32_t nkmax[3] = {0, 0, 0};
  std::vector<int32_t> orbit_of;  // (nx, ny, nz, spin, isospin) -> orbital, -1 if absent

  int32_t orbitof(int32_t x, int32_t y, int32_t z, int32_t s, int32_t t) const;
};

// Packed representation of one hhpp channel: pairs with a<b and i<j.
struct PackedChannel {
  int32_t n_hh = 0, n_pp = 0;      // ordered (reference) sizes
  int32_t H = 0, P = 0;            // packed sizes
  std::vector<int32_t> hh_of_packed;  // packed -> ordered row index
  std::vector<int32_t> pp_of_packed;
  std::vector<int32_t> hh_packed;  // ordered -> signed packed index+1 (0: i==j)
  std::vector<int32_t> pp_packed;
  int64_t t_off = 0;               // offset of the packed T block (P x H)
  int64_t amp_off = 0;             // offset of the ordered block (n_pp x n_hh)
  int32_t hhhh = -1;               // matching hhhh channel
};

struct Layout {
  Basis b;
  ChannelGrid grid[7];             // pair-sum kinds 1..6
  ChannelFamily fam[7];            // 1 hhhh, 2 hhhp, 3 hhpp, 4 hphp, 5 hppp, 6 pppp
  ChannelGrid phgrid[4];           // difference kinds 1 phhp, 2 hphp, 3 hpph
  ChannelFamily ph[4];
  // ordered pair -> position+1 in its channel list (reference hh_hhpp%ival etc.)
  std::vector<int32_t> hh_hhpp, pp_hhpp, hh_hhhh, hp_hphp, hh_hhhp, hp_hhhp, hp_hppp, pp_hppp;
  std::vector<int32_t> ph_ph_phhp, hp_ph_phhp;
  // packed engine tables
  std::vector<PackedChannel> pk;
  int64_t n_amps = 0;              // ordered T2 elements
  int64_t n_tpacked = 0;           // packed T2 elements

  int32_t chan3_of_pair(int32_t p, int32_t q) const;  // hhpp channel (0-based) or -1
  int32_t pair_index(const std::vector<int32_t> &m, int32_t p, int32_t q) const {
    return m[(size_t)p * b.ns + q];
  }
  uint64_t hash() const;
};

Basis build_basis(int32_t nmax, int32_t A, bool snm, double density, const double theta[3]);
void build_layout(Layout &L);  // from L.b
std::string describe(const Layout &L);

}  // namespace ccx
