// Device image of the layout: plain structs of device pointers passed to kernels.
#pragma once

#include <cstdint>
#include <vector_types.h>

namespace ccx {

// Packed (a<b, i<j) hhpp channel tables and the particle-hole ring tables.
struct DevLayout {
  int ns, A, NP;  // states, holes, particles
  int nch;        // hhpp channels
  const int *P, *H;             // packed sizes per channel
  const int64_t *t_off;         // T/R block offsets (P*H, column-major, pp fastest)
  const int64_t *vpp_off;       // V_pppp' offsets (P*P, row ab' major: [ab'*P + cd'])
  const int64_t *hh2_off;       // X / I9 / V_hhhh' offsets (H*H column-major)
  const int *pp_off, *hh_off;   // offsets into the packed pair arrays
  const int2 *pp_orb, *hh_orb;  // packed pair orbitals
  const int *pp_row, *hh_row;   // packed pair -> ordered row of the reference block
  const int2 *pp_slot;          // [(a-A)*NP + (b-A)] -> (channel, signed packed index)
  const int2 *hh_slot;          // [i*A + j]          -> (channel, signed packed index)
  const int *partner;           // [ns] other-spin orbital with the same n and tz, or -1
  // ring (phhp) channels
  int nph;
  const int *n_ph, *n_hp;
  const int64_t *tph_off;       // T_ph / R_ph offsets (n_ph*n_hp column-major)
  const int64_t *i4_off;        // I4 / W offsets (n_hp*n_hp)
  const int64_t *vph_off;       // V_ph offsets (n_hp*n_ph)
  const int *ph_off, *hp_off;
  const int2 *ph_orb;           // (a particle, i hole) rows
  const int2 *hp_orb;           // (j hole, b particle) columns
  const int2 *ph_slot;          // [(a-A)*A + i] -> (channel, row)
  const int2 *hp_slot;          // [j*NP + (b-A)] -> (channel, column)
  // element tiles: {channel, start}
  const int2 *ttile;
  int nttile;
  const int2 *phtile;
  int nphtile;
  const int2 *vtile;            // tiles over V_pppp' elements
  int nvtile;
};

constexpr int kTileElems = 1024;

// Orbital data used by the device potentials.
struct DevOrbits {
  int ns;
  const int *nx, *ny, *nz, *sz, *tz;
  const double *kx, *ky, *kz, *e;
  double volume;
};

}  // namespace ccx
