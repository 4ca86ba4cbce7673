// T2 checkpoint files (host only): amplitudes of one lattice behind a header carrying
// the lattice's layout hash and the hash of its momenta (the twist).
#pragma once

#include <cstdint>
#include <string>

#include "layout.hpp"

namespace ccx {

// FNV-1a over the box length and the orbital momenta kx, ky, kz
uint64_t geometry_hash(const Layout &L);
// t2: 2 * L.n_amps doubles (ccx_get_t2_all order); errors throw EngineError(1, ...)
void write_t2_checkpoint(const Layout &L, const std::string &path, const double *t2);
// any_twist: accept a checkpoint of the same channel structure at another twist or box
void read_t2_checkpoint(const Layout &L, const std::string &path, bool any_twist, double *t2);

}  // namespace ccx
