// T2 checkpoint files: the amplitudes of one lattice (all channels concatenated in the
// reference's t2_ccm order, complex interleaved, as ccx_get_t2_all returns them) behind
// a header that names the lattice they belong to.
//
// The reference keeps no checkpoint (every run starts from MP2); this is the export /
// import that harvests converged amplitudes (for resuming a solve, or as training data
// and starting points of the learned warm start) and refuses them on another lattice.
//
// Layout (little-endian, 96-byte header, then the data):
//   char     magic[8]      "CCXT2CK" + NUL
//   uint32   version       1
//   uint32   byte_order    0x01020304 as written
//   uint64   layout_hash   Layout::hash(): states, spins, isospins, channel tables
//   uint64   geometry_hash FNV-1a over the box length and the orbital momenta (twist)
//   int64    n_amps        complex amplitudes that follow
//   int32    n_states, n_holes
//   double   box_length
//   uint64   data_hash     FNV-1a over the data bytes
//   uint8    reserved[32]  zero
//   double   data[2 * n_amps]
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "checkpoint.hpp"
#include "engine.hpp"

namespace ccx {

namespace {

constexpr char kMagic[8] = {'C', 'C', 'X', 'T', '2', 'C', 'K', '\0'};
constexpr uint32_t kVersion = 1;
constexpr uint32_t kByteOrder = 0x01020304u;

struct Header {
  char magic[8];
  uint32_t version, byte_order;
  uint64_t layout_hash, geometry_hash;
  int64_t n_amps;
  int32_t n_states, n_holes;
  double box_length;
  uint64_t data_hash;
  uint8_t reserved[32];
};
static_assert(sizeof(Header) == 96, "checkpoint header is 96 bytes");

struct Fnv {
  uint64_t h = 1469598103934665603ULL;
  void mix(const void *p, size_t n) {
    const unsigned char *c = (const unsigned char *)p;
    for (size_t i = 0; i < n; ++i) {
      h ^= c[i];
      h *= 1099511628211ULL;
    }
  }
};

struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

[[noreturn]] void io_error(const std::string &what, const std::string &path) {
  throw EngineError(1, what + " '" + path + "': " + std::strerror(errno));
}

}  // namespace

uint64_t geometry_hash(const Layout &L) {
  Fnv h;
  h.mix(&L.b.L, sizeof L.b.L);
  for (const std::vector<double> *k : {&L.b.kx, &L.b.ky, &L.b.kz}) h.mix(k->data(), k->size() * sizeof(double));
  return h.h;
}

void write_t2_checkpoint(const Layout &L, const std::string &path, const double *t2) {
  if (!t2) throw EngineError(1, "null amplitude buffer");
  Header hd{};
  std::memcpy(hd.magic, kMagic, sizeof kMagic);
  hd.version = kVersion;
  hd.byte_order = kByteOrder;
  hd.layout_hash = L.hash();
  hd.geometry_hash = geometry_hash(L);
  hd.n_amps = L.n_amps;
  hd.n_states = L.b.ns;
  hd.n_holes = L.b.A;
  hd.box_length = L.b.L;
  const size_t bytes = (size_t)2 * (size_t)L.n_amps * sizeof(double);
  Fnv d;
  d.mix(t2, bytes);
  hd.data_hash = d.h;
  // written to a temporary name and renamed, so that a reader never sees half a file
  const std::string tmp = path + ".part";
  {
    File out;
    out.f = std::fopen(tmp.c_str(), "wb");
    if (!out.f) io_error("cannot create checkpoint", tmp);
    if (std::fwrite(&hd, sizeof hd, 1, out.f) != 1 || (bytes && std::fwrite(t2, bytes, 1, out.f) != 1))
      io_error("cannot write checkpoint", tmp);
    if (std::fflush(out.f) != 0) io_error("cannot write checkpoint", tmp);
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) io_error("cannot rename checkpoint to", path);
}

void read_t2_checkpoint(const Layout &L, const std::string &path, bool any_twist, double *t2) {
  if (!t2) throw EngineError(1, "null amplitude buffer");
  File in;
  in.f = std::fopen(path.c_str(), "rb");
  if (!in.f) io_error("cannot open checkpoint", path);
  Header hd{};
  if (std::fread(&hd, sizeof hd, 1, in.f) != 1) throw EngineError(1, "checkpoint '" + path + "' is truncated (header)");
  if (std::memcmp(hd.magic, kMagic, sizeof kMagic) != 0) throw EngineError(1, "'" + path + "' is not a T2 checkpoint");
  if (hd.byte_order != kByteOrder) throw EngineError(1, "checkpoint '" + path + "' was written with another byte order");
  if (hd.version != kVersion)
    throw EngineError(1, "checkpoint '" + path + "' has version " + std::to_string(hd.version) + ", expected " +
                             std::to_string(kVersion));
  if (hd.layout_hash != L.hash() || hd.n_amps != L.n_amps || hd.n_states != L.b.ns || hd.n_holes != L.b.A)
    throw EngineError(1, "checkpoint '" + path + "' belongs to another lattice (states, holes or channel tables differ)");
  if (!any_twist && hd.geometry_hash != geometry_hash(L))
    throw EngineError(1, "checkpoint '" + path + "' was written at another twist or box length");
  const size_t bytes = (size_t)2 * (size_t)L.n_amps * sizeof(double);
  // read into a scratch buffer: the caller's buffer is left untouched on any error
  std::unique_ptr<double[]> buf(new double[2 * (size_t)L.n_amps + 1]);
  if (bytes && std::fread(buf.get(), bytes, 1, in.f) != 1)
    throw EngineError(1, "checkpoint '" + path + "' is truncated (amplitudes)");
  char extra;
  if (std::fread(&extra, 1, 1, in.f) != 0) throw EngineError(1, "checkpoint '" + path + "' has trailing bytes");
  Fnv d;
  d.mix(buf.get(), bytes);
  if (d.h != hd.data_hash) throw EngineError(1, "checkpoint '" + path + "' is corrupt (data checksum)");
  std::memcpy(t2, buf.get(), bytes);
}

}  // namespace ccx
