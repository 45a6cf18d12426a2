// host_model.h — host-side unit cell / lattice spec shared by the builder.
#pragma once
#include <stdint.h>

#include <array>
#include <string>
#include <vector>

#include "tbk_internal.h"

#if defined(__CUDACC__)
#define TBK_HD __host__ __device__ __forceinline__
#else
#define TBK_HD inline
#endif

namespace tbk {

// Counter-based seeded uniforms (SplitMix64 finaliser, Steele/Lea/Flood 2014):
// u01(seed, stream, idx) in [0,1) with 53 random bits.  Integer-only, so host and
// device draw identical values.
TBK_HD uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
TBK_HD double u01(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t k = mix64(seed ^ mix64(stream + 0x632BE59BD9B4E019ull));
  uint64_t h = mix64(k + idx * 0xD1B54A32D192ED03ull);
  return (double)(h >> 11) * 0x1.0p-53;
}
constexpr uint64_t kDisorderStream = 0xD150D3Dull;
constexpr uint64_t kRemoveStream = 0x5ACA7C1Eull;   // remove_atoms_random draws

struct Hop {
  int32_t from, to;
  int32_t v[3];
  double tr, ti;
};

struct Cell {
  int dim = 0, n_atoms = 0;
  double bases[9];               // column c (lattice vector c) at bases[3c .. 3c+2]
  std::vector<std::string> names;
  std::vector<double> pos;       // n_atoms x 3
  std::vector<Hop> hops;         // canonical (from >= to), insertion order
  int warnings = 0;

  double hop_distance(int from, int to, const int32_t* v) const;
  int find_hop(int from, int to, const int32_t* v) const;
  bool hopping_exists(int from, int to, const int32_t* v) const;
  void add_direct(int from, int to, const int32_t* v, double tr, double ti);
  int nn_shell(int from, int nn, std::vector<std::array<int32_t, 4>>& out) const;
};

enum GaugeKind { GAUGE_NONE = 0, GAUGE_LINEAR = 1, GAUGE_SITES = 2 };
enum ScalarKind { SCALAR_NONE = 0, SCALAR_SITES = 1, SCALAR_DISORDER = 2 };

}  // namespace tbk

struct tbk_cell_s : public tbk::Cell {};

struct tbk_lattice_s {
  tbk::Cell cell;
  int32_t span[3];
  int64_t total = 0;
  int gauge_kind = tbk::GAUGE_NONE;
  double gauge_linear[12];            // G (row-major 3x3), then c
  std::vector<double> gauge_sites;    // total x 3
  int scalar_kind = tbk::SCALAR_NONE;
  std::vector<double> scalar_sites;   // total
  double disorder_W = 0.0;
  uint64_t disorder_seed = 0;
  std::vector<uint8_t> removed;       // total (empty = none)
};
