// pp_shuffle.cpp -- deterministic label shuffle for the label-randomisation
// null model (the reference shuffles with std::shuffle over a seeded mt19937,
// src/PARAPROBE_SolverHdl.cpp:2882-2894, whose output is implementation
// defined).  This is a plain Fisher-Yates pass; random draws come from
// splitmix64 (Steele, Lea and Flood 2014) and are reduced to [0, i] with
// Lemire's multiply-and-reject method, so the permutation is the same on every
// platform for a given seed.
#include <cstdint>
#include <cstring>

#include "pp_host.h"

namespace pp_host {

namespace {
struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  // uniform in [0, bound)
  uint64_t below(uint64_t bound) {
    for (;;) {
      const uint64_t x = next();
      const unsigned __int128 m = (unsigned __int128)x * bound;
      const uint64_t lo = (uint64_t)m;
      if (lo >= bound || lo >= (0 - bound) % bound) return (uint64_t)(m >> 64);
    }
  }
};
}  // namespace

void shuffle_labels(const uint8_t* label, uint64_t n, uint64_t seed, uint8_t* out) {
  if (n == 0) return;
  std::memmove(out, label, n);
  SplitMix64 g{seed};
  for (uint64_t i = n - 1; i > 0; --i) {
    const uint64_t j = g.below(i + 1);
    const uint8_t t = out[i];
    out[i] = out[j];
    out[j] = t;
  }
}

}  // namespace pp_host
