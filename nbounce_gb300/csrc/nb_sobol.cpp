// Sobol-Burley sample table: the data behind `sobol_burley` binding 2 of the reference pass
// (src/pathtracing/pathtracer.rs:56-71, read by pathtracing.wgsl:151-159).
//
// The reference fills it with sobol_burley 0.5.0's sample_4d(i, d, 0), a crate outside the
// reference tree.  This is Burley's published method ("Practical Hash-based Owen
// Scrambling", JCGT 9(4), 2020): 4D Sobol points (Joe-Kuo direction numbers) whose index is
// shuffled and whose coordinates are Owen-scrambled, both by nested uniform scrambling =
// bit reversal + Laine-Karras permutation + bit reversal.  Seeds are derived per dimension
// set (index shuffle) and per dimension (scramble) with the "lowbias32" integer hash.
// Output floats are the top 24 bits of the scrambled 32-bit coordinate times 2^-24.

#include <cstdint>

#include "nb_internal.h"
#include "sobol_directions.inc"

namespace nb {
namespace {

inline uint32_t bit_reverse(uint32_t x) {
  x = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
  x = ((x >> 2) & 0x33333333u) | ((x & 0x33333333u) << 2);
  x = ((x >> 4) & 0x0F0F0F0Fu) | ((x & 0x0F0F0F0Fu) << 4);
  x = ((x >> 8) & 0x00FF00FFu) | ((x & 0x00FF00FFu) << 8);
  return (x >> 16) | (x << 16);
}

// Laine-Karras permutation, multipliers from Burley 2020 (listing 2)
inline uint32_t laine_karras(uint32_t x, uint32_t seed) {
  x += seed;
  x ^= x * 0x6c50b47cu;
  x ^= x * 0xb82f1e52u;
  x ^= x * 0xc7afe638u;
  x ^= x * 0x8d22f6e6u;
  return x;
}

inline uint32_t owen_scramble(uint32_t x, uint32_t seed) { return bit_reverse(laine_karras(bit_reverse(x), seed)); }

inline uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

inline uint32_t sobol_coordinate(uint32_t index, uint32_t dim) {
  uint32_t x = 0;
  const unsigned int* v = kSobolDirections[dim];
  for (int k = 0; index; ++k, index >>= 1)
    if (index & 1u) x ^= v[k];
  return x;
}

}  // namespace

void sobol_burley_table(uint32_t n_samples, uint32_t n_dimsets, uint32_t seed, float* out) {
  const uint32_t seed_hash = lowbias32(seed);
  const uint32_t dim_seed = lowbias32(seed ^ 0x85ebca6bu);
  for (uint32_t d = 0; d < n_dimsets; ++d) {
    const uint32_t shuffle_seed = lowbias32(d ^ seed_hash);
    uint32_t scramble_seed[4];
    for (uint32_t k = 0; k < 4; ++k) scramble_seed[k] = lowbias32((4u * d + k) ^ 0x9e3779b9u ^ dim_seed);
    for (uint32_t i = 0; i < n_samples; ++i) {
      const uint32_t shuffled = owen_scramble(i, shuffle_seed);
      float* o = out + 4 * ((size_t)i * n_dimsets + d);
      for (uint32_t k = 0; k < 4; ++k) {
        uint32_t x = owen_scramble(sobol_coordinate(shuffled, 4u * d + k), scramble_seed[k]);
        o[k] = (float)(x >> 8) * (1.0f / 16777216.0f);
      }
    }
  }
}

}  // namespace nb
