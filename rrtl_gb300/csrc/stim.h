// Counter-based stimulus and output hashing shared by every engine.
//
// Stimulus bits are a pure function of (seed, stream, cycle, index), so a
// kernel can generate a lane's inputs for any cycle without reading HBM and
// a CPU checker regenerates the same bits. The mixer is the SplitMix64
// finaliser (Steele, Lea, Flood: "Fast splittable pseudorandom number
// generators", OOPSLA 2014).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define RRTL_HD __host__ __device__ __forceinline__
#else
#define RRTL_HD inline
#endif

namespace rrtl {

RRTL_HD uint64_t smix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// 32 stimulus bits for (seed, stream, cycle, idx).
RRTL_HD uint32_t stim_word(uint64_t seed, uint64_t stream, uint64_t cycle, uint64_t idx) {
  uint64_t k = smix64(seed ^ (stream * 0xD6E8FEB86659FD93ull));
  return (uint32_t)smix64(k ^ (cycle * 0xA0761D6478BD642Full) ^ (idx * 0xE7037ED1A0B428DBull));
}

// Value of limb `limb` of a RANDOM input of `width` bits on global lane
// `lane`: 1-bit inputs take bit (lane % 32) of the word for lane/32, so a
// bit-sliced engine draws one word per 32 lanes; wider inputs draw one word
// per limb. RANDOM_UNIFORM gives every lane the value of global lane 0.
RRTL_HD uint32_t stim_lane_limb(uint64_t seed, uint64_t stream, uint64_t cycle, uint64_t lane, uint32_t width,
                                uint32_t limb) {
  if (width == 1) return (stim_word(seed, stream, cycle, lane >> 5) >> (uint32_t)(lane & 31u)) & 1u;
  uint32_t v = stim_word(seed, stream ^ ((uint64_t)limb << 40), cycle, lane);
  uint32_t nl = (width + 31) / 32;
  if (limb + 1 == nl && (width & 31)) v &= (1u << (width & 31)) - 1u;
  return v;
}

// The 32-lane word of a 1-bit RANDOM_UNIFORM input: every lane takes the bit
// global lane 0 would take under RANDOM.
RRTL_HD uint32_t stim_uniform_word(uint64_t seed, uint64_t stream, uint64_t cycle) {
  return (stim_word(seed, stream, cycle, 0) & 1u) ? 0xFFFFFFFFu : 0u;
}

// One term of the per-cycle output hash. `idx` is the 32-lane word index for
// 1-bit recorded signals (value = the packed word, lanes past the batch end
// cleared) and lane*limbs+limb for wider ones; the per-cycle hash is the
// wrapping sum of all terms, so any evaluation order and either engine agree.
RRTL_HD uint64_t hash_salt(uint64_t cycle, uint32_t rec) {
  return smix64((cycle << 20) ^ (uint64_t)rec ^ 0x5851F42D4C957F2Dull);
}
RRTL_HD uint64_t hash_term_salted(uint64_t salt, uint64_t idx, uint32_t value) {
  return smix64((uint64_t)value ^ (idx << 32) ^ salt);
}
RRTL_HD uint64_t hash_term(uint64_t cycle, uint32_t rec, uint64_t idx, uint32_t value) {
  return hash_term_salted(hash_salt(cycle, rec), idx, value);
}

}  // namespace rrtl
