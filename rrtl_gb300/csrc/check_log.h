// Device-side mismatch log of trace replay (the reference's replay result
// buffer, crates/rrtl-gpu-sim/src/lib.rs:1022-1024: a count word followed by
// six-word records (step, check index, lane, limb, expected, actual)).
#pragma once

#include <stdint.h>

namespace rrtl {

#if defined(__CUDACC__)
__device__ __forceinline__ void log_mismatch(uint32_t* log, uint32_t cap, uint64_t step, uint32_t check, uint32_t lane,
                                             uint32_t limb, uint32_t expected, uint32_t actual) {
  const uint32_t i = atomicAdd(log, 1u);
  if (i < cap) {
    uint32_t* e = log + 1 + (size_t)i * 6;
    e[0] = (uint32_t)step;
    e[1] = check;
    e[2] = lane;
    e[3] = limb;
    e[4] = expected;
    e[5] = actual;
  }
}
#endif

}  // namespace rrtl
