// Device helpers of the bit-sliced gate engine shared by the fused and plain
// kernels (gate_kernels.cu) and the per-design compiled gate kernels
// (gate_jit.cpp, compiled at run time by NVRTC, which is why this header
// includes only headers handed to NVRTC with it).
#pragma once

#include <stdint.h>

#include "../../include/rrtl_cuda.h"
#include "check_log.h"
#include "gate_dev.h"
#include "stim.h"

namespace rrtl {

// LOP3 with an immediate truth table: input a <-> 0xF0, b <-> 0xCC, c <-> 0xAA.
template <int L>
__device__ __forceinline__ uint32_t lop3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("lop3.b32 %0, %1, %2, %3, %4;" : "=r"(d) : "r"(a), "r"(b), "r"(c), "n"(L));
  return d;
}

// Lanes of 32-lane word gw that exist in a batch of `lanes` lanes.
__device__ __forceinline__ uint32_t valid_mask(uint32_t gw, uint32_t lanes) {
  uint32_t base = gw * 32u;
  if (base >= lanes) return 0u;
  uint32_t n = lanes - base;
  return n >= 32u ? 0xFFFFFFFFu : ((1u << n) - 1u);
}

__device__ __forceinline__ uint32_t stim_value(const GateStimDev& s, const GateRunDev& R, uint64_t c, uint32_t gw,
                                               uint32_t cur) {
  switch (s.kind) {
    case RRTL_STIM_RANDOM: return stim_word(R.seed, s.param, c, R.word_base + gw);
    case RRTL_STIM_RANDOM_UNIFORM: return stim_uniform_word(R.seed, s.param, c);
    case RRTL_STIM_PULSE: return c < s.param ? 0xFFFFFFFFu : 0u;
    case RRTL_STIM_CONST: return (s.param & 1u) ? 0xFFFFFFFFu : 0u;
    case RRTL_STIM_TRACE:
      return gw < R.words ? R.in_trace[((size_t)c * R.n_trace_cols + s.param) * R.words + gw] : 0u;
    default: return cur;
  }
}

// Trace check of recorded net k on 32-lane word gw at cycle c: every lane
// whose bit differs from the expected word is logged (limb 0).
__device__ __forceinline__ void check_word(const GateRunDev& R, uint64_t c, uint32_t k, uint32_t gw, uint32_t v) {
  const uint32_t idx = R.chk_idx[(size_t)c * R.n_rec + k];
  if (idx == 0xFFFFFFFFu) return;
  const uint32_t exp = R.chk_exp[((size_t)c * R.n_rec + k) * R.words + gw];
  uint32_t mm = (v ^ exp) & valid_mask(gw, R.lanes);
  while (mm) {
    const uint32_t b = __ffs(mm) - 1u;
    log_mismatch(R.chk_log, R.chk_cap, c, idx, gw * 32u + b, 0u, (exp >> b) & 1u, (v >> b) & 1u);
    mm &= mm - 1u;
  }
}

}  // namespace rrtl
