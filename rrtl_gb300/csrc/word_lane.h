// Run protocol of one word-engine lane, shared by the interpreted word kernel
// (word_kernels.cu) and the per-design compiled kernels (word_jit.cpp), so
// both engines step a lane through exactly the same sequence:
//
//   per cycle: stimulus -> settle -> record (trace, hash, detect, checks)
//              -> clock edge (register capture, memory writes, commit)
//
// with a settle before the first cycle when the run asks for one and a
// closing settle after the last. This is the reference's replay order
// (inputs, settle, check, tick: crates/rrtl-sim-ir/src/lib.rs:9540-9568).
//
// An engine type L provides
//   uint32_t get(uint32_t word), set(uint32_t word, uint32_t v)
//                                one signal word of the lane
//   void settle()                comb stream, then the async-reset stream
//   void edge()                  tick_next, tick_commit, register commit
// and the run's stimulus table, record table and record mode come in as a
// spec (WordRunSpec over R.stim and R.rec or copies of them in shared memory,
// or a generated type holding them as compile-time constants).
//
// The header is also compiled at run time by NVRTC, so it includes only
// headers that are handed to NVRTC with it.
#pragma once

#include <stdint.h>

#include "../../include/rrtl_cuda.h"
#include "check_log.h"
#include "stim.h"
#include "word_dev.h"

namespace rrtl {

// The run's stimulus table, record table and record mode as read at run
// time (a generated kernel may instead pass a type whose tables are
// compile-time constants, so the loops below unroll and fold away).
struct WordRunSpec {
  const WordStimDev* ST;
  const WordRecDev* RT;
  uint32_t ns, nr, md;
  __device__ __forceinline__ uint32_t n_stim() const { return ns; }
  __device__ __forceinline__ WordStimDev stim(uint32_t k) const { return ST[k]; }
  __device__ __forceinline__ uint32_t n_rec() const { return nr; }
  __device__ __forceinline__ WordRecDev rec(uint32_t k) const { return RT[k]; }
  __device__ __forceinline__ uint32_t mode() const { return md; }
};

// Stimulus of cycle c (absolute cycle ca) into the lane's input signals.
template <class L, class S>
__device__ __forceinline__ void word_stimulus(const WordRunDev& R, uint32_t lane, L& W, const S& spec,
                                              unsigned long long c, unsigned long long ca, bool live) {
#pragma unroll
  for (uint32_t k = 0; k < spec.n_stim(); ++k) {
    const WordStimDev s = spec.stim(k);
    if (s.kind == RRTL_STIM_HOLD) continue;
    for (uint32_t l = 0; l < s.limbs; ++l) {
      uint32_t v = 0;
      if (s.kind == RRTL_STIM_RANDOM) v = stim_lane_limb(R.seed, s.param, ca, R.lane_base + lane, s.width, l);
      else if (s.kind == RRTL_STIM_RANDOM_UNIFORM) v = stim_lane_limb(R.seed, s.param, ca, 0ull, s.width, l);
      else if (s.kind == RRTL_STIM_PULSE) v = (l == 0 && ca < s.param) ? 1u : 0u;
      else if (s.kind == RRTL_STIM_CONST) v = l < 2 ? (uint32_t)(s.param >> (32 * l)) : 0u;
      else if (s.kind == RRTL_STIM_TRACE)
        v = live ? R.in_trace[((size_t)c * R.n_trace_cols + s.param + l) * R.lanes + lane] : 0u;
      if (l + 1 == s.limbs && (s.width & 31u)) v &= (1u << (s.width & 31u)) - 1u;
      W.set(s.sig_off + l, v);
    }
  }
}

// Record stage of cycle c (trace, hash, detection, checks); the whole warp
// takes part (shuffles and ballots).
template <class L, class S>
__device__ __forceinline__ void word_record(const WordRunDev& R, uint32_t lane, L& W, const S& spec,
                                            unsigned long long c, unsigned long long ca, bool live, bool& detected) {
  if (!spec.n_rec()) return;
  const uint32_t mode = spec.mode();
  unsigned long long h = 0ull;
  bool diff = false;
  unsigned long long salts = 0ull;  // hash salt of record (k & ~31) + this lane's index in the warp
#pragma unroll
  for (uint32_t k = 0; k < spec.n_rec(); ++k) {
    const WordRecDev rc = spec.rec(k);
    if (mode & RRTL_REC_HASH) {
      // one salt per lane of the warp, shared by shuffles (the whole warp runs this loop)
      if ((k & 31u) == 0) salts = hash_salt(ca, k + (threadIdx.x & 31u));
    }
    const unsigned long long salt = (mode & RRTL_REC_HASH) ? __shfl_sync(0xFFFFFFFFu, salts, k & 31u) : 0ull;
    for (uint32_t l = 0; l < rc.limbs; ++l) {
      uint32_t v = W.get(rc.sig_off + l);
      if (l + 1 == rc.limbs && (rc.width & 31u)) v &= (1u << (rc.width & 31u)) - 1u;
      if (mode & RRTL_REC_DETECT) diff |= __shfl_sync(0xFFFFFFFFu, v, 0) != v;
      if ((mode & RRTL_REC_HASH) && rc.width == 1) {
        // 1-bit signals hash as 32-lane packed words, the gate engine's unit
        const uint32_t packed = __ballot_sync(0xFFFFFFFFu, live && (v & 1u));
        if ((threadIdx.x & 31u) == 0 && live) h += hash_term_salted(salt, (R.lane_base + lane) >> 5, packed);
      }
      if (!live) continue;
      if (mode & RRTL_REC_TRACE) R.out_trace[((size_t)c * R.rec_limbs + rc.base + l) * R.lanes + lane] = v;
      if (mode & RRTL_REC_CHECK) {
        const size_t row = (size_t)c * R.rec_limbs + rc.base + l;
        const uint32_t idx = R.chk_idx[row];
        if (idx != 0xFFFFFFFFu) {
          const uint32_t exp = R.chk_exp[row * R.lanes + lane];
          if (exp != v) log_mismatch(R.chk_log, R.chk_cap, ca, idx, lane, l, exp, v);
        }
      }
      if ((mode & RRTL_REC_HASH) && rc.width != 1)
        h += hash_term_salted(salt, (R.lane_base + lane) * rc.limbs + l, v);
    }
  }
  if (mode & RRTL_REC_HASH) {
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xFFFFFFFFu, h, o);
    if ((threadIdx.x & 31u) == 0 && h) atomicAdd(R.out_hash + c, h);
  }
  if ((mode & RRTL_REC_DETECT) && live && diff && !detected) {
    detected = true;
    R.detect[lane] = (uint32_t)ca;
  }
}

template <class L, class S>
__device__ __forceinline__ void word_lane_cycles(const WordRunDev& R, uint32_t lane, L& W, const S& spec) {
  const bool live = lane < R.lanes;
  // a lane detected by an earlier launch of the same run stays detected
  bool detected = (spec.mode() & RRTL_REC_DETECT) && live && R.detect[lane] != 0xFFFFFFFFu;
  if (R.start_settle) W.settle();
  for (unsigned long long c = 0; c < R.cycles; ++c) {
    const unsigned long long ca = R.cycle_base + c;
    word_stimulus(R, lane, W, spec, c, ca, live);
    W.settle();
    word_record(R, lane, W, spec, c, ca, live, detected);
    W.edge();
  }
  if (R.final_settle) W.settle();
}

// ---- per-design compiled kernels
//
// A compiled lane keeps its value slots in registers. Its signal words are
// registers too (kRegSignals: the generated lane type holds them as members
// and reaches them by a switch when the stimulus or record table names one
// at run time) or, for designs with many signal words, rows of shared memory
// or HBM through sv/svs. Memories listed in WordJitPlace are staged in shared
// memory for the launch ([word][thread], so any per-lane address is bank
// conflict free); the others stay word-major in HBM.
struct JitLaneBase {
  static constexpr bool kRegSignals = false;
  uint32_t* sv;                     // signal word 0 of this lane (kRegSignals false)
  size_t svs;                       // signal word stride
  uint32_t* mb[kJitPlacedMems];     // word 0 of memory k for this lane
  size_t ms[kJitPlacedMems];        // its word stride
  uint32_t* gm;                     // R.mems + lane (memories past kJitPlacedMems)
  size_t LP;                        // lanes_pad
  __device__ __forceinline__ uint32_t& SV(uint32_t off) const { return sv[(size_t)off * svs]; }
  __device__ __forceinline__ uint32_t get(uint32_t off) const { return SV(off); }
  __device__ __forceinline__ void set(uint32_t off, uint32_t v) const { SV(off) = v; }
  __device__ __forceinline__ uint32_t& MK(uint32_t k, size_t w) const { return mb[k][w * ms[k]]; }
  __device__ __forceinline__ uint32_t& MG(size_t w) const { return gm[w * LP]; }
};

// Stimulus and record tables of up to this many entries are copied to
// shared memory for the launch.
constexpr uint32_t kJitTableEntries = 64;

// The run tables of a kernel compiled for any run: copied to shared memory
// for the launch when they are short.
struct JitDynamicRun {
  WordStimDev st[kJitTableEntries];
  WordRecDev rt[kJitTableEntries];
  __device__ __forceinline__ WordRunSpec load(const WordRunDev& R) {
    const bool st_smem = R.n_stim <= kJitTableEntries, rt_smem = R.n_rec <= kJitTableEntries;
    if (st_smem)
      for (uint32_t i = threadIdx.x; i < R.n_stim; i += blockDim.x) st[i] = R.stim[i];
    if (rt_smem)
      for (uint32_t i = threadIdx.x; i < R.n_rec; i += blockDim.x) rt[i] = R.rec[i];
    return WordRunSpec{st_smem ? st : R.stim, rt_smem ? rt : R.rec, R.n_stim, R.n_rec, R.mode};
  }
};

// Kernel body of a compiled design: stage in, run the cycles, stage out.
// `spec` is a WordRunSpec over tables that `tables` filled, or a type whose
// tables are compile-time constants.
template <class L, class S>
__device__ __forceinline__ void word_jit_run(const WordRunDev& R, const WordJitPlace& Pl, uint32_t* jsm, const S& spec) {
  const uint32_t lane = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t T = blockDim.x;
  uint32_t* my = jsm + threadIdx.x;
  L W;
  W.LP = R.lanes_pad;
  W.gm = R.mems + lane;
  if constexpr (L::kRegSignals) {
    W.load(R.values + lane, R.lanes_pad);
  } else if (Pl.sig_smem) {
    W.sv = my;
    W.svs = T;
    for (uint32_t w = 0; w < Pl.n_sig_words; ++w) my[(size_t)w * T] = R.values[(size_t)w * R.lanes_pad + lane];
  } else {
    W.sv = R.values + lane;
    W.svs = R.lanes_pad;
  }
#pragma unroll
  for (uint32_t k = 0; k < kJitPlacedMems; ++k) {
    if (k >= Pl.n_mems) break;
    uint32_t* g = R.mems + (size_t)Pl.mem_off[k] * R.lanes_pad + lane;
    if (Pl.smem_row[k] != 0xFFFFFFFFu) {
      uint32_t* s = my + (size_t)Pl.smem_row[k] * T;
      for (uint32_t w = 0; w < Pl.mem_words[k]; ++w) s[(size_t)w * T] = g[(size_t)w * R.lanes_pad];
      W.mb[k] = s;
      W.ms[k] = T;
    } else {
      W.mb[k] = g;
      W.ms[k] = R.lanes_pad;
    }
  }
  __syncthreads();  // shared-memory run tables are in place
  word_lane_cycles(R, lane, W, spec);
  if constexpr (L::kRegSignals) {
    W.store(R.values + lane, R.lanes_pad);
  } else if (Pl.sig_smem) {
    for (uint32_t w = 0; w < Pl.n_sig_words; ++w) R.values[(size_t)w * R.lanes_pad + lane] = my[(size_t)w * T];
  }
#pragma unroll
  for (uint32_t k = 0; k < kJitPlacedMems; ++k) {
    if (k >= Pl.n_mems) break;
    if (Pl.smem_row[k] == 0xFFFFFFFFu || !Pl.written[k]) continue;
    uint32_t* g = R.mems + (size_t)Pl.mem_off[k] * R.lanes_pad + lane;
    const uint32_t* s = my + (size_t)Pl.smem_row[k] * T;
    for (uint32_t w = 0; w < Pl.mem_words[k]; ++w) g[(size_t)w * R.lanes_pad] = s[(size_t)w * T];
  }
}

// ---- two-warp split of a compiled kernel
//
// For lane counts that leave warp schedulers idle, a block runs 32 lanes on
// two warps: warp p evaluates the cones of its share of the register
// captures and memory writes (the lane type's settle_part / edge_part), each
// from its own copy of the lane's signals; warp 0 also computes everything the
// record stage reads and records. Per cycle: stimulus (both), settle_part,
// record (warp 0), barrier (every read of the cycle is done), edge_part
// (captures, memory writes, commits of owned registers), owned register words
// out to the exchange rows, barrier, the other warp's register words in. At
// the end warp 0 gathers every register, runs the closing settle over the
// whole design and writes the lane back.
__device__ __forceinline__ void jit_pair_barrier() { asm volatile("bar.sync 1, 64;" ::: "memory"); }

template <class L, class S>
__device__ __forceinline__ void word_jit_run_split(const WordRunDev& R, const WordJitPlace& Pl, uint32_t* jsm,
                                                   const S& spec) {
  const uint32_t part = threadIdx.x >> 5, lid = threadIdx.x & 31u;
  const uint32_t lane = blockIdx.x * 32u + lid;
  uint32_t* my = jsm + lid;  // shared-memory rows of 32 lanes
  uint32_t* X = jsm + (size_t)Pl.x_row * 32u;
  L W;
  W.LP = R.lanes_pad;
  W.gm = R.mems + lane;
  W.load(R.values + lane, R.lanes_pad);
#pragma unroll
  for (uint32_t k = 0; k < kJitPlacedMems; ++k) {
    if (k >= Pl.n_mems) break;
    uint32_t* g = R.mems + (size_t)Pl.mem_off[k] * R.lanes_pad + lane;
    if (Pl.smem_row[k] != 0xFFFFFFFFu) {
      uint32_t* sm = my + (size_t)Pl.smem_row[k] * 32u;
      if (part == 0)
        for (uint32_t w = 0; w < Pl.mem_words[k]; ++w) sm[(size_t)w * 32u] = g[(size_t)w * R.lanes_pad];
      W.mb[k] = sm;
      W.ms[k] = 32u;
    } else {
      W.mb[k] = g;
      W.ms[k] = R.lanes_pad;
    }
  }
  jit_pair_barrier();
  const bool live = lane < R.lanes;
  bool detected = (spec.mode() & RRTL_REC_DETECT) && live && part == 0 && R.detect[lane] != 0xFFFFFFFFu;
  if (R.start_settle && part == 0) W.settle();
  for (unsigned long long c = 0; c < R.cycles; ++c) {
    const unsigned long long ca = R.cycle_base + c;
    word_stimulus(R, lane, W, spec, c, ca, live);
    W.settle_part(part);
    if (part == 0) word_record(R, lane, W, spec, c, ca, live, detected);
    jit_pair_barrier();
    W.edge_part(part);
    W.xout(part, X, lid);
    jit_pair_barrier();
    W.xin(part, X, lid);
  }
  if (part != 0) return;
  if (R.cycles) W.xin_all(X, lid);
  if (R.final_settle) W.settle();
  W.store(R.values + lane, R.lanes_pad);
#pragma unroll
  for (uint32_t k = 0; k < kJitPlacedMems; ++k) {
    if (k >= Pl.n_mems) break;
    if (Pl.smem_row[k] == 0xFFFFFFFFu || !Pl.written[k]) continue;
    uint32_t* g = R.mems + (size_t)Pl.mem_off[k] * R.lanes_pad + lane;
    const uint32_t* sm = my + (size_t)Pl.smem_row[k] * 32u;
    for (uint32_t w = 0; w < Pl.mem_words[k]; ++w) g[(size_t)w * R.lanes_pad] = sm[(size_t)w * 32u];
  }
}

}  // namespace rrtl
