// Device-side descriptors of a gate program and of one run over a batch.
// Shared by the CUDA kernels and the host runtime.
#pragma once

#include <stdint.h>

namespace rrtl {

// Warps of the fused gate kernel's CTA; a staged piece carries one run range
// per warp. One CTA of 16 warps per SM: measured on the 50k-gate netlist
// (65,536 lanes x 1,000 cycles) 3% faster than 32 warps (fewer per-piece
// dispatches and barrier arrivals for the same cell work) and 30% faster
// than 8 (too few warps to cover shared-memory latency).
#ifndef RRTL_FUSED_WARPS
#define RRTL_FUSED_WARPS 16
#endif
constexpr uint32_t kGateFusedWarps = RRTL_FUSED_WARPS;
// 32-lane words one thread of the fused kernel owns for a tile of W words
// (one 32/64/128-bit shared access moves them); a warp step covers V groups.
#ifndef RRTL_FUSED_V
#define RRTL_FUSED_V 4
#endif
#if defined(__CUDACC__)
__host__ __device__
#endif
constexpr uint32_t gate_fused_vec(uint32_t W) {
  return (uint32_t)RRTL_FUSED_V <= W ? (uint32_t)RRTL_FUSED_V : (W >= 2 ? 2u : 1u);
}
// CTAs of the fused kernels meant to share an SM (each then gets that share
// of its shared memory); one, since a tile's nets fill most of it.
#ifndef RRTL_FUSED_CTAS_PER_SM
#define RRTL_FUSED_CTAS_PER_SM 1
#endif
constexpr uint32_t kGateFusedCtasPerSm = RRTL_FUSED_CTAS_PER_SM;

struct GateStimDev {
  uint32_t slot;  // on-chip slot (fused path)
  uint32_t net;   // global net row (plain path)
  uint32_t kind;  // RRTL_STIM_*
  uint32_t pad;
  uint64_t param;
};

struct GateRecDev {
  uint32_t slot;
  uint32_t net;
};

// One stuck-at force on one 32-lane word: v = (v & ~mask) | (val & mask).
struct GateForceDev {
  uint32_t slot;
  uint32_t net;
  uint32_t word;  // word inside the tile (fused tiles are W words, plain tiles 8)
  uint32_t mask;
  uint32_t val;
  uint32_t pad;
};

// Register commit entry. flags: 1 has reset, 2 active-low reset, 4 reset value 1.
struct GateRegDev {
  uint32_t q, d, rst, flags;
};

// One staged piece (see PieceBlob): where it lies in the blob, its size and
// the size of its run header.
struct GatePieceDev {
  uint32_t group_begin, n_groups, level, last_of_level;
  uint32_t off_words, bytes, pad0, pad1;
};

struct GateProgDev {
  // fused path (slots in shared memory)
  const uint32_t* blob;        // staged pieces: run headers and packed slot records (PieceBlob)
  const GatePieceDev* pieces;
  uint32_t n_pieces, n_slots, n_levels, piece_groups;
  uint32_t ring_bytes;         // bytes of one ring buffer (largest piece)
  uint32_t hdr_bytes;          // run header of every staged piece
  const uint32_t* src_net;     // sources loaded per tile and written back
  const uint32_t* src_slot;
  uint32_t n_src;
  const GateRegDev* sregs;     // slot-based commit list
  const uint32_t* wb_net;      // [groups*group] global net of each cell's signal output, or ~0
  // plain path (nets in HBM)
  const uint4* grecs;          // [groups*group] {a, b, c, out | lut << 24}
  const uint32_t* level_group_begin;  // [n_levels+1]
  const GateRegDev* gregs;     // net-based commit list
  uint32_t n_regs;
  uint32_t const0_slot, const1_slot;
  uint32_t group;              // cells per group G = 32 / W, W = words per fused tile
};

struct GateRunDev {
  unsigned long long cycles, seed;
  uint32_t n_stim;
  const GateStimDev* stim;
  uint32_t n_rec;
  const GateRecDev* rec;
  uint32_t mode;
  uint32_t n_trace_cols;
  const uint32_t* in_trace;   // [cycle][col][words]
  uint32_t* out_trace;        // [cycle][rec][words]
  unsigned long long* out_hash;
  uint32_t* detect;           // [lanes]
  uint32_t lanes, words, words_pad, n_tiles;
  const uint32_t* force_off;  // [n_tiles*(n_levels+2)]: per tile, per stage (0 = after commit, L+1 = after level L)
  const GateForceDev* forces;
  uint32_t has_forces;
  uint32_t final_settle;
  uint32_t* nets;             // [rows][words_pad]
  uint32_t* err;              // device status word
  unsigned long long cycle_base;  // absolute cycle of the launch's first cycle (stimulus, records)
  unsigned long long word_base;   // global 32-lane word of the batch's word 0 (RANDOM stimulus, hash terms)
  // trace checks (RRTL_REC_CHECK): per cycle and recorded net, the check index
  // (~0: none) and the expected words; mismatches go to an atomic log
  const uint32_t* chk_idx;    // [cycle][rec]
  const uint32_t* chk_exp;    // [cycle][rec][words]
  uint32_t* chk_log;          // [1 + 6*cap]: count, then (step, check, lane, limb, expected, actual)
  uint32_t chk_cap;
};

// One job of the device-side queue: a run over one batch with its program.
struct GateJobDev {
  GateProgDev P;
  GateRunDev R;
};

// One queue item: cycles [c0, c0 + ncyc) of one tile of one job; flags bit 0:
// the job's closing settle follows.
struct GateItemDev {
  uint32_t job, tile;
  unsigned long long c0;
  uint32_t ncyc, flags;
};

struct GateQueueDev {
  const GateJobDev* jobs;
  const GateItemDev* items;
  uint32_t n_items;
  uint32_t* next;  // [0] atomic item counter, [1] launch status (both zeroed before the launch): a CTA
                   // that could not drain its copies at exit fails every job of the launch
};

}  // namespace rrtl
