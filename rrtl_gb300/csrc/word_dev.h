// Device-side descriptors of a word program (lane-per-thread engine).
#pragma once

#include <stdint.h>

namespace rrtl {

enum WOp : uint8_t {
  W_LIT = 0,   // dst = lits[aux]
  W_SIG,       // dst = signal at word offset aux (limbs from flags bit0: 2 limbs)
  W_NOT, W_AND, W_OR, W_XOR, W_ADD, W_SUB, W_MUL,
  W_EQ, W_NE,  // dst = a == b (values already fit their widths)
  W_LT,        // unsigned a < b at operand width aux
  W_LTS,       // signed a < b at operand width aux
  W_MUX,       // dst = (a & 1) ? b : c
  W_SLICE,     // dst = a >> aux
  W_MASK,      // zext / trunc / cast / move
  W_SEXT,      // sign-extend from width aux
  W_CAT,       // dst = (a << aux) | b
  W_MEMRD,     // dst = mem[aux][a] (0 when a >= depth)
  W_STORE,     // signal[aux] = a
  W_ASTORE,    // if reset(aux2) asserted: signal[aux] = a
  W_CAPTURE,   // cap[aux] = reset(aux2) asserted ? lits[aux3] : a
  W_MEMWR,     // if (a & 1) and b < depth: mem[aux][b] = c
};

// flags: bit0 two limbs (signal/memory access), bit1 has reset, bit2 active-low reset.
// Values of 65 to 128 bits take a pair of value slots (s: bits 0-63, s+1: bits
// 64-127). An instruction with kWWide set computes on 128 bits: kWPairD says
// its result is a pair, kWPairA/B/C which operands are pairs (a single slot
// reads as a value below 2^64). Wide signal accesses
// (W_SIG, W_STORE, W_ASTORE, W_CAPTURE) carry their limb count in `c`; wide
// literals and capture reset values are two consecutive `lits` entries.
enum : uint8_t { kWWide = 8, kWPairA = 16, kWPairB = 32, kWPairC = 64, kWPairD = 128 };
struct WInstr {
  uint8_t op;
  uint8_t flags;
  uint16_t width;  // result width (stores: destination width)
  uint16_t dst, a, b, c;  // value slots
  uint32_t aux, aux2, aux3;
};

struct WMemDev {
  uint32_t offset;  // first memory word of this memory inside one lane's block
  uint32_t depth;
  uint32_t limbs;
  uint32_t width;
};

struct WCommitDev {
  uint32_t cap_off, sig_off, limbs, pad;
};

struct WordProgDev {
  const WInstr* code;
  uint32_t comb_b, comb_e, async_b, async_e, next_b, next_e, commit_b, commit_e;
  const unsigned long long* lits;
  const WMemDev* mems;
  const WCommitDev* commits;
  uint32_t n_commits;
  uint32_t n_vslots;
  uint32_t n_sig_words;  // signal value words per lane
  uint32_t sig_smem;     // 1: a block keeps its lanes' signal values in shared memory for the launch
};

struct WordStimDev {
  uint32_t sig_off, limbs, width, kind;
  uint64_t param;
};

struct WordRecDev {
  uint32_t sig_off, limbs, width, base;  // base: first limb row of this record in a cycle's trace rows
};

struct WordRunDev {
  unsigned long long cycles, seed;
  uint32_t n_stim;
  const WordStimDev* stim;
  uint32_t n_rec;
  const WordRecDev* rec;
  uint32_t rec_limbs;
  uint32_t mode;
  uint32_t n_trace_cols;
  const uint32_t* in_trace;   // [cycle][col][lanes]
  uint32_t* out_trace;        // [cycle][rec limb rows][lanes]
  unsigned long long* out_hash;
  uint32_t* detect;
  uint32_t lanes, lanes_pad;
  uint32_t* values;           // [signal word][lanes_pad]
  uint32_t* mems;             // [memory word][lanes_pad]
  uint32_t* caps;             // [capture word][lanes_pad]
  unsigned long long* vspill; // [slot][lanes_pad] value slots when they do not fit shared memory
  uint32_t final_settle;
  uint32_t start_settle;      // settle before the first cycle (eval)
  unsigned long long cycle_base;  // absolute index of this launch's first cycle (stimulus, hash, detect);
                                  // buffers are indexed from the launch's first cycle
  unsigned long long lane_base;   // global lane of the batch's lane 0 (RANDOM stimulus, hash terms)
  uint32_t* err;
  // trace checks (RRTL_REC_CHECK), per cycle and recorded limb row
  const uint32_t* chk_idx;    // [cycle][rec limb rows], ~0 = no check
  const uint32_t* chk_exp;    // [cycle][rec limb rows][lanes]
  uint32_t* chk_log;          // [1 + 6*cap]
  uint32_t chk_cap;
};

// Shared-memory placement of one launch of a compiled word kernel. Rows are
// [row][thread] u32 words: the signal words first (when staged), then each
// staged memory. Memories past kJitPlacedMems always stay in HBM.
constexpr uint32_t kJitPlacedMems = 8;
struct WordJitPlace {
  uint32_t sig_smem;      // 1: signal words staged from row 0
  uint32_t n_sig_words;
  uint32_t n_mems;        // memories with an entry below (min(memories, kJitPlacedMems))
  uint32_t x_row;         // split kernels: first row of the register exchange area
  uint32_t mem_off[kJitPlacedMems];    // first word of memory k in a lane's memory block
  uint32_t mem_words[kJitPlacedMems];  // depth x limbs
  uint32_t smem_row[kJitPlacedMems];   // first shared-memory row, ~0 = stays in HBM
  uint32_t written[kJitPlacedMems];    // 1: the design writes memory k (copied back after the launch)
};

// One run of the multi-job word kernel: blocks [block_begin, next job's
// block_begin) simulate its lanes, 128 per block.
struct WordJobDev {
  WordProgDev P;
  WordRunDev R;
  uint32_t block_begin, pad;
};

}  // namespace rrtl
