// Word program: lowering of a machine program for the lane-per-thread engine.
//
// Values of up to 64 bits live in 64-bit value slots, values of 65 to 128
// bits in slot pairs (see kWWide in word_dev.h); signals and memories
// stay in their packed u32-limb layout (crates/rrtl-sim-ir/src/lib.rs:12698-12722),
// stored word-major [word][lane] so a warp's accesses coalesce.
//
// Schedule: inside one comb level (the machine packets lowered from one
// packed packet, crates/rrtl-sim-ir/src/lib.rs:2997-3048) the reference
// evaluates every instruction, then applies every store. When no instruction
// of the level reads a signal the same level stores (true of any acyclic
// design, whose levels only read lower levels), storing right after each
// value is computed is equivalent, and a depth-first order per store keeps
// few values live. Levels that do read their own stores keep the reference
// order. Register captures go to a capture buffer; memory writes always run
// after every read of their block, as in the reference.
#pragma once

#include <cstdint>
#include <vector>

#include "lower.h"
#include "word_dev.h"

namespace rrtl {

struct WordProgram {
  std::vector<WInstr> code;
  uint32_t comb_b = 0, comb_e = 0, async_b = 0, async_e = 0, next_b = 0, next_e = 0, commit_b = 0, commit_e = 0;
  std::vector<unsigned long long> lits;
  std::vector<WMemDev> mems;
  std::vector<WCommitDev> commits;
  uint32_t n_vslots = 0;
  uint32_t total_capture_words = 0;
  uint32_t n_sig_words = 0;  // signal value words per lane
  uint64_t source_instrs = 0;
};

// Throws RrtlError("E_WORD_SCOPE", ...) for values wider than 128 bits.
WordProgram build_word_program(const MachineProgram& mp);

}  // namespace rrtl
