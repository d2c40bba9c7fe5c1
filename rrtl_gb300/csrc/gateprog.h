// Bit-sliced gate program: the GPU lowering of a gate-level machine program.
//
// Scope is the reference's bit-parallel engine (crates/rrtl-sim-ir/src/bitparallel.rs:1-17):
// every signal 1 bit, ops Signal/Lit/Not/And/Or/Xor/Mux, registers with
// optional synchronous reset, no memories. Each 32-lane word of a net is one
// u32 (bit k = lane 32*w + k).
//
// Lowering steps:
//  1. Every comb-assigned signal becomes a net produced by one LUT3 cell whose
//     truth table is the assignment's expression over at most three leaf nets
//     (other signals, internal nets, constants). Sub-expressions whose support
//     exceeds three leaves become internal nets. Cells never look through
//     another signal's net, so a stuck-at force on any signal net behaves as
//     in BitParallelSimulator::settle (bitparallel.rs:256-300).
//  2. Register next-state expressions (tick_next) become cells too; their
//     outputs are the D nets read by the commit.
//  3. Cells are levelized (level = 1 + deepest input producer) and, within a
//     level, sorted by truth table and padded to groups of G = 32/W cells that
//     share one table, W being the words per tile (8, 4, 2 or 1): a warp
//     evaluates one group, G cells x W words, with one truth table.
//  4. Nets get on-chip slots by liveness over the level order; sources
//     (inputs, constants) keep permanent slots, registers keep theirs except
//     between their last read and the commit.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "lower.h"

namespace rrtl {

constexpr uint32_t kPadWords = 8;     // net rows are padded to a multiple of 8 words (plain-kernel tile)
constexpr uint32_t kNetConst0 = 0;    // all-zero net
constexpr uint32_t kNetConst1 = 1;    // all-ones net
constexpr uint32_t kMaxSlots = 65535; // 16-bit slot fields in packed records

struct GateCell {
  uint8_t lut = 0;      // LOP3 table: input a <-> 0xF0, b <-> 0xCC, c <-> 0xAA
  uint32_t in[3] = {kNetConst0, kNetConst0, kNetConst0};
  uint32_t out = 0;     // net
  int32_t level = 0;
  bool pad = false;     // padding cell (writes the scratch slot)
};

struct GateReg {
  uint32_t signal;   // packed signal index
  uint32_t q_net;
  uint32_t d_net;
  uint32_t rst_net;  // kNetConst0 when no reset
  bool has_reset, active_low, reset_value;
};

// Bounded piece of one level's cells: the unit staged into shared memory.
struct GatePiece {
  uint32_t level;
  uint32_t group_begin;  // index of the first group in the level-ordered group array
  uint32_t n_groups;
  bool last_of_level;
  uint32_t seg_begin, seg_end;  // runs of one truth table inside the piece
};

// A run of groups inside a piece that share one truth table (group indices
// relative to the piece).
struct GateSegment {
  uint32_t lut, begin, end;
};

struct GateProgram {
  uint32_t tile_words = 8;              // W: 32-lane words per tile in the fused kernel
  uint32_t group = 4;                   // G = 32 / W cells per group
  uint32_t n_signals = 0;
  uint32_t n_nets = 0;                  // global net array rows
  std::vector<uint32_t> signal_net;     // packed signal -> net
  std::vector<int32_t> net_signal;      // net -> packed signal or -1
  std::vector<uint8_t> net_is_source;   // constants, inputs, registers, undriven signals
  std::vector<int32_t> net_level;       // producing cell level, -1 for sources
  std::vector<GateCell> cells;          // level-ordered, grouped, padded
  uint32_t n_real_cells = 0;
  uint32_t n_levels = 0;
  std::vector<uint32_t> level_group_begin;  // per level, first group; size n_levels+1
  std::vector<GateReg> regs;
  // on-chip slots
  std::vector<int32_t> net_slot;  // -1: not resident
  std::vector<uint8_t> net_end_live;  // holds its value in its slot when the cycle's settle ends
  uint32_t n_slots = 0;           // including the scratch slot (slot 0)
  std::vector<uint32_t> source_nets;  // nets loaded into slots at tile start (and written back)
  std::vector<GatePiece> pieces;
  std::vector<GateSegment> segments;
  uint32_t piece_groups = 0;      // max groups per piece
  uint64_t source_instrs = 0;
};

// Reorder a cell's inputs so its truth table is its permutation class's
// smallest; lut_is_canonical says whether a table is such a representative.
void canonicalize_inputs(GateCell& c);
bool lut_is_canonical(uint8_t lut);

// Throws RrtlError("E_GATE_SCOPE", ...) when the program is outside the gate engine's scope.
GateProgram build_gate_program(const MachineProgram& mp, uint32_t tile_words = 8);

// The registers in commit order: groups of G (one shared-memory wavefront of
// the fused kernel's vector commit) whose D rows, and whose Q rows, fall in
// distinct bank residues where the residues allow it.
std::vector<uint32_t> commit_order(const GateProgram& gp);

// Split every level into nearly equal pieces of at most `piece_groups` groups
// and record the truth-table runs of each piece.
void build_pieces(GateProgram& gp, uint32_t piece_groups);

// Packed 8-byte record for one cell in shared memory: four 16-bit slot
// fields a, b, c, out (the truth table comes from the piece's runs).
inline uint64_t pack_smem_record(uint32_t a, uint32_t b, uint32_t c, uint32_t out) {
  return (uint64_t)a | ((uint64_t)b << 16) | ((uint64_t)c << 32) | ((uint64_t)out << 48);
}

// One truth-table run of a warp's share of a piece: groups [b, e) relative to
// the piece, all with table `lut` (b, e < 4096).
inline uint32_t pack_run(uint32_t lut, uint32_t b, uint32_t e) { return lut | (b << 8) | (e << 20); }

// The pieces as the fused kernel stages them: per piece a header of
// `hdr_bytes` (the same for every piece), then the packed records of its
// cells (group-major, G per group). Header words 2k and 2k+1 belong to warp
// k: its first truth-table run (pack_run; 0 if it has none) and, as
// `first | last << 16`, the range of its further runs in the list that starts
// at word 2*warps. Warp shares are contiguous, balanced by cost: a warp step
// covers `steps_per` groups and each run costs `run_cost` steps more; warp 0,
// which also keeps the ring full, gets `lead_weight` of a normal share.
// Every piece starts on a 16-byte boundary (bulk-copy rules).
struct PieceBlob {
  std::vector<uint32_t> words;
  std::vector<uint32_t> off_words;  // per piece: first word
  std::vector<uint32_t> bytes;      // per piece: header + records
  uint32_t hdr_bytes = 0;
  uint32_t max_bytes = 0;
};
PieceBlob build_piece_blob(const GateProgram& gp, uint32_t warps, double lead_weight, uint32_t steps_per,
                           double run_cost);

}  // namespace rrtl
