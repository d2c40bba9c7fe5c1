// Packed simulation IR and its machine form.
//
// Restates the reference's lowering pipeline:
//   lower_to_packed_program  crates/rrtl-sim-ir/src/lib.rs:592-659, 12306-12840
//   lower_to_machine_program crates/rrtl-sim-ir/src/lib.rs:661-672, 2997-3178
// The data types follow crates/rrtl-sim-ir/src/lib.rs:67-321. Signal storage
// is flattened into u32 limbs (`offset`, `limbs = ceil(width/32)`), memories
// into per-lane word ranges, and the design into four streams:
// async_reset_comb, comb (levelized), tick_next (register captures) and
// tick_commit (memory writes).
#pragma once

#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "design.h"

namespace rrtl {

struct ValueLayout {
  uint32_t width = 1;
  BitType ty;
  uint32_t offset = 0;
  uint32_t limbs = 1;
};

enum class PSK : uint8_t { Input, Output, Wire, Reg };

struct PackedSignal {
  std::string name;  // "<instance path>.<signal name>"
  bool top = false;  // belongs to the top module (has a source handle)
  uint32_t src_id = 0;
  std::string owner_path;
  ValueLayout layout;
  PSK kind = PSK::Wire;
};

struct PackedMemory {
  std::string name;
  uint32_t src_id = 0;
  bool top = false;
  std::string owner_path;
  uint32_t addr_width = 0;
  uint64_t depth = 0;
  ValueLayout data_layout;
  uint64_t offset = 0;  // word offset inside one lane's memory block
};

struct PackedReset {
  uint32_t signal = 0;
  std::vector<uint32_t> value;
  bool async = false;
  bool active_low = false;
  bool operator==(const PackedReset& o) const {
    return signal == o.signal && value == o.value && async == o.async && active_low == o.active_low;
  }
};

enum class PK : uint8_t {
  Lit, Signal, Not, And, Or, Xor, Add, Sub, Mul, Eq, Ne, Lt, Mux, Slice, Zext, Sext, Trunc, Cast, Concat, MemRead
};

struct PackedExpr {
  PK kind = PK::Lit;
  BitType ty;
  std::vector<uint32_t> lit;  // Lit limbs
  uint32_t index = 0;         // Signal index / memory index
  uint32_t lsb = 0;           // Slice
  bool is_signed = false;     // Lt
  std::vector<PackedExpr> args;
  size_t hash = 0;            // structural hash, filled by finish()
  void finish();
  bool operator==(const PackedExpr& o) const;
};

enum class POK : uint8_t { Assign, CaptureReg, MemoryWrite };

struct PackedOp {
  POK kind = POK::Assign;
  uint32_t dst = 0;  // signal (Assign/CaptureReg) or memory (MemoryWrite)
  PackedExpr expr;   // Assign expr / CaptureReg next / MemoryWrite enable
  PackedExpr addr, data;
  bool has_reset = false;
  PackedReset reset;
};

struct PackedProgram {
  std::string top;
  std::vector<PackedSignal> signals;
  std::vector<PackedMemory> memories;
  std::vector<std::vector<PackedOp>> async_reset_comb, comb, tick_next, tick_commit;  // packets
  std::unordered_map<uint32_t, uint32_t> top_signal_index;  // top-module SignalId -> packed index
  std::unordered_map<uint32_t, uint32_t> top_memory_index;  // top-module SignalId -> memory index
  uint64_t total_signal_words = 0;
  uint64_t total_memory_words_per_lane = 0;
};

// Machine form --------------------------------------------------------------

typedef PK IK;  // instruction kinds mirror expression kinds one to one

struct Instr {
  uint32_t dst = 0;
  BitType ty;
  IK kind = IK::Lit;
  std::vector<uint32_t> ops;  // operand value ids (Mux: cond, then, else)
  std::vector<uint32_t> lit;
  uint32_t index = 0;  // Signal / MemRead memory
  uint32_t lsb = 0;
  bool is_signed = false;
};

enum class EffK : uint8_t { StoreSignal, CaptureReg, MemoryWrite };

struct Effect {
  EffK kind = EffK::StoreSignal;
  uint32_t dst = 0;    // signal or memory
  uint32_t value = 0;  // StoreSignal / CaptureReg value, MemoryWrite data
  uint32_t enable = 0, addr = 0;
  bool has_reset = false;
  PackedReset reset;
};

struct MPacket {
  std::vector<Instr> instrs;
  std::vector<Effect> effects;
};

struct Block {
  std::vector<MPacket> packets;
  uint32_t num_values = 0;          // max value id + 1
  std::vector<uint32_t> value_width;  // width of each value id
};

struct MachineProgram {
  PackedProgram source;
  Block async_reset_comb, comb, tick_next, tick_commit;
};

PackedProgram lower_to_packed_program(const Design& d, const std::string& top);
MachineProgram lower_to_machine_program(const PackedProgram& p);

// Instruction operand ids for dependency analysis (crates/rrtl-sim-ir/src/lib.rs:3180+).
const std::vector<uint32_t>& instr_deps(const Instr& i);

}  // namespace rrtl
