// Design IR: the RTL data model the batch simulator compiles from.
//
// Mirrors the reference's `rrtl_ir` types (crates/rrtl-ir/src/lib.rs:8-30
// BitType, :212-282 Expr, :434-475 SignalKind/Reset, :553-575 Module) and the
// parts of `rrtl_core::compile` (crates/rrtl-core/src/lib.rs:1057-1068,
// 3432-3602) that decide expression types. A design arrives as the serde-JSON
// encoding of `rrtl_ir::Design`, so a Rust caller can hand over
// `serde_json::to_string(design.ir())` unchanged.
#pragma once

#include <cstdint>
#include <optional>
#include <string>
#include <vector>

#include "json.h"

namespace rrtl {

typedef unsigned __int128 u128;
typedef __int128 i128;

struct BitType {
  uint32_t width = 1;
  bool is_signed = false;
  bool operator==(const BitType& o) const { return width == o.width && is_signed == o.is_signed; }
  bool operator!=(const BitType& o) const { return !(*this == o); }
};
inline BitType uint_t(uint32_t w) { return BitType{w, false}; }
inline BitType sint_t(uint32_t w) { return BitType{w, true}; }

struct SigRef {
  uint32_t module = 0;
  uint32_t id = 0;
  bool operator==(const SigRef& o) const { return module == o.module && id == o.id; }
};

enum class EK : uint8_t {
  Lit, Signal, Not, And, Or, Xor, Add, Sub, Mul, Eq, Ne, Lt, Mux, Slice, Zext, Sext, Trunc, Cast, Concat, MemRead
};

// Expression tree node (crates/rrtl-ir/src/lib.rs:212-254).
struct Expr {
  EK kind = EK::Lit;
  i128 value = 0;        // Lit
  BitType ty;            // Lit type
  SigRef sig;            // Signal / MemRead memory
  uint32_t lsb = 0;      // Slice
  uint32_t width = 0;    // Slice / Zext / Sext / Trunc target width
  bool cast_signed = false;  // Cast target signedness
  std::vector<Expr> args;    // operands in source order (Mux: cond, then, else)
};

enum class SigKind : uint8_t { Input, Output, Inout, Wire, Reg, Mem };

struct Reset {
  SigRef signal;
  i128 value = 0;
  bool async = false;       // ResetKind::Async
  bool active_low = false;  // ResetPolarity::ActiveLow
};

struct SignalInfo {
  SigRef handle;
  std::string name;
  uint32_t width = 1;
  BitType ty;
  SigKind kind = SigKind::Wire;
  // Reg
  std::optional<SigRef> clock;
  std::optional<Reset> reset;
  std::optional<Expr> next;
  // Mem
  uint32_t addr_width = 0;
  uint32_t data_width = 0;
  uint64_t depth = 0;
};

struct Assignment {
  SigRef dst;
  Expr expr;
};

struct MemoryWrite {
  SigRef mem;
  SigRef clock;
  Expr enable, addr, data;
};

struct InitialRegisterValue {
  SigRef signal;
  i128 value = 0;
};

struct InitialMemoryValue {
  SigRef mem;
  uint64_t addr = 0;
  i128 value = 0;
};

struct Instance {
  std::string name;
  std::string module;
  std::vector<std::pair<std::string, SigRef>> connections;
};

struct Module {
  uint32_t id = 0;
  std::string name;
  bool is_external = false;
  std::vector<SignalInfo> signals;
  std::vector<Assignment> assignments;
  std::vector<MemoryWrite> memory_writes;
  std::vector<InitialRegisterValue> initial_register_values;
  std::vector<InitialMemoryValue> initial_memory_values;
  std::vector<Instance> instances;
  size_t n_assertions = 0;
  size_t n_cover_points = 0;

  const SignalInfo* signal(SigRef s) const {
    if (s.module != id || s.id >= signals.size()) return nullptr;
    return &signals[s.id];
  }
};

struct Design {
  std::vector<Module> modules;
  const Module* find_module(const std::string& name) const {
    for (auto& m : modules)
      if (m.name == name) return &m;
    return nullptr;
  }
};

// Error carrying a stable diagnostic code like the reference's
// `Diagnostic { code, message }` (crates/rrtl-ir/src/lib.rs:612-640).
struct RrtlError : std::runtime_error {
  std::string code;
  RrtlError(std::string c, const std::string& msg) : std::runtime_error(c + ": " + msg), code(std::move(c)) {}
};

// Parse the serde-JSON encoding of `rrtl_ir::Design`.
Design design_from_json(const char* text, size_t len);

// Expression type as computed by `expr_type` in the reference compiler
// (crates/rrtl-core/src/lib.rs:5424-5605). Throws RrtlError with the reference's
// diagnostic code on the type errors that would change simulation meaning.
BitType expr_type(const Module& m, const Expr& e);

// The subset of `validate_design` (crates/rrtl-core/src/lib.rs:3417) that the
// simulators rely on: every expression types, assignment and register widths
// match their destination, registers have a clock and a next.
void validate(const Design& d);

uint32_t limbs_for(uint32_t width);        // ceil(width/32), at least 1
uint32_t final_limb_mask(uint32_t width);  // mask of the top limb
std::vector<uint32_t> encode_limbs(i128 value, BitType ty);

}  // namespace rrtl
