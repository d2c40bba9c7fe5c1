// Bit-sliced evaluation of multi-bit designs on the gate engine.
//
// The reference's BitSliceSimulator (crates/rrtl-sim-ir/src/bitslice.rs:1-402)
// stores a W-bit signal as W bit-planes (plane p = bit p of every lane, 64
// lanes per u64) and evaluates bitwise ops and muxes per plane, add/sub as a
// ripple carry across planes, eq/ne as xor planes OR-reduced, and
// slice/concat/extension as plane reindexing. Here that is a lowering: the
// flattened packed program is rewritten as a design of 1-bit signals (one per
// plane, named "<signal>[p]") whose assignments are those per-plane
// operations, and that design runs on the bit-sliced gate engine (32 lanes
// per u32 word; fused, compiled or plain kernels). Every plane operation has
// at most three plane operands, so it is one LUT3 cell.
//
// Scope (the reference's, plus unsigned/signed compare): And/Or/Xor/Not/Mux/
// Eq/Ne/Lt/Add/Sub and Slice/Concat/Zext/Sext/Trunc/Cast over Signal/Lit,
// registers with synchronous reset. No memories, no multiply (the reference
// rejects both), no asynchronous reset (the gate engine has none).
// Out-of-scope designs throw RrtlError("E_BITSLICE", ...).
#pragma once

#include <string>

#include "design.h"
#include "lower.h"

namespace rrtl {

// The one-module design of 1-bit signals that evaluates `P` plane by plane.
// Its top module keeps the name P.top; plane p of packed signal s is the
// signal "<s.name without the top prefix>[p]"; all registers are clocked by
// an added input "__bitslice_clk".
Design bitslice_design(const PackedProgram& P);

// serde-JSON encoding of a design (the format design_from_json reads).
std::string design_to_json(const Design& d);

}  // namespace rrtl
