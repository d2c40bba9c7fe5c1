// Instance folding: a design whose top is a flat wrapper of N independent
// instances of one child module runs as the child alone over N x L lanes
// (lane = instance * L + local lane) instead of N flattened copies over L
// lanes. Structural analysis only, after analyze_instance_fold
// (crates/rrtl-sim-ir/src/instance_fold.rs:42-97); the caller lowers the
// child module as the design's top and demultiplexes I/O by lane block, as
// InstanceFoldSimulator does (crates/rrtl-gpu-sim/src/instance_fold.rs).
#pragma once

#include <optional>
#include <string>
#include <vector>

#include "design.h"

namespace rrtl {

struct FoldConnection {
  std::string top_signal;  // the top module's signal name
  uint32_t instance = 0;
  std::string port;        // the child module's port name
  bool output = false;     // the port is a child output (else input)
};

struct InstanceFold {
  std::string child;
  std::vector<std::string> instance_names;
  std::vector<FoldConnection> connections;
};

// The fold plan of `top`, or nullopt with `why` set when the design is not a
// flat wrapper of at least two independent instances of one non-external
// module: the top has no registers, memories, assignments or memory writes
// of its own; no signal is driven by two instance outputs; no instance
// output feeds an instance input (shared inputs such as a clock are
// allowed); inout ports are not folded.
std::optional<InstanceFold> analyze_instance_fold(const Design& d, const std::string& top, std::string* why);

// The plan as JSON: {"child": ..., "instances": [...], "connections":
// [[top_signal, instance, port, "in"|"out"], ...]}.
std::string instance_fold_json(const InstanceFold& f);

}  // namespace rrtl
