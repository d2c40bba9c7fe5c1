// Per-design compiled gate kernels (bit-sliced, 32 lanes per u32 word).
//
// The reference's fastest GPU path is a per-design compiled gate kernel
// (the OpenCL/CUDA emitter gpu_codegen::emit_kernel,
// crates/rrtl-sim-ir/src/gpu_codegen.rs:503-557, measured on crc32 in
// docs/rrtl-optimizations.md:1725-1734). Here a gate program (gateprog.h)
// with its run's stimulus and record tables is emitted as straight-line CUDA
// C++: one thread per 32-lane word for all cycles, every net a register, one
// LOP3 per cell in level order, the register commit and the record stage
// unrolled with the run's nets as constants. It serves runs without stuck-at
// forces on designs of up to kGateJitMaxCells cells; others run the fused
// kernel.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gate_dev.h"
#include "gateprog.h"
#include "word_jit.h"

namespace rrtl {

constexpr size_t kGateJitMaxCells = 8192;
constexpr uint32_t kGateJitThreads = 64;

// A gate run's stimulus table (net, kind, param), record table (net) and
// record mode: what the compiled kernel bakes in.
struct GateRunTables {
  std::vector<GateStimDev> stim;
  std::vector<GateRecDev> rec;
  uint32_t mode = 0;
  std::string key() const;
};

std::string gate_jit_source(const GateProgram& gp, const GateRunTables& run);

// Emit, compile and load; never throws (failures leave ok = false).
void gate_jit_build(const GateProgram& gp, const GateRunTables& run, int device, JitKernel* J);

cudaError_t launch_gate_jit(const JitKernel& J, const GateRunDev& R, cudaStream_t st);

// The fused kernel compiled for one design and tile width
// (`rrtl_gate_fused_jit`): the same code as gate_fused_kernel<W>
// (gate_fused.h), with the run dispatch listing only the truth-table classes
// the design's cells use, so the dispatch and the code it jumps into stay
// small enough for the split piece barrier (fused_tile's kSplit), whose
// second copy of every loop the 80-class generic kernel cannot afford.
// Measured on the 50k-gate netlist (11 of the 80 classes): 78.5 ms per
// 1,000-cycle step at 65,536 lanes, with its own piece blob balanced for the
// split barrier, against 87.5 for the generic kernel.
std::string gate_fused_jit_source(const GateProgram& gp);
void gate_fused_jit_build(const GateProgram& gp, int device, JitKernel* J);
cudaError_t launch_gate_fused_jit(const JitKernel& J, const GateProgDev& P, const GateRunDev& R, uint32_t grid,
                                  size_t smem, cudaStream_t st);

}  // namespace rrtl
