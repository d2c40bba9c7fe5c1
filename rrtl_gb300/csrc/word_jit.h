// Per-design compiled word kernels.
//
// The reference emits a design as straight-line per-lane GPU code (WGSL
// tick_many, crates/rrtl-gpu-sim/src/lib.rs:2857-2890, 3082-4126; the CUDA
// emitter gpu_codegen::emit_kernel, crates/rrtl-sim-ir/src/gpu_codegen.rs:503-557).
// Here the word program (wordprog.h) is emitted as CUDA C++, one statement per
// word instruction in program order, compiled at design load by NVRTC for the
// device's architecture and launched through the runtime's library API. The
// run protocol around it (stimulus, record, commit order) is the same header
// the interpreted kernel uses (word_lane.h).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "word_dev.h"
#include "wordprog.h"

namespace rrtl {

// A run's stimulus table, record table and record mode: what a kernel
// compiled for one run bakes in.
struct WordRunTables {
  std::vector<WordStimDev> stim;
  std::vector<WordRecDev> rec;
  uint32_t mode = 0;
  std::string key() const;
};

// Runs with more table entries than this use the kernel compiled for any run.
constexpr size_t kJitRunTableMax = 64;
// Kernels compiled for specific runs kept per design.
constexpr size_t kJitRunKernelsPerDesign = 64;

// Two-warp split of a run's compiled kernel: which instructions each warp
// evaluates (the cones of its register captures and memory writes; warp 0
// also what the record stage reads), and the register words the warps
// exchange at the clock edge.
struct WordSplitPlan {
  std::vector<uint8_t> in[2];        // per instruction: evaluated by warp p
  std::vector<uint32_t> xwords;      // register signal words, in exchange-row order
  std::vector<uint8_t> owner;        // per exchange word: the warp that captures it
  std::vector<uint8_t> need[2];      // per exchange word: warp p reads it from the other warp
  std::vector<uint8_t> commit_owner; // per commit entry
  size_t sizes[2] = {0, 0};
};

// Split plan of `wp` for `run`; false (with the reason) when the design does
// not split: asynchronous resets, combinational feedback, signals beyond the
// register limit, or partitions too uneven to gain.
bool word_split_plan(const WordProgram& wp, const WordRunTables& run, WordSplitPlan* sp, std::string* why);

// One NVRTC-compiled kernel (a compiled word or gate kernel) loaded as a
// library; destroyed with the design that owns it.
struct JitKernel {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t fn = nullptr;
  std::atomic<bool> ready{false};  // the build finished (the fields below are final)
  bool ok = false;
  std::string error;     // why there is no compiled kernel (empty when ok)
  double compile_ms = 0; // emit + NVRTC + load
  size_t source_bytes = 0;
  size_t static_smem = 0;        // the kernel's static shared memory (stimulus/record tables)
  bool reg_signals = false;      // signal words live in registers (no signal staging)
  bool split = false;            // two warps per 32 lanes (word_jit_run_split)
  uint32_t n_xwords = 0;         // register words exchanged between the two warps
  std::vector<uint8_t> written;  // per memory: the design writes it
  ~JitKernel();
};

// Largest word program that is compiled (bigger ones run interpreted).
constexpr size_t kJitMaxInstrs = 20000;
// Designs with at most this many signal words keep them in registers.
constexpr uint32_t kJitRegSignals = 256;

// CUDA C++ source of a word program's compiled kernel `rrtl_word_jit`: for
// any run, or with `run` for that run's tables only.
std::string word_jit_source(const WordProgram& wp, const WordRunTables* run = nullptr,
                            const WordSplitPlan* split = nullptr);

// Compile `src` for `arch` (e.g. "sm_103a") with NVRTC; returns the cubin,
// or an empty vector with `log` holding the compiler's messages.
std::vector<char> word_jit_compile(const std::string& src, const std::string& arch, std::string* log);

// Load and exercise NVRTC once (a trivial compile) so later compiles skip
// its start-up cost; a no-op when NVRTC is absent.
void jit_warm();

// Compile CUDA source `src` with NVRTC for `device` and load its kernel
// `name` into J. Never throws: failures leave ok = false and the reason in
// error.
void jit_build_kernel(const std::string& src, int device, const char* name, JitKernel* J);

// Emit, compile and load the kernel of `wp` on the current device. Never
// throws: failures leave ok = false and the reason in error.
void word_jit_build(const WordProgram& wp, int device, JitKernel* out, const WordRunTables* run = nullptr,
                    const WordSplitPlan* split = nullptr);

// Shared-memory placement for one launch over `lanes_pad` lanes and `cycles`
// cycles; returns the dynamic shared memory bytes per 128-lane block.
size_t word_jit_place(const WordProgram& wp, const JitKernel& J, uint32_t n_sig_words, uint32_t lanes_pad,
                      uint64_t cycles, uint32_t sm_count, size_t max_smem_block, size_t max_smem_sm,
                      WordJitPlace* out);

cudaError_t launch_word_jit(const JitKernel& J, const WordRunDev& R, const WordJitPlace& Pl, size_t smem,
                            cudaStream_t st);

}  // namespace rrtl
