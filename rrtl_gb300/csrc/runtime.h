// Host runtime objects behind the C ABI (include/rrtl_cuda.h).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/rrtl_cuda.h"
#include "gate_dev.h"
#include "gateprog.h"
#include "lower.h"
#include "word_dev.h"
#include "wordprog.h"

namespace rrtl {

struct ApiError {
  rrtl_status status;
  std::string msg;
};

[[noreturn]] inline void fail(rrtl_status st, const std::string& msg) { throw ApiError{st, msg}; }

void cuda_check(cudaError_t e, const char* what);

// Device buffer owned by the library (grow-only when used as scratch).
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf();
  void reserve(size_t n);
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

template <class T>
void upload(DevBuf& b, const std::vector<T>& v) {
  b.reserve(std::max<size_t>(v.size() * sizeof(T), 16));
  if (!v.empty()) cuda_check(cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
}

// The gate program for one fused tile width W, with its device copy.
struct GateVariant {
  uint32_t W = 8;
  GateProgram gp;
  std::vector<uint8_t> end_live;  // net is resident at the end of a cycle (recordable on the fused path)
  GateProgDev gdev{};
  bool fused_ok = false;
  size_t fused_smem = 0;
  uint32_t fused_ctas = 1;  // resident fused CTAs per SM
  DevBuf d_srecs, d_pieces, d_src_net, d_src_slot, d_sregs, d_wb, d_grecs, d_lgb, d_gregs;
};

// Per-tile, per-stage force table of a batch for one tile width.
struct ForceTable {
  bool valid = false;
  bool any = false;
  DevBuf d_off, d_forces;
};

}  // namespace rrtl

// Handles are reference counted: a design holds its context and a batch its
// design, so destroying a parent first only drops the caller's reference and
// the parent is released with its last child.
struct rrtl_ctx {
  int refs = 1;
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t sm_count = 0;
  size_t max_smem = 0;      // opt-in shared memory per block
  size_t max_smem_sm = 0;   // shared memory per SM
  cudaEvent_t events[8] = {};
};

struct rrtl_design {
  int refs = 1;
  rrtl_ctx* ctx = nullptr;
  rrtl::Design design;
  std::string top;
  rrtl::MachineProgram mp;
  uint32_t engine = 0;
  // gate engine: one program per fused tile width W (index log2 W), built on
  // demand; nets, levels and registers are the same in every variant
  std::unique_ptr<rrtl::GateVariant> gvar[4];
  uint32_t gate_base = 3;   // log2 W of the variant built at load time
  uint32_t gate_w_max = 0;  // widest W whose slots fit on chip, 0 if none
  const rrtl::GateProgram& gp() const { return gvar[gate_base]->gp; }
  // word engine
  rrtl::WordProgram wp;
  rrtl::WordProgDev wdev{};
  rrtl::DevBuf d_wcode, d_wcap, d_wlit;
};

struct rrtl_batch {
  rrtl_design* d = nullptr;
  uint32_t lanes = 0;
  uint32_t path = RRTL_PATH_FUSED;
  float last_ms = 0.f;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  rrtl::DevBuf d_err;
  // gate engine state
  uint32_t words = 0, words_pad = 0, rows = 0;
  uint32_t tile_words = 0;  // requested fused tile width, 0 = chosen per run
  uint32_t last_tile_words = 0;  // tile width of the last fused run, 0 after a plain run
  rrtl::DevBuf d_nets;
  std::vector<rrtl_fault> faults;
  rrtl::ForceTable forces_plain, forces_fused[4];  // plain: 8-word tiles; fused: per log2 W
  // word engine state
  uint32_t lanes_pad = 0;
  rrtl::DevBuf d_values, d_mem, d_caps;
  // per-run scratch
  rrtl::DevBuf d_stim, d_rec, d_in_trace, d_out_trace, d_hash, d_detect;
};
