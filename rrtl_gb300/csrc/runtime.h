// Host runtime objects behind the C ABI (include/rrtl_cuda.h).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/rrtl_cuda.h"
#include "gate_dev.h"
#include "gate_jit.h"
#include "gateprog.h"
#include "lower.h"
#include "word_dev.h"
#include "word_jit.h"
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
  // the same pieces with warp shares balanced for the split piece barrier of
  // the per-design compiled kernel (gdev when they would not fit)
  GateProgDev gdev_split{};
  size_t fused_smem_split = 0;
  DevBuf d_srecs_split, d_pieces_split;
  uint32_t fused_ctas = 1;  // resident fused CTAs per SM
  double tile_cycle_cost = 0;  // estimated warp steps of one tile-cycle (job ordering)
  DevBuf d_srecs, d_pieces, d_src_net, d_src_slot, d_sregs, d_wb, d_grecs, d_lgb, d_gregs;
};

// Per-tile, per-stage force table of a batch for one tile width.
struct ForceTable {
  bool valid = false;
  bool any = false;
  DevBuf d_off, d_forces;
};

// A gate-engine run made ready for a launch: program variant, device run
// descriptor and the sizes of its outputs.
struct GatePrepared {
  GateVariant* v = nullptr;
  GateRunDev R{};
  GateRunTables tables;  // host copies of the run's stimulus and record tables
  bool fused = false;
  uint32_t W = 0;
  size_t trace_out_bytes = 0, hash_bytes = 0, det_bytes = 0;
  bool want_trace = false, want_hash = false, want_det = false;
};

// A word-engine run made ready for chunked launches.
struct WordPrepared {
  WordRunDev R{};
  WordRunTables tables;  // host copies of the run's stimulus and record tables
  bool smem_slots = false;
  uint32_t rec_limbs = 0;
  size_t trace_out_bytes = 0, hash_bytes = 0, det_bytes = 0;
  bool want_trace = false, want_hash = false, want_det = false;
};

// One submitted job of the device job queue.
struct QueueJob {
  uint64_t id = 0;
  rrtl_batch* batch = nullptr;
  rrtl_run run{};
  std::vector<rrtl_stim> stim;    // owned copies of the run's arrays
  std::vector<uint32_t> record;
  uint32_t status = 0;            // RRTL_JOB_*
  uint32_t launch = 0;            // launch that carries it
  GatePrepared prep;
};

// Jobs submitted to a context and the device buffers of its queue launches.
struct JobQueue {
  uint64_t next_id = 1;
  uint32_t launches = 0;
  std::vector<QueueJob> jobs;                 // queued or running
  std::unordered_map<uint64_t, uint32_t> finished;  // id -> RRTL_JOB_DONE / RRTL_JOB_FAILED
  DevBuf d_jobs, d_items, d_next;
  size_t smem_set = 0;                        // dynamic shared memory the queue kernel is prepared for
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;   // around the last launch
  float last_ms = 0.f;
  uint32_t last_items = 0;
  ~JobQueue();
};

// Device tables of a trace replay's checks (RRTL_REC_CHECK).
struct CheckTables {
  const uint32_t* idx = nullptr;
  const uint32_t* exp = nullptr;
  uint32_t* log = nullptr;
  uint32_t cap = 0;
};

// Runtime internals shared by the C ABI and the serving loop.
GatePrepared gate_prepare(rrtl_batch* b, const rrtl_run& run, bool device_ptrs, bool want_fused,
                          const CheckTables* chk = nullptr);
void gate_copy_out(rrtl_batch* b, const GatePrepared& g, const rrtl_run& run);
void gate_plain_launches(const GatePrepared& g, uint64_t cycles, cudaStream_t st, bool graph);
WordPrepared word_prepare(rrtl_batch* b, const rrtl_run& run, bool device_ptrs, bool start_settle,
                          const CheckTables* chk = nullptr);
cudaError_t word_chunk(const rrtl_design* d, const WordPrepared& g, uint64_t c0, uint64_t n, bool last, cudaStream_t st);
void word_copy_out(rrtl_batch* b, const WordPrepared& g, const rrtl_run& run);
size_t gate_queue_static_smem();
cudaError_t gate_queue_prepare(size_t smem);
cudaError_t launch_gate_queue(const GateQueueDev& Q, uint32_t grid, size_t smem, cudaStream_t st);
cudaError_t launch_gate_fused(const GateProgDev& P, const GateRunDev& R, uint32_t grid, size_t smem, cudaStream_t st);
cudaError_t launch_mbar_wait_check(uint32_t limit, uint32_t* out, cudaStream_t st);
void set_last_error(const std::string& msg);
WordRunDev word_chunk_desc(const WordPrepared& g, uint64_t c0, uint64_t n, bool last);
// The compiled gate kernel for this run's tables (built on first use and
// kept per design), or nullptr when the design or run does not qualify.
const JitKernel* gate_jit_for_run(rrtl_design* d, const GateRunTables& t);
// Whether a fused-path run of `words` 32-lane words should use the compiled
// gate kernel: the autotuner's choice for the lane bucket, else designs whose
// live nets fit in registers.
bool gate_jit_preferred(rrtl_design* d, uint32_t words);
constexpr uint32_t kTunedCompiled = 0xFFFFFFFFu;
// Designs whose peak of live nets (the fused program's slot count) is at
// most this use the compiled gate kernel unless tuned otherwise: beyond it
// the nets no longer fit the registers of one thread and spill.
constexpr uint32_t kGateJitAutoSlots = 192;
// Designs of narrow levels (fewer cells per level on average than this) use
// it too: the fused kernel's per-level barrier then dominates and most of its
// warps idle, which costs more than spilled nets.
constexpr uint32_t kGateJitNarrowLevel = 48;
// Host-side preparation a run of `lanes` lanes will need (the gate
// program variant of its tile width, or the word kernel compiled for its
// tables), done ahead so that the serving loop's admission finds it built.
void design_warm_for_run(rrtl_design* d, uint32_t lanes, const rrtl_run& run);
// Throws E_WORD_SCOPE when the interpreted word kernel cannot hold the design's value slots.
void word_require_interp(const rrtl_design* d, const WordPrepared& g);
// The design's compiled word kernel, built on first use; nullptr when the design runs interpreted.
const JitKernel* word_jit_get(rrtl_design* d);
// The kernel compiled for this run's tables (built on first use and kept per
// design), else the design's general compiled kernel, else nullptr.
// lanes_pad: the batch's padded lanes (0: no two-warp split).
const JitKernel* word_jit_for_run(rrtl_design* d, const WordRunTables& t, uint32_t lanes_pad = 0);
cudaError_t launch_word_multi(const WordJobDev* jobs, uint32_t n_jobs, uint32_t blocks, size_t smem, cudaStream_t st);
cudaError_t word_multi_prepare(size_t smem);
// Device address of the allocation-free entry point's scratch array for the
// current device (cudaGetSymbolAddress; the device must be current).
cudaError_t noalloc_scratch_lookup(uint32_t** out);
constexpr uint32_t kWordBlockLanes = 128;
constexpr size_t kWordSmemLimit = 96 * 1024;

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
  std::unique_ptr<rrtl::JobQueue> queue;
  // device address of the allocation-free entry point's fixed scratch array,
  // looked up when the context is created (with its device current), so it
  // lives and dies with the context
  uint32_t* noalloc_scratch = nullptr;
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
  std::map<uint32_t, uint32_t> tuned_w;  // measured best W by lane bucket (ceil log2 of 32-lane words);
                                         // rrtl::kTunedCompiled: the compiled gate kernel
  const rrtl::GateProgram& gp() const { return gvar[gate_base]->gp; }
  // word engine
  rrtl::WordProgram wp;
  rrtl::WordProgDev wdev{};
  rrtl::DevBuf d_wcode, d_wcap, d_wlit;
  std::mutex gvar_mu;  // builds of gvar entries (serving producers prepare designs concurrently)
  std::mutex wjit_mu;
  // compiled word kernels: "general" (any run, built on the first fused run)
  // and one per run tables
  std::map<std::string, std::unique_ptr<rrtl::JitKernel>> wjit_runs;
  std::map<std::string, std::unique_ptr<rrtl::JitKernel>> gjit_runs;  // compiled gate kernels, per run tables
  std::map<std::string, std::unique_ptr<rrtl::JitKernel>> gfused_jit;  // compiled fused kernels, per tile width
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
  bool queued = false;      // a job of this batch is in the context's job queue
  uint32_t last_tile_words = 0;  // tile width of the last fused run, 0 after a plain run
  rrtl::DevBuf d_nets;
  std::vector<rrtl_fault> faults;
  rrtl::ForceTable forces_plain, forces_fused[4];  // plain: 8-word tiles; fused: per log2 W
  // word engine state
  uint32_t lanes_pad = 0;
  rrtl::DevBuf d_values, d_mem, d_caps;
  // per-run scratch
  rrtl::DevBuf d_stim, d_rec, d_in_trace, d_out_trace, d_hash, d_detect;
  rrtl::DevBuf d_chk_idx, d_chk_exp, d_chk_log;  // trace replay
};
