// C ABI implementation (include/rrtl_cuda.h): contexts, compiled designs,
// lane batches and runs. All device memory is owned here; caller buffers are
// only touched during a call.
#include "runtime.h"
#include "bitslice.h"
#include "instance_fold.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

namespace rrtl {

// kernels (gate_kernels.cu, word_kernels.cu)
size_t gate_fused_smem_bytes(const GateProgDev& P);
cudaError_t gate_fused_prepare(const GateProgDev& P, size_t smem);
cudaError_t gate_queue_prepare(size_t smem);
size_t gate_queue_static_smem();
cudaError_t launch_gate_queue(const GateQueueDev& Q, uint32_t grid, size_t smem, cudaStream_t st);
int gate_fused_ctas_per_sm(const GateProgDev& P, size_t smem);
cudaError_t launch_gate_fused(const GateProgDev& P, const GateRunDev& R, uint32_t grid, size_t smem, cudaStream_t st);
cudaError_t launch_gate_plain(const GateProgDev& P, const GateRunDev& R, uint64_t c, int phase, cudaStream_t st);
cudaError_t launch_word(const WordProgDev& P, const WordRunDev& R, bool smem_slots, cudaStream_t st);
cudaError_t word_prepare(size_t smem);

constexpr uint32_t kWordThreads = kWordBlockLanes;
constexpr size_t kWordSmemBudget = kWordSmemLimit;

void cuda_check(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation) fail(RRTL_E_OOM, std::string("E_OOM: ") + what + ": " + cudaGetErrorString(e));
  if (e != cudaSuccess) fail(RRTL_E_DEVICE, std::string("E_DEVICE: ") + what + ": " + cudaGetErrorString(e));
}

JobQueue::~JobQueue() {
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
}

DevBuf::~DevBuf() {
  if (p) cudaFree(p);
}

void DevBuf::reserve(size_t n) {
  if (n <= bytes) return;
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
  cuda_check(cudaMalloc(&p, n), "cudaMalloc");
  bytes = n;
}

}  // namespace rrtl

using namespace rrtl;

static thread_local std::string g_last_error;

namespace rrtl {
// Error reporting for entry points defined outside this file.
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace rrtl

template <class F>
static rrtl_status guard(F&& f) {
  try {
    f();
    g_last_error.clear();
    return RRTL_OK;
  } catch (const ApiError& e) {
    g_last_error = e.msg;
    return e.status;
  } catch (const RrtlError& e) {
    g_last_error = e.what();
    return e.code.rfind("E_GATE_SCOPE", 0) == 0 || e.code.rfind("E_WORD_SCOPE", 0) == 0 ? RRTL_E_UNSUPPORTED
                                                                                         : RRTL_E_DESIGN;
  } catch (const std::bad_alloc&) {
    g_last_error = "E_OOM: host allocation failed";
    return RRTL_E_OOM;
  } catch (const std::exception& e) {
    g_last_error = std::string("E_INTERNAL: ") + e.what();
    return RRTL_E_ARG;
  }
}

#define REQUIRE(cond, st, msg) \
  do {                         \
    if (!(cond)) fail(st, msg); \
  } while (0)

// ------------------------------------------------------------------ helpers --

namespace rrtl {

uint32_t round_up(uint32_t x, uint32_t m) { return (x + m - 1) / m * m; }

void set_device(rrtl_ctx* c) { cuda_check(cudaSetDevice(c->device), "cudaSetDevice"); }

const PackedSignal& signal_of(rrtl_design* d, uint32_t s) {
  REQUIRE(s < d->mp.source.signals.size(), RRTL_E_SIGNAL, "E_GPU_SIGNAL: signal index out of range");
  return d->mp.source.signals[s];
}

constexpr uint32_t kRingBufs = 4;  // record ring buffers of the fused kernel
// Share of a piece's groups given to warp 0, which also keeps the ring full.
#ifndef RRTL_LEAD_WARP_WEIGHT
#define RRTL_LEAD_WARP_WEIGHT 0.7
#endif
constexpr double kLeadWarpWeight = RRTL_LEAD_WARP_WEIGHT;
// Dispatch cost of one truth-table run, in warp steps (work split of a piece).
#ifndef RRTL_RUN_COST
#define RRTL_RUN_COST 4.0
#endif
constexpr double kRunCost = RRTL_RUN_COST;
// The same two weights for the blob of the per-design compiled kernel,
// whose split piece barrier lets a warp that arrives late start its next
// piece late: lighter lead-warp relief and a cheaper run balance best there
// (50k-gate netlist, 65,536 lanes: 83.7 ms per step at 0.7 / 4 steps, 78.8
// at 0.85 / 2; the CTA-barrier kernels lose 2% at 0.85).
#ifndef RRTL_LEAD_WARP_WEIGHT_SPLIT
#define RRTL_LEAD_WARP_WEIGHT_SPLIT 0.85
#endif
#ifndef RRTL_RUN_COST_SPLIT
#define RRTL_RUN_COST_SPLIT 2.0
#endif
constexpr double kLeadWarpWeightSplit = RRTL_LEAD_WARP_WEIGHT_SPLIT;
constexpr double kRunCostSplit = RRTL_RUN_COST_SPLIT;

uint32_t log2_words(uint32_t W) { return W == 8 ? 3u : W == 4 ? 2u : W == 2 ? 1u : 0u; }

// Build and upload the gate program for fused tile width W. The fused path
// needs the slots (W words each), a 4-deep record ring and the piece/segment
// tables in one CTA's shared memory; pieces take what the slots leave (up to
// 512 groups) and shrink until the tables fit too.
GateVariant* gate_variant(rrtl_design* d, uint32_t W) {
  uint32_t li = log2_words(W);
  std::lock_guard<std::mutex> lk(d->gvar_mu);
  if (d->gvar[li]) return d->gvar[li].get();
  auto v = std::make_unique<GateVariant>();
  v->W = W;
  v->gp = build_gate_program(d->mp, W);
  GateProgram& gp = v->gp;
  const uint32_t G = gp.group;
  REQUIRE(gp.n_nets + 1 < (1u << 24), RRTL_E_UNSUPPORTED, "E_GATE_SCOPE: more than 16M nets");
  const uint32_t scratch_net = gp.n_nets;  // extra row for padding cells
  std::vector<uint4> grecs(gp.cells.size());
  std::vector<uint32_t> wb(gp.cells.size(), 0xFFFFFFFFu);
  for (size_t i = 0; i < gp.cells.size(); ++i) {
    const GateCell& c = gp.cells[i];
    uint32_t out = c.pad ? scratch_net : c.out;
    grecs[i] = make_uint4(c.in[0], c.in[1], c.in[2], out | ((uint32_t)c.lut << 24));
    if (!c.pad && gp.net_signal[c.out] >= 0) wb[i] = c.out;
  }
  std::vector<GateRegDev> gregs, sregs;
  for (auto& r : gp.regs) {
    uint32_t fl = (r.has_reset ? 1u : 0u) | (r.active_low ? 2u : 0u) | (r.reset_value ? 4u : 0u);
    gregs.push_back(GateRegDev{r.q_net, r.d_net, r.rst_net, fl});
  }
  upload(v->d_grecs, grecs);
  upload(v->d_wb, wb);
  upload(v->d_lgb, gp.level_group_begin);
  upload(v->d_gregs, gregs);

  // shared memory of one CTA: all of it, or an equal share when several
  // CTAs of fewer warps are meant to share an SM (1 KB per CTA is reserved)
  const size_t max_smem = kGateFusedCtasPerSm == 1
                              ? d->ctx->max_smem
                              : std::min(d->ctx->max_smem, d->ctx->max_smem_sm / kGateFusedCtasPerSm - 1024);
  const size_t slot_bytes = (((size_t)gp.n_slots * W * 4 + 15) & ~(size_t)15) + 128;  // slots + header
  const size_t group_bytes = (size_t)G * 8;                                           // records of one group
  v->fused_ok = gp.n_slots <= kMaxSlots && slot_bytes + kRingBufs * 8 * group_bytes <= max_smem;
  uint32_t piece_groups = 8;
  PieceBlob blob;
  if (v->fused_ok) {
    size_t per_buf = (max_smem - slot_bytes) / kRingBufs;
    piece_groups = (uint32_t)std::min<size_t>(512, per_buf / group_bytes) & ~7u;
    for (;;) {
      build_pieces(gp, piece_groups);
      blob = build_piece_blob(gp, kGateFusedWarps, kLeadWarpWeight, gate_fused_vec(W), kRunCost);
      size_t need = slot_bytes + gp.pieces.size() * sizeof(GatePieceDev) + (size_t)kRingBufs * blob.max_bytes;
      if (need <= max_smem) break;
      if (piece_groups <= 8) {
        v->fused_ok = false;
        break;
      }
      piece_groups -= 8;
    }
  } else {
    build_pieces(gp, 256);
  }
  for (const GatePiece& pc : gp.pieces)
    v->tile_cycle_cost += std::ceil((double)pc.n_groups / (kGateFusedWarps * (double)gate_fused_vec(W))) + 4.0;
  if (v->fused_ok) {
    std::vector<GatePieceDev> pieces;
    for (size_t i = 0; i < gp.pieces.size(); ++i) {
      const GatePiece& p = gp.pieces[i];
      pieces.push_back(GatePieceDev{p.group_begin, p.n_groups, p.level, p.last_of_level ? 1u : 0u, blob.off_words[i],
                                    blob.bytes[i], 0, 0});
    }
    std::vector<uint32_t> src_slot;
    for (uint32_t n : gp.source_nets) src_slot.push_back((uint32_t)gp.net_slot[n]);
    for (uint32_t k : commit_order(gp)) {
      const GateReg& r = gp.regs[k];
      uint32_t fl = (r.has_reset ? 1u : 0u) | (r.active_low ? 2u : 0u) | (r.reset_value ? 4u : 0u);
      sregs.push_back(GateRegDev{(uint32_t)gp.net_slot[r.q_net], (uint32_t)gp.net_slot[r.d_net],
                                 (uint32_t)gp.net_slot[r.rst_net], fl});
    }
    upload(v->d_srecs, blob.words);
    upload(v->d_pieces, pieces);
    upload(v->d_src_net, gp.source_nets);
    upload(v->d_src_slot, src_slot);
    upload(v->d_sregs, sregs);
  }
  GateProgDev& P = v->gdev;
  P = GateProgDev{};
  P.blob = v->d_srecs.as<uint32_t>();
  P.pieces = v->d_pieces.as<GatePieceDev>();
  P.ring_bytes = blob.max_bytes;
  P.hdr_bytes = blob.hdr_bytes;
  P.n_pieces = (uint32_t)gp.pieces.size();
  P.n_slots = gp.n_slots;
  P.n_levels = gp.n_levels;
  P.piece_groups = piece_groups;
  P.src_net = v->d_src_net.as<uint32_t>();
  P.src_slot = v->d_src_slot.as<uint32_t>();
  P.n_src = (uint32_t)gp.source_nets.size();
  P.sregs = v->d_sregs.as<GateRegDev>();
  P.wb_net = v->d_wb.as<uint32_t>();
  P.grecs = v->d_grecs.as<uint4>();
  P.level_group_begin = v->d_lgb.as<uint32_t>();
  P.gregs = v->d_gregs.as<GateRegDev>();
  P.n_regs = (uint32_t)gp.regs.size();
  P.const0_slot = v->fused_ok ? (uint32_t)gp.net_slot[kNetConst0] : 0;
  P.const1_slot = v->fused_ok ? (uint32_t)gp.net_slot[kNetConst1] : 0;
  P.group = G;
  if (v->fused_ok) {
    v->fused_smem = gate_fused_smem_bytes(P);
    if (v->fused_smem > max_smem) {
      v->fused_ok = false;
    } else {
      // the limit is per kernel, not per design: allow the device maximum so
      // every design's variant of this width can launch
      cuda_check(gate_fused_prepare(P, d->ctx->max_smem), "gate_fused_prepare");
      v->fused_ctas = (uint32_t)gate_fused_ctas_per_sm(P, v->fused_smem);
    }
  }
  v->gdev_split = v->gdev;
  v->fused_smem_split = v->fused_smem;
  if (v->fused_ok) {
    PieceBlob bs = build_piece_blob(gp, kGateFusedWarps, kLeadWarpWeightSplit, gate_fused_vec(W), kRunCostSplit);
    GateProgDev Ps = v->gdev;
    Ps.ring_bytes = bs.max_bytes;
    Ps.hdr_bytes = bs.hdr_bytes;
    const size_t need = gate_fused_smem_bytes(Ps);
    if (need <= max_smem) {
      std::vector<GatePieceDev> pieces;
      for (size_t i = 0; i < gp.pieces.size(); ++i) {
        const GatePiece& pc = gp.pieces[i];
        pieces.push_back(GatePieceDev{pc.group_begin, pc.n_groups, pc.level, pc.last_of_level ? 1u : 0u,
                                      bs.off_words[i], bs.bytes[i], 0, 0});
      }
      upload(v->d_srecs_split, bs.words);
      upload(v->d_pieces_split, pieces);
      Ps.blob = v->d_srecs_split.as<uint32_t>();
      Ps.pieces = v->d_pieces_split.as<GatePieceDev>();
      v->gdev_split = Ps;
      v->fused_smem_split = need;
    }
  }
  // nets that hold their end-of-cycle value in a slot (recordable on the fused path)
  v->end_live = gp.net_end_live;
  d->gvar[li] = std::move(v);
  return d->gvar[li].get();
}

// Load-time variant: the widest tile whose slots fit on chip. Slot counts
// barely depend on W, so a miss at W = 8 predicts the width that fits.
void build_gate_variants(rrtl_design* d) {
  GateVariant* v8 = gate_variant(d, 8);
  d->gate_base = 3;
  d->gate_w_max = v8->fused_ok ? 8 : 0;
  if (v8->fused_ok || v8->gp.n_slots > kMaxSlots) return;
  for (uint32_t W = 4; W >= 1; W /= 2) {
    size_t need = (size_t)v8->gp.n_slots * W * 4 + 128 + kRingBufs * 8 * (32 / W) * 8;
    if (need > d->ctx->max_smem && W > 1) continue;
    GateVariant* v = gate_variant(d, W);
    if (v->fused_ok) {
      d->gate_base = log2_words(W);
      d->gate_w_max = W;
      return;
    }
  }
}

// Fused tile width for a run over `words` 32-lane words. Cost model per SM:
// every tile runs every level; a warp evaluates one group of G = 32/W cells
// per step, the CTA's warps (kGateFusedWarps) share a level, and each level
// piece ends in a barrier worth about kBarrierSteps group steps. A step costs more at small
// W because G cells rarely find their inputs in G distinct shared-memory
// banks (kStepCost, by log2 W). Tiles are spread over the SMs in whole rounds.
uint32_t lane_bucket(uint32_t words) {
  uint32_t b = 0;
  while ((1u << b) < words) ++b;
  return b;
}

uint32_t choose_tile_words(rrtl_design* d, uint32_t words) {
  auto tuned = d->tuned_w.find(lane_bucket(words));
  if (tuned != d->tuned_w.end() && tuned->second != kTunedCompiled) return tuned->second;
  constexpr double kBarrierSteps = 4.0;
  constexpr double kStepCost[4] = {1.45, 1.25, 1.1, 1.0};
  const GateProgram& gp = d->gp();
  const uint32_t sms = d->ctx->sm_count * kGateFusedCtasPerSm;
  double best = INFINITY;
  uint32_t best_w = d->gate_w_max;
  for (uint32_t W = d->gate_w_max; W >= 1; W /= 2) {
    const uint32_t G = 32 / W;
    double per_tile = 0;
    for (uint32_t L = 0; L < gp.n_levels; ++L) {
      double cells = (double)(gp.level_group_begin[L + 1] - gp.level_group_begin[L]) * gp.group;
      double groups = std::ceil(cells / G);
      per_tile += std::ceil(groups / (double)kGateFusedWarps) * kStepCost[log2_words(W)] +
                  kBarrierSteps * std::max(1.0, std::ceil(groups / 512.0));
    }
    uint32_t tiles = (words + W - 1) / W;
    double t = std::ceil((double)tiles / sms) * per_tile;
    if (t < best * 0.97) {  // a narrower tile must win clearly
      best = t;
      best_w = W;
    }
  }
  return best_w;
}

void upload_word_program(rrtl_design* d) {
  const WordProgram& wp = d->wp;
  upload(d->d_wcode, wp.code);
  upload(d->d_wlit, wp.lits);
  // memories and commits share one buffer
  std::vector<uint8_t> blob(wp.mems.size() * sizeof(WMemDev) + wp.commits.size() * sizeof(WCommitDev) + 16);
  if (!wp.mems.empty()) memcpy(blob.data(), wp.mems.data(), wp.mems.size() * sizeof(WMemDev));
  if (!wp.commits.empty())
    memcpy(blob.data() + wp.mems.size() * sizeof(WMemDev), wp.commits.data(), wp.commits.size() * sizeof(WCommitDev));
  upload(d->d_wcap, blob);
  WordProgDev& W = d->wdev;
  W = WordProgDev{};
  W.code = d->d_wcode.as<WInstr>();
  W.comb_b = wp.comb_b; W.comb_e = wp.comb_e;
  W.async_b = wp.async_b; W.async_e = wp.async_e;
  W.next_b = wp.next_b; W.next_e = wp.next_e;
  W.commit_b = wp.commit_b; W.commit_e = wp.commit_e;
  W.lits = d->d_wlit.as<unsigned long long>();
  W.mems = d->d_wcap.as<WMemDev>();
  W.commits = reinterpret_cast<const WCommitDev*>(d->d_wcap.as<uint8_t>() + wp.mems.size() * sizeof(WMemDev));
  W.n_commits = (uint32_t)wp.commits.size();
  W.n_vslots = std::max<uint32_t>(wp.n_vslots, 1);
  W.n_sig_words = (uint32_t)d->mp.source.total_signal_words;
  size_t smem = (size_t)W.n_vslots * kWordThreads * 8u;
  // signal values stay in shared memory for a launch when they fit beside the slots
  const size_t sig = (size_t)W.n_sig_words * kWordThreads * 4u;
  W.sig_smem = smem + sig <= kWordSmemBudget ? 1u : 0u;
  if (smem <= kWordSmemBudget) cuda_check(word_prepare(kWordSmemBudget), "word_prepare");
}

bool word_smem_slots(rrtl_design* d) { return (size_t)d->wdev.n_vslots * kWordThreads * 8u <= kWordSmemBudget; }

struct Timer {
  rrtl_batch* b;
  explicit Timer(rrtl_batch* bb) : b(bb) { cuda_check(cudaEventRecord(b->ev0, b->d->ctx->stream), "event"); }
  void stop() { cuda_check(cudaEventRecord(b->ev1, b->d->ctx->stream), "event"); }
};

void check_err_word(rrtl_batch* b) {
  uint32_t e = 0;
  cuda_check(cudaMemcpyAsync(&e, b->d_err.p, 4, cudaMemcpyDeviceToHost, b->d->ctx->stream), "err");
  cuda_check(cudaStreamSynchronize(b->d->ctx->stream), "sync");
  if (e) {
    cudaMemsetAsync(b->d_err.p, 0, 4, b->d->ctx->stream);
    fail((rrtl_status)e, "E_TIMEOUT: a bounded device wait gave up");
  }
}

// Forces grouped per tile of `tile_words` words and per stage (stage 0 after
// commit, L+1 after level L). `v` gives the on-chip slots of the fused path
// (null for the plain path, which addresses nets).
void build_forces(rrtl_batch* b, ForceTable& ft, uint32_t tile_words, const GateVariant* v) {
  const GateProgram& gp = b->d->gp();
  const uint32_t stages = gp.n_levels + 1;
  const uint32_t n_tiles = b->words_pad / tile_words;
  std::map<std::tuple<uint32_t, uint32_t, uint32_t, uint32_t>, std::pair<uint32_t, uint32_t>> merged;  // (tile, stage, net, word)
  for (auto& f : b->faults) {
    uint32_t net = gp.signal_net[f.signal];
    int32_t lv = gp.net_level[net];
    uint32_t stage = lv < 0 ? 0u : (uint32_t)lv + 1u;
    uint32_t gw = f.lane / 32, bit = f.lane % 32;
    auto& mv = merged[std::make_tuple(gw / tile_words, stage, net, gw % tile_words)];
    mv.first |= 1u << bit;
    if (f.value) mv.second |= 1u << bit;
    else mv.second &= ~(1u << bit);
  }
  std::vector<GateForceDev> fs;
  std::vector<uint32_t> off((size_t)n_tiles * (stages + 1), 0);
  size_t k = 0;
  auto it = merged.begin();
  for (uint32_t t = 0; t < n_tiles; ++t)
    for (uint32_t s = 0; s <= stages; ++s) {
      off[(size_t)t * (stages + 1) + s] = (uint32_t)k;
      if (s == stages) continue;
      while (it != merged.end() && std::get<0>(it->first) == t && std::get<1>(it->first) == s) {
        uint32_t net = std::get<2>(it->first);
        int32_t slot = v ? v->gp.net_slot[net] : 0;
        fs.push_back(GateForceDev{(uint32_t)std::max(slot, 0), net, std::get<3>(it->first), it->second.first,
                                  it->second.second, 0});
        ++k;
        ++it;
      }
    }
  // the per-tile table stores stages+1 boundaries; the last boundary of tile t is the first of tile t+1
  for (uint32_t t = 0; t < n_tiles; ++t)
    off[(size_t)t * (stages + 1) + stages] = t + 1 < n_tiles ? off[(size_t)(t + 1) * (stages + 1)] : (uint32_t)k;
  upload(ft.d_forces, fs);
  upload(ft.d_off, off);
  ft.any = !fs.empty();
  ft.valid = true;
}

void invalidate_forces(rrtl_batch* b) {
  b->forces_plain.valid = false;
  for (auto& f : b->forces_fused) f.valid = false;
}

// ---- gate engine run
// Validate a run, pick the program variant and upload its stimulus and record
// tables; stages host input traces and zeroes hash/detect outputs on the
// context stream. `want_fused` asks for the fused path (it falls back to the
// plain path when a recorded net does not stay on chip to the end of a cycle).
GatePrepared gate_prepare(rrtl_batch* b, const rrtl_run& run, bool device_ptrs, bool want_fused,
                          const CheckTables* chk) {
  rrtl_design* d = b->d;
  cudaStream_t st = d->ctx->stream;
  GatePrepared g;
  const uint32_t W = want_fused ? (b->tile_words ? b->tile_words : choose_tile_words(d, b->words)) : 0;
  GateVariant* v = W ? gate_variant(d, W) : d->gvar[d->gate_base].get();
  const GateProgram& gp = v->gp;
  bool fused = W && v->fused_ok;
  std::vector<GateStimDev> stim;
  for (uint32_t i = 0; i < run.n_stim; ++i) {
    const rrtl_stim& s = run.stim[i];
    signal_of(d, s.signal);
    uint32_t net = gp.signal_net[s.signal];
    REQUIRE(gp.net_is_source[net], RRTL_E_ARG, "E_GPU_STIM: stimulus targets a combinationally driven signal");
    REQUIRE(s.kind <= RRTL_STIM_RANDOM_UNIFORM, RRTL_E_ARG, "E_GPU_STIM: unknown stimulus kind");
    if (s.kind == RRTL_STIM_TRACE)
      REQUIRE(s.param < run.n_trace_cols && run.input_trace, RRTL_E_ARG, "E_GPU_STIM: trace column out of range");
    stim.push_back(GateStimDev{0u, net, s.kind, 0, s.param});
  }
  std::vector<GateRecDev> rec;
  for (uint32_t i = 0; i < run.n_record; ++i) {
    signal_of(d, run.record[i]);
    uint32_t net = gp.signal_net[run.record[i]];
    if (fused && !v->end_live[net]) fused = false;  // value not held to the end of the cycle: use the plain path
    rec.push_back(GateRecDev{0u, net});
  }
  if (fused) {
    for (auto& r : rec) r.slot = (uint32_t)gp.net_slot[r.net];
    for (auto& s : stim) s.slot = (uint32_t)gp.net_slot[s.net];
  }
  REQUIRE(!(run.record_mode & (RRTL_REC_TRACE | RRTL_REC_HASH | RRTL_REC_DETECT)) || run.n_record > 0, RRTL_E_ARG,
          "E_GPU_RECORD: recording needs at least one signal");
  REQUIRE(run.cycles < (1ull << 32), RRTL_E_ARG, "E_GPU_STEPS: cycle count exceeds 2^32");
  upload(b->d_stim, stim);
  upload(b->d_rec, rec);
  g.tables.stim = stim;
  g.tables.rec = rec;
  g.tables.mode = run.record_mode;

  GateRunDev& R = g.R;
  R.cycles = run.cycles;
  R.seed = run.seed;
  R.n_stim = (uint32_t)stim.size();
  R.stim = b->d_stim.as<GateStimDev>();
  R.n_rec = (uint32_t)rec.size();
  R.rec = b->d_rec.as<GateRecDev>();
  R.mode = run.record_mode;
  R.n_trace_cols = run.n_trace_cols;
  R.lanes = b->lanes;
  R.words = b->words;
  R.words_pad = b->words_pad;
  R.n_tiles = b->words_pad / (fused ? W : kPadWords);
  ForceTable& ft = fused ? b->forces_fused[log2_words(W)] : b->forces_plain;
  if (!ft.valid) build_forces(b, ft, fused ? W : kPadWords, fused ? v : nullptr);
  R.force_off = ft.d_off.as<uint32_t>();
  R.forces = ft.d_forces.as<GateForceDev>();
  R.has_forces = ft.any ? 1u : 0u;
  R.final_settle = 1;
  R.nets = b->d_nets.as<uint32_t>();
  R.err = b->d_err.as<uint32_t>();
  R.cycle_base = 0;
  REQUIRE(run.lane_base % 32 == 0 && run.lane_base < (1ull << 40), RRTL_E_ARG,
          "E_GPU_LANE_BASE: lane_base must be a multiple of 32 below 2^40");
  R.word_base = run.lane_base / 32;
  REQUIRE(!(run.record_mode & RRTL_REC_CHECK) || chk, RRTL_E_ARG, "E_GPU_RECORD: checks are for trace replay");
  if (chk) {
    R.chk_idx = chk->idx;
    R.chk_exp = chk->exp;
    R.chk_log = chk->log;
    R.chk_cap = chk->cap;
  }

  size_t trace_in_bytes = (size_t)run.cycles * run.n_trace_cols * b->words * 4;
  g.trace_out_bytes = (size_t)run.cycles * run.n_record * b->words * 4;
  g.hash_bytes = (size_t)run.cycles * 8;
  g.det_bytes = (size_t)b->lanes * 4;
  g.want_trace = run.record_mode & RRTL_REC_TRACE;
  g.want_hash = run.record_mode & RRTL_REC_HASH;
  g.want_det = run.record_mode & RRTL_REC_DETECT;
  REQUIRE(!g.want_trace || run.out_trace, RRTL_E_ARG, "E_GPU_RECORD: out_trace is null");
  REQUIRE(!g.want_hash || run.out_hash, RRTL_E_ARG, "E_GPU_RECORD: out_hash is null");
  REQUIRE(!g.want_det || run.detect, RRTL_E_ARG, "E_GPU_RECORD: detect is null");
  if (device_ptrs) {
    R.in_trace = run.input_trace;
    R.out_trace = run.out_trace;
    R.out_hash = reinterpret_cast<unsigned long long*>(run.out_hash);
    R.detect = run.detect;
  } else {
    if (trace_in_bytes) {
      b->d_in_trace.reserve(trace_in_bytes);
      cuda_check(cudaMemcpyAsync(b->d_in_trace.p, run.input_trace, trace_in_bytes, cudaMemcpyHostToDevice, st), "h2d trace");
      R.in_trace = b->d_in_trace.as<uint32_t>();
    }
    if (g.want_trace) {
      b->d_out_trace.reserve(std::max<size_t>(g.trace_out_bytes, 16));
      R.out_trace = b->d_out_trace.as<uint32_t>();
    }
    if (g.want_hash) {
      b->d_hash.reserve(std::max<size_t>(g.hash_bytes, 16));
      R.out_hash = b->d_hash.as<unsigned long long>();
    }
    if (g.want_det) {
      b->d_detect.reserve(std::max<size_t>(g.det_bytes, 16));
      R.detect = b->d_detect.as<uint32_t>();
    }
  }
  if (g.want_hash) cuda_check(cudaMemsetAsync(R.out_hash, 0, g.hash_bytes, st), "memset hash");
  if (g.want_det) cuda_check(cudaMemsetAsync(R.detect, 0xFF, g.det_bytes, st), "memset detect");
  g.v = v;
  g.fused = fused;
  g.W = fused ? W : 0;
  return g;
}

// Copy a prepared run's recorded outputs to the caller's host buffers.
void gate_copy_out(rrtl_batch* b, const GatePrepared& g, const rrtl_run& run) {
  cudaStream_t st = b->d->ctx->stream;
  if (g.want_trace)
    cuda_check(cudaMemcpyAsync(run.out_trace, g.R.out_trace, g.trace_out_bytes, cudaMemcpyDeviceToHost, st), "d2h trace");
  if (g.want_hash)
    cuda_check(cudaMemcpyAsync(run.out_hash, g.R.out_hash, g.hash_bytes, cudaMemcpyDeviceToHost, st), "d2h hash");
  if (g.want_det) cuda_check(cudaMemcpyAsync(run.detect, g.R.detect, g.det_bytes, cudaMemcpyDeviceToHost, st), "d2h detect");
}

// The plain path: one launch per cycle plus the closing settle. With `graph`
// the launches are captured into a CUDA graph and replayed as one submission.
void gate_plain_launches(const GatePrepared& g, uint64_t cycles, cudaStream_t st, bool graph) {
  if (!graph) {
    for (uint64_t c = 0; c < cycles; ++c) cuda_check(launch_gate_plain(g.v->gdev, g.R, c, 0, st), "gate_plain_kernel");
    cuda_check(launch_gate_plain(g.v->gdev, g.R, 0, 1, st), "gate_plain_kernel");
    return;
  }
  cudaGraph_t graph_h = nullptr;
  cudaGraphExec_t exec = nullptr;
  cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
  cudaError_t e = cudaSuccess;
  for (uint64_t c = 0; c < cycles && e == cudaSuccess; ++c) e = launch_gate_plain(g.v->gdev, g.R, c, 0, st);
  if (e == cudaSuccess) e = launch_gate_plain(g.v->gdev, g.R, 0, 1, st);
  cudaError_t e2 = cudaStreamEndCapture(st, &graph_h);
  cuda_check(e, "gate_plain_kernel (capture)");
  cuda_check(e2, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&exec, graph_h, 0);
  cudaGraphDestroy(graph_h);
  cuda_check(e, "cudaGraphInstantiate");
  e = cudaGraphLaunch(exec, st);
  cudaGraphExecDestroy(exec);
  cuda_check(e, "cudaGraphLaunch");
}

// A per-design kernel cache entry is built once, outside the lock: a thread
// that finds an entry another thread is still building gets nullptr and
// falls back (general kernel, interpreter or fused kernel) instead of waiting,
// so a compile on one thread never stalls another (the serving loop).
template <class Build>
const JitKernel* jit_cache_get(std::mutex& mu, std::map<std::string, std::unique_ptr<JitKernel>>& cache,
                             const std::string& key, Build build) {
  JitKernel* J = nullptr;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      JitKernel* e = it->second.get();
      return e->ready.load(std::memory_order_acquire) && e->ok ? e : nullptr;
    }
    if (cache.size() >= kJitRunKernelsPerDesign) return nullptr;
    J = cache.emplace(key, std::make_unique<JitKernel>()).first->second.get();
  }
  build(J);
  J->ready.store(true, std::memory_order_release);
  return J->ok ? J : nullptr;
}

const JitKernel* gate_jit_for_run(rrtl_design* d, const GateRunTables& t) {
  const char* env = getenv("RRTL_GATE_JIT");
  if ((env && env[0] == '0') || d->gp().n_real_cells > kGateJitMaxCells || t.stim.size() > kJitRunTableMax ||
      t.rec.size() > kJitRunTableMax)
    return nullptr;
  return jit_cache_get(d->wjit_mu, d->gjit_runs, t.key(),
                       [&](JitKernel* J) { gate_jit_build(d->gp(), t, d->ctx->device, J); });
}

// The fused kernel compiled for this design's truth-table classes at tile
// width v->W (nullptr: the generic fused kernel runs). RRTL_FUSED_JIT=0 keeps
// the generic kernel (A/B switch).
const JitKernel* fused_jit_for(rrtl_design* d, GateVariant* v) {
  const char* env = getenv("RRTL_FUSED_JIT");
  if ((env && env[0] == '0') || !v->fused_ok) return nullptr;
  return jit_cache_get(d->wjit_mu, d->gfused_jit, "W" + std::to_string(v->W),
                       [&](JitKernel* J) { gate_fused_jit_build(v->gp, d->ctx->device, J); });
}

bool gate_jit_preferred(rrtl_design* d, uint32_t words) {
  const char* env = getenv("RRTL_GATE_JIT");
  if (env && env[0] == '2') return true;  // A/B switch: every design within the compiled kernel's size limit
  auto tuned = d->tuned_w.find(lane_bucket(words));
  if (tuned != d->tuned_w.end()) return tuned->second == kTunedCompiled;
  const GateProgram& gp = d->gp();
  if (gp.n_real_cells > kGateJitMaxCells) return false;
  return gp.n_slots <= kGateJitAutoSlots || gp.n_real_cells < (uint64_t)kGateJitNarrowLevel * std::max(1u, gp.n_levels);
}

void gate_run(rrtl_batch* b, const rrtl_run& run, bool device_ptrs, const CheckTables* chk = nullptr,
              bool force_compiled = false) {
  rrtl_design* d = b->d;
  cudaStream_t st = d->ctx->stream;
  GatePrepared g = gate_prepare(b, run, device_ptrs, b->path == RRTL_PATH_FUSED, chk);
  // the compiled gate kernel: automatic tile width, no stuck-at forces; built before the timed region
  const JitKernel* J = nullptr;
  if (b->path == RRTL_PATH_FUSED && !g.R.has_forces && (force_compiled || (b->tile_words == 0 && gate_jit_preferred(d, b->words))))
    J = gate_jit_for_run(d, g.tables);
  // the fused kernel compiled for the design's truth-table classes, also built before the timed region
  const JitKernel* F = !J && g.fused ? fused_jit_for(d, g.v) : nullptr;
  Timer tm(b);
  if (J) {
    g.R.cycle_base = 0;
    cuda_check(launch_gate_jit(*J, g.R, st), "rrtl_gate_jit");
    g.W = 0;
  } else if (g.fused) {
    uint32_t grid = std::min<uint32_t>(g.R.n_tiles, d->ctx->sm_count * g.v->fused_ctas);
    if (F)
      cuda_check(launch_gate_fused_jit(*F, g.v->gdev_split, g.R, grid, g.v->fused_smem_split, st),
                 "rrtl_gate_fused_jit");
    else
      cuda_check(launch_gate_fused(g.v->gdev, g.R, grid, g.v->fused_smem, st), "gate_fused_kernel");
  } else {
    gate_plain_launches(g, run.cycles, st, b->path == RRTL_PATH_PLAIN_GRAPH && run.cycles > 0);
  }
  b->last_tile_words = g.W;
  tm.stop();
  if (!device_ptrs) {
    gate_copy_out(b, g, run);
    check_err_word(b);
    cuda_check(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1), "elapsed");
  }
}

// ---- word engine run
// Validate a word-engine run and upload its stimulus and record tables;
// stages host input traces and zeroes hash/detect outputs on the context
// stream. `start_settle`: settle before the first cycle.
WordPrepared word_prepare(rrtl_batch* b, const rrtl_run& run, bool device_ptrs, bool start_settle,
                          const CheckTables* chk) {
  rrtl_design* d = b->d;
  cudaStream_t st = d->ctx->stream;
  WordPrepared g;
  std::vector<WordStimDev> stim;
  for (uint32_t i = 0; i < run.n_stim; ++i) {
    const rrtl_stim& s = run.stim[i];
    const PackedSignal& ps = signal_of(d, s.signal);
    REQUIRE(s.kind <= RRTL_STIM_RANDOM_UNIFORM, RRTL_E_ARG, "E_GPU_STIM: unknown stimulus kind");
    if (s.kind == RRTL_STIM_TRACE)
      REQUIRE(s.param < run.n_trace_cols && run.input_trace, RRTL_E_ARG, "E_GPU_STIM: trace column out of range");
    stim.push_back(WordStimDev{ps.layout.offset, ps.layout.limbs, ps.layout.width, s.kind, s.param});
  }
  std::vector<WordRecDev> rec;
  uint32_t rec_limbs = 0;
  for (uint32_t i = 0; i < run.n_record; ++i) {
    const PackedSignal& ps = signal_of(d, run.record[i]);
    rec.push_back(WordRecDev{ps.layout.offset, ps.layout.limbs, ps.layout.width, rec_limbs});
    rec_limbs += ps.layout.limbs;
  }
  REQUIRE(!(run.record_mode & (RRTL_REC_TRACE | RRTL_REC_HASH | RRTL_REC_DETECT)) || run.n_record > 0, RRTL_E_ARG,
          "E_GPU_RECORD: recording needs at least one signal");
  upload(b->d_stim, stim);
  upload(b->d_rec, rec);
  g.tables.stim = stim;
  g.tables.rec = rec;
  g.tables.mode = run.record_mode;
  WordRunDev& R = g.R;
  R.cycles = run.cycles;
  R.seed = run.seed;
  R.n_stim = (uint32_t)stim.size();
  R.stim = b->d_stim.as<WordStimDev>();
  R.n_rec = (uint32_t)rec.size();
  R.rec = b->d_rec.as<WordRecDev>();
  R.rec_limbs = rec_limbs;
  R.mode = run.record_mode;
  R.n_trace_cols = run.n_trace_cols;
  R.lanes = b->lanes;
  R.lanes_pad = b->lanes_pad;
  R.values = b->d_values.as<uint32_t>();
  R.mems = b->d_mem.as<uint32_t>();
  R.caps = b->d_caps.as<uint32_t>();
  R.final_settle = 1;
  R.start_settle = start_settle;
  R.err = b->d_err.as<uint32_t>();
  R.vspill = nullptr;
  REQUIRE(run.lane_base % 32 == 0 && run.lane_base < (1ull << 40), RRTL_E_ARG,
          "E_GPU_LANE_BASE: lane_base must be a multiple of 32 below 2^40");
  R.lane_base = run.lane_base;
  REQUIRE(!(run.record_mode & RRTL_REC_CHECK) || chk, RRTL_E_ARG, "E_GPU_RECORD: checks are for trace replay");
  if (chk) {
    R.chk_idx = chk->idx;
    R.chk_exp = chk->exp;
    R.chk_log = chk->log;
    R.chk_cap = chk->cap;
  }
  g.smem_slots = word_smem_slots(d);
  g.rec_limbs = rec_limbs;
  size_t trace_in_bytes = (size_t)run.cycles * run.n_trace_cols * b->lanes * 4;
  g.trace_out_bytes = (size_t)run.cycles * rec_limbs * b->lanes * 4;
  g.hash_bytes = (size_t)run.cycles * 8;
  g.det_bytes = (size_t)b->lanes * 4;
  g.want_trace = run.record_mode & RRTL_REC_TRACE;
  g.want_hash = run.record_mode & RRTL_REC_HASH;
  g.want_det = run.record_mode & RRTL_REC_DETECT;
  REQUIRE(!g.want_trace || run.out_trace, RRTL_E_ARG, "E_GPU_RECORD: out_trace is null");
  REQUIRE(!g.want_hash || run.out_hash, RRTL_E_ARG, "E_GPU_RECORD: out_hash is null");
  REQUIRE(!g.want_det || run.detect, RRTL_E_ARG, "E_GPU_RECORD: detect is null");
  if (device_ptrs) {
    R.in_trace = run.input_trace;
    R.out_trace = run.out_trace;
    R.out_hash = reinterpret_cast<unsigned long long*>(run.out_hash);
    R.detect = run.detect;
  } else {
    if (trace_in_bytes) {
      b->d_in_trace.reserve(trace_in_bytes);
      cuda_check(cudaMemcpyAsync(b->d_in_trace.p, run.input_trace, trace_in_bytes, cudaMemcpyHostToDevice, st), "h2d trace");
      R.in_trace = b->d_in_trace.as<uint32_t>();
    }
    if (g.want_trace) {
      b->d_out_trace.reserve(std::max<size_t>(g.trace_out_bytes, 16));
      R.out_trace = b->d_out_trace.as<uint32_t>();
    }
    if (g.want_hash) {
      b->d_hash.reserve(std::max<size_t>(g.hash_bytes, 16));
      R.out_hash = b->d_hash.as<unsigned long long>();
    }
    if (g.want_det) {
      b->d_detect.reserve(std::max<size_t>(g.det_bytes, 16));
      R.detect = b->d_detect.as<uint32_t>();
    }
  }
  if (g.want_hash) cuda_check(cudaMemsetAsync(R.out_hash, 0, g.hash_bytes, st), "memset hash");
  if (g.want_det) cuda_check(cudaMemsetAsync(R.detect, 0xFF, g.det_bytes, st), "memset detect");
  return g;
}

// The interpreted word kernel keeps a block's value slots in shared memory
// (the compiled kernel keeps them in registers and has no such limit).
void word_require_interp(const rrtl_design* d, const WordPrepared& g) {
  REQUIRE(g.smem_slots, RRTL_E_UNSUPPORTED,
          "E_WORD_SCOPE: design needs " + std::to_string(d->wdev.n_vslots) +
              " live value slots, more than the interpreted word kernel holds in shared memory");
}

// Launch cycles [c0, c0 + n) of a prepared word run (one kernel; the settle
// before the first cycle only when c0 == 0, the closing one if `last`).
WordRunDev word_chunk_desc(const WordPrepared& g, uint64_t c0, uint64_t n, bool last) {
  WordRunDev R1 = g.R;
  R1.cycles = n;
  R1.start_settle = c0 == 0 ? g.R.start_settle : 0;
  R1.final_settle = last ? 1u : 0u;
  // per-cycle pointers shift so cycle c0 of the run is cycle 0 of the launch's buffers
  R1.in_trace = g.R.in_trace ? g.R.in_trace + (size_t)c0 * g.R.n_trace_cols * g.R.lanes : nullptr;
  R1.out_trace = g.R.out_trace ? g.R.out_trace + (size_t)c0 * g.rec_limbs * g.R.lanes : nullptr;
  R1.out_hash = g.R.out_hash ? g.R.out_hash + c0 : nullptr;
  R1.chk_idx = g.R.chk_idx ? g.R.chk_idx + (size_t)c0 * g.rec_limbs : nullptr;
  R1.chk_exp = g.R.chk_exp ? g.R.chk_exp + (size_t)c0 * g.rec_limbs * g.R.lanes : nullptr;
  R1.cycle_base = c0;
  return R1;
}

cudaError_t word_chunk(const rrtl_design* d, const WordPrepared& g, uint64_t c0, uint64_t n, bool last, cudaStream_t st) {
  return launch_word(d->wdev, word_chunk_desc(g, c0, n, last), g.smem_slots, st);
}

void word_copy_out(rrtl_batch* b, const WordPrepared& g, const rrtl_run& run) {
  cudaStream_t st = b->d->ctx->stream;
  if (g.want_trace)
    cuda_check(cudaMemcpyAsync(run.out_trace, g.R.out_trace, g.trace_out_bytes, cudaMemcpyDeviceToHost, st), "d2h trace");
  if (g.want_hash)
    cuda_check(cudaMemcpyAsync(run.out_hash, g.R.out_hash, g.hash_bytes, cudaMemcpyDeviceToHost, st), "d2h hash");
  if (g.want_det) cuda_check(cudaMemcpyAsync(run.detect, g.R.detect, g.det_bytes, cudaMemcpyDeviceToHost, st), "d2h detect");
}

// The design's compiled word kernel for any run, built on first use (nullptr
// when the design runs interpreted; the reason stays in the "general" cache
// entry's error).
const JitKernel* word_jit_get(rrtl_design* d) {
  const char* env = getenv("RRTL_WORD_JIT");
  if (env && env[0] == '0') return nullptr;
  return jit_cache_get(d->wjit_mu, d->wjit_runs, "general",
                       [&](JitKernel* J) { word_jit_build(d->wp, d->ctx->device, J); });
}

const JitKernel* word_jit_for_run(rrtl_design* d, const WordRunTables& t, uint32_t lanes_pad) {
  const JitKernel* any = word_jit_get(d);
  const char* env = getenv("RRTL_WORD_JIT_RUNS");
  if (!any || (env && env[0] == '0') || t.stim.size() > kJitRunTableMax || t.rec.size() > kJitRunTableMax) return any;
  // two warps per 32 lanes on request only (RRTL_WORD_JIT_SPLIT=2): measured
  // slower than one warp on the pipelined CPU even at 4,096 lanes
  const char* senv = getenv("RRTL_WORD_JIT_SPLIT");
  if (lanes_pad && senv && senv[0] == '2') {
    const JitKernel* S = jit_cache_get(d->wjit_mu, d->wjit_runs, t.key() + "|split", [&](JitKernel* J) {
      WordSplitPlan plan;
      std::string why;
      if (word_split_plan(d->wp, t, &plan, &why)) word_jit_build(d->wp, d->ctx->device, J, &t, &plan);
      else J->error = "no split: " + why;
    });
    if (S) return S;
  }
  const JitKernel* R = jit_cache_get(d->wjit_mu, d->wjit_runs, t.key(),
                                   [&](JitKernel* J) { word_jit_build(d->wp, d->ctx->device, J, &t); });
  return R ? R : any;
}

void design_warm_for_run(rrtl_design* d, uint32_t lanes, const rrtl_run& run) {
  set_device(d->ctx);
  if (d->engine == RRTL_ENGINE_GATE) {
    if (d->gate_w_max) gate_variant(d, choose_tile_words(d, (lanes + 31) / 32));
    return;
  }
  WordRunTables t;
  uint32_t base = 0;
  for (uint32_t i = 0; i < run.n_stim; ++i) {
    const PackedSignal& ps = signal_of(d, run.stim[i].signal);
    t.stim.push_back(WordStimDev{ps.layout.offset, ps.layout.limbs, ps.layout.width, run.stim[i].kind, run.stim[i].param});
  }
  for (uint32_t i = 0; i < run.n_record; ++i) {
    const PackedSignal& ps = signal_of(d, run.record[i]);
    t.rec.push_back(WordRecDev{ps.layout.offset, ps.layout.limbs, ps.layout.width, base});
    base += ps.layout.limbs;
  }
  t.mode = run.record_mode;
  word_jit_for_run(d, t, (lanes + 127) / 128 * 128);
}

void word_run(rrtl_batch* b, const rrtl_run& run, bool device_ptrs, bool start_settle, bool final_settle,
              const CheckTables* chk = nullptr) {
  rrtl_design* d = b->d;
  rrtl_ctx* ctx = d->ctx;
  cudaStream_t st = ctx->stream;
  WordPrepared g = word_prepare(b, run, device_ptrs, start_settle, chk);
  g.R.final_settle = final_settle;
  const bool per_cycle = (b->path == RRTL_PATH_PLAIN || b->path == RRTL_PATH_PLAIN_GRAPH) && run.cycles > 1;
  // compile before the timed region opens
  const JitKernel* J = !per_cycle && b->path == RRTL_PATH_FUSED ? word_jit_for_run(d, g.tables, b->lanes_pad) : nullptr;
  if (!J) word_require_interp(d, g);
  Timer tm(b);
  if (per_cycle) {
    // one launch per cycle: the baseline path (captured into a CUDA graph on RRTL_PATH_PLAIN_GRAPH)
    const bool graph = b->path == RRTL_PATH_PLAIN_GRAPH;
    if (graph) cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    cudaError_t ce = cudaSuccess;
    for (uint64_t c = 0; c < run.cycles && ce == cudaSuccess; ++c)
      ce = word_chunk(d, g, c, 1, c + 1 == run.cycles && final_settle, st);
    if (graph) {
      cudaGraph_t gh = nullptr;
      cudaError_t e2 = cudaStreamEndCapture(st, &gh);
      cuda_check(ce, "word_kernel (capture)");
      cuda_check(e2, "cudaStreamEndCapture");
      cudaGraphExec_t exec = nullptr;
      cudaError_t e3 = cudaGraphInstantiate(&exec, gh, 0);
      cudaGraphDestroy(gh);
      cuda_check(e3, "cudaGraphInstantiate");
      e3 = cudaGraphLaunch(exec, st);
      cudaGraphExecDestroy(exec);
      cuda_check(e3, "cudaGraphLaunch");
    } else {
      cuda_check(ce, "word_kernel");
    }
  } else if (J) {
    WordJitPlace pl;
    const size_t smem = word_jit_place(d->wp, *J, d->wdev.n_sig_words, b->lanes_pad, run.cycles, ctx->sm_count,
                                       ctx->max_smem, ctx->max_smem_sm, &pl);
    cuda_check(launch_word_jit(*J, g.R, pl, smem, st), "rrtl_word_jit");
  } else {
    cuda_check(launch_word(d->wdev, g.R, g.smem_slots, st), "word_kernel");
  }
  tm.stop();
  if (!device_ptrs) {
    word_copy_out(b, g, run);
    check_err_word(b);
    cuda_check(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1), "elapsed");
  }
}

// ---- device job queue

JobQueue& queue_of(rrtl_ctx* c) {
  if (!c->queue) {
    c->queue = std::make_unique<JobQueue>();
    cuda_check(cudaEventCreate(&c->queue->ev0), "event");
    cuda_check(cudaEventCreate(&c->queue->ev1), "event");
  }
  return *c->queue;
}

// Copy results of every job of the finished launches out and record their
// status. Called once the stream has passed the launches' end.
void queue_finish(rrtl_ctx* c) {
  JobQueue& Q = queue_of(c);
  // launch status: a CTA that could not drain its copies fails every job of the launch
  uint32_t launch_err = 0;
  if (Q.d_next.p && cudaMemcpy(&launch_err, Q.d_next.as<uint32_t>() + 1, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    launch_err = RRTL_E_DEVICE;
  std::vector<QueueJob> keep;
  for (QueueJob& j : Q.jobs) {
    if (j.status != RRTL_JOB_RUNNING) {
      keep.push_back(std::move(j));
      continue;
    }
    rrtl_batch* b = j.batch;
    uint32_t e = launch_err;
    cudaError_t ce = e ? cudaSuccess : cudaMemcpy(&e, b->d_err.p, 4, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && e == 0) {
      try {
        gate_copy_out(b, j.prep, j.run);
        cuda_check(cudaStreamSynchronize(c->stream), "sync");
        j.status = RRTL_JOB_DONE;
      } catch (const ApiError&) {
        j.status = RRTL_JOB_FAILED;
      }
    } else {
      cudaMemset(b->d_err.p, 0, 4);
      j.status = RRTL_JOB_FAILED;
    }
    b->queued = false;
    Q.finished[j.id] = j.status;
  }
  Q.jobs.swap(keep);
}

uint64_t queue_submit(rrtl_ctx* c, const rrtl_job& job) {
  rrtl_batch* b = job.batch;
  REQUIRE(b, RRTL_E_ARG, "E_ARG: job has no batch");
  REQUIRE(b->d->ctx == c, RRTL_E_ARG, "E_QUEUE: the job's batch belongs to another context");
  REQUIRE(b->d->engine == RRTL_ENGINE_GATE, RRTL_E_UNSUPPORTED, "E_QUEUE: the job queue runs gate-engine batches");
  REQUIRE(!b->queued, RRTL_E_ARG, "E_QUEUE: the batch already has a job in the queue");
  REQUIRE(job.run.n_stim == 0 || job.run.stim, RRTL_E_ARG, "E_ARG: stim is null");
  REQUIRE(job.run.n_record == 0 || job.run.record, RRTL_E_ARG, "E_ARG: record is null");
  JobQueue& Q = queue_of(c);
  QueueJob j;
  j.id = Q.next_id++;
  j.batch = b;
  j.run = job.run;
  j.stim.assign(job.run.stim, job.run.stim + job.run.n_stim);
  j.record.assign(job.run.record, job.run.record + job.run.n_record);
  j.run.stim = j.stim.data();
  j.run.record = j.record.data();
  j.status = RRTL_JOB_QUEUED;
  b->queued = true;
  Q.jobs.push_back(std::move(j));
  Q.jobs.back().run.stim = Q.jobs.back().stim.data();
  Q.jobs.back().run.record = Q.jobs.back().record.data();
  return Q.jobs.back().id;
}

// One persistent launch over every queued job: each job's tiles become items
// (all cycles of one tile), listed longest first; jobs whose recorded nets
// leave the chip, or whose shared memory exceeds what the queue kernel can
// take, run on their own kernels first on the same stream.
void queue_launch(rrtl_ctx* c) {
  JobQueue& Q = queue_of(c);
  cudaStream_t st = c->stream;
  const size_t qmax = c->max_smem - gate_queue_static_smem();
  std::vector<GateJobDev> jobs;
  std::vector<std::pair<double, GateItemDev>> items;
  size_t smem = 0;
  const uint32_t launch = ++Q.launches;
  cuda_check(cudaEventRecord(Q.ev0, st), "event");
  for (QueueJob& j : Q.jobs) {
    if (j.status != RRTL_JOB_QUEUED) continue;
    rrtl_batch* b = j.batch;
    b->path = RRTL_PATH_FUSED;
    j.prep = gate_prepare(b, j.run, false, true);
    j.status = RRTL_JOB_RUNNING;
    j.launch = launch;
    const GatePrepared& g = j.prep;
    if (!g.fused || g.v->fused_smem > qmax) {
      if (g.fused) {
        uint32_t grid = std::min<uint32_t>(g.R.n_tiles, c->sm_count * g.v->fused_ctas);
        cuda_check(launch_gate_fused(g.v->gdev, g.R, grid, g.v->fused_smem, st), "gate_fused_kernel");
      } else {
        gate_plain_launches(g, j.run.cycles, st, false);
      }
      b->last_tile_words = g.W;
      continue;
    }
    const uint32_t ji = (uint32_t)jobs.size();
    jobs.push_back(GateJobDev{g.v->gdev, g.R});
    smem = std::max(smem, g.v->fused_smem);
    const double cost = (double)(j.run.cycles + 1) * g.v->tile_cycle_cost;
    for (uint32_t t = 0; t < g.R.n_tiles; ++t)
      items.push_back({cost, GateItemDev{ji, t, 0ull, (uint32_t)j.run.cycles, 1u}});
    b->last_tile_words = g.W;
  }
  std::stable_sort(items.begin(), items.end(),
                   [](const std::pair<double, GateItemDev>& x, const std::pair<double, GateItemDev>& y) {
                     return x.first > y.first;
                   });
  Q.last_items = (uint32_t)items.size();
  if (!items.empty()) {
    std::vector<GateItemDev> flat;
    flat.reserve(items.size());
    for (auto& it : items) flat.push_back(it.second);
    upload(Q.d_jobs, jobs);
    upload(Q.d_items, flat);
    Q.d_next.reserve(16);
    cuda_check(cudaMemsetAsync(Q.d_next.p, 0, 8, st), "memset queue");
    if (!Q.smem_set) {
      // the limit is per kernel: allow every job this queue can take
      cuda_check(gate_queue_prepare(qmax), "gate_queue_prepare");
      Q.smem_set = qmax;
    }
    GateQueueDev QD{Q.d_jobs.as<GateJobDev>(), Q.d_items.as<GateItemDev>(), (uint32_t)flat.size(), Q.d_next.as<uint32_t>()};
    const uint32_t grid = std::min<uint32_t>((uint32_t)flat.size(), c->sm_count);
    cuda_check(launch_gate_queue(QD, grid, smem, st), "gate_queue_kernel");
  }
  cuda_check(cudaEventRecord(Q.ev1, st), "event");
}

// Trace replay (GpuBatchSimulator::replay_lane_trace, crates/rrtl-gpu-sim/src/lib.rs:989-1357):
// per step the step's input ops are stored, the design settles, the step's
// checks compare signal limbs per lane with expected values and log
// mismatches, and the clock ticks. Sparse input ops become dense trace
// columns (a signal keeps its last value between ops, starting from the
// batch's current state); checks ride on the record stage.
uint64_t batch_replay(rrtl_batch* b, const rrtl_trace& t, uint32_t cap, uint32_t* log) {
  rrtl_design* d = b->d;
  const bool gate = d->engine == RRTL_ENGINE_GATE;
  const uint32_t unit = gate ? b->words : b->lanes;  // 32-bit values per column per step
  REQUIRE(t.steps < (1ull << 32), RRTL_E_ARG, "E_GPU_TRACE_STEPS: trace replay step count exceeds 2^32");
  REQUIRE(t.n_inputs == 0 || t.inputs, RRTL_E_ARG, "E_ARG: inputs is null");
  REQUIRE(t.n_checks == 0 || t.checks, RRTL_E_ARG, "E_ARG: checks is null");
  const uint64_t steps = t.steps;
  auto limbs_of = [&](uint32_t sig) { return signal_of(d, sig).layout.limbs; };
  // input columns: every limb of every driven signal
  std::map<uint32_t, uint32_t> in_col;
  uint32_t ncols = 0;
  for (uint32_t i = 0; i < t.n_inputs; ++i) {
    const rrtl_trace_input& op = t.inputs[i];
    const PackedSignal& ps = signal_of(d, op.signal);
    REQUIRE(op.limb < ps.layout.limbs, RRTL_E_ARG, "E_GPU_TRACE_INPUTS: limb out of range");
    REQUIRE(op.step < steps, RRTL_E_ARG, "E_GPU_TRACE_INPUTS: step out of range");
    REQUIRE(op.values, RRTL_E_ARG, "E_ARG: input values are null");
    REQUIRE(!gate || ps.layout.width == 1, RRTL_E_ARG, "E_GPU_WIDE_SIGNAL: the gate engine replays 1-bit signals");
    if (!in_col.count(op.signal)) {
      in_col[op.signal] = ncols;
      ncols += ps.layout.limbs;
    }
  }
  std::vector<uint32_t> cur((size_t)ncols * unit, 0), trace((size_t)steps * ncols * unit, 0);
  for (auto& kv : in_col) {
    uint32_t* dst = cur.data() + (size_t)kv.second * unit;
    if (gate) {
      const uint32_t net = d->gp().signal_net[kv.first];
      cuda_check(cudaStreamSynchronize(d->ctx->stream), "sync");
      cuda_check(cudaMemcpy(dst, b->d_nets.as<uint32_t>() + (size_t)net * b->words_pad, (size_t)b->words * 4,
                            cudaMemcpyDeviceToHost),
                 "d2h signal");
    } else {
      std::vector<uint32_t> v((size_t)limbs_of(kv.first) * b->lanes);
      rrtl_status st = rrtl_batch_get_signal_limbs(b, kv.first, v.data(), v.size());
      if (st) fail(st, g_last_error);
      std::copy(v.begin(), v.end(), dst);
    }
  }
  std::vector<uint32_t> order(t.n_inputs);
  for (uint32_t i = 0; i < t.n_inputs; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return t.inputs[x].step < t.inputs[y].step; });
  size_t k = 0;
  for (uint64_t s = 0; s < steps; ++s) {
    for (; k < order.size() && t.inputs[order[k]].step == s; ++k) {
      const rrtl_trace_input& op = t.inputs[order[k]];
      uint32_t* dst = cur.data() + (size_t)(in_col[op.signal] + op.limb) * unit;
      if (gate) {
        std::fill(dst, dst + unit, 0u);
        for (uint32_t l = 0; l < b->lanes; ++l)
          if (op.values[l] & 1u) dst[l / 32] |= 1u << (l % 32);
      } else {
        std::copy(op.values, op.values + b->lanes, dst);
      }
    }
    std::copy(cur.begin(), cur.end(), trace.begin() + (size_t)s * ncols * unit);
  }
  std::vector<rrtl_stim> stim;
  for (auto& kv : in_col) stim.push_back(rrtl_stim{kv.first, RRTL_STIM_TRACE, kv.second});
  // checks: recorded signals, one row per limb
  std::map<uint32_t, uint32_t> rec_row;
  std::vector<uint32_t> rec;
  uint32_t rows = 0;
  for (uint32_t i = 0; i < t.n_checks; ++i) {
    const rrtl_trace_check& op = t.checks[i];
    const PackedSignal& ps = signal_of(d, op.signal);
    REQUIRE(op.limb < ps.layout.limbs, RRTL_E_ARG, "E_GPU_TRACE_CHECKS: limb out of range");
    REQUIRE(op.step < steps, RRTL_E_ARG, "E_GPU_TRACE_CHECKS: step out of range");
    REQUIRE(op.expected, RRTL_E_ARG, "E_ARG: expected values are null");
    REQUIRE(!gate || ps.layout.width == 1, RRTL_E_ARG, "E_GPU_WIDE_SIGNAL: the gate engine replays 1-bit signals");
    if (!rec_row.count(op.signal)) {
      rec_row[op.signal] = rows;
      rec.push_back(op.signal);
      rows += gate ? 1 : ps.layout.limbs;
    }
  }
  std::vector<uint32_t> idx((size_t)steps * rows, 0xFFFFFFFFu), exp((size_t)steps * rows * unit, 0);
  for (uint32_t i = 0; i < t.n_checks; ++i) {
    const rrtl_trace_check& op = t.checks[i];
    const size_t row = (size_t)op.step * rows + rec_row[op.signal] + op.limb;
    idx[row] = op.check_index;
    uint32_t* dst = exp.data() + row * unit;
    if (gate) {
      std::fill(dst, dst + unit, 0u);
      for (uint32_t l = 0; l < b->lanes; ++l)
        if (op.expected[l] & 1u) dst[l / 32] |= 1u << (l % 32);
    } else {
      const uint32_t width = signal_of(d, op.signal).layout.width;
      const bool last = op.limb + 1 == limbs_of(op.signal);
      for (uint32_t l = 0; l < b->lanes; ++l) dst[l] = last ? op.expected[l] & final_limb_mask(width) : op.expected[l];
    }
  }
  upload(b->d_chk_idx, idx);
  upload(b->d_chk_exp, exp);
  b->d_chk_log.reserve(std::max<size_t>((1 + (size_t)cap * 6) * 4, 16));
  cudaStream_t st = d->ctx->stream;
  cuda_check(cudaMemsetAsync(b->d_chk_log.p, 0, 4, st), "memset log");
  CheckTables ct;
  ct.idx = b->d_chk_idx.as<uint32_t>();
  ct.exp = b->d_chk_exp.as<uint32_t>();
  ct.log = b->d_chk_log.as<uint32_t>();
  ct.cap = cap;
  rrtl_run r{};
  r.cycles = steps;
  r.n_stim = (uint32_t)stim.size();
  r.stim = stim.data();
  r.n_record = (uint32_t)rec.size();
  r.record = rec.data();
  r.record_mode = rec.empty() ? 0u : (uint32_t)RRTL_REC_CHECK;
  r.n_trace_cols = ncols;
  r.input_trace = ncols ? trace.data() : nullptr;
  if (gate) gate_run(b, r, false, &ct);
  else word_run(b, r, false, false, true, &ct);
  uint32_t count = 0;
  cuda_check(cudaMemcpy(&count, b->d_chk_log.p, 4, cudaMemcpyDeviceToHost), "d2h log");
  const uint32_t kept = std::min(count, cap);
  if (log) {
    log[0] = count;
    if (kept) cuda_check(cudaMemcpy(log + 1, b->d_chk_log.as<uint32_t>() + 1, (size_t)kept * 6 * 4, cudaMemcpyDeviceToHost), "d2h log");
  }
  return count;
}

void batch_eval(rrtl_batch* b) {
  rrtl_run r{};
  if (b->d->engine == RRTL_ENGINE_GATE) gate_run(b, r, false);
  else word_run(b, r, false, true, false);
}

void batch_tick_many(rrtl_batch* b, uint64_t steps, bool sync) {
  rrtl_run r{};
  r.cycles = steps;
  if (b->d->engine == RRTL_ENGINE_GATE) gate_run(b, r, !sync);
  else word_run(b, r, !sync, true, true);
  if (sync) check_err_word(b);
}

}  // namespace rrtl

// -------------------------------------------------------------------- C ABI --

extern "C" {

const char* rrtl_last_error(void) { return g_last_error.c_str(); }

rrtl_status rrtl_ctx_create(int32_t device, rrtl_ctx** out) {
  return guard([&] {
    REQUIRE(out, RRTL_E_ARG, "E_ARG: out is null");
    int n = 0;
    cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    REQUIRE(device >= 0 && device < n, RRTL_E_ARG, "E_ARG: no such device");
    auto* c = new rrtl_ctx;
    c->device = device;
    try {
      set_device(c);
      cuda_check(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
      int sms = 0, smem = 0, smem_sm = 0;
      cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "attr");
      cuda_check(cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "attr");
      cuda_check(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device), "attr");
      c->sm_count = (uint32_t)sms;
      c->max_smem = (size_t)smem;
      c->max_smem_sm = (size_t)smem_sm;
      for (auto& e : c->events) cuda_check(cudaEventCreate(&e), "event");
      cuda_check(noalloc_scratch_lookup(&c->noalloc_scratch), "noalloc scratch lookup");
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
  });
}

static void ctx_release(rrtl_ctx* ctx) {
  if (--ctx->refs > 0) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& e : ctx->events)
    if (e) cudaEventDestroy(e);
  ctx->queue.reset();
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

static void design_release(rrtl_design* d) {
  if (--d->refs > 0) return;
  rrtl_ctx* ctx = d->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete d;  // frees the device program while the context is still alive
  ctx_release(ctx);
}

rrtl_status rrtl_ctx_destroy(rrtl_ctx* ctx) {
  return guard([&] {
    if (!ctx) return;
    ctx_release(ctx);
  });
}

rrtl_status rrtl_ctx_sm_count(rrtl_ctx* ctx, uint32_t* out) {
  return guard([&] {
    REQUIRE(ctx && out, RRTL_E_ARG, "E_ARG: null argument");
    *out = ctx->sm_count;
  });
}

rrtl_status rrtl_ctx_event_record(rrtl_ctx* ctx, uint32_t slot) {
  return guard([&] {
    REQUIRE(ctx && slot < 8, RRTL_E_ARG, "E_ARG: bad event slot");
    set_device(ctx);
    cuda_check(cudaEventRecord(ctx->events[slot], ctx->stream), "cudaEventRecord");
  });
}

rrtl_status rrtl_ctx_event_elapsed(rrtl_ctx* ctx, uint32_t a, uint32_t b, float* ms) {
  return guard([&] {
    REQUIRE(ctx && a < 8 && b < 8 && ms, RRTL_E_ARG, "E_ARG: bad event slot");
    set_device(ctx);
    cuda_check(cudaEventSynchronize(ctx->events[b]), "cudaEventSynchronize");
    cuda_check(cudaEventElapsedTime(ms, ctx->events[a], ctx->events[b]), "cudaEventElapsedTime");
  });
}

rrtl_status rrtl_ctx_synchronize(rrtl_ctx* ctx) {
  return guard([&] {
    REQUIRE(ctx, RRTL_E_ARG, "E_ARG: null argument");
    set_device(ctx);
    cuda_check(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  });
}

rrtl_status rrtl_ctx_check_wait_timeout(rrtl_ctx* ctx, uint32_t polls, uint32_t* wait_status, uint32_t* completed) {
  return guard([&] {
    REQUIRE(ctx && wait_status && completed, RRTL_E_ARG, "E_ARG: null argument");
    REQUIRE(polls >= 1 && polls <= (1u << 22), RRTL_E_ARG, "E_ARG: polls must be in 1..2^22");
    set_device(ctx);
    DevBuf out;
    out.reserve(16);
    cuda_check(cudaMemsetAsync(out.p, 0xFF, 16, ctx->stream), "memset");
    cuda_check(launch_mbar_wait_check(polls, out.as<uint32_t>(), ctx->stream), "wait check launch");
    uint32_t h[2] = {0, 0};
    cuda_check(cudaMemcpyAsync(h, out.p, sizeof h, cudaMemcpyDeviceToHost, ctx->stream), "d2h wait check");
    cuda_check(cudaStreamSynchronize(ctx->stream), "sync");
    *wait_status = h[0];
    *completed = h[1];
  });
}

static void load_design(rrtl_ctx* ctx, Design design, const std::string& top, rrtl_design** out);

rrtl_status rrtl_design_load_json(rrtl_ctx* ctx, const char* json, size_t len, const char* top, rrtl_design** out) {
  return guard([&] {
    REQUIRE(ctx && json && top && out, RRTL_E_ARG, "E_ARG: null argument");
    set_device(ctx);
    load_design(ctx, design_from_json(json, len), top, out);
  });
}

rrtl_status rrtl_design_load_bitslice(rrtl_ctx* ctx, const char* json, size_t len, const char* top, rrtl_design** out) {
  return guard([&] {
    REQUIRE(ctx && json && top && out, RRTL_E_ARG, "E_ARG: null argument");
    set_device(ctx);
    Design planes;
    try {
      planes = bitslice_design(lower_to_packed_program(design_from_json(json, len), top));
    } catch (const RrtlError& e) {
      if (e.code == "E_BITSLICE") fail(RRTL_E_UNSUPPORTED, e.what());
      throw;
    }
    load_design(ctx, std::move(planes), top, out);
    if ((*out)->engine != RRTL_ENGINE_GATE) {
      rrtl_design_destroy(*out);
      *out = nullptr;
      fail(RRTL_E_UNSUPPORTED, "E_BITSLICE: the plane design is outside the gate engine");
    }
  });
}

rrtl_status rrtl_bitslice_json(const char* json, size_t len, const char* top, char* out, size_t cap, size_t* out_len) {
  return guard([&] {
    REQUIRE(json && top, RRTL_E_ARG, "E_ARG: null argument");
    std::string js;
    try {
      js = design_to_json(bitslice_design(lower_to_packed_program(design_from_json(json, len), top)));
    } catch (const RrtlError& e) {
      if (e.code == "E_BITSLICE") fail(RRTL_E_UNSUPPORTED, e.what());
      throw;
    }
    if (out_len) *out_len = js.size();
    if (out && cap) {
      const size_t n = std::min(cap - 1, js.size());
      memcpy(out, js.data(), n);
      out[n] = 0;
    }
  });
}

static void load_design(rrtl_ctx* ctx, Design design, const std::string& top, rrtl_design** out) {
  {
    auto d = std::make_unique<rrtl_design>();
    d->ctx = ctx;
    d->design = std::move(design);
    d->top = top;
    PackedProgram pp = lower_to_packed_program(d->design, top);
    d->mp = lower_to_machine_program(pp);
    bool gate = true;
    try {
      build_gate_variants(d.get());
    } catch (const RrtlError& e) {
      if (e.code != "E_GATE_SCOPE") throw;
      gate = false;
    }
    if (gate) {
      d->engine = RRTL_ENGINE_GATE;
    } else {
      d->engine = RRTL_ENGINE_WORD;
      d->wp = build_word_program(d->mp);
      upload_word_program(d.get());
    }
    ctx->refs++;
    *out = d.release();
  }
}

rrtl_status rrtl_design_destroy(rrtl_design* d) {
  return guard([&] {
    if (!d) return;
    design_release(d);
  });
}

rrtl_status rrtl_design_word_jit(rrtl_design* d, uint32_t* active, float* compile_ms) {
  std::string why;
  const rrtl_status st = guard([&] {
    REQUIRE(d && active, RRTL_E_ARG, "E_ARG: null argument");
    *active = 0;
    if (compile_ms) *compile_ms = 0.f;
    if (d->engine != RRTL_ENGINE_WORD) {
      why = "the design runs on the gate engine";
      return;
    }
    set_device(d->ctx);
    const JitKernel* J = word_jit_get(d);
    *active = J ? 1u : 0u;
    std::lock_guard<std::mutex> lk(d->wjit_mu);
    auto it = d->wjit_runs.find("general");
    const JitKernel* E = it != d->wjit_runs.end() && it->second->ready.load() ? it->second.get() : nullptr;
    if (compile_ms && E) *compile_ms = (float)E->compile_ms;
    if (!J) why = E ? E->error : std::string("compiled word kernels are off (RRTL_WORD_JIT=0) or still building");
  });
  if (st == RRTL_OK && !why.empty()) g_last_error = why;
  return st;
}

rrtl_status rrtl_word_jit_emit(const char* json, size_t len, const char* top, const rrtl_run* run, const char* arch,
                               char* source, size_t source_cap, size_t* source_len, uint32_t* cubin_bytes, char* log,
                               size_t log_cap, uint32_t flags) {
  return guard([&] {
    REQUIRE(json && top, RRTL_E_ARG, "E_ARG: null argument");
    if (cubin_bytes) *cubin_bytes = 0;
    if (log && log_cap) log[0] = 0;
    Design dz = design_from_json(json, len);
    MachineProgram mp = lower_to_machine_program(lower_to_packed_program(dz, top));
    WordProgram wp;
    try {
      wp = build_word_program(mp);
    } catch (const RrtlError& e) {
      fail(RRTL_E_UNSUPPORTED, e.what());
    }
    WordRunTables tabs;
    if (run) {
      const PackedProgram& P = mp.source;
      auto sig = [&](uint32_t i) -> const PackedSignal& {
        REQUIRE(i < P.signals.size(), RRTL_E_SIGNAL, "E_GPU_SIGNAL: signal index out of range");
        return P.signals[i];
      };
      for (uint32_t i = 0; i < run->n_stim; ++i) {
        const PackedSignal& ps = sig(run->stim[i].signal);
        tabs.stim.push_back(WordStimDev{ps.layout.offset, ps.layout.limbs, ps.layout.width, run->stim[i].kind,
                                        run->stim[i].param});
      }
      uint32_t base = 0;
      for (uint32_t i = 0; i < run->n_record; ++i) {
        const PackedSignal& ps = sig(run->record[i]);
        tabs.rec.push_back(WordRecDev{ps.layout.offset, ps.layout.limbs, ps.layout.width, base});
        base += ps.layout.limbs;
      }
      tabs.mode = run->record_mode;
    }
    WordSplitPlan plan;
    const bool split = run && (flags & RRTL_JIT_SPLIT);
    if (split) {
      std::string why;
      REQUIRE(word_split_plan(wp, tabs, &plan, &why), RRTL_E_UNSUPPORTED, "E_WORD_JIT_SPLIT: " + why);
    }
    const std::string src = word_jit_source(wp, run ? &tabs : nullptr, split ? &plan : nullptr);
    if (source_len) *source_len = src.size();
    if (source && source_cap) {
      const size_t n = std::min(source_cap - 1, src.size());
      memcpy(source, src.data(), n);
      source[n] = 0;
    }
    if (!arch) return;
    std::string lg;
    std::vector<char> cubin = word_jit_compile(src, arch, &lg);
    if (log && log_cap) {
      const size_t n = std::min(log_cap - 1, lg.size());
      memcpy(log, lg.data(), n);
      log[n] = 0;
    }
    REQUIRE(!cubin.empty(), RRTL_E_UNSUPPORTED, "E_WORD_JIT: " + lg.substr(0, 400));
    if (cubin_bytes) *cubin_bytes = (uint32_t)cubin.size();
  });
}

rrtl_status rrtl_gate_jit_emit(const char* json, size_t len, const char* top, const rrtl_run* run, const char* arch,
                               char* source, size_t source_cap, size_t* source_len, uint32_t* cubin_bytes, char* log,
                               size_t log_cap) {
  return guard([&] {
    REQUIRE(json && top && run, RRTL_E_ARG, "E_ARG: null argument");
    if (cubin_bytes) *cubin_bytes = 0;
    if (log && log_cap) log[0] = 0;
    Design dz = design_from_json(json, len);
    MachineProgram mp = lower_to_machine_program(lower_to_packed_program(dz, top));
    GateProgram gp;
    try {
      gp = build_gate_program(mp, 8);
    } catch (const RrtlError& e) {
      fail(RRTL_E_UNSUPPORTED, e.what());
    }
    GateRunTables tabs;
    for (uint32_t i = 0; i < run->n_stim; ++i) {
      REQUIRE(run->stim[i].signal < gp.n_signals, RRTL_E_SIGNAL, "E_GPU_SIGNAL: signal index out of range");
      tabs.stim.push_back(GateStimDev{0u, gp.signal_net[run->stim[i].signal], run->stim[i].kind, 0u, run->stim[i].param});
    }
    for (uint32_t i = 0; i < run->n_record; ++i) {
      REQUIRE(run->record[i] < gp.n_signals, RRTL_E_SIGNAL, "E_GPU_SIGNAL: signal index out of range");
      tabs.rec.push_back(GateRecDev{0u, gp.signal_net[run->record[i]]});
    }
    tabs.mode = run->record_mode;
    const std::string src = gate_jit_source(gp, tabs);
    if (source_len) *source_len = src.size();
    if (source && source_cap) {
      const size_t n = std::min(source_cap - 1, src.size());
      memcpy(source, src.data(), n);
      source[n] = 0;
    }
    if (!arch) return;
    std::string lg;
    std::vector<char> cubin = word_jit_compile(src, arch, &lg);
    if (log && log_cap) {
      const size_t n = std::min(log_cap - 1, lg.size());
      memcpy(log, lg.data(), n);
      log[n] = 0;
    }
    REQUIRE(!cubin.empty(), RRTL_E_UNSUPPORTED, "E_GATE_JIT: " + lg.substr(0, 400));
    if (cubin_bytes) *cubin_bytes = (uint32_t)cubin.size();
  });
}

rrtl_status rrtl_gate_program_info_get(const char* json, size_t len, const char* top, uint32_t tile_words,
                                       rrtl_gate_program_info* out) {
  return guard([&] {
    REQUIRE(json && top && out, RRTL_E_ARG, "E_ARG: null argument");
    REQUIRE(tile_words == 1 || tile_words == 2 || tile_words == 4 || tile_words == 8, RRTL_E_ARG,
            "E_ARG: tile width must be 1, 2, 4 or 8 words");
    Design dz = design_from_json(json, len);
    MachineProgram mp = lower_to_machine_program(lower_to_packed_program(dz, top));
    GateProgram gp;
    try {
      gp = build_gate_program(mp, tile_words);
    } catch (const RrtlError& e) {
      fail(RRTL_E_UNSUPPORTED, e.what());
    }
    rrtl_gate_program_info I{};
    const uint32_t G = gp.group;
    I.tile_words = tile_words;
    I.group = G;
    I.levels = gp.n_levels;
    I.slots = gp.n_slots;
    std::vector<uint8_t> seen(256, 0);
    // largest number of distinct rows that share a bank residue among `rows`
    auto wavefronts = [&](std::vector<uint32_t>& rows) {
      std::sort(rows.begin(), rows.end());
      rows.erase(std::unique(rows.begin(), rows.end()), rows.end());
      std::vector<uint32_t> per(G, 0);
      uint32_t mx = 0;
      for (uint32_t r : rows) mx = std::max(mx, ++per[r % G]);
      return mx;
    };
    std::vector<uint32_t> rows;
    const int32_t c0 = gp.net_slot[kNetConst0];
    for (size_t g = 0; g + G <= gp.cells.size(); g += G) {
      const uint8_t lut = gp.cells[g].lut;
      seen[lut] = 1;
      ++I.groups;
      const bool use[3] = {(lut & 0x0F) != ((lut >> 4) & 0x0F), (lut & 0x33) != ((lut >> 2) & 0x33),
                           (lut & 0x55) != ((lut >> 1) & 0x55)};
      for (int p = 0; p < 3; ++p) {
        if (!use[p]) continue;
        rows.clear();
        for (uint32_t k = 0; k < G; ++k) {
          const GateCell& c = gp.cells[g + k];
          rows.push_back((uint32_t)(c.pad ? c0 : gp.net_slot[c.in[p]]));
        }
        I.operand_wavefronts += wavefronts(rows);
        I.operand_rows += 1;
      }
      for (uint32_t k = 0; k < G; ++k) {
        if (gp.cells[g + k].pad) ++I.pad_cells;
        else ++I.cells;
      }
    }
    for (int l = 0; l < 256; ++l) I.classes += seen[l];
    const std::vector<uint32_t> ord = commit_order(gp);
    for (size_t i = 0; i < ord.size(); i += G) {
      rows.clear();
      for (size_t k = i; k < std::min(ord.size(), i + G); ++k) rows.push_back((uint32_t)gp.net_slot[gp.regs[ord[k]].d_net]);
      I.commit_wavefronts += wavefronts(rows);
      ++I.commit_groups;
    }
    *out = I;
  });
}

rrtl_status rrtl_gate_fused_jit_emit(const char* json, size_t len, const char* top, uint32_t tile_words,
                                     const char* arch, char* source, size_t source_cap, size_t* source_len,
                                     uint32_t* cubin_bytes, char* log, size_t log_cap) {
  return guard([&] {
    REQUIRE(json && top, RRTL_E_ARG, "E_ARG: null argument");
    REQUIRE(tile_words == 1 || tile_words == 2 || tile_words == 4 || tile_words == 8, RRTL_E_ARG,
            "E_ARG: tile width must be 1, 2, 4 or 8 words");
    if (cubin_bytes) *cubin_bytes = 0;
    if (log && log_cap) log[0] = 0;
    Design dz = design_from_json(json, len);
    MachineProgram mp = lower_to_machine_program(lower_to_packed_program(dz, top));
    GateProgram gp;
    try {
      gp = build_gate_program(mp, tile_words);
    } catch (const RrtlError& e) {
      fail(RRTL_E_UNSUPPORTED, e.what());
    }
    const std::string src = gate_fused_jit_source(gp);
    if (source_len) *source_len = src.size();
    if (source && source_cap) {
      const size_t n = std::min(source_cap - 1, src.size());
      memcpy(source, src.data(), n);
      source[n] = 0;
    }
    if (!arch) return;
    std::string lg;
    std::vector<char> cubin = word_jit_compile(src, arch, &lg);
    if (log && log_cap) {
      const size_t n = std::min(log_cap - 1, lg.size());
      memcpy(log, lg.data(), n);
      log[n] = 0;
    }
    REQUIRE(!cubin.empty(), RRTL_E_UNSUPPORTED, "E_GATE_JIT: " + lg.substr(0, 400));
    if (cubin_bytes) *cubin_bytes = (uint32_t)cubin.size();
  });
}

rrtl_status rrtl_instance_fold_plan(const char* json, size_t len, const char* top, char* plan, size_t cap,
                                    size_t* plan_len) {
  return guard([&] {
    REQUIRE(json && top, RRTL_E_ARG, "E_ARG: null argument");
    Design dz = design_from_json(json, len);
    std::string why;
    auto f = analyze_instance_fold(dz, top, &why);
    REQUIRE(f.has_value(), RRTL_E_UNSUPPORTED, "E_INSTANCE_FOLD: " + why);
    const std::string js = instance_fold_json(*f);
    if (plan_len) *plan_len = js.size();
    if (plan && cap) {
      const size_t n = std::min(cap - 1, js.size());
      memcpy(plan, js.data(), n);
      plan[n] = 0;
    }
  });
}

rrtl_status rrtl_design_info_get(rrtl_design* d, rrtl_design_info* out) {
  return guard([&] {
    REQUIRE(d && out, RRTL_E_ARG, "E_ARG: null argument");
    rrtl_design_info i{};
    const PackedProgram& P = d->mp.source;
    i.n_signals = (uint32_t)P.signals.size();
    i.n_memories = (uint32_t)P.memories.size();
    i.total_signal_words = P.total_signal_words;
    i.total_memory_words_per_lane = P.total_memory_words_per_lane;
    i.engine = d->engine;
    if (d->engine == RRTL_ENGINE_GATE) {
      const GateProgram& gp = d->gp();
      i.n_gates = gp.n_real_cells;
      i.n_levels = gp.n_levels;
      i.n_nets = gp.n_nets;
      i.n_slots = d->gate_w_max ? gp.n_slots : 0;
      i.n_regs = (uint32_t)gp.regs.size();
      i.source_instrs = gp.source_instrs;
    } else {
      i.n_gates = (uint32_t)d->wp.code.size();
      i.n_levels = (uint32_t)d->mp.comb.packets.size();
      i.n_slots = d->wp.n_vslots;
      i.n_regs = (uint32_t)d->wp.commits.size();
      i.source_instrs = d->wp.source_instrs;
    }
    *out = i;
  });
}

rrtl_status rrtl_design_signal(rrtl_design* d, const char* name, uint32_t* index, uint32_t* width, uint32_t* kind) {
  return guard([&] {
    REQUIRE(d && name, RRTL_E_ARG, "E_ARG: null argument");
    std::string full = d->top + "." + name;
    const auto& S = d->mp.source.signals;
    for (size_t i = 0; i < S.size(); ++i)
      if (S[i].name == name || S[i].name == full) {
        if (index) *index = (uint32_t)i;
        if (width) *width = S[i].layout.width;
        if (kind) *kind = (uint32_t)S[i].kind;
        return;
      }
    fail(RRTL_E_SIGNAL, std::string("E_GPU_SIGNAL: no signal `") + name + "`");
  });
}

rrtl_status rrtl_design_memory(rrtl_design* d, const char* name, uint32_t* index, uint64_t* depth, uint32_t* width) {
  return guard([&] {
    REQUIRE(d && name, RRTL_E_ARG, "E_ARG: null argument");
    std::string full = d->top + "." + name;
    const auto& M = d->mp.source.memories;
    for (size_t i = 0; i < M.size(); ++i)
      if (M[i].name == name || M[i].name == full) {
        if (index) *index = (uint32_t)i;
        if (depth) *depth = M[i].depth;
        if (width) *width = M[i].data_layout.width;
        return;
      }
    fail(RRTL_E_SIGNAL, std::string("E_GPU_MEMORY: no memory `") + name + "`");
  });
}

rrtl_status rrtl_batch_create(rrtl_design* d, uint32_t lanes, rrtl_batch** out) {
  return guard([&] {
    REQUIRE(d && out, RRTL_E_ARG, "E_ARG: null argument");
    REQUIRE(lanes > 0, RRTL_E_LANES, "E_GPU_LANES: GPU simulator requires at least one lane");
    REQUIRE(lanes <= (1u << 30), RRTL_E_LANES, "E_GPU_LANES: too many lanes");
    set_device(d->ctx);
    auto b = std::make_unique<rrtl_batch>();
    b->d = d;
    b->lanes = lanes;
    cuda_check(cudaEventCreate(&b->ev0), "event");
    cuda_check(cudaEventCreate(&b->ev1), "event");
    b->d_err.reserve(16);
    cuda_check(cudaMemset(b->d_err.p, 0, 16), "memset");
    if (d->engine == RRTL_ENGINE_GATE) {
      b->words = (lanes + 31) / 32;
      b->words_pad = round_up(b->words, kPadWords);
      b->rows = d->gp().n_nets + 1;
      size_t bytes = (size_t)b->rows * b->words_pad * 4;
      b->d_nets.reserve(bytes);
      cuda_check(cudaMemset(b->d_nets.p, 0, bytes), "memset nets");
      cuda_check(cudaMemset(b->d_nets.as<uint8_t>() + (size_t)kNetConst1 * b->words_pad * 4, 0xFF, (size_t)b->words_pad * 4),
                 "memset const1");
    } else {
      b->lanes_pad = round_up(lanes, kWordThreads);
      const PackedProgram& P = d->mp.source;
      size_t vb = std::max<size_t>((size_t)P.total_signal_words * b->lanes_pad * 4, 16);
      size_t mb = std::max<size_t>((size_t)P.total_memory_words_per_lane * b->lanes_pad * 4, 16);
      size_t cb = std::max<size_t>((size_t)d->wp.total_capture_words * b->lanes_pad * 4, 16);
      b->d_values.reserve(vb);
      b->d_mem.reserve(mb);
      b->d_caps.reserve(cb);
      cuda_check(cudaMemset(b->d_values.p, 0, vb), "memset");
      cuda_check(cudaMemset(b->d_mem.p, 0, mb), "memset");
    }
    batch_eval(b.get());
    d->refs++;
    *out = b.release();
  });
}

rrtl_status rrtl_batch_destroy(rrtl_batch* b) {
  return guard([&] {
    if (!b) return;
    rrtl_design* d = b->d;
    cudaSetDevice(d->ctx->device);
    cudaStreamSynchronize(d->ctx->stream);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    delete b;
    design_release(d);
  });
}

rrtl_status rrtl_batch_lanes(rrtl_batch* b, uint32_t* out) {
  return guard([&] {
    REQUIRE(b && out, RRTL_E_ARG, "E_ARG: null argument");
    *out = b->lanes;
  });
}

static void gate_set_bits(rrtl_batch* b, uint32_t signal, const uint32_t* words) {
  uint32_t net = b->d->gp().signal_net[signal];
  std::vector<uint32_t> row(b->words_pad, 0);
  for (uint32_t w = 0; w < b->words; ++w) {
    uint32_t valid = b->lanes - w * 32;
    row[w] = valid >= 32 ? words[w] : (words[w] & ((1u << valid) - 1u));
  }
  cuda_check(cudaMemcpyAsync(b->d_nets.as<uint32_t>() + (size_t)net * b->words_pad, row.data(), (size_t)b->words_pad * 4,
                             cudaMemcpyHostToDevice, b->d->ctx->stream),
             "h2d signal");
  cuda_check(cudaStreamSynchronize(b->d->ctx->stream), "sync");
}

static void gate_get_bits(rrtl_batch* b, uint32_t signal, uint32_t* words) {
  uint32_t net = b->d->gp().signal_net[signal];
  cuda_check(cudaMemcpyAsync(words, b->d_nets.as<uint32_t>() + (size_t)net * b->words_pad, (size_t)b->words * 4,
                             cudaMemcpyDeviceToHost, b->d->ctx->stream),
             "d2h signal");
  cuda_check(cudaStreamSynchronize(b->d->ctx->stream), "sync");
  uint32_t valid = b->lanes - (b->words - 1) * 32;
  if (valid < 32) words[b->words - 1] &= (1u << valid) - 1u;
}

rrtl_status rrtl_batch_set_input_limbs(rrtl_batch* b, uint32_t signal, const uint32_t* data, size_t n) {
  return guard([&] {
    REQUIRE(b && data, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    const PackedSignal& ps = signal_of(b->d, signal);
    REQUIRE(n == (size_t)ps.layout.limbs * b->lanes, RRTL_E_ARG,
            "E_GPU_LANE_VALUES: expected " + std::to_string((size_t)ps.layout.limbs * b->lanes) + " values, got " + std::to_string(n));
    if (b->d->engine == RRTL_ENGINE_GATE) {
      std::vector<uint32_t> words(b->words, 0);
      for (uint32_t l = 0; l < b->lanes; ++l)
        if (data[l] & 1u) words[l / 32] |= 1u << (l % 32);
      gate_set_bits(b, signal, words.data());
    } else {
      uint32_t limbs = ps.layout.limbs;
      std::vector<uint32_t> rows((size_t)limbs * b->lanes_pad, 0);
      for (uint32_t k = 0; k < limbs; ++k)
        for (uint32_t l = 0; l < b->lanes; ++l) {
          uint32_t v = data[(size_t)k * b->lanes + l];
          if (k + 1 == limbs) v &= final_limb_mask(ps.layout.width);
          rows[(size_t)k * b->lanes_pad + l] = v;
        }
      cuda_check(cudaMemcpyAsync(b->d_values.as<uint32_t>() + (size_t)ps.layout.offset * b->lanes_pad, rows.data(),
                                 rows.size() * 4, cudaMemcpyHostToDevice, b->d->ctx->stream),
                 "h2d signal");
      cuda_check(cudaStreamSynchronize(b->d->ctx->stream), "sync");
    }
  });
}

rrtl_status rrtl_batch_get_signal_limbs(rrtl_batch* b, uint32_t signal, uint32_t* out, size_t n) {
  return guard([&] {
    REQUIRE(b && out, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    const PackedSignal& ps = signal_of(b->d, signal);
    REQUIRE(n == (size_t)ps.layout.limbs * b->lanes, RRTL_E_ARG, "E_GPU_LANE_VALUES: output size mismatch");
    check_err_word(b);
    if (b->d->engine == RRTL_ENGINE_GATE) {
      std::vector<uint32_t> words(b->words);
      gate_get_bits(b, signal, words.data());
      for (uint32_t l = 0; l < b->lanes; ++l) out[l] = (words[l / 32] >> (l % 32)) & 1u;
    } else {
      uint32_t limbs = ps.layout.limbs;
      std::vector<uint32_t> rows((size_t)limbs * b->lanes_pad);
      cuda_check(cudaMemcpyAsync(rows.data(), b->d_values.as<uint32_t>() + (size_t)ps.layout.offset * b->lanes_pad,
                                 rows.size() * 4, cudaMemcpyDeviceToHost, b->d->ctx->stream),
                 "d2h signal");
      cuda_check(cudaStreamSynchronize(b->d->ctx->stream), "sync");
      for (uint32_t k = 0; k < limbs; ++k)
        for (uint32_t l = 0; l < b->lanes; ++l) {
          uint32_t v = rows[(size_t)k * b->lanes_pad + l];
          if (k + 1 == limbs) v &= final_limb_mask(ps.layout.width);
          out[(size_t)k * b->lanes + l] = v;
        }
    }
  });
}

rrtl_status rrtl_batch_set_input_bits(rrtl_batch* b, uint32_t signal, const uint32_t* words, size_t n) {
  return guard([&] {
    REQUIRE(b && words, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    const PackedSignal& ps = signal_of(b->d, signal);
    REQUIRE(ps.layout.width == 1, RRTL_E_ARG, "E_GPU_WIDE_SIGNAL: bit-packed access needs a 1-bit signal");
    REQUIRE(n == (b->lanes + 31) / 32, RRTL_E_ARG, "E_GPU_LANE_VALUES: expected ceil(lanes/32) words");
    if (b->d->engine == RRTL_ENGINE_GATE) {
      gate_set_bits(b, signal, words);
    } else {
      std::vector<uint32_t> v(b->lanes);
      for (uint32_t l = 0; l < b->lanes; ++l) v[l] = (words[l / 32] >> (l % 32)) & 1u;
      rrtl_status st = rrtl_batch_set_input_limbs(b, signal, v.data(), v.size());
      if (st) fail(st, g_last_error);
    }
  });
}

rrtl_status rrtl_batch_get_signal_bits(rrtl_batch* b, uint32_t signal, uint32_t* out, size_t n) {
  return guard([&] {
    REQUIRE(b && out, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    const PackedSignal& ps = signal_of(b->d, signal);
    REQUIRE(ps.layout.width == 1, RRTL_E_ARG, "E_GPU_WIDE_SIGNAL: bit-packed access needs a 1-bit signal");
    REQUIRE(n == (b->lanes + 31) / 32, RRTL_E_ARG, "E_GPU_LANE_VALUES: expected ceil(lanes/32) words");
    check_err_word(b);
    if (b->d->engine == RRTL_ENGINE_GATE) {
      gate_get_bits(b, signal, out);
    } else {
      std::vector<uint32_t> v(b->lanes);
      rrtl_status st = rrtl_batch_get_signal_limbs(b, signal, v.data(), v.size());
      if (st) fail(st, g_last_error);
      memset(out, 0, n * 4);
      for (uint32_t l = 0; l < b->lanes; ++l) out[l / 32] |= (v[l] & 1u) << (l % 32);
    }
  });
}

rrtl_status rrtl_batch_get_signals_bits(rrtl_batch* b, const uint32_t* signals, size_t n, uint32_t* out, size_t n_out) {
  return guard([&] {
    REQUIRE(b && (signals || n == 0) && (out || n == 0), RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    uint32_t words = (b->lanes + 31) / 32;
    REQUIRE(n_out == n * words, RRTL_E_ARG, "E_GPU_LANE_VALUES: expected n*ceil(lanes/32) words");
    for (size_t i = 0; i < n; ++i)
      REQUIRE(signal_of(b->d, signals[i]).layout.width == 1, RRTL_E_ARG, "E_GPU_WIDE_SIGNAL: bit-packed access needs 1-bit signals");
    check_err_word(b);
    if (b->d->engine == RRTL_ENGINE_GATE) {
      cudaStream_t st = b->d->ctx->stream;
      // one 2-D copy per run of consecutive net rows
      for (size_t i = 0; i < n;) {
        uint32_t net = b->d->gp().signal_net[signals[i]];
        size_t j = i + 1;
        while (j < n && b->d->gp().signal_net[signals[j]] == net + (j - i)) ++j;
        cuda_check(cudaMemcpy2DAsync(out + i * words, (size_t)words * 4, b->d_nets.as<uint32_t>() + (size_t)net * b->words_pad,
                                     (size_t)b->words_pad * 4, (size_t)words * 4, j - i, cudaMemcpyDeviceToHost, st),
                   "d2h signals");
        i = j;
      }
      cuda_check(cudaStreamSynchronize(st), "sync");
      uint32_t valid = b->lanes - (words - 1) * 32;
      if (valid < 32)
        for (size_t i = 0; i < n; ++i) out[i * words + words - 1] &= (1u << valid) - 1u;
    } else {
      for (size_t i = 0; i < n; ++i) {
        rrtl_status stt = rrtl_batch_get_signal_bits(b, signals[i], out + i * words, words);
        if (stt) fail(stt, g_last_error);
      }
    }
  });
}

rrtl_status rrtl_batch_set_memory_limbs(rrtl_batch* b, uint32_t memory, const uint32_t* data, size_t n) {
  return guard([&] {
    REQUIRE(b && data, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    const auto& M = b->d->mp.source.memories;
    REQUIRE(memory < M.size(), RRTL_E_SIGNAL, "E_GPU_MEMORY: memory index out of range");
    REQUIRE(b->d->engine == RRTL_ENGINE_WORD, RRTL_E_UNSUPPORTED, "E_GPU_MEMORY: engine has no memories");
    const PackedMemory& m = M[memory];
    uint32_t limbs = m.data_layout.limbs;
    size_t words = (size_t)m.depth * limbs;
    REQUIRE(n == words * b->lanes, RRTL_E_ARG, "E_GPU_MEMORY_VALUES: expected depth*limbs*lanes values");
    std::vector<uint32_t> rows(words * b->lanes_pad, 0);
    for (size_t wv = 0; wv < words; ++wv)
      for (uint32_t l = 0; l < b->lanes; ++l) {
        uint32_t v = data[wv * b->lanes + l];
        if (wv % limbs == limbs - 1) v &= final_limb_mask(m.data_layout.width);
        rows[wv * b->lanes_pad + l] = v;
      }
    cuda_check(cudaMemcpyAsync(b->d_mem.as<uint32_t>() + (size_t)m.offset * b->lanes_pad, rows.data(), rows.size() * 4,
                               cudaMemcpyHostToDevice, b->d->ctx->stream),
               "h2d memory");
    cuda_check(cudaStreamSynchronize(b->d->ctx->stream), "sync");
  });
}

rrtl_status rrtl_batch_get_memory_limbs(rrtl_batch* b, uint32_t memory, uint32_t* out, size_t n) {
  return guard([&] {
    REQUIRE(b && out, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    const auto& M = b->d->mp.source.memories;
    REQUIRE(memory < M.size(), RRTL_E_SIGNAL, "E_GPU_MEMORY: memory index out of range");
    REQUIRE(b->d->engine == RRTL_ENGINE_WORD, RRTL_E_UNSUPPORTED, "E_GPU_MEMORY: engine has no memories");
    const PackedMemory& m = M[memory];
    uint32_t limbs = m.data_layout.limbs;
    size_t words = (size_t)m.depth * limbs;
    REQUIRE(n == words * b->lanes, RRTL_E_ARG, "E_GPU_MEMORY_VALUES: expected depth*limbs*lanes values");
    check_err_word(b);
    std::vector<uint32_t> rows(words * b->lanes_pad);
    cuda_check(cudaMemcpyAsync(rows.data(), b->d_mem.as<uint32_t>() + (size_t)m.offset * b->lanes_pad, rows.size() * 4,
                               cudaMemcpyDeviceToHost, b->d->ctx->stream),
               "d2h memory");
    cuda_check(cudaStreamSynchronize(b->d->ctx->stream), "sync");
    for (size_t wv = 0; wv < words; ++wv)
      for (uint32_t l = 0; l < b->lanes; ++l) {
        uint32_t v = rows[wv * b->lanes_pad + l];
        if (wv % limbs == limbs - 1) v &= final_limb_mask(m.data_layout.width);
        out[wv * b->lanes + l] = v;
      }
  });
}

rrtl_status rrtl_batch_eval(rrtl_batch* b) {
  return guard([&] {
    REQUIRE(b, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    batch_eval(b);
  });
}

rrtl_status rrtl_batch_tick(rrtl_batch* b) {
  return guard([&] {
    REQUIRE(b, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    batch_tick_many(b, 1, true);
  });
}

rrtl_status rrtl_batch_tick_many(rrtl_batch* b, uint64_t steps) {
  return guard([&] {
    REQUIRE(b, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    REQUIRE(steps < (1ull << 32), RRTL_E_ARG, "E_GPU_STEPS: tick_many step count exceeds 2^32");
    if (steps == 0) return;
    batch_tick_many(b, steps, false);
  });
}

rrtl_status rrtl_batch_synchronize(rrtl_batch* b) {
  return guard([&] {
    REQUIRE(b, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    check_err_word(b);
    cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
  });
}

rrtl_status rrtl_batch_run(rrtl_batch* b, const rrtl_run* run) {
  return guard([&] {
    REQUIRE(b && run, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    REQUIRE(run->n_stim == 0 || run->stim, RRTL_E_ARG, "E_ARG: stim is null");
    REQUIRE(run->n_record == 0 || run->record, RRTL_E_ARG, "E_ARG: record is null");
    if (b->d->engine == RRTL_ENGINE_GATE) gate_run(b, *run, false);
    else word_run(b, *run, false, false, true);
  });
}

rrtl_status rrtl_batch_run_device(rrtl_batch* b, const rrtl_run* run) {
  return guard([&] {
    REQUIRE(b && run, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    REQUIRE(run->n_stim == 0 || run->stim, RRTL_E_ARG, "E_ARG: stim is null");
    REQUIRE(run->n_record == 0 || run->record, RRTL_E_ARG, "E_ARG: record is null");
    if (b->d->engine == RRTL_ENGINE_GATE) gate_run(b, *run, true);
    else word_run(b, *run, true, false, true);
  });
}

rrtl_status rrtl_batch_replay_trace(rrtl_batch* b, const rrtl_trace* trace, uint32_t max_mismatches, uint32_t* log,
                                    uint64_t* n_mismatches) {
  return guard([&] {
    REQUIRE(b && trace, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    const uint64_t n = batch_replay(b, *trace, std::max<uint32_t>(max_mismatches, 1), log);
    if (n_mismatches) *n_mismatches = n;
  });
}

rrtl_status rrtl_batch_set_faults(rrtl_batch* b, const rrtl_fault* faults, size_t n) {
  return guard([&] {
    REQUIRE(b && (faults || n == 0), RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    REQUIRE(b->d->engine == RRTL_ENGINE_GATE, RRTL_E_UNSUPPORTED, "E_FAULT: fault injection needs the gate engine");
    const GateProgram& gp = b->d->gp();
    for (size_t i = 0; i < n; ++i) {
      const rrtl_fault& f = faults[i];
      REQUIRE(f.lane < b->lanes, RRTL_E_ARG, "E_FAULT_LANE: lane out of range");
      REQUIRE(f.lane % 32 != 0, RRTL_E_ARG, "E_FAULT_LANE: lane 0 of each 32-lane word is the fault-free reference");
      const PackedSignal& ps = signal_of(b->d, f.signal);
      REQUIRE(ps.kind != PSK::Input, RRTL_E_ARG, "E_FAULT_NET: stuck-at faults go on wires, outputs or registers");
      uint32_t net = gp.signal_net[f.signal];
      REQUIRE(!gp.net_is_source[net] || ps.kind == PSK::Reg, RRTL_E_ARG, "E_FAULT_NET: undriven signal");
      REQUIRE(f.value <= 1, RRTL_E_ARG, "E_FAULT: stuck-at value must be 0 or 1");
    }
    b->faults.assign(faults, faults + n);
    invalidate_forces(b);
  });
}

rrtl_status rrtl_batch_snapshot(rrtl_batch* b, uint32_t* values, size_t nv, uint32_t* memories, size_t nm) {
  return guard([&] {
    REQUIRE(b, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    const PackedProgram& P = b->d->mp.source;
    REQUIRE(nv == (size_t)P.total_signal_words * b->lanes, RRTL_E_ARG, "E_SIM_IR_STORAGE_VALUES: size mismatch");
    REQUIRE(nm == (size_t)P.total_memory_words_per_lane * b->lanes, RRTL_E_ARG, "E_SIM_IR_STORAGE_MEMORIES: size mismatch");
    check_err_word(b);
    if (b->d->engine == RRTL_ENGINE_GATE) {
      std::vector<uint32_t> words(b->words);
      for (uint32_t s = 0; s < P.signals.size(); ++s) {
        gate_get_bits(b, s, words.data());
        for (uint32_t l = 0; l < b->lanes; ++l) values[(size_t)P.signals[s].layout.offset * b->lanes + l] = (words[l / 32] >> (l % 32)) & 1u;
      }
    } else {
      std::vector<uint32_t> rows((size_t)P.total_signal_words * b->lanes_pad);
      cuda_check(cudaMemcpy(rows.data(), b->d_values.p, rows.size() * 4, cudaMemcpyDeviceToHost), "d2h");
      for (size_t wv = 0; wv < P.total_signal_words; ++wv)
        for (uint32_t l = 0; l < b->lanes; ++l) values[wv * b->lanes + l] = rows[wv * b->lanes_pad + l];
      if (nm) {
        std::vector<uint32_t> mrows((size_t)P.total_memory_words_per_lane * b->lanes_pad);
        cuda_check(cudaMemcpy(mrows.data(), b->d_mem.p, mrows.size() * 4, cudaMemcpyDeviceToHost), "d2h");
        for (size_t wv = 0; wv < P.total_memory_words_per_lane; ++wv)
          for (uint32_t l = 0; l < b->lanes; ++l)
            memories[(size_t)l * P.total_memory_words_per_lane + wv] = mrows[wv * b->lanes_pad + l];
      }
    }
  });
}

rrtl_status rrtl_batch_restore(rrtl_batch* b, const uint32_t* values, size_t nv, const uint32_t* memories, size_t nm) {
  return guard([&] {
    REQUIRE(b, RRTL_E_ARG, "E_ARG: null argument");
    set_device(b->d->ctx);
    const PackedProgram& P = b->d->mp.source;
    REQUIRE(nv == (size_t)P.total_signal_words * b->lanes, RRTL_E_ARG, "E_SIM_IR_STORAGE_VALUES: size mismatch");
    REQUIRE(nm == (size_t)P.total_memory_words_per_lane * b->lanes, RRTL_E_ARG, "E_SIM_IR_STORAGE_MEMORIES: size mismatch");
    if (b->d->engine == RRTL_ENGINE_GATE) {
      std::vector<uint32_t> words(b->words);
      for (uint32_t s = 0; s < P.signals.size(); ++s) {
        std::fill(words.begin(), words.end(), 0u);
        for (uint32_t l = 0; l < b->lanes; ++l)
          if (values[(size_t)P.signals[s].layout.offset * b->lanes + l] & 1u) words[l / 32] |= 1u << (l % 32);
        gate_set_bits(b, s, words.data());
      }
    } else {
      std::vector<uint32_t> rows((size_t)P.total_signal_words * b->lanes_pad, 0);
      for (size_t wv = 0; wv < P.total_signal_words; ++wv)
        for (uint32_t l = 0; l < b->lanes; ++l) rows[wv * b->lanes_pad + l] = values[wv * b->lanes + l];
      cuda_check(cudaMemcpy(b->d_values.p, rows.data(), rows.size() * 4, cudaMemcpyHostToDevice), "h2d");
      if (nm) {
        std::vector<uint32_t> mrows((size_t)P.total_memory_words_per_lane * b->lanes_pad, 0);
        for (size_t wv = 0; wv < P.total_memory_words_per_lane; ++wv)
          for (uint32_t l = 0; l < b->lanes; ++l)
            mrows[wv * b->lanes_pad + l] = memories[(size_t)l * P.total_memory_words_per_lane + wv];
        cuda_check(cudaMemcpy(b->d_mem.p, mrows.data(), mrows.size() * 4, cudaMemcpyHostToDevice), "h2d");
      }
    }
  });
}

rrtl_status rrtl_batch_set_path(rrtl_batch* b, uint32_t path) {
  return guard([&] {
    REQUIRE(b, RRTL_E_ARG, "E_ARG: null argument");
    REQUIRE(path <= RRTL_PATH_WORD_INTERP, RRTL_E_ARG, "E_ARG: unknown path");
    b->path = path == RRTL_PATH_WORD_INTERP && b->d->engine == RRTL_ENGINE_GATE ? (uint32_t)RRTL_PATH_FUSED : path;
  });
}

rrtl_status rrtl_queue_submit(rrtl_ctx* ctx, const rrtl_job* job, uint64_t* id) {
  return guard([&] {
    REQUIRE(ctx && job && id, RRTL_E_ARG, "E_ARG: null argument");
    set_device(ctx);
    *id = queue_submit(ctx, *job);
  });
}

rrtl_status rrtl_queue_launch(rrtl_ctx* ctx) {
  return guard([&] {
    REQUIRE(ctx, RRTL_E_ARG, "E_ARG: null argument");
    set_device(ctx);
    queue_launch(ctx);
  });
}

rrtl_status rrtl_queue_wait(rrtl_ctx* ctx) {
  return guard([&] {
    REQUIRE(ctx, RRTL_E_ARG, "E_ARG: null argument");
    set_device(ctx);
    JobQueue& Q = queue_of(ctx);
    cuda_check(cudaStreamSynchronize(ctx->stream), "sync");
    cuda_check(cudaEventElapsedTime(&Q.last_ms, Q.ev0, Q.ev1), "elapsed");
    queue_finish(ctx);
  });
}

rrtl_status rrtl_queue_poll(rrtl_ctx* ctx, uint64_t id, uint32_t* status) {
  return guard([&] {
    REQUIRE(ctx && status, RRTL_E_ARG, "E_ARG: null argument");
    set_device(ctx);
    JobQueue& Q = queue_of(ctx);
    auto it = Q.finished.find(id);
    if (it != Q.finished.end()) {
      *status = it->second;
      return;
    }
    for (QueueJob& j : Q.jobs)
      if (j.id == id) {
        if (j.status == RRTL_JOB_RUNNING && cudaEventQuery(Q.ev1) == cudaSuccess) {
          cuda_check(cudaStreamSynchronize(ctx->stream), "sync");
          cudaEventElapsedTime(&Q.last_ms, Q.ev0, Q.ev1);
          queue_finish(ctx);
          *status = Q.finished.at(id);
        } else {
          *status = j.status;
        }
        return;
      }
    fail(RRTL_E_ARG, "E_QUEUE: unknown job id");
  });
}

rrtl_status rrtl_queue_last_ms(rrtl_ctx* ctx, float* ms) {
  return guard([&] {
    REQUIRE(ctx && ms, RRTL_E_ARG, "E_ARG: null argument");
    *ms = queue_of(ctx).last_ms;
  });
}

// Measured tile-width choice: time `cycles` cycles of a scratch batch of
// `lanes` lanes (every input random) at each width whose slots fit on chip,
// keep the fastest for batches of this size (lane bucket = ceil(log2 words)).
rrtl_status rrtl_design_autotune(rrtl_design* d, uint32_t lanes, uint32_t cycles, uint32_t* best_words, float* best_ms) {
  return guard([&] {
    REQUIRE(d, RRTL_E_ARG, "E_ARG: null argument");
    REQUIRE(lanes > 0, RRTL_E_LANES, "E_GPU_AUTOTUNE_LANES: autotuning needs at least one lane");
    REQUIRE(cycles > 0, RRTL_E_ARG, "E_GPU_AUTOTUNE_STEPS: autotuning needs at least one cycle");
    set_device(d->ctx);
    if (d->engine != RRTL_ENGINE_GATE || !d->gate_w_max) {
      if (best_words) *best_words = 0;
      if (best_ms) *best_ms = 0.f;
      return;
    }
    const GateProgram& gp = d->gp();
    std::vector<rrtl_stim> stim;
    for (uint32_t sig = 0; sig < gp.n_signals; ++sig)
      if (d->mp.source.signals[sig].kind == PSK::Input) stim.push_back(rrtl_stim{sig, RRTL_STIM_RANDOM, sig});
    rrtl_run run{};
    run.cycles = cycles;
    run.seed = 1;
    run.n_stim = (uint32_t)stim.size();
    run.stim = stim.data();
    const uint32_t words = (lanes + 31) / 32;
    uint32_t best = d->gate_w_max;
    float best_t = INFINITY;
    d->tuned_w.erase(lane_bucket(words));
    for (uint32_t W = d->gate_w_max; W >= 1; W /= 2) {
      if (!gate_variant(d, W)->fused_ok) continue;
      rrtl_batch* b = nullptr;
      rrtl_status st = rrtl_batch_create(d, lanes, &b);
      if (st) fail(st, g_last_error);
      b->tile_words = W;
      float t = INFINITY;
      try {
        for (int rep = 0; rep < 3; ++rep) {
          gate_run(b, run, false);
          if (rep) t = std::min(t, b->last_ms);
        }
      } catch (...) {
        rrtl_batch_destroy(b);
        throw;
      }
      rrtl_batch_destroy(b);
      if (t < best_t) {
        best_t = t;
        best = W;
      }
    }
    // the compiled gate kernel, when the design qualifies
    if (d->gp().n_real_cells <= kGateJitMaxCells) {
      rrtl_batch* b = nullptr;
      rrtl_status st = rrtl_batch_create(d, lanes, &b);
      if (st) fail(st, g_last_error);
      float t = INFINITY;
      try {
        for (int rep = 0; rep < 3; ++rep) {
          gate_run(b, run, false, nullptr, true);
          if (rep && b->last_tile_words == 0) t = std::min(t, b->last_ms);
        }
      } catch (...) {
        rrtl_batch_destroy(b);
        throw;
      }
      rrtl_batch_destroy(b);
      if (t < best_t) {
        best_t = t;
        best = kTunedCompiled;
      }
    }
    d->tuned_w[lane_bucket(words)] = best;
    if (best_words) *best_words = best == kTunedCompiled ? 0u : best;
    if (best_ms) *best_ms = best_t;
  });
}

// ---- autotune recommendation table
namespace {

struct TuneRecord {
  std::string case_name;
  uint64_t lanes = 0, steps = 0;
  uint32_t tile_words = 0;
  bool has_metric = false;
  uint64_t metric_ns = 0;
};

std::vector<TuneRecord> parse_tune_table(const char* table, size_t len) {
  std::vector<TuneRecord> out;
  try {
    const json::Value v = json::Parser(table, len).parse();
    if (!v.is_arr()) throw std::runtime_error("expected an array of records");
    for (const json::Value& r : v.arr) {
      TuneRecord t;
      t.case_name = r.at("case").str();
      t.lanes = r.at("lanes").u64();
      t.steps = r.at("steps").u64();
      t.tile_words = r.at("tile_words").u32();
      if (t.tile_words != 0 && t.tile_words != 1 && t.tile_words != 2 && t.tile_words != 4 && t.tile_words != 8)
        throw std::runtime_error("tile_words must be 0, 1, 2, 4 or 8");
      const json::Value* m = r.find("autotune_metric_ns");
      if (m && !m->is_null()) {
        t.has_metric = true;
        t.metric_ns = m->u64();
      }
      out.push_back(std::move(t));
    }
  } catch (const std::exception& e) {
    fail(RRTL_E_ARG, std::string("E_GPU_AUTOTUNE_JSON: failed to load GPU autotune recommendations: ") + e.what());
  }
  return out;
}

// The reference's match rule: exact (case, lanes, steps), or the record of the
// same case with the smallest (|lane difference|, |step difference|, metric
// (absent last), lanes, steps).
uint32_t find_tune_record(const std::vector<TuneRecord>& items, const std::string& case_name, uint64_t lanes,
                          uint64_t steps, uint32_t mode) {
  REQUIRE(mode == RRTL_AUTOTUNE_EXACT || mode == RRTL_AUTOTUNE_NEAREST, RRTL_E_ARG, "E_ARG: unknown match mode");
  auto diff = [](uint64_t a, uint64_t b) { return a > b ? a - b : b - a; };
  int best = -1;
  for (size_t i = 0; i < items.size(); ++i) {
    const TuneRecord& r = items[i];
    if (r.case_name != case_name) continue;
    if (mode == RRTL_AUTOTUNE_EXACT) {
      if (r.lanes == lanes && r.steps == steps) {
        best = (int)i;
        break;
      }
      continue;
    }
    if (best < 0) {
      best = (int)i;
      continue;
    }
    const TuneRecord& b = items[best];
    auto key = [&](const TuneRecord& x) {
      return std::make_tuple(diff(x.lanes, lanes), diff(x.steps, steps), x.has_metric ? x.metric_ns : ~0ull, x.lanes,
                             x.steps);
    };
    if (key(r) < key(b)) best = (int)i;
  }
  if (best < 0)
    fail(RRTL_E_ARG, "E_GPU_AUTOTUNE_RECOMMENDATION: no GPU autotune recommendation for case `" + case_name +
                         "` lanes=" + std::to_string(lanes) + " steps=" + std::to_string(steps));
  return (uint32_t)best;
}

}  // namespace

rrtl_status rrtl_autotune_find(const char* table, size_t table_len, const char* case_name, uint64_t lanes,
                               uint64_t steps, uint32_t mode, uint32_t* index) {
  return guard([&] {
    REQUIRE(table && case_name && index, RRTL_E_ARG, "E_ARG: null argument");
    *index = find_tune_record(parse_tune_table(table, table_len), case_name, lanes, steps, mode);
  });
}

rrtl_status rrtl_design_autotune_recommend(rrtl_design* d, const char* case_name, uint32_t lanes, uint32_t steps,
                                           char* out, size_t cap, size_t* len) {
  return guard([&] {
    REQUIRE(d && case_name, RRTL_E_ARG, "E_ARG: null argument");
    uint32_t w = 0;
    float ms = 0.f;
    const rrtl_status st = rrtl_design_autotune(d, lanes, steps, &w, &ms);
    if (st) fail(st, g_last_error);
    std::string name;
    for (const char* p = case_name; *p; ++p) {
      if (*p == '"' || *p == '\\') name += '\\';
      if ((unsigned char)*p >= 0x20) name += *p;
    }
    const bool measured = d->engine == RRTL_ENGINE_GATE && d->gate_w_max;
    const std::string js = "{\"case\": \"" + name + "\", \"lanes\": " + std::to_string(lanes) +
                           ", \"steps\": " + std::to_string(steps) + ", \"tile_words\": " + std::to_string(w) +
                           ", \"autotune_metric\": \"kernel_ms\", \"autotune_metric_ns\": " +
                           (measured ? std::to_string((uint64_t)((double)ms * 1e6)) : std::string("null")) + "}";
    if (len) *len = js.size();
    if (out && cap) {
      const size_t n = std::min(cap - 1, js.size());
      memcpy(out, js.data(), n);
      out[n] = 0;
    }
  });
}

rrtl_status rrtl_design_autotune_apply(rrtl_design* d, const char* table, size_t table_len, const char* case_name,
                                       uint32_t lanes, uint64_t steps, uint32_t mode, uint32_t* tile_words) {
  return guard([&] {
    REQUIRE(d && table && case_name, RRTL_E_ARG, "E_ARG: null argument");
    REQUIRE(lanes > 0, RRTL_E_LANES, "E_GPU_AUTOTUNE_LANES: a recommendation applies to at least one lane");
    const std::vector<TuneRecord> items = parse_tune_table(table, table_len);
    const TuneRecord& r = items[find_tune_record(items, case_name, lanes, steps, mode)];
    REQUIRE(d->engine == RRTL_ENGINE_GATE && d->gate_w_max, RRTL_E_UNSUPPORTED,
            "E_GPU_AUTOTUNE_RECOMMENDATION: tile widths apply to gate-engine designs on the fused path");
    set_device(d->ctx);
    uint32_t choice = r.tile_words;
    if (choice == 0) {
      REQUIRE(d->gp().n_real_cells <= kGateJitMaxCells, RRTL_E_ARG,
              "E_GPU_AUTOTUNE_RECOMMENDATION: the compiled gate kernel does not take a design of this size");
      choice = kTunedCompiled;
    } else {
      REQUIRE(choice <= d->gate_w_max && gate_variant(d, choice)->fused_ok, RRTL_E_ARG,
              "E_GPU_AUTOTUNE_RECOMMENDATION: tile width " + std::to_string(choice) +
                  " does not fit this design's slots");
    }
    d->tuned_w[lane_bucket((lanes + 31) / 32)] = choice;
    if (tile_words) *tile_words = r.tile_words;
  });
}

rrtl_status rrtl_batch_set_tile_words(rrtl_batch* b, uint32_t words) {
  return guard([&] {
    REQUIRE(b, RRTL_E_ARG, "E_ARG: null argument");
    REQUIRE(words == 0 || words == 1 || words == 2 || words == 4 || words == 8, RRTL_E_ARG,
            "E_ARG: tile width must be 0, 1, 2, 4 or 8 words");
    REQUIRE(b->d->engine == RRTL_ENGINE_GATE || words == 0, RRTL_E_UNSUPPORTED, "E_ARG: tile width is a gate-engine setting");
    set_device(b->d->ctx);
    if (words) {
      GateVariant* v = gate_variant(b->d, words);
      REQUIRE(v->fused_ok, RRTL_E_UNSUPPORTED,
              "E_GATE_SCOPE: " + std::to_string(v->gp.n_slots) + " net slots of " + std::to_string(words) +
                  " words do not fit in shared memory");
    }
    b->tile_words = words;
  });
}

rrtl_status rrtl_batch_tile_words(rrtl_batch* b, uint32_t* words) {
  return guard([&] {
    REQUIRE(b && words, RRTL_E_ARG, "E_ARG: null argument");
    *words = b->last_tile_words;
  });
}

rrtl_status rrtl_batch_last_kernel_ms(rrtl_batch* b, float* ms) {
  return guard([&] {
    REQUIRE(b && ms, RRTL_E_ARG, "E_ARG: null argument");
    *ms = b->last_ms;
  });
}

}  // extern "C"
