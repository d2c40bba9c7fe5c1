// Serving loop (rrtl_server_*, include/rrtl_cuda.h): continuous batching of
// simulation requests on one GPU.
//
// Producer threads submit requests; one device-owner thread admits them as
// device memory frees up (each request gets its own lane batch, resident
// until it finishes) and drives rounds. A round advances every active
// request by up to `chunk_cycles` cycles: the gate-engine requests together
// in one launch of the persistent job-queue kernel (one item per tile and
// chunk), the word-engine requests as one launch of their compiled kernel
// each (side by side on a few streams) or, for designs without one,
// together in one launch of the interpreted multi-job word kernel. Requests
// that arrive during a round join at the next one, so new work overlaps the
// requests already on the device. A request's results are those of the same
// run alone on a fresh batch: every chunk continues from the state the last
// one left in the batch's device state.
//
// This is the single-GPU form of the reference's lane-shard scheduler
// (DistributedRuntime, crates/rrtl-runtime/src/lib.rs:6785-7760) reduced to
// a job queue, driven as a request loop.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>

#include "runtime.h"

using namespace rrtl;

namespace {

constexpr uint64_t kMinChunk = 8;  // adaptive chunks never fall below this many cycles
constexpr int kJitStreams = 4;     // compiled word kernels of a round run side by side on these

uint64_t now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct Request {
  uint64_t id = 0;
  rrtl_design* design = nullptr;
  uint32_t lanes = 0;
  rrtl_run run{};
  std::vector<rrtl_stim> stim;
  std::vector<uint32_t> record;
  std::vector<rrtl_fault> faults;
  std::vector<std::pair<uint32_t, std::vector<uint32_t>>> mem_init;
  uint32_t status = RRTL_JOB_QUEUED;
  std::string error;
  uint64_t t_submit = 0, t_admit = 0, t_done = 0;
  size_t bytes = 0;
  // device-owner thread only
  rrtl_batch* batch = nullptr;
  bool gate = false, fused = false;
  GatePrepared gp;
  WordPrepared wp;
  const JitKernel* jit = nullptr;  // the design's compiled word kernel, if any
  uint64_t done_cycles = 0;
  uint64_t chunk = 0;  // cycles of the current round
};

// Device bytes a request holds while active (lane state and run outputs).
size_t request_bytes(const Request& r) {
  const rrtl_design* d = r.design;
  const uint64_t cyc = r.run.cycles;
  size_t out = cyc * 8 + (size_t)r.lanes * 4;
  if (d->engine == RRTL_ENGINE_GATE) {
    const size_t words = ((r.lanes + 31) / 32 + 7) / 8 * 8;
    out += (size_t)(d->gp().n_nets + 1) * words * 4;
    if (r.run.record_mode & RRTL_REC_TRACE) out += cyc * r.run.n_record * words * 4;
  } else {
    const size_t lp = (r.lanes + 127) / 128 * 128;
    const PackedProgram& P = d->mp.source;
    out += ((size_t)P.total_signal_words + P.total_memory_words_per_lane + d->wp.total_capture_words) * lp * 4;
    if (r.run.record_mode & RRTL_REC_TRACE) out += cyc * r.run.n_record * 2 * lp * 4;
  }
  return out + (1u << 16);
}

}  // namespace

struct rrtl_server {
  rrtl_ctx* ctx = nullptr;
  size_t budget = 0;
  uint32_t chunk = 256;
  uint32_t max_active = 0;
  double round_ms = 0;      // target round time (0: fixed chunks)
  uint32_t policy = RRTL_SERVE_FAIR;
  double ms_per_cost = 0;   // calibrated device time of one unit of tile-cycle cost
  double ms_per_wcycle = 0; // calibrated device time of one cycle of a compiled word kernel
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> pending;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> all;
  uint64_t next_id = 1;
  bool stop = false;
  std::thread owner;
  // device-owner thread state
  std::vector<std::shared_ptr<Request>> active;
  size_t used = 0;
  DevBuf d_jobs, d_items, d_next, d_wjobs;
  bool queue_ready = false;
  size_t word_smem_set = 0;
  cudaStream_t word_stream = nullptr;  // word-engine launches overlap the gate queue kernel
  cudaEvent_t staged = nullptr;        // this round's uploads and memsets are done on the context stream
  cudaStream_t jit_stream[kJitStreams] = {};
  cudaEvent_t jit_ev[kJitStreams][2] = {};
  // statistics (under mu)
  uint64_t rounds = 0, completed = 0, failed = 0, lane_cycles = 0, busy_ns = 0;

  void loop();
  void admit(std::vector<std::shared_ptr<Request>>& fresh);
  void round();
  void finish(Request& r, uint32_t status, const std::string& err);
};

void rrtl_server::finish(Request& r, uint32_t status, const std::string& err) {
  if (r.batch) {
    rrtl_batch_destroy(r.batch);
    r.batch = nullptr;
  }
  used -= std::min(used, r.bytes);
  std::lock_guard<std::mutex> lk(mu);
  r.status = status;
  r.error = err;
  r.t_done = now_ns();
  if (status == RRTL_JOB_DONE) {
    ++completed;
    lane_cycles += (uint64_t)r.lanes * r.run.cycles;
  } else {
    ++failed;
  }
  cv_done.notify_all();
}

// Create the lane batch of each newly admitted request and prepare its run.
void rrtl_server::admit(std::vector<std::shared_ptr<Request>>& fresh) {
  for (auto& rp : fresh) {
    Request& r = *rp;
    try {
      rrtl_status st = rrtl_batch_create(r.design, r.lanes, &r.batch);
      if (st) fail(st, rrtl_last_error());
      if (!r.faults.empty()) {
        st = rrtl_batch_set_faults(r.batch, r.faults.data(), r.faults.size());
        if (st) fail(st, rrtl_last_error());
      }
      for (auto& mi : r.mem_init) {
        st = rrtl_batch_set_memory_limbs(r.batch, mi.first, mi.second.data(), mi.second.size());
        if (st) fail(st, rrtl_last_error());
      }

      r.gate = r.design->engine == RRTL_ENGINE_GATE;
      if (r.gate) {
        r.gp = gate_prepare(r.batch, r.run, false, true);
        r.fused = r.gp.fused && r.gp.v->fused_smem <= ctx->max_smem - gate_queue_static_smem();
      } else {
        r.wp = word_prepare(r.batch, r.run, false, false);
        r.jit = word_jit_for_run(r.design, r.wp.tables, r.wp.R.lanes_pad);  // compiled once per design and run tables
        if (!r.jit) word_require_interp(r.design, r.wp);
      }
      active.push_back(rp);
    } catch (const ApiError& e) {
      finish(r, RRTL_JOB_FAILED, e.msg);
    } catch (const std::exception& e) {
      finish(r, RRTL_JOB_FAILED, std::string("E_INTERNAL: ") + e.what());
    }
  }
}

// Advance every active request by up to `chunk` cycles, then retire the
// finished ones.
void rrtl_server::round() {
  cudaStream_t st = ctx->stream;
  const uint64_t t0 = now_ns();
  std::vector<GateJobDev> jobs;
  std::vector<GateItemDev> items;
  std::vector<WordJobDev> wjobs;
  std::vector<Request*> jit_reqs;
  std::vector<WordRunDev> jit_descs;
  uint32_t wblocks = 0;
  size_t smem = 0, wsmem = 0;
  std::vector<std::pair<double, uint32_t>> order;
  // adaptive chunks: every gate request's tiles get about the same cost c per
  // round, with c chosen so the round (its longest tile, or all tiles spread
  // over the SMs) lasts about round_ms
  double cost_per_tile_round = 0;
  // shortest remaining first: the gate-engine requests with the least work
  // left, as many as fill the SMs twice, share the round; the others advance
  // by the minimum chunk only, so short requests are not held to the pace of
  // long ones
  std::unordered_set<const Request*> front;
  if (policy == RRTL_SERVE_SHORTEST_FIRST) {
    std::vector<std::pair<double, const Request*>> rem;
    for (auto& rp : active)
      if (rp->gate && rp->fused)
        rem.push_back({(double)(rp->run.cycles - rp->done_cycles) * rp->gp.v->tile_cycle_cost * rp->gp.R.n_tiles,
                       rp.get()});
    std::sort(rem.begin(), rem.end(), [](const std::pair<double, const Request*>& x,
                                         const std::pair<double, const Request*>& y) { return x.first < y.first; });
    double tiles = 0;
    for (auto& x : rem) {
      if (tiles >= 2.0 * ctx->sm_count) break;
      front.insert(x.second);
      tiles += x.second->gp.R.n_tiles;
    }
  }
  auto in_front = [&](const Request* r) { return policy != RRTL_SERVE_SHORTEST_FIRST || front.count(r) > 0; };
  if (round_ms > 0 && ms_per_cost > 0) {
    double tiles = 0;
    for (auto& rp : active)
      if (rp->gate && rp->fused && in_front(rp.get())) tiles += rp->gp.R.n_tiles;
    cost_per_tile_round = round_ms / ms_per_cost / std::max(1.0, tiles / std::max<uint32_t>(1, ctx->sm_count));
  }
  for (auto& rp : active) {
    Request& r = *rp;
    const uint64_t left = r.run.cycles - r.done_cycles;
    if (r.gate && !r.fused) {
      // recorded nets leave the chip or the program is too large for the queue kernel: whole run, plain path
      r.chunk = left;
      gate_plain_launches(r.gp, r.run.cycles, st, false);
      continue;
    }
    r.chunk = std::min<uint64_t>(left, chunk);
    if (r.gate && !in_front(&r)) {
      r.chunk = std::min<uint64_t>(left, kMinChunk);
    } else if (r.gate && cost_per_tile_round > 0) {
      const uint64_t want = (uint64_t)std::max((double)kMinChunk, cost_per_tile_round / std::max(r.gp.v->tile_cycle_cost, 1e-9));
      r.chunk = std::min<uint64_t>(left, want);
    }
    const bool last = r.done_cycles + r.chunk == r.run.cycles;
    if (r.gate) {
      const uint32_t ji = (uint32_t)jobs.size();
      jobs.push_back(GateJobDev{r.gp.v->gdev, r.gp.R});
      smem = std::max(smem, r.gp.v->fused_smem);
      const double cost = (double)(r.chunk + 1) * r.gp.v->tile_cycle_cost;
      for (uint32_t t = 0; t < r.gp.R.n_tiles; ++t) {
        order.push_back({cost, (uint32_t)items.size()});
        items.push_back(GateItemDev{ji, t, (unsigned long long)r.done_cycles, (uint32_t)r.chunk, last ? 1u : 0u});
      }
    } else if (r.jit) {
      if (round_ms > 0 && ms_per_wcycle > 0)
        r.chunk = std::min<uint64_t>(left, std::max<uint64_t>(kMinChunk, (uint64_t)(round_ms / ms_per_wcycle)));
      const bool lastj = r.done_cycles + r.chunk == r.run.cycles;
      jit_reqs.push_back(&r);
      jit_descs.push_back(word_chunk_desc(r.wp, r.done_cycles, r.chunk, lastj));
    } else {
      WordJobDev wj{};
      wj.P = r.design->wdev;
      wj.R = word_chunk_desc(r.wp, r.done_cycles, r.chunk, last);
      wj.block_begin = wblocks;
      wblocks += r.wp.R.lanes_pad / kWordBlockLanes;
      wsmem = std::max(wsmem, (size_t)r.design->wdev.n_vslots * kWordBlockLanes * 8 +
                                  (r.design->wdev.sig_smem ? (size_t)r.design->wdev.n_sig_words * kWordBlockLanes * 4 : 0));
      wjobs.push_back(wj);
    }
  }
  if (!jit_reqs.empty() || !wjobs.empty()) cuda_check(cudaEventRecord(staged, st), "event");
  // compiled word kernels: one launch per request, spread over the side streams
  uint64_t jit_cycles[kJitStreams] = {};
  const int n_js = std::min<int>(kJitStreams, (int)jit_reqs.size());
  for (int k = 0; k < n_js; ++k) {
    cuda_check(cudaStreamWaitEvent(jit_stream[k], staged, 0), "wait event");
    cuda_check(cudaEventRecord(jit_ev[k][0], jit_stream[k]), "event");
  }
  for (size_t i = 0; i < jit_reqs.size(); ++i) {
    Request& r = *jit_reqs[i];
    const int k = (int)(i % kJitStreams);
    WordJitPlace pl;
    const size_t jsmem = word_jit_place(r.design->wp, *r.jit, r.design->wdev.n_sig_words, r.wp.R.lanes_pad, r.chunk,
                                        ctx->sm_count, ctx->max_smem, ctx->max_smem_sm, &pl);
    cuda_check(launch_word_jit(*r.jit, jit_descs[i], pl, jsmem, jit_stream[k]), "rrtl_word_jit");
    jit_cycles[k] += r.chunk;
  }
  for (int k = 0; k < n_js; ++k) cuda_check(cudaEventRecord(jit_ev[k][1], jit_stream[k]), "event");
  if (!wjobs.empty()) {
    // one launch for every interpreted word-engine request, on the second stream, after this round's staging
    if (wsmem > word_smem_set) {
      cuda_check(word_multi_prepare(kWordSmemLimit), "word_multi_prepare");
      word_smem_set = kWordSmemLimit;
    }
    upload(d_wjobs, wjobs);
    cuda_check(cudaEventRecord(staged, st), "event");  // after the job table upload
    cuda_check(cudaStreamWaitEvent(word_stream, staged, 0), "wait event");
    cuda_check(launch_word_multi(d_wjobs.as<WordJobDev>(), (uint32_t)wjobs.size(), wblocks, wsmem, word_stream),
               "word_multi_kernel");
  }
  double max_cost = 0, sum_cost = 0;
  for (auto& o : order) {
    max_cost = std::max(max_cost, o.first);
    sum_cost += o.first;
  }
  const double crit = std::max(max_cost, sum_cost / std::max<uint32_t>(1, ctx->sm_count));
  if (!items.empty()) {
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<double, uint32_t>& a, const std::pair<double, uint32_t>& b) { return a.first > b.first; });
    std::vector<GateItemDev> sorted;
    sorted.reserve(items.size());
    for (auto& o : order) sorted.push_back(items[o.second]);
    const size_t qmax = ctx->max_smem - gate_queue_static_smem();
    if (!queue_ready) {
      cuda_check(gate_queue_prepare(qmax), "gate_queue_prepare");
      queue_ready = true;
    }
    upload(d_jobs, jobs);
    upload(d_items, sorted);
    d_next.reserve(16);
    cuda_check(cudaMemsetAsync(d_next.p, 0, 8, st), "memset queue");
    GateQueueDev QD{d_jobs.as<GateJobDev>(), d_items.as<GateItemDev>(), (uint32_t)sorted.size(), d_next.as<uint32_t>()};
    cuda_check(launch_gate_queue(QD, std::min<uint32_t>((uint32_t)sorted.size(), ctx->sm_count), smem, st),
               "gate_queue_kernel");
  }
  cuda_check(cudaStreamSynchronize(st), "sync");
  const uint64_t t_gate = now_ns();
  cuda_check(cudaStreamSynchronize(word_stream), "sync");
  double wcyc = 0;
  for (int k = 0; k < n_js; ++k) {
    cuda_check(cudaEventSynchronize(jit_ev[k][1]), "sync");
    float ms = 0;
    cuda_check(cudaEventElapsedTime(&ms, jit_ev[k][0], jit_ev[k][1]), "elapsed");
    if (jit_cycles[k]) wcyc = std::max(wcyc, (double)ms / (double)jit_cycles[k]);
  }
  if (wcyc > 0) ms_per_wcycle = ms_per_wcycle > 0 ? 0.7 * ms_per_wcycle + 0.3 * wcyc : wcyc;
  if (crit > 0 && !items.empty()) {
    // calibrate: the round's gate part took about its critical cost
    const double m = (double)(t_gate - t0) / 1e6 / crit;
    ms_per_cost = ms_per_cost > 0 ? 0.7 * ms_per_cost + 0.3 * m : m;
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    ++rounds;
    busy_ns += now_ns() - t0;
  }
  // launch status of the queue kernel: a CTA that could not drain its copies
  // fails every request the launch served
  uint32_t launch_err = 0;
  if (!items.empty() && cudaMemcpy(&launch_err, d_next.as<uint32_t>() + 1, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    launch_err = RRTL_E_DEVICE;
  std::vector<std::shared_ptr<Request>> keep;
  for (auto& rp : active) {
    Request& r = *rp;
    if (launch_err && r.gate && r.fused) {
      finish(r, RRTL_JOB_FAILED, "E_TIMEOUT: a bounded device wait of the round's queue launch gave up");
      continue;
    }
    r.done_cycles += r.chunk;
    if (r.done_cycles < r.run.cycles) {
      keep.push_back(rp);
      continue;
    }
    uint32_t e = 0;
    cudaMemcpy(&e, r.batch->d_err.p, 4, cudaMemcpyDeviceToHost);
    if (e) {
      finish(r, RRTL_JOB_FAILED, "E_TIMEOUT: a bounded device wait gave up");
      continue;
    }
    try {
      if (r.gate) gate_copy_out(r.batch, r.gp, r.run);
      else word_copy_out(r.batch, r.wp, r.run);
      cuda_check(cudaStreamSynchronize(st), "sync");
      finish(r, RRTL_JOB_DONE, "");
    } catch (const ApiError& ex) {
      finish(r, RRTL_JOB_FAILED, ex.msg);
    }
  }
  active.swap(keep);
}

void rrtl_server::loop() {
  cudaSetDevice(ctx->device);
  bool streams_ok = cudaStreamCreateWithFlags(&word_stream, cudaStreamNonBlocking) == cudaSuccess &&
                    cudaEventCreateWithFlags(&staged, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < kJitStreams && streams_ok; ++k)
    streams_ok = cudaStreamCreateWithFlags(&jit_stream[k], cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreate(&jit_ev[k][0]) == cudaSuccess && cudaEventCreate(&jit_ev[k][1]) == cudaSuccess;
  if (!streams_ok) {
    // without its streams the loop cannot run: fail every request as it arrives
    for (;;) {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] { return stop || !pending.empty(); });
      while (!pending.empty()) {
        Request& r = *pending.front();
        r.status = RRTL_JOB_FAILED;
        r.error = "E_DEVICE: serving loop could not create its stream";
        r.t_done = now_ns();
        ++failed;
        pending.pop_front();
      }
      cv_done.notify_all();
      if (stop) return;
    }
  }
  for (;;) {
    std::vector<std::shared_ptr<Request>> fresh;
    {
      std::unique_lock<std::mutex> lk(mu);
      if (active.empty()) cv_work.wait(lk, [&] { return stop || !pending.empty(); });
      if (stop && pending.empty() && active.empty()) {
      lk.unlock();
      cudaEventDestroy(staged);
      cudaStreamDestroy(word_stream);
      for (int k = 0; k < kJitStreams; ++k) {
        cudaStreamDestroy(jit_stream[k]);
        cudaEventDestroy(jit_ev[k][0]);
        cudaEventDestroy(jit_ev[k][1]);
      }
      return;
    }
      // admission: first come first served while the device memory budget and the slot count allow
      while (!pending.empty()) {
        Request& r = *pending.front();
        const bool room = used + r.bytes <= budget || (active.empty() && fresh.empty());
        if (!room || (max_active && active.size() + fresh.size() >= max_active)) break;
        used += r.bytes;
        r.status = RRTL_JOB_RUNNING;
        r.t_admit = now_ns();
        fresh.push_back(pending.front());
        pending.pop_front();
      }
    }
    admit(fresh);
    if (active.empty()) continue;
    try {
      round();
    } catch (const ApiError& e) {
      // a launch failed: every active request fails with it
      for (auto& rp : active) finish(*rp, RRTL_JOB_FAILED, e.msg);
      active.clear();
    }
  }
}

template <class F>
static rrtl_status sguard(F&& f) {
  try {
    f();
    return RRTL_OK;
  } catch (const ApiError& e) {
    set_last_error(e.msg);
    return e.status;
  } catch (const std::exception& e) {
    set_last_error(std::string("E_INTERNAL: ") + e.what());
    return RRTL_E_ARG;
  }
}

extern "C" {

rrtl_status rrtl_server_create(rrtl_ctx* ctx, const rrtl_server_opts* opts, rrtl_server** out) {
  return sguard([&] {
    if (!ctx || !out) fail(RRTL_E_ARG, "E_ARG: null argument");
    cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
    auto s = std::make_unique<rrtl_server>();
    s->ctx = ctx;
    size_t free_b = 0, total_b = 0;
    cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    s->budget = opts && opts->hbm_budget ? (size_t)opts->hbm_budget : free_b / 10 * 9;
    s->chunk = opts && opts->chunk_cycles ? opts->chunk_cycles : 256;
    s->max_active = opts ? opts->max_active : 0;
    s->round_ms = opts ? opts->round_us / 1000.0 : 0.0;
    s->policy = opts ? opts->policy : RRTL_SERVE_FAIR;
    if (s->policy > RRTL_SERVE_SHORTEST_FIRST) fail(RRTL_E_ARG, "E_ARG: unknown serving policy");
    // the first NVRTC compile of a process pays for loading the compiler;
    // pay it here rather than in the first word request's admission
    jit_warm();
    ctx->refs++;
    rrtl_server* raw = s.release();
    raw->owner = std::thread([raw] { raw->loop(); });
    *out = raw;
  });
}

rrtl_status rrtl_server_submit(rrtl_server* s, const rrtl_request* req, uint64_t* id) {
  return sguard([&] {
    if (!s || !req || !id || !req->design) fail(RRTL_E_ARG, "E_ARG: null argument");
    if (req->design->ctx != s->ctx) fail(RRTL_E_ARG, "E_SERVER: the design belongs to another context");
    if (req->lanes == 0) fail(RRTL_E_LANES, "E_GPU_LANES: GPU simulator requires at least one lane");
    if (req->run.n_stim && !req->run.stim) fail(RRTL_E_ARG, "E_ARG: stim is null");
    if (req->run.n_record && !req->run.record) fail(RRTL_E_ARG, "E_ARG: record is null");
    if (req->n_faults && !req->faults) fail(RRTL_E_ARG, "E_ARG: faults is null");
    auto r = std::make_shared<Request>();
    r->design = req->design;
    r->lanes = req->lanes;
    r->run = req->run;
    r->stim.assign(req->run.stim, req->run.stim + req->run.n_stim);
    r->record.assign(req->run.record, req->run.record + req->run.n_record);
    r->faults.assign(req->faults, req->faults + req->n_faults);
    if (req->n_mem_init && !req->mem_init) fail(RRTL_E_ARG, "E_ARG: mem_init is null");
    for (uint32_t i = 0; i < req->n_mem_init; ++i) {
      const rrtl_mem_init& mi = req->mem_init[i];
      if (mi.n && !mi.data) fail(RRTL_E_ARG, "E_ARG: mem_init data is null");
      r->mem_init.emplace_back(mi.memory, std::vector<uint32_t>(mi.data, mi.data + mi.n));
    }
    r->run.stim = r->stim.data();
    r->run.record = r->record.data();
    r->bytes = request_bytes(*r);
    r->t_submit = now_ns();
    // build what admission will need (a tile-width variant, a compiled word
    // kernel) on the submitting thread, so the device loop never stalls on it;
    // a failure here surfaces again at admission
    try {
      design_warm_for_run(r->design, r->lanes, r->run);
    } catch (...) {
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->stop) fail(RRTL_E_ARG, "E_SERVER: the server is shutting down");
      r->id = s->next_id++;
      s->all[r->id] = r;
      s->pending.push_back(r);
      *id = r->id;
    }
    s->cv_work.notify_one();
  });
}

rrtl_status rrtl_server_info(rrtl_server* s, uint64_t id, rrtl_request_info* info) {
  return sguard([&] {
    if (!s || !info) fail(RRTL_E_ARG, "E_ARG: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) fail(RRTL_E_ARG, "E_SERVER: unknown request id");
    const Request& r = *it->second;
    info->status = r.status;
    info->submit_ns = r.t_submit;
    info->admit_ns = r.t_admit;
    info->done_ns = r.t_done;
  });
}

rrtl_status rrtl_server_wait(rrtl_server* s, uint64_t id, uint32_t timeout_ms) {
  return sguard([&] {
    if (!s) fail(RRTL_E_ARG, "E_ARG: null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) fail(RRTL_E_ARG, "E_SERVER: unknown request id");
    std::shared_ptr<Request> r = it->second;
    auto done = [&] { return r->status == RRTL_JOB_DONE || r->status == RRTL_JOB_FAILED; };
    if (timeout_ms) {
      if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done))
        fail(RRTL_E_TIMEOUT, "E_TIMEOUT: request not finished");
    } else {
      s->cv_done.wait(lk, done);
    }
    if (r->status == RRTL_JOB_FAILED) fail(RRTL_E_DEVICE, r->error.empty() ? "E_SERVER: request failed" : r->error);
  });
}

rrtl_status rrtl_server_drain(rrtl_server* s) {
  return sguard([&] {
    if (!s) fail(RRTL_E_ARG, "E_ARG: null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] {
      for (auto& kv : s->all)
        if (kv.second->status != RRTL_JOB_DONE && kv.second->status != RRTL_JOB_FAILED) return false;
      return true;
    });
  });
}

rrtl_status rrtl_server_stats_get(rrtl_server* s, rrtl_server_stats* out) {
  return sguard([&] {
    if (!s || !out) fail(RRTL_E_ARG, "E_ARG: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    out->rounds = s->rounds;
    out->completed = s->completed;
    out->failed = s->failed;
    out->lane_cycles = s->lane_cycles;
    out->busy_ns = s->busy_ns;
    out->pending = s->pending.size();
  });
}

rrtl_status rrtl_server_release(rrtl_server* s, uint64_t id) {
  return sguard([&] {
    if (!s) fail(RRTL_E_ARG, "E_ARG: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) fail(RRTL_E_ARG, "E_SERVER: unknown request id");
    if (it->second->status != RRTL_JOB_DONE && it->second->status != RRTL_JOB_FAILED)
      fail(RRTL_E_ARG, "E_SERVER: request not finished");
    s->all.erase(it);
  });
}

rrtl_status rrtl_server_destroy(rrtl_server* s) {
  return sguard([&] {
    if (!s) return;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->owner.joinable()) s->owner.join();
    rrtl_ctx* ctx = s->ctx;
    delete s;
    rrtl_ctx_destroy(ctx);
  });
}

}  // extern "C"
