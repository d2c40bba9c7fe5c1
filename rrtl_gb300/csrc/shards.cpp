// Lane-shard runtime (rrtl_runtime_*, include/rrtl_cuda.h): the single-GPU
// form of the reference's DistributedRuntime shard plan
// (crates/rrtl-runtime/src/lib.rs:168-175 RuntimeShardInfo, :6785-7760).
//
// A runtime splits `total` lanes of one design into contiguous shards, each
// starting on a 32-lane word, and keeps one lane batch per shard. A run goes
// to every shard with lane_base = the shard's first lane, so random stimulus
// and hash terms follow global lanes: gate-engine shards run as jobs of one
// launch of the device job queue, word-engine shards one after another on
// the context stream. Outputs come back in global-lane order: per-cycle
// hashes add up (wrapping) to the hash of the whole run, detection vectors
// and traces are placed at each shard's lanes, and input traces are cut per
// shard.
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "runtime.h"

using namespace rrtl;

struct rrtl_runtime {
  rrtl_design* d = nullptr;
  uint64_t total = 0;
  std::vector<rrtl_shard_info> shards;
  std::vector<rrtl_batch*> batches;
};

namespace {

void check_status(rrtl_status st) {
  if (st != RRTL_OK) fail(st, rrtl_last_error());
}

template <class F>
rrtl_status rguard(F&& f) {
  try {
    f();
    set_last_error("");
    return RRTL_OK;
  } catch (const ApiError& e) {
    set_last_error(e.msg);
    return e.status;
  } catch (const std::bad_alloc&) {
    set_last_error("E_OOM: host allocation failed");
    return RRTL_E_OOM;
  } catch (const std::exception& e) {
    set_last_error(std::string("E_INTERNAL: ") + e.what());
    return RRTL_E_ARG;
  }
}

// Contiguous shards of `total` lanes over `n` shards, each starting on a
// multiple of 32 lanes (the unit stimulus and hashes are keyed on).
std::vector<rrtl_shard_info> plan_shards(uint64_t total, uint32_t n) {
  if (total == 0) fail(RRTL_E_LANES, "E_GPU_LANES: GPU simulator requires at least one lane");
  if (n == 0) fail(RRTL_E_ARG, "E_ARG: at least one shard");
  const uint64_t words = (total + 31) / 32;
  if (n > words) fail(RRTL_E_ARG, "E_RUNTIME_SHARDS: more shards than 32-lane words");
  std::vector<rrtl_shard_info> out;
  for (uint32_t k = 0; k < n; ++k) {
    const uint64_t a = std::min(total, words * k / n * 32), b = std::min(total, words * (k + 1) / n * 32);
    if (b - a > 0xFFFFFFFFull) fail(RRTL_E_LANES, "E_GPU_LANES: a shard holds more than 2^32 - 1 lanes");
    out.push_back(rrtl_shard_info{k, (uint32_t)(b - a), a});
  }
  return out;
}

}  // namespace

extern "C" {

rrtl_status rrtl_shard_plan(uint64_t total_lanes, uint32_t n, rrtl_shard_info* out) {
  return rguard([&] {
    if (!out) fail(RRTL_E_ARG, "E_ARG: null argument");
    std::vector<rrtl_shard_info> p = plan_shards(total_lanes, n);
    std::memcpy(out, p.data(), p.size() * sizeof(rrtl_shard_info));
  });
}

rrtl_status rrtl_runtime_create(rrtl_design* d, uint64_t total_lanes, uint32_t n, rrtl_runtime** out) {
  return rguard([&] {
    if (!d || !out) fail(RRTL_E_ARG, "E_ARG: null argument");
    auto rt = std::make_unique<rrtl_runtime>();
    rt->d = d;
    rt->total = total_lanes;
    rt->shards = plan_shards(total_lanes, n);
    try {
      for (const rrtl_shard_info& s : rt->shards) {
        rrtl_batch* b = nullptr;
        check_status(rrtl_batch_create(d, s.lanes, &b));
        rt->batches.push_back(b);
      }
    } catch (...) {
      for (rrtl_batch* b : rt->batches) rrtl_batch_destroy(b);
      throw;
    }
    *out = rt.release();
  });
}

rrtl_status rrtl_runtime_destroy(rrtl_runtime* rt) {
  return rguard([&] {
    if (!rt) return;
    for (rrtl_batch* b : rt->batches) rrtl_batch_destroy(b);
    delete rt;
  });
}

rrtl_status rrtl_runtime_shard(rrtl_runtime* rt, uint32_t k, rrtl_shard_info* info, rrtl_batch** batch) {
  return rguard([&] {
    if (!rt) fail(RRTL_E_ARG, "E_ARG: null argument");
    if (k >= rt->shards.size()) fail(RRTL_E_ARG, "E_RUNTIME_SHARDS: no such shard");
    if (info) *info = rt->shards[k];
    if (batch) *batch = rt->batches[k];
  });
}

rrtl_status rrtl_runtime_set_faults(rrtl_runtime* rt, const rrtl_fault* faults, size_t n) {
  return rguard([&] {
    if (!rt || (n && !faults)) fail(RRTL_E_ARG, "E_ARG: null argument");
    std::vector<std::vector<rrtl_fault>> per(rt->shards.size());
    for (size_t i = 0; i < n; ++i) {
      rrtl_fault f = faults[i];
      if (f.lane >= rt->total) fail(RRTL_E_ARG, "E_GPU_FAULT: lane out of range");
      size_t k = 0;
      while (k + 1 < rt->shards.size() && f.lane >= rt->shards[k + 1].start_lane) ++k;
      f.lane -= (uint32_t)rt->shards[k].start_lane;
      per[k].push_back(f);
    }
    for (size_t k = 0; k < per.size(); ++k)
      check_status(rrtl_batch_set_faults(rt->batches[k], per[k].data(), per[k].size()));
  });
}

rrtl_status rrtl_runtime_run(rrtl_runtime* rt, const rrtl_run* run) {
  return rguard([&] {
    if (!rt || !run) fail(RRTL_E_ARG, "E_ARG: null argument");
    rrtl_design* d = rt->d;
    const bool gate = d->engine == RRTL_ENGINE_GATE;
    const size_t S = rt->shards.size();
    const uint64_t cyc = run->cycles;
    const uint32_t mode = run->record_mode;
    const uint64_t total_words = (rt->total + 31) / 32;
    // units of one trace row: 32-lane words (gate engine) or lanes (word engine)
    auto units = [&](const rrtl_shard_info& s) { return gate ? (uint64_t)(s.lanes + 31) / 32 : (uint64_t)s.lanes; };
    auto first = [&](const rrtl_shard_info& s) { return gate ? s.start_lane / 32 : s.start_lane; };
    const uint64_t all_units = gate ? total_words : rt->total;
    uint32_t rows = run->n_record;  // trace rows per cycle: recorded signals (gate) or their limbs (word)
    if (!gate) {
      rows = 0;
      for (uint32_t i = 0; i < run->n_record; ++i) {
        if (run->record[i] >= d->mp.source.signals.size()) fail(RRTL_E_SIGNAL, "E_GPU_SIGNAL: signal index out of range");
        rows += d->mp.source.signals[run->record[i]].layout.limbs;
      }
    }
    std::vector<std::vector<uint64_t>> hashes(S);
    std::vector<std::vector<uint32_t>> traces(S), inputs(S);
    std::vector<rrtl_run> runs(S);
    for (size_t k = 0; k < S; ++k) {
      const rrtl_shard_info& s = rt->shards[k];
      rrtl_run r = *run;
      r.lane_base = run->lane_base + s.start_lane;
      if (mode & RRTL_REC_HASH) {
        if (!run->out_hash) fail(RRTL_E_ARG, "E_GPU_RECORD: out_hash is null");
        hashes[k].assign(cyc, 0);
        r.out_hash = hashes[k].data();
      }
      if (mode & RRTL_REC_DETECT) {
        if (!run->detect) fail(RRTL_E_ARG, "E_GPU_RECORD: detect is null");
        r.detect = run->detect + s.start_lane;  // a shard's detection vector is its lanes' slice
      }
      if (mode & RRTL_REC_TRACE) {
        if (!run->out_trace) fail(RRTL_E_ARG, "E_GPU_RECORD: out_trace is null");
        traces[k].assign(cyc * rows * units(s), 0);
        r.out_trace = traces[k].data();
      }
      if (run->n_trace_cols) {
        if (!run->input_trace) fail(RRTL_E_ARG, "E_GPU_STIM: input_trace is null");
        const uint64_t u = units(s), f0 = first(s);
        inputs[k].resize(cyc * run->n_trace_cols * u);
        for (uint64_t c = 0; c < cyc; ++c)
          for (uint32_t col = 0; col < run->n_trace_cols; ++col)
            std::memcpy(inputs[k].data() + (c * run->n_trace_cols + col) * u,
                        run->input_trace + (c * run->n_trace_cols + col) * all_units + f0, u * 4);
        r.input_trace = inputs[k].data();
      }
      runs[k] = r;
    }
    if (gate) {
      std::vector<uint64_t> ids(S);
      for (size_t k = 0; k < S; ++k) {
        rrtl_job job{rt->batches[k], runs[k]};
        check_status(rrtl_queue_submit(d->ctx, &job, &ids[k]));
      }
      check_status(rrtl_queue_launch(d->ctx));
      check_status(rrtl_queue_wait(d->ctx));
      for (size_t k = 0; k < S; ++k) {
        uint32_t st = 0;
        check_status(rrtl_queue_poll(d->ctx, ids[k], &st));
        if (st != RRTL_JOB_DONE) fail(RRTL_E_DEVICE, "E_RUNTIME_SHARDS: shard " + std::to_string(k) + " failed");
      }
    } else {
      for (size_t k = 0; k < S; ++k) check_status(rrtl_batch_run(rt->batches[k], &runs[k]));
    }
    if (mode & RRTL_REC_HASH) {
      for (uint64_t c = 0; c < cyc; ++c) {
        uint64_t h = 0;
        for (size_t k = 0; k < S; ++k) h += hashes[k][c];
        run->out_hash[c] = h;
      }
    }
    if (mode & RRTL_REC_TRACE) {
      for (size_t k = 0; k < S; ++k) {
        const uint64_t u = units(rt->shards[k]), f0 = first(rt->shards[k]);
        for (uint64_t c = 0; c < cyc; ++c)
          for (uint32_t q = 0; q < rows; ++q)
            std::memcpy(run->out_trace + (c * rows + q) * all_units + f0, traces[k].data() + (c * rows + q) * u, u * 4);
      }
    }
  });
}

}  // extern "C"
