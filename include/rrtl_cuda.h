/*
 * rrtl_cuda.h — C ABI of the GB300 batched cycle-simulation engine.
 *
 * This is the drop-in boundary for RRTL's batch simulator. The reference
 * exposes the same capability as the Rust type `GpuBatchSimulator`
 * (crates/rrtl-gpu-sim/src/lib.rs:458-1512) and the design-as-data
 * `InterpGpuSimulator` (crates/rrtl-gpu-sim/src/interp.rs:1772-2069), selected
 * through `RuntimeBackend::Gpu` (crates/rrtl-runtime/src/lib.rs:29-40). Each
 * entry point below names the method it replaces.
 *
 * Conventions
 *  - Every function returns rrtl_status (0 = OK). rrtl_last_error() returns
 *    the message of the calling thread's last failure, prefixed by a stable
 *    code mirroring the reference diagnostics (E_GPU_LANES, E_GPU_SIGNAL, ...).
 *  - Handles are opaque. The library owns all device memory; caller buffers
 *    are only read or written during the call.
 *  - Host lane arrays are signal-major [limb][lane], the reference's
 *    `(offset + limb) * lanes + lane` order (crates/rrtl-gpu-sim/src/lib.rs:1637-1639).
 *    The top limb is masked to the signal width on set and on get.
 *  - Memories are exchanged as [addr][limb][lane].
 *  - Signals are addressed by packed signal index (position in the packed
 *    program, crates/rrtl-sim-ir/src/lib.rs:12340-12414); look it up by name
 *    with rrtl_design_signal().
 *  - One thread drives a batch at a time (the Rust API is `&mut self`).
 *  - Destroy calls may come in any order: a design keeps its context and a
 *    batch its design alive until the last of them is destroyed.
 */
#ifndef RRTL_CUDA_H
#define RRTL_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t rrtl_status;

enum {
  RRTL_OK = 0,
  RRTL_E_ARG = 1,        /* bad argument (E_GPU_LANE_VALUES, E_GPU_MEMORY_VALUES, ...) */
  RRTL_E_DESIGN = 2,     /* design rejected by the compiler / lowering (E_SIM_IR_*, E_EXPR_TYPE, ...) */
  RRTL_E_SIGNAL = 3,     /* unknown signal or memory (E_GPU_SIGNAL, E_GPU_MEMORY) */
  RRTL_E_DEVICE = 4,     /* CUDA error */
  RRTL_E_OOM = 5,        /* device allocation failed */
  RRTL_E_TIMEOUT = 6,    /* a bounded device wait gave up */
  RRTL_E_UNSUPPORTED = 7,/* feature outside this engine's scope */
  RRTL_E_LANES = 8       /* lanes == 0 or lanes beyond the limit (E_GPU_LANES) */
};

typedef struct rrtl_ctx rrtl_ctx;
typedef struct rrtl_design rrtl_design;
typedef struct rrtl_batch rrtl_batch;

/* Message of the calling thread's last failure ("" when none). */
const char* rrtl_last_error(void);

/* ---- context ------------------------------------------------------------ */

/* Device context with its own CUDA stream. Replaces the wgpu adapter/device/
 * queue setup in GpuBatchSimulator::new_async (crates/rrtl-gpu-sim/src/lib.rs:612-642). */
rrtl_status rrtl_ctx_create(int32_t device, rrtl_ctx** out);
rrtl_status rrtl_ctx_destroy(rrtl_ctx* ctx);
/* Number of streaming multiprocessors of the context's device. */
rrtl_status rrtl_ctx_sm_count(rrtl_ctx* ctx, uint32_t* out);
/* Device timing on the context stream (no reference counterpart; the Rust
 * API times with wall clocks, crates/rrtl-gpu-sim/src/lib.rs:305-322).
 * Records CUDA event `slot` (0..7) on the stream; elapsed_ms synchronises on
 * event `b` and returns the time from event `a` to event `b`. */
rrtl_status rrtl_ctx_event_record(rrtl_ctx* ctx, uint32_t slot);
rrtl_status rrtl_ctx_event_elapsed(rrtl_ctx* ctx, uint32_t a, uint32_t b, float* ms);
rrtl_status rrtl_ctx_synchronize(rrtl_ctx* ctx);
/* Failure-detection self-check of the bounded device wait that the fused and
 * queue kernels use for their copies (no reference counterpart). One CTA
 * waits `polls` polls (1..2^22) on an mbarrier that nothing arrives on:
 * *wait_status is RRTL_E_TIMEOUT when that wait gave up, as it must (RRTL_OK
 * would mean it did not). It then arrives once and waits again: *completed
 * is 1 when that wait finished. No copy is in flight; the context stays
 * usable. */
rrtl_status rrtl_ctx_check_wait_timeout(rrtl_ctx* ctx, uint32_t polls, uint32_t* wait_status, uint32_t* completed);

/* ---- compiled design ---------------------------------------------------- */

/* Compile once: parse the serde-JSON of `rrtl_ir::Design`, flatten and lower
 * it (lower_to_packed_program / lower_to_machine_program,
 * crates/rrtl-sim-ir/src/lib.rs:592-672) and upload the device program.
 * Replaces GpuBatchSimulator::new / new_from_compiled (crates/rrtl-gpu-sim/src/lib.rs:497-530). */
rrtl_status rrtl_design_load_json(rrtl_ctx* ctx, const char* json, size_t len, const char* top, rrtl_design** out);
rrtl_status rrtl_design_destroy(rrtl_design* design);

typedef struct {
  uint32_t n_signals;          /* packed signals */
  uint32_t n_memories;
  uint64_t total_signal_words; /* PackedProgram::total_signal_words */
  uint64_t total_memory_words_per_lane;
  uint32_t engine;             /* RRTL_ENGINE_GATE (bit-sliced) or RRTL_ENGINE_WORD */
  uint32_t n_gates;            /* gate engine: LUT3 cells after mapping; word engine: instructions */
  uint32_t n_levels;           /* gate engine: logic levels; word engine: comb packets */
  uint32_t n_nets;             /* gate engine: materialised nets */
  uint32_t n_slots;            /* gate engine: on-chip net slots after liveness allocation */
  uint32_t n_regs;             /* registers (flip-flops for the gate engine) */
  uint64_t source_instrs;      /* machine-program instructions, all streams */
} rrtl_design_info;

enum { RRTL_ENGINE_GATE = 1, RRTL_ENGINE_WORD = 2 };

rrtl_status rrtl_design_info_get(rrtl_design* design, rrtl_design_info* out);
/* Look up a packed signal by name: either "<top>.<name>" or "<name>" for a
 * top-level signal. Writes its index, width and kind (0 in, 1 out, 2 wire, 3 reg). */
rrtl_status rrtl_design_signal(rrtl_design* design, const char* name, uint32_t* index, uint32_t* width, uint32_t* kind);
rrtl_status rrtl_design_memory(rrtl_design* design, const char* name, uint32_t* index, uint64_t* depth, uint32_t* width);

/* ---- lane batch ---------------------------------------------------------- */

/* Device lane state for `lanes` independent instances, zero-initialised and
 * settled (PackedSimulator::new evaluates comb once, crates/rrtl-sim-ir/src/lib.rs:3033-3060).
 * lanes == 0 fails with RRTL_E_LANES (E_GPU_LANES, crates/rrtl-gpu-sim/src/lib.rs:525-529). */
rrtl_status rrtl_batch_create(rrtl_design* design, uint32_t lanes, rrtl_batch** out);
rrtl_status rrtl_batch_destroy(rrtl_batch* b);
rrtl_status rrtl_batch_lanes(rrtl_batch* b, uint32_t* out);

/* GpuBatchSimulator::set_input_limbs (crates/rrtl-gpu-sim/src/lib.rs:836-843).
 * `lane_limbs` is [limbs][lanes]; n must equal limbs*lanes. Like the reference
 * it does not re-settle (crates/rrtl-gpu-sim/src/lib.rs:1514-1555). */
rrtl_status rrtl_batch_set_input_limbs(rrtl_batch* b, uint32_t signal, const uint32_t* lane_limbs, size_t n);
/* GpuBatchSimulator::get_signal_limbs (crates/rrtl-gpu-sim/src/lib.rs:860-876). Synchronises. */
rrtl_status rrtl_batch_get_signal_limbs(rrtl_batch* b, uint32_t signal, uint32_t* out, size_t n);
/* Bit-packed forms for 1-bit signals: word w bit k is lane 32*w+k. n = ceil(lanes/32). */
rrtl_status rrtl_batch_set_input_bits(rrtl_batch* b, uint32_t signal, const uint32_t* words, size_t n);
rrtl_status rrtl_batch_get_signal_bits(rrtl_batch* b, uint32_t signal, uint32_t* out, size_t n);

/* Bit-packed values of several 1-bit signals at once: out is [n][ceil(lanes/32)]. */
rrtl_status rrtl_batch_get_signals_bits(rrtl_batch* b, const uint32_t* signals, size_t n, uint32_t* out, size_t n_out);

/* GpuBatchSimulator::set_memory_limbs / get_memory_limbs
 * (crates/rrtl-gpu-sim/src/lib.rs:903-951). Layout [addr][limb][lane]. */
rrtl_status rrtl_batch_set_memory_limbs(rrtl_batch* b, uint32_t memory, const uint32_t* data, size_t n);
rrtl_status rrtl_batch_get_memory_limbs(rrtl_batch* b, uint32_t memory, uint32_t* out, size_t n);

/* GpuBatchSimulator::eval_combinational (crates/rrtl-gpu-sim/src/lib.rs:953-957). */
rrtl_status rrtl_batch_eval(rrtl_batch* b);
/* GpuBatchSimulator::tick: settle, capture, commit, settle (crates/rrtl-gpu-sim/src/lib.rs:966-971). */
rrtl_status rrtl_batch_tick(rrtl_batch* b);
/* GpuBatchSimulator::tick_many with inputs held (crates/rrtl-gpu-sim/src/lib.rs:973-987).
 * Asynchronous on the context stream like InterpGpuSimulator::tick_many
 * (crates/rrtl-gpu-sim/src/interp.rs:2020-2042); getters synchronise. */
rrtl_status rrtl_batch_tick_many(rrtl_batch* b, uint64_t steps);
rrtl_status rrtl_batch_synchronize(rrtl_batch* b);

/* ---- per-cycle stimulus and recording (trace replay) ----------------------
 * One run advances `cycles` clock cycles. Per cycle c, in order:
 *   1. every stimulated input takes its value for cycle c;
 *   2. the design settles (comb, then async resets);
 *   3. recorded signals are sampled (trace / hash / fault detection);
 *   4. registers capture, memories write, registers commit (then stuck-at
 *      forces on registers are re-applied).
 * This is the reference's replay step order: inputs, settle, check, tick
 * (crates/rrtl-sim-ir/src/lib.rs:9540-9568; crates/rrtl-gpu-sim/src/lib.rs:2892-3078).
 * After the last cycle the design is settled again, so getters see the state
 * a final tick would leave. */
enum {
  RRTL_STIM_HOLD = 0,   /* keep the current value */
  RRTL_STIM_RANDOM = 1, /* uniform bits from the counter hash (param = stream id), drawn per global lane */
  RRTL_STIM_PULSE = 2,  /* 1 for cycles < param, then 0 (a reset pulse) */
  RRTL_STIM_CONST = 3,  /* constant param on every lane */
  RRTL_STIM_TRACE = 4,  /* from input_trace column `param` */
  RRTL_STIM_RANDOM_UNIFORM = 5 /* uniform bits from the counter hash keyed on (seed, param, cycle) only: the
                                  same value on every lane, namely the value RANDOM gives global lane 0. This
                                  is fault simulation's stimulus: the golden lane and every faulted lane see
                                  one input sequence (set_signal_all, crates/rrtl-sim-ir/examples/fault_sim.rs:66-76) */
};

typedef struct {
  uint32_t signal;
  uint32_t kind;
  uint64_t param;
} rrtl_stim;

enum { RRTL_REC_TRACE = 1, RRTL_REC_HASH = 2, RRTL_REC_DETECT = 4, RRTL_REC_CHECK = 8 /* trace replay only */ };

typedef struct {
  uint64_t cycles;
  uint64_t seed;
  uint32_t n_stim;
  const rrtl_stim* stim;
  uint32_t n_record;
  const uint32_t* record;      /* recorded signals (1-bit for the gate engine) */
  uint32_t record_mode;        /* RRTL_REC_* bitmask */
  uint32_t n_trace_cols;       /* columns of input_trace */
  const uint32_t* input_trace; /* gate engine: [cycle][col][word]; word engine: [cycle][col][lane], limb l of a
                                  RRTL_STIM_TRACE signal read from column param + l */
  uint32_t* out_trace;         /* gate engine: [cycle][rec][word]; word engine: [cycle][rec][limb][lane] */
  uint64_t* out_hash;          /* [cycle] per-cycle output hash */
  uint32_t* detect;            /* [lanes] first cycle a lane's recorded signals differ from lane 0 of its
                                  32-lane word; 0xFFFFFFFF if never (gate engine only) */
  uint64_t lane_base;          /* global index of the batch's lane 0, a multiple of 32: RANDOM stimulus and the
                                  hash terms are keyed on global lanes (words), so batches at lane_base 0, L,
                                  2L, ... of one seed are shards of one run of their total lanes, and their
                                  per-cycle hashes add up (wrapping) to that run's (the reference's shard plan,
                                  RuntimeShardInfo::start_lane, crates/rrtl-runtime/src/lib.rs:168-175).
                                  Traces, input traces and detect stay indexed by the batch's own lanes. */
} rrtl_run;

/* Runs on the device. Host pointers in `run` are copied in and out inside the
 * call (use rrtl_batch_run_device for device-resident buffers). */
rrtl_status rrtl_batch_run(rrtl_batch* b, const rrtl_run* run);

/* Same, with every buffer pointer in `run` a device pointer of the batch's
 * device; returns without synchronising. */
rrtl_status rrtl_batch_run_device(rrtl_batch* b, const rrtl_run* run);

/* ---- trace replay (GpuBatchSimulator::replay_lane_trace, crates/rrtl-gpu-sim/src/lib.rs:989-1357;
 * plan types GpuTraceReplayPlan / GpuTraceInputOp / GpuTraceCheckOp, :276-300) ----------------------
 * Per step: the step's input ops store their lane values, the design settles,
 * the step's checks compare one limb of a signal per lane with the expected
 * values, and the clock ticks; after the last step the design settles. A
 * signal keeps its value between input ops (starting from the batch state).
 * Mismatches go to `log` = [count, then (step, check_index, lane, limb,
 * expected, actual) for up to max_mismatches of them, in no fixed order];
 * *n_mismatches is the full count. Gate engine: 1-bit signals, limb 0. */
typedef struct {
  uint64_t step;
  uint32_t signal;
  uint32_t limb;
  const uint32_t* values;    /* [lanes] */
} rrtl_trace_input;

typedef struct {
  uint64_t step;
  uint32_t check_index;
  uint32_t signal;
  uint32_t limb;
  uint32_t pad;
  const uint32_t* expected;  /* [lanes] */
} rrtl_trace_check;

typedef struct {
  uint64_t steps;
  uint32_t n_inputs;
  const rrtl_trace_input* inputs;
  uint32_t n_checks;
  const rrtl_trace_check* checks;
} rrtl_trace;

rrtl_status rrtl_batch_replay_trace(rrtl_batch* b, const rrtl_trace* trace, uint32_t max_mismatches, uint32_t* log,
                                    uint64_t* n_mismatches);

/* ---- fault injection (BitParallelSimulator::set_force, crates/rrtl-sim-ir/src/bitparallel.rs:96-126) */
typedef struct {
  uint32_t lane;
  uint32_t signal;  /* packed signal index of a wire, output or register net */
  uint32_t value;   /* stuck-at value, 0 or 1 */
} rrtl_fault;

/* Replace the batch's fault list. Gate engine only. Lane 0 of every 32-lane
 * word is the fault-free reference for RRTL_REC_DETECT, so faults on those
 * lanes are rejected. */
rrtl_status rrtl_batch_set_faults(rrtl_batch* b, const rrtl_fault* faults, size_t n);

/* ---- snapshots (GpuBatchSimulator::snapshot_storage / restore_storage,
 * crates/rrtl-gpu-sim/src/lib.rs:1363-1408) ------------------------------- */
/* values: total_signal_words*lanes words in [(offset+limb)][lane] order (the
 * PackedSimulatorStorage::values layout); memories: total_memory_words_per_lane*lanes
 * words in [lane][word] order (PackedSimulatorStorage::memories). */
rrtl_status rrtl_batch_snapshot(rrtl_batch* b, uint32_t* values, size_t nv, uint32_t* memories, size_t nm);
rrtl_status rrtl_batch_restore(rrtl_batch* b, const uint32_t* values, size_t nv, const uint32_t* memories, size_t nm);

/* ---- execution path selection -------------------------------------------
 * RRTL_PATH_FUSED: persistent multi-cycle kernel with on-chip net slots (default).
 * RRTL_PATH_PLAIN: one kernel launch per cycle, nets in HBM (the baseline).
 * RRTL_PATH_PLAIN_GRAPH: the plain path's per-cycle launches of one run
 *   captured into a CUDA graph and submitted as one graph launch.
 * RRTL_PATH_WORD_INTERP: word engine, one launch of the interpreted kernel
 *   for the whole run even when the design has a compiled kernel (the fused
 *   path runs the compiled one); gate-engine batches treat it as FUSED. */
enum { RRTL_PATH_FUSED = 0, RRTL_PATH_PLAIN = 1, RRTL_PATH_PLAIN_GRAPH = 2, RRTL_PATH_WORD_INTERP = 3 };
rrtl_status rrtl_batch_set_path(rrtl_batch* b, uint32_t path);

/* Gate engine, fused path: 32-lane words per tile (8, 4, 2 or 1; 0 = chosen
 * per run from the design's level profile and the batch's size). A tile's
 * nets occupy W words of shared memory each, so designs with many live nets
 * run narrower tiles. No counterpart in the reference (an engine tuning knob).
 * rrtl_batch_tile_words reports the width of the last fused run (0 after a
 * run on the plain path). */
rrtl_status rrtl_batch_set_tile_words(rrtl_batch* b, uint32_t words);

/* Autotuner (the reference's GPU autotune, crates/rrtl-gpu-sim/src/lib.rs:103-172,
 * 2712-2721, re-aimed at this engine's knob): times `cycles` cycles of a
 * scratch batch of `lanes` lanes at every tile width that fits and makes the
 * fastest the choice for batches of that size (same power-of-two bucket of
 * 32-lane words). Gate engine; the word engine has no width and reports 0. */
rrtl_status rrtl_design_autotune(rrtl_design* design, uint32_t lanes, uint32_t cycles, uint32_t* best_words,
                                 float* best_ms);
rrtl_status rrtl_batch_tile_words(rrtl_batch* b, uint32_t* words);

/* Autotune recommendation table (the reference's GpuAutotuneRecommendation
 * records, crates/rrtl-gpu-sim/src/lib.rs:58-189): a JSON array of objects
 * {"case": string, "lanes": n, "steps": n, "tile_words": 8|4|2|1|0,
 *  "autotune_metric": string, "autotune_metric_ns": n or null}, tile_words 0
 * meaning the compiled gate kernel. The table is the caller's to keep (a
 * file); the library writes one record and reads a table.
 *
 * rrtl_design_autotune_recommend runs rrtl_design_autotune for `lanes` lanes
 * and `steps` cycles and writes that record for `case_name` (JSON text, NUL
 * terminated; *len is its length, also when cap is too small).
 *
 * rrtl_autotune_find picks a record as the reference does
 * (find_gpu_autotune_recommendation_with_mode, :123-144): mode
 * RRTL_AUTOTUNE_EXACT needs case, lanes and steps equal; RRTL_AUTOTUNE_NEAREST
 * takes the record of the same case with the smallest lane distance, then
 * step distance, then metric, lanes and steps (autotune_match_key,
 * :175-189). No device. RRTL_E_ARG with E_GPU_AUTOTUNE_JSON for a table that
 * does not parse; RRTL_E_ARG with E_GPU_AUTOTUNE_RECOMMENDATION when no
 * record matches (:160-170).
 *
 * rrtl_design_autotune_apply finds the record the same way and makes its
 * choice the design's for batches of `lanes` lanes (the power-of-two bucket
 * rrtl_design_autotune fills); *tile_words gets the choice. RRTL_E_ARG with
 * E_GPU_AUTOTUNE_RECOMMENDATION when the record's choice does not fit this
 * design (a width whose slots do not fit, or the compiled kernel for a
 * design past its size limit). */
enum { RRTL_AUTOTUNE_EXACT = 0, RRTL_AUTOTUNE_NEAREST = 1 };
rrtl_status rrtl_design_autotune_recommend(rrtl_design* design, const char* case_name, uint32_t lanes,
                                           uint32_t steps, char* json, size_t cap, size_t* len);
rrtl_status rrtl_autotune_find(const char* table, size_t table_len, const char* case_name, uint64_t lanes,
                               uint64_t steps, uint32_t mode, uint32_t* index);
rrtl_status rrtl_design_autotune_apply(rrtl_design* design, const char* table, size_t table_len,
                                       const char* case_name, uint32_t lanes, uint64_t steps, uint32_t mode,
                                       uint32_t* tile_words);

/* Device time of the last run/tick_many in milliseconds (CUDA events on the
 * context stream around the kernels of that call). */
rrtl_status rrtl_batch_last_kernel_ms(rrtl_batch* b, float* ms);

/* ---- device job queue ------------------------------------------------------
 * The single-GPU form of the reference's lane-shard scheduler
 * (DistributedRuntime, crates/rrtl-runtime/src/lib.rs:6785-7760): jobs are
 * runs on gate-engine batches of any design, lane count, cycle count and
 * fault list. rrtl_queue_launch packs every queued job into one persistent
 * kernel that drains a device-side list of (job, tile) items, longest first,
 * so uneven jobs share the GPU. A job's results are exactly those of
 * rrtl_batch_run on the same batch. The run's arrays are copied at submit;
 * its output buffers must stay valid until the job is finished. A batch
 * holds at most one unfinished job. No counterpart in the reference's API
 * (its scheduler is a Rust type, not a C ABI). */
typedef struct {
  rrtl_batch* batch;
  rrtl_run run;
} rrtl_job;

enum { RRTL_JOB_QUEUED = 0, RRTL_JOB_RUNNING = 1, RRTL_JOB_DONE = 2, RRTL_JOB_FAILED = 3 };

rrtl_status rrtl_queue_submit(rrtl_ctx* ctx, const rrtl_job* job, uint64_t* id);
/* Launch every queued job (asynchronous). */
rrtl_status rrtl_queue_launch(rrtl_ctx* ctx);
/* Wait for every launched job and copy its outputs to the caller's buffers. */
rrtl_status rrtl_queue_wait(rrtl_ctx* ctx);
/* RRTL_JOB_*; a finished launch is completed (outputs copied) by the poll. */
rrtl_status rrtl_queue_poll(rrtl_ctx* ctx, uint64_t id, uint32_t* status);
/* Device time of the last launch (ms), valid after rrtl_queue_wait. */
rrtl_status rrtl_queue_last_ms(rrtl_ctx* ctx, float* ms);

/* ---- lane-shard runtime ------------------------------------------------------
 * The reference's DistributedRuntime splits a run's lanes into contiguous
 * shards (RuntimeShardInfo{worker, start_lane, lanes},
 * crates/rrtl-runtime/src/lib.rs:168-175) and runs each on a worker engine
 * (:6785-7760); RuntimeEngine::Gpu holds its GPU engine (:7785-7792). Here a
 * runtime holds one lane batch per shard of one design on one GPU: a run goes
 * to every shard with lane_base = the run's lane_base + the shard's first
 * lane (so stimulus and hashes follow global lanes); gate-engine shards run
 * as the jobs of one device job-queue launch, word-engine shards one after
 * another. Outputs are in global-lane order: out_hash is the wrapping sum of
 * the shards' hashes (the hash of the whole run), detect and out_trace hold
 * every shard's lanes at their global positions, and input_trace columns are
 * cut per shard. Shards start on multiples of 32 lanes. */
typedef struct {
  uint32_t worker;      /* shard index */
  uint32_t lanes;
  uint64_t start_lane;  /* global index of the shard's lane 0 */
} rrtl_shard_info;

typedef struct rrtl_runtime rrtl_runtime;

/* Contiguous shards of total_lanes lanes over n shards (out: n entries). */
rrtl_status rrtl_shard_plan(uint64_t total_lanes, uint32_t n, rrtl_shard_info* out);
rrtl_status rrtl_runtime_create(rrtl_design* design, uint64_t total_lanes, uint32_t shards, rrtl_runtime** out);
rrtl_status rrtl_runtime_destroy(rrtl_runtime* rt);
/* Shard k's plan entry and lane batch (the batch belongs to the runtime). */
rrtl_status rrtl_runtime_shard(rrtl_runtime* rt, uint32_t k, rrtl_shard_info* info, rrtl_batch** batch);
/* Stuck-at faults on global lanes, handed to the shards that hold them (gate engine). */
rrtl_status rrtl_runtime_set_faults(rrtl_runtime* rt, const rrtl_fault* faults, size_t n);
/* One run over every shard; host buffers as for rrtl_batch_run, sized for all lanes. */
rrtl_status rrtl_runtime_run(rrtl_runtime* rt, const rrtl_run* run);

/* ---- serving loop ----------------------------------------------------------
 * Continuous batching of simulation requests on one GPU. Producer threads
 * submit requests (a design, a lane count, a run and optional faults); a
 * device-owner thread admits them first come first served while their device
 * state fits the memory budget, keeps each request's lane state on the device
 * until it finishes, and drives rounds in which every active request advances
 * by up to `chunk_cycles` cycles (gate-engine requests share one launch of
 * the persistent job-queue kernel). Requests arriving during a round join at
 * the next one. Each result equals the same run alone on a fresh batch. While
 * a server runs, its context must not be used from other threads except
 * through rrtl_server_* calls. No counterpart in the reference's API. */
typedef struct rrtl_server rrtl_server;

typedef struct {
  uint64_t hbm_budget;    /* bytes of device memory for request state; 0 = 90% of free memory */
  uint32_t chunk_cycles;  /* cycles each active request advances per round; 0 = 256 */
  uint32_t max_active;    /* requests on the device at once; 0 = no limit */
  uint32_t round_us;      /* target round time: gate-engine chunks are sized per request from its
                             program's cost so a round lasts about this long; 0 = fixed chunks */
  uint32_t policy;        /* RRTL_SERVE_FAIR: every active request shares each round;
                             RRTL_SERVE_SHORTEST_FIRST: the gate-engine requests with the least work left
                             (as many as fill the SMs twice) share the round, the others advance by a minimum
                             chunk, so short requests are not held to the pace of long ones */
} rrtl_server_opts;

enum { RRTL_SERVE_FAIR = 0, RRTL_SERVE_SHORTEST_FIRST = 1 };

typedef struct {
  uint32_t memory;        /* memory index (rrtl_design_memory) */
  const uint32_t* data;   /* [addr][limb][lane], as rrtl_batch_set_memory_limbs */
  size_t n;
} rrtl_mem_init;

typedef struct {
  rrtl_design* design;
  uint32_t lanes;
  uint32_t n_faults;
  const rrtl_fault* faults;      /* gate engine: stuck-at faults of the request's lanes */
  uint32_t n_mem_init;
  const rrtl_mem_init* mem_init; /* word engine: memory contents loaded before the run */
  rrtl_run run;                  /* host output buffers, filled when the request finishes */
} rrtl_request;

typedef struct {
  uint32_t status;   /* RRTL_JOB_* */
  uint64_t submit_ns, admit_ns, done_ns;  /* steady-clock times (0 = not yet) */
} rrtl_request_info;

typedef struct {
  uint64_t rounds, completed, failed, lane_cycles, busy_ns, pending;
} rrtl_server_stats;

rrtl_status rrtl_server_create(rrtl_ctx* ctx, const rrtl_server_opts* opts, rrtl_server** out);
/* Thread-safe. The request's arrays are copied; its output buffers must stay
 * valid until it finishes. */
rrtl_status rrtl_server_submit(rrtl_server* s, const rrtl_request* req, uint64_t* id);
rrtl_status rrtl_server_info(rrtl_server* s, uint64_t id, rrtl_request_info* info);
/* Block until the request finishes (timeout_ms 0 = no limit); returns its error if it failed. */
rrtl_status rrtl_server_wait(rrtl_server* s, uint64_t id, uint32_t timeout_ms);
rrtl_status rrtl_server_drain(rrtl_server* s);
rrtl_status rrtl_server_stats_get(rrtl_server* s, rrtl_server_stats* out);
/* Forget a finished request (its id becomes unknown). */
rrtl_status rrtl_server_release(rrtl_server* s, uint64_t id);
/* Finish every submitted request, stop the owner thread, free the server. */
rrtl_status rrtl_server_destroy(rrtl_server* s);

/* ---- allocation-free tick_many (word engine) -----------------------------
 * No counterpart in the reference: it exists for callers that may not call
 * cudaMalloc or cudaFree, such as a serving process that has divided device
 * memory among tenants up front and forbids later allocations, or a
 * latency-critical loop that cannot risk the implicit device synchronisation
 * cudaFree (and at times cudaMalloc) performs.
 *
 * Runs tick_many(steps) of a word-engine design (settle, then per step
 * capture, memory write, commit, settle) on lane state the caller owns:
 *   values   device array [total_signal_words][lanes_pad] of u32
 *   memories device array [total_memory_words_per_lane][lanes_pad] of u32
 *            (may be NULL when the design has no memories)
 * with lanes_pad = lanes rounded up to a multiple of 128; the word at
 * [word][lane] is limb `word` of lane `lane` in the PackedSimulatorStorage
 * order. The call allocates nothing: the register capture buffer it needs
 * lives in a fixed device array of 2^20 u32 words that the library defines,
 * so total capture words (one per register limb) x lanes_pad may not exceed
 * 2^20; larger requests fail with RRTL_E_ARG (E_NOALLOC_SIZE). Every GPU that
 * loads the library holds that array until the process exits. rrtl_ctx_create
 * looks up the array's device address (with the context's device current)
 * and the context keeps it, so this call does no set-up of its own.
 * `values` and `memories` must be device (or managed) memory of the design's
 * device: other pointers (host memory, another device's memory) fail with
 * RRTL_E_ARG before anything is launched. The call runs on the context's
 * stream, which does not wait for the legacy default stream or for the
 * caller's streams: finish every write to `values` and `memories` (for
 * example with a stream or device synchronise) before calling. All calls
 * share the array and it keeps the previous call's contents, which every call
 * overwrites before reading; calls whose work overlaps on the GPU race on it.
 * steps == 0 returns without launching anything. Returns after the work
 * finishes. */
rrtl_status rrtl_word_tick_many_noalloc(rrtl_design* design, uint32_t* values, uint32_t* memories, uint32_t lanes,
                                        uint64_t steps);

/* ---- per-design compiled word kernels ------------------------------------
 * A word-engine design is also emitted as straight-line CUDA C++ (one
 * statement per word instruction, value slots in registers) and compiled by
 * NVRTC for the device on its first fused run; the fused path then runs the
 * compiled kernel and RRTL_PATH_WORD_INTERP the interpreted one. This
 * replaces the reference's generated per-design kernels (WGSL tick_many,
 * crates/rrtl-gpu-sim/src/lib.rs:2857-2890, and gpu_codegen::emit_kernel,
 * crates/rrtl-sim-ir/src/gpu_codegen.rs:503-557). Designs over 20,000 word
 * instructions, or hosts without NVRTC, run interpreted.
 *
 * rrtl_design_word_jit: compiles the design's kernel if that has not been
 * tried yet; *active = 1 when the compiled kernel is in use, *compile_ms the
 * time emit + compile + load took. For a gate-engine design *active = 0.
 * rrtl_last_error() holds the reason when *active = 0. */
rrtl_status rrtl_design_word_jit(rrtl_design* design, uint32_t* active, float* compile_ms);

/* Emit (and, when arch is not NULL, e.g. "sm_103a", compile) the compiled
 * word kernel of a design without a device: for tests and inspection. With
 * run NULL the kernel serves any run; otherwise it is the kernel compiled for
 * that run's stimulus table, record table and record mode (the fused path
 * builds one per distinct set of tables, up to 64 per design, and runs with
 * more than 64 stimulus or record entries use the general one).
 * source: buffer of source_cap bytes for the NUL-terminated CUDA source (may
 * be NULL); *source_len its length. *cubin_bytes the compiled image's size
 * (0 when not compiled); log (may be NULL) the compiler's messages.
 * RRTL_E_UNSUPPORTED when the design is outside the word engine's scope
 * (values over 128 bits) or the compiler fails. Values of 65 to 128 bits
 * compute on 128-bit integers in pairs of value slots. */
rrtl_status rrtl_word_jit_emit(const char* json, size_t len, const char* top, const rrtl_run* run, const char* arch,
                               char* source, size_t source_cap, size_t* source_len, uint32_t* cubin_bytes, char* log,
                               size_t log_cap, uint32_t flags);
/* flags bit 0 (RRTL_JIT_SPLIT): with run, the two-warp form (two warps per 32
 * lanes, each evaluating the cones of its share of the registers and memory
 * writes, registers exchanged through shared memory at the clock edge), which
 * the fused path runs when the environment sets RRTL_WORD_JIT_SPLIT=2 (it
 * measured slower than one warp per 32 lanes); RRTL_E_UNSUPPORTED when the
 * design does not split
 * (asynchronous resets, combinational feedback, very uneven cones). */
enum { RRTL_JIT_SPLIT = 1 };

/* ---- per-design compiled gate kernels ---------------------------------------
 * A gate-engine run on the fused path without stuck-at forces, with an
 * automatic tile width, on a design of up to 8,192 cells, runs a gate kernel
 * compiled for the design and the run's tables: one thread per 32-lane word,
 * every net a register, one LOP3 per cell (the reference's per-design
 * compiled kernel, crates/rrtl-sim-ir/src/gpu_codegen.rs:503-557). Designs
 * whose live nets fit in registers (at most 192 at once) use it unless the
 * autotuner measured a tile width faster for the lane count (larger designs
 * spill and run faster on the fused kernel); rrtl_design_autotune times it as a candidate and
 * reports it as best_words = 0. rrtl_batch_tile_words reads 0 after such a
 * run. This call emits (and with arch compiles) that kernel without a device,
 * like rrtl_word_jit_emit; run is required (its signals are packed indices).
 * RRTL_E_UNSUPPORTED when the design is outside the gate engine. */
rrtl_status rrtl_gate_jit_emit(const char* json, size_t len, const char* top, const rrtl_run* run, const char* arch,
                               char* source, size_t source_cap, size_t* source_len, uint32_t* cubin_bytes, char* log,
                               size_t log_cap);

/* The fused gate kernel compiled for one design (fused path of
 * rrtl_batch_run on the gate engine): the generic kernel's code with a run
 * dispatch over only the truth-table classes the design's cells use, which
 * leaves room for a split barrier between pieces in runs without stuck-at
 * forces (about 10% faster on a 50k-gate netlist: 11 of 80 classes). Built on the first such run of a tile width and cached with the
 * design; RRTL_FUSED_JIT=0 in the environment keeps the generic kernel. This
 * call emits (and with arch compiles) it for tile width tile_words (1, 2, 4
 * or 8) without a device. RRTL_E_UNSUPPORTED when the design is outside the
 * gate engine. */
rrtl_status rrtl_gate_fused_jit_emit(const char* json, size_t len, const char* top, uint32_t tile_words,
                                     const char* arch, char* source, size_t source_cap, size_t* source_len,
                                     uint32_t* cubin_bytes, char* log, size_t log_cap);

/* The gate lowering of a design at one fused tile width, without a device
 * (no reference counterpart: the reference's interpreter encodes one record
 * per gate and has no shared-memory layout). Shared-memory accounting per
 * cycle of one tile: every group of G = 32/W cells reads each used input
 * position in one access per quarter-warp, which takes as many wavefronts as
 * the largest number of distinct slot rows sharing a bank residue
 * (operand_wavefronts) against one per distinct row set (operand_rows, the
 * conflict-free floor); the vector commit reads the D rows of G registers
 * per wavefront in commit order (commit_wavefronts against commit_groups).
 * RRTL_E_UNSUPPORTED when the design is outside the gate engine. */
typedef struct {
  uint32_t tile_words, group;  /* W and G = 32 / W */
  uint32_t cells, pad_cells, groups, levels, slots, classes;
  uint64_t operand_rows, operand_wavefronts;
  uint64_t commit_groups, commit_wavefronts;
} rrtl_gate_program_info;
rrtl_status rrtl_gate_program_info_get(const char* json, size_t len, const char* top, uint32_t tile_words,
                                       rrtl_gate_program_info* out);

/* ---- bit-sliced multi-bit designs --------------------------------------------
 * The reference's BitSliceSimulator (crates/rrtl-sim-ir/src/bitslice.rs:1-402)
 * keeps a W-bit signal as W bit-planes across lanes. rrtl_design_load_bitslice
 * rewrites a design's flattened packed program into 1-bit plane signals
 * ("<signal>[p]", plane p = bit p of every lane) whose per-plane operations
 * (bitwise, mux, ripple add/sub, xor/OR-reduce eq/ne, borrow-chain lt,
 * plane reindexing for slice/concat/extension) run on the bit-sliced gate
 * engine, 32 lanes per u32 word. Scope: no memories, no multiply, no
 * asynchronous reset (E_BITSLICE, RRTL_E_UNSUPPORTED). Inputs and outputs
 * are the planes: set and read them with the 1-bit signal calls (lane bits
 * packed 32 per word). rrtl_bitslice_json returns the plane design as
 * design JSON without a device (for inspection and the oracle). */
rrtl_status rrtl_design_load_bitslice(rrtl_ctx* ctx, const char* json, size_t len, const char* top, rrtl_design** out);
rrtl_status rrtl_bitslice_json(const char* json, size_t len, const char* top, char* out, size_t cap, size_t* out_len);

/* ---- instance folding ------------------------------------------------------
 * A top that is a flat wrapper of N >= 2 independent instances of one module
 * (no logic of its own, no instance output feeding an instance input, no
 * signal driven by two instances; shared inputs such as a clock allowed)
 * simulates as that child module over N x L lanes, instance i on lanes
 * [i*L, (i+1)*L): load the design with the child as top
 * (rrtl_design_load_json(ctx, json, len, child, ...)) and create a batch of
 * N x L lanes. This replaces analyze_instance_fold
 * (crates/rrtl-sim-ir/src/instance_fold.rs:42-97) and the plan side of
 * InstanceFoldPlan (crates/rrtl-gpu-sim/src/instance_fold.rs). No device is
 * needed. plan: buffer of cap bytes for the NUL-terminated JSON plan
 * {"child", "instances": [names], "connections": [[top_signal, instance,
 * port, "in"|"out"], ...]}; *plan_len its length. RRTL_E_UNSUPPORTED
 * (E_INSTANCE_FOLD: reason) when the design does not fold. */
rrtl_status rrtl_instance_fold_plan(const char* json, size_t len, const char* top, char* plan, size_t cap,
                                    size_t* plan_len);

#ifdef __cplusplus
}
#endif

#endif /* RRTL_CUDA_H */
