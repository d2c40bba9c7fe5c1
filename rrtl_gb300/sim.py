"""Python mirror of the reference's batch simulator API over the C ABI.

`GpuBatchSimulator` follows `rrtl_gpu_sim::GpuBatchSimulator`
(crates/rrtl-gpu-sim/src/lib.rs:458-1512): compile once, set inputs per lane,
tick / tick_many, read signals, memories and snapshots. Every call goes
through librrtl_gb300.so (include/rrtl_cuda.h); there is no CPU fallback, and
loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes
import json
import os
from ctypes import POINTER, byref, c_char_p, c_float, c_int32, c_size_t, c_uint32, c_uint64, c_void_p
from typing import Iterable, Optional, Sequence, Union

import numpy as np

from . import builder as _b

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "librrtl_gb300.so")

STIM_HOLD, STIM_RANDOM, STIM_PULSE, STIM_CONST, STIM_TRACE, STIM_RANDOM_UNIFORM = 0, 1, 2, 3, 4, 5
REC_TRACE, REC_HASH, REC_DETECT, REC_CHECK = 1, 2, 4, 8
PATH_FUSED, PATH_PLAIN, PATH_PLAIN_GRAPH, PATH_WORD_INTERP = 0, 1, 2, 3
JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3
ENGINE_GATE, ENGINE_WORD = 1, 2
SERVE_FAIR, SERVE_SHORTEST_FIRST = 0, 1

_STATUS = {
    1: "RRTL_E_ARG",
    2: "RRTL_E_DESIGN",
    3: "RRTL_E_SIGNAL",
    4: "RRTL_E_DEVICE",
    5: "RRTL_E_OOM",
    6: "RRTL_E_TIMEOUT",
    7: "RRTL_E_UNSUPPORTED",
    8: "RRTL_E_LANES",
}


class RrtlError(RuntimeError):
    """A failed C-ABI call: `status` is the rrtl_status, `code` the diagnostic code."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.code = message.split(":", 1)[0] if ":" in message else message
        super().__init__(f"{_STATUS.get(status, status)}: {message}")


class Stim(ctypes.Structure):
    _fields_ = [("signal", c_uint32), ("kind", c_uint32), ("param", c_uint64)]


class Run(ctypes.Structure):
    _fields_ = [
        ("cycles", c_uint64),
        ("seed", c_uint64),
        ("n_stim", c_uint32),
        ("stim", POINTER(Stim)),
        ("n_record", c_uint32),
        ("record", POINTER(c_uint32)),
        ("record_mode", c_uint32),
        ("n_trace_cols", c_uint32),
        ("input_trace", POINTER(c_uint32)),
        ("out_trace", POINTER(c_uint32)),
        ("out_hash", POINTER(c_uint64)),
        ("detect", POINTER(c_uint32)),
        ("lane_base", c_uint64),
    ]


class TraceInput(ctypes.Structure):
    _fields_ = [("step", c_uint64), ("signal", c_uint32), ("limb", c_uint32), ("values", POINTER(c_uint32))]


class TraceCheck(ctypes.Structure):
    _fields_ = [("step", c_uint64), ("check_index", c_uint32), ("signal", c_uint32), ("limb", c_uint32),
                ("pad", c_uint32), ("expected", POINTER(c_uint32))]


class Trace(ctypes.Structure):
    _fields_ = [("steps", c_uint64), ("n_inputs", c_uint32), ("inputs", POINTER(TraceInput)),
                ("n_checks", c_uint32), ("checks", POINTER(TraceCheck))]


class Job(ctypes.Structure):
    _fields_ = [("batch", c_void_p), ("run", Run)]


class Fault(ctypes.Structure):
    _fields_ = [("lane", c_uint32), ("signal", c_uint32), ("value", c_uint32)]


class GateProgramInfo(ctypes.Structure):
    _fields_ = [("tile_words", c_uint32), ("group", c_uint32), ("cells", c_uint32), ("pad_cells", c_uint32),
                ("groups", c_uint32), ("levels", c_uint32), ("slots", c_uint32), ("classes", c_uint32),
                ("operand_rows", c_uint64), ("operand_wavefronts", c_uint64), ("commit_groups", c_uint64),
                ("commit_wavefronts", c_uint64)]


class ShardInfo(ctypes.Structure):
    _fields_ = [("worker", c_uint32), ("lanes", c_uint32), ("start_lane", c_uint64)]


class DesignInfo(ctypes.Structure):
    _fields_ = [
        ("n_signals", c_uint32),
        ("n_memories", c_uint32),
        ("total_signal_words", c_uint64),
        ("total_memory_words_per_lane", c_uint64),
        ("engine", c_uint32),
        ("n_gates", c_uint32),
        ("n_levels", c_uint32),
        ("n_nets", c_uint32),
        ("n_slots", c_uint32),
        ("n_regs", c_uint32),
        ("source_instrs", c_uint64),
    ]


# Exported C-ABI symbols, as declared in include/rrtl_cuda.h.
EXPORTS = (
    "rrtl_last_error",
    "rrtl_ctx_create",
    "rrtl_ctx_destroy",
    "rrtl_ctx_sm_count",
    "rrtl_ctx_event_record",
    "rrtl_ctx_event_elapsed",
    "rrtl_ctx_synchronize",
    "rrtl_ctx_check_wait_timeout",
    "rrtl_design_load_json",
    "rrtl_design_destroy",
    "rrtl_design_info_get",
    "rrtl_design_signal",
    "rrtl_design_memory",
    "rrtl_batch_create",
    "rrtl_batch_destroy",
    "rrtl_batch_lanes",
    "rrtl_batch_set_input_limbs",
    "rrtl_batch_get_signal_limbs",
    "rrtl_batch_set_input_bits",
    "rrtl_batch_get_signal_bits",
    "rrtl_batch_get_signals_bits",
    "rrtl_batch_set_memory_limbs",
    "rrtl_batch_get_memory_limbs",
    "rrtl_batch_eval",
    "rrtl_batch_tick",
    "rrtl_batch_tick_many",
    "rrtl_batch_synchronize",
    "rrtl_batch_run",
    "rrtl_batch_run_device",
    "rrtl_batch_set_faults",
    "rrtl_batch_replay_trace",
    "rrtl_batch_snapshot",
    "rrtl_batch_restore",
    "rrtl_batch_set_path",
    "rrtl_batch_set_tile_words",
    "rrtl_design_autotune",
    "rrtl_queue_submit",
    "rrtl_queue_launch",
    "rrtl_queue_wait",
    "rrtl_queue_poll",
    "rrtl_queue_last_ms",
    "rrtl_server_create",
    "rrtl_server_submit",
    "rrtl_server_info",
    "rrtl_server_wait",
    "rrtl_server_drain",
    "rrtl_server_stats_get",
    "rrtl_server_release",
    "rrtl_server_destroy",
    "rrtl_batch_tile_words",
    "rrtl_batch_last_kernel_ms",
    "rrtl_word_tick_many_noalloc",
    "rrtl_design_word_jit",
    "rrtl_word_jit_emit",
    "rrtl_instance_fold_plan",
    "rrtl_gate_jit_emit",
    "rrtl_gate_fused_jit_emit",
    "rrtl_gate_program_info_get",
    "rrtl_design_autotune_recommend",
    "rrtl_autotune_find",
    "rrtl_design_autotune_apply",
    "rrtl_design_load_bitslice",
    "rrtl_bitslice_json",
    "rrtl_shard_plan",
    "rrtl_runtime_create",
    "rrtl_runtime_destroy",
    "rrtl_runtime_shard",
    "rrtl_runtime_set_faults",
    "rrtl_runtime_run",
)

_lib = None


def lib():
    """Load librrtl_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run rrtl_gb300.build.build() first")
    L = ctypes.CDLL(LIB_PATH)
    L.rrtl_last_error.restype = c_char_p
    P = POINTER
    sigs = {
        "rrtl_ctx_create": [c_int32, P(c_void_p)],
        "rrtl_ctx_destroy": [c_void_p],
        "rrtl_ctx_sm_count": [c_void_p, P(c_uint32)],
        "rrtl_ctx_event_record": [c_void_p, c_uint32],
        "rrtl_ctx_event_elapsed": [c_void_p, c_uint32, c_uint32, P(c_float)],
        "rrtl_ctx_synchronize": [c_void_p],
        "rrtl_ctx_check_wait_timeout": [c_void_p, c_uint32, P(c_uint32), P(c_uint32)],
        "rrtl_design_load_json": [c_void_p, c_char_p, c_size_t, c_char_p, P(c_void_p)],
        "rrtl_design_destroy": [c_void_p],
        "rrtl_design_info_get": [c_void_p, P(DesignInfo)],
        "rrtl_design_signal": [c_void_p, c_char_p, P(c_uint32), P(c_uint32), P(c_uint32)],
        "rrtl_design_memory": [c_void_p, c_char_p, P(c_uint32), P(c_uint64), P(c_uint32)],
        "rrtl_batch_create": [c_void_p, c_uint32, P(c_void_p)],
        "rrtl_batch_destroy": [c_void_p],
        "rrtl_batch_lanes": [c_void_p, P(c_uint32)],
        "rrtl_batch_set_input_limbs": [c_void_p, c_uint32, P(c_uint32), c_size_t],
        "rrtl_batch_get_signal_limbs": [c_void_p, c_uint32, P(c_uint32), c_size_t],
        "rrtl_batch_set_input_bits": [c_void_p, c_uint32, P(c_uint32), c_size_t],
        "rrtl_batch_get_signal_bits": [c_void_p, c_uint32, P(c_uint32), c_size_t],
        "rrtl_batch_get_signals_bits": [c_void_p, P(c_uint32), c_size_t, P(c_uint32), c_size_t],
        "rrtl_batch_set_memory_limbs": [c_void_p, c_uint32, P(c_uint32), c_size_t],
        "rrtl_batch_get_memory_limbs": [c_void_p, c_uint32, P(c_uint32), c_size_t],
        "rrtl_batch_eval": [c_void_p],
        "rrtl_batch_tick": [c_void_p],
        "rrtl_batch_tick_many": [c_void_p, c_uint64],
        "rrtl_batch_synchronize": [c_void_p],
        "rrtl_batch_run": [c_void_p, P(Run)],
        "rrtl_batch_run_device": [c_void_p, P(Run)],
        "rrtl_batch_set_faults": [c_void_p, P(Fault), c_size_t],
        "rrtl_batch_replay_trace": [c_void_p, P(Trace), c_uint32, P(c_uint32), P(c_uint64)],
        "rrtl_batch_snapshot": [c_void_p, P(c_uint32), c_size_t, P(c_uint32), c_size_t],
        "rrtl_batch_restore": [c_void_p, P(c_uint32), c_size_t, P(c_uint32), c_size_t],
        "rrtl_batch_set_path": [c_void_p, c_uint32],
        "rrtl_batch_set_tile_words": [c_void_p, c_uint32],
        "rrtl_design_autotune": [c_void_p, c_uint32, c_uint32, P(c_uint32), P(c_float)],
        "rrtl_queue_submit": [c_void_p, P(Job), P(c_uint64)],
        "rrtl_queue_launch": [c_void_p],
        "rrtl_queue_wait": [c_void_p],
        "rrtl_queue_poll": [c_void_p, c_uint64, P(c_uint32)],
        "rrtl_queue_last_ms": [c_void_p, P(c_float)],
        "rrtl_server_create": [c_void_p, P(ServerOpts), P(c_void_p)],
        "rrtl_server_submit": [c_void_p, P(Request), P(c_uint64)],
        "rrtl_server_info": [c_void_p, c_uint64, P(RequestInfo)],
        "rrtl_server_wait": [c_void_p, c_uint64, c_uint32],
        "rrtl_server_drain": [c_void_p],
        "rrtl_server_stats_get": [c_void_p, P(ServerStats)],
        "rrtl_server_release": [c_void_p, c_uint64],
        "rrtl_server_destroy": [c_void_p],
        "rrtl_batch_tile_words": [c_void_p, P(c_uint32)],
        "rrtl_batch_last_kernel_ms": [c_void_p, P(c_float)],
        "rrtl_word_tick_many_noalloc": [c_void_p, c_void_p, c_void_p, c_uint32, c_uint64],
        "rrtl_design_word_jit": [c_void_p, P(c_uint32), P(c_float)],
        "rrtl_word_jit_emit": [c_char_p, c_size_t, c_char_p, c_void_p, c_char_p, c_char_p, c_size_t, P(c_size_t),
                               P(c_uint32), c_char_p, c_size_t, c_uint32],
        "rrtl_instance_fold_plan": [c_char_p, c_size_t, c_char_p, c_char_p, c_size_t, P(c_size_t)],
        "rrtl_design_load_bitslice": [c_void_p, c_char_p, c_size_t, c_char_p, P(c_void_p)],
        "rrtl_bitslice_json": [c_char_p, c_size_t, c_char_p, c_char_p, c_size_t, P(c_size_t)],
        "rrtl_gate_jit_emit": [c_char_p, c_size_t, c_char_p, c_void_p, c_char_p, c_char_p, c_size_t, P(c_size_t),
                               P(c_uint32), c_char_p, c_size_t],
        "rrtl_gate_fused_jit_emit": [c_char_p, c_size_t, c_char_p, c_uint32, c_char_p, c_char_p, c_size_t, P(c_size_t),
                                     P(c_uint32), c_char_p, c_size_t],
        "rrtl_gate_program_info_get": [c_char_p, c_size_t, c_char_p, c_uint32, P(GateProgramInfo)],
        "rrtl_design_autotune_recommend": [c_void_p, c_char_p, c_uint32, c_uint32, c_char_p, c_size_t, P(c_size_t)],
        "rrtl_autotune_find": [c_char_p, c_size_t, c_char_p, c_uint64, c_uint64, c_uint32, P(c_uint32)],
        "rrtl_design_autotune_apply": [c_void_p, c_char_p, c_size_t, c_char_p, c_uint32, c_uint64, c_uint32,
                                       P(c_uint32)],
        "rrtl_shard_plan": [c_uint64, c_uint32, P(ShardInfo)],
        "rrtl_runtime_create": [c_void_p, c_uint64, c_uint32, P(c_void_p)],
        "rrtl_runtime_destroy": [c_void_p],
        "rrtl_runtime_shard": [c_void_p, c_uint32, P(ShardInfo), P(c_void_p)],
        "rrtl_runtime_set_faults": [c_void_p, P(Fault), c_size_t],
        "rrtl_runtime_run": [c_void_p, P(Run)],
    }
    for name, args in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = c_int32
    _lib = L
    return L


def check(status: int):
    if status != 0:
        raise RrtlError(status, lib().rrtl_last_error().decode())


def _u32p(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_uint32))


class Context:
    """One device plus its stream (rrtl_ctx)."""

    def __init__(self, device: int = 0):
        self.h = c_void_p()
        check(lib().rrtl_ctx_create(device, byref(self.h)))

    @property
    def sm_count(self) -> int:
        n = c_uint32()
        check(lib().rrtl_ctx_sm_count(self.h, byref(n)))
        return n.value

    def record(self, slot: int):
        check(lib().rrtl_ctx_event_record(self.h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        f = c_float()
        check(lib().rrtl_ctx_event_elapsed(self.h, a, b, byref(f)))
        return f.value

    def synchronize(self):
        check(lib().rrtl_ctx_synchronize(self.h))

    def check_wait_timeout(self, polls: int = 256):
        """Run the bounded-wait self-check: (status of a wait on an mbarrier
        nothing arrives on -- RRTL_E_TIMEOUT is the expected answer --, whether
        the wait after one arrival completed)."""
        st, done = c_uint32(), c_uint32()
        check(lib().rrtl_ctx_check_wait_timeout(self.h, polls, byref(st), byref(done)))
        return st.value, bool(done.value)

    # -- device job queue (rrtl_queue_*)
    def submit(self, batch: "GpuBatchSimulator", cycles: int, seed: int = 0, stim: Iterable = (),
               record: Iterable = (), mode: int = 0, input_trace: Optional[np.ndarray] = None,
               lane_base: int = 0) -> "QueuedJob":
        """Queue a run on `batch`; its outputs fill the returned job's arrays once it finishes."""
        out = batch.alloc_outputs(cycles, list(record), mode)
        r = batch.make_run(cycles, seed, stim, record, mode, input_trace, out["trace"], out["hash"], out["detect"],
                           lane_base)
        j = Job()
        j.batch = batch.h
        j.run = r
        jid = c_uint64()
        check(lib().rrtl_queue_submit(self.h, byref(j), byref(jid)))
        job = QueuedJob(self, jid.value, out, (r, batch))
        return job

    def launch(self):
        check(lib().rrtl_queue_launch(self.h))

    def wait(self):
        check(lib().rrtl_queue_wait(self.h))

    def poll(self, job_id: int) -> int:
        v = c_uint32()
        check(lib().rrtl_queue_poll(self.h, job_id, byref(v)))
        return v.value

    @property
    def queue_ms(self) -> float:
        f = c_float()
        check(lib().rrtl_queue_last_ms(self.h, byref(f)))
        return f.value

    def close(self):
        if self.h:
            lib().rrtl_ctx_destroy(self.h)
            self.h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class QueuedJob:
    """A job in a context's device queue; `outputs` holds trace/hash/detect arrays."""

    def __init__(self, ctx: Context, job_id: int, outputs: dict, keep):
        self.ctx, self.id, self.outputs, self._keep = ctx, job_id, outputs, keep

    @property
    def status(self) -> int:
        return self.ctx.poll(self.id)


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def word_jit_emit(design: Union[_b.Design, str], top: str, arch: Optional[str] = None, run: Optional["Run"] = None,
                  split: bool = False):
    """CUDA source of a design's compiled word kernel (for any run, or for the
    tables of `run`, a Run whose signals are packed indices), and with `arch`
    its NVRTC compile (no device needed): (source, cubin bytes, compiler log)."""
    text = design.to_json() if isinstance(design, _b.Design) else design
    raw = text.encode()
    rp = ctypes.cast(byref(run), c_void_p) if run is not None else None
    n = c_size_t()
    fl = 1 if split else 0
    check(lib().rrtl_word_jit_emit(raw, len(raw), top.encode(), rp, None, None, 0, byref(n), None, None, 0, fl))
    src = ctypes.create_string_buffer(n.value + 1)
    logb = ctypes.create_string_buffer(1 << 16)
    cub = c_uint32()
    check(lib().rrtl_word_jit_emit(raw, len(raw), top.encode(), rp, arch.encode() if arch else None, src,
                                   n.value + 1, byref(n), byref(cub), logb, len(logb), fl))
    return src.value.decode(), cub.value, logb.value.decode()


def gate_jit_emit(design: Union[_b.Design, str], top: str, run: "Run", arch: Optional[str] = None):
    """CUDA source of the compiled gate kernel for `run`'s tables (a Run whose
    signals are packed indices), and with `arch` its NVRTC compile (no device
    needed): (source, cubin bytes, compiler log)."""
    text = design.to_json() if isinstance(design, _b.Design) else design
    raw = text.encode()
    rp = ctypes.cast(byref(run), c_void_p)
    n = c_size_t()
    check(lib().rrtl_gate_jit_emit(raw, len(raw), top.encode(), rp, None, None, 0, byref(n), None, None, 0))
    src = ctypes.create_string_buffer(n.value + 1)
    logb = ctypes.create_string_buffer(1 << 16)
    cub = c_uint32()
    check(lib().rrtl_gate_jit_emit(raw, len(raw), top.encode(), rp, arch.encode() if arch else None, src,
                                   n.value + 1, byref(n), byref(cub), logb, len(logb)))
    return src.value.decode(), cub.value, logb.value.decode()


AUTOTUNE_EXACT, AUTOTUNE_NEAREST = 0, 1


def autotune_find(table, case: str, lanes: int, steps: int, nearest: bool = False) -> int:
    """Index of the recommendation for (case, lanes, steps) in `table` (a list
    of records or its JSON text), by the reference's exact or nearest rule
    (rrtl_autotune_find; no device)."""
    import json as _json

    text = table if isinstance(table, str) else _json.dumps(table)
    raw = text.encode()
    i = c_uint32()
    check(lib().rrtl_autotune_find(raw, len(raw), case.encode(), lanes, steps,
                                   AUTOTUNE_NEAREST if nearest else AUTOTUNE_EXACT, byref(i)))
    return i.value


def gate_program_info(design: Union[_b.Design, str], top: str, tile_words: int = 8) -> dict:
    """The gate lowering at one fused tile width (rrtl_gate_program_info_get):
    cell, group, level, slot and class counts and the shared-memory
    wavefronts of its operand reads and register commit against their
    conflict-free floors."""
    text = design.to_json() if isinstance(design, _b.Design) else design
    raw = text.encode()
    info = GateProgramInfo()
    check(lib().rrtl_gate_program_info_get(raw, len(raw), top.encode(), tile_words, byref(info)))
    return {name: getattr(info, name) for name, _ in GateProgramInfo._fields_}


def gate_fused_jit_emit(design: Union[_b.Design, str], top: str, tile_words: int = 8, arch: Optional[str] = None):
    """CUDA source of the fused gate kernel compiled for the design's
    truth-table classes at `tile_words`, and with `arch` its NVRTC compile (no
    device needed): (source, cubin bytes, compiler log)."""
    text = design.to_json() if isinstance(design, _b.Design) else design
    raw = text.encode()
    n = c_size_t()
    check(lib().rrtl_gate_fused_jit_emit(raw, len(raw), top.encode(), tile_words, None, None, 0, byref(n), None, None,
                                         0))
    src = ctypes.create_string_buffer(n.value + 1)
    logb = ctypes.create_string_buffer(1 << 16)
    cub = c_uint32()
    check(lib().rrtl_gate_fused_jit_emit(raw, len(raw), top.encode(), tile_words, arch.encode() if arch else None, src,
                                         n.value + 1, byref(n), byref(cub), logb, len(logb)))
    return src.value.decode(), cub.value, logb.value.decode()


class CompiledDesign:
    """A design compiled and uploaded once (rrtl_design)."""

    def __init__(self, design: Union[_b.Design, str], top: str, ctx: Optional[Context] = None, bitslice: bool = False):
        self.ctx = ctx or default_context()
        text = design.to_json() if isinstance(design, _b.Design) else design
        raw = text.encode()
        self.h = c_void_p()
        load = lib().rrtl_design_load_bitslice if bitslice else lib().rrtl_design_load_json
        check(load(self.ctx.h, raw, len(raw), top.encode(), byref(self.h)))
        self.top = top
        self._cache = {}

    @property
    def info(self) -> DesignInfo:
        i = DesignInfo()
        check(lib().rrtl_design_info_get(self.h, byref(i)))
        return i

    def signal(self, name: str):
        """(index, width, kind) of a signal by name."""
        if name in self._cache:
            return self._cache[name]
        idx, w, k = c_uint32(), c_uint32(), c_uint32()
        check(lib().rrtl_design_signal(self.h, name.encode(), byref(idx), byref(w), byref(k)))
        self._cache[name] = (idx.value, w.value, k.value)
        return self._cache[name]

    def autotune(self, lanes: int, cycles: int = 32):
        """Time every fitting tile width on `lanes` lanes; returns (best words, ms of `cycles` cycles)."""
        w, ms = c_uint32(), c_float()
        check(lib().rrtl_design_autotune(self.h, lanes, cycles, byref(w), byref(ms)))
        return w.value, ms.value

    def autotune_recommend(self, case: str, lanes: int, steps: int = 32) -> dict:
        """Autotune for `lanes` lanes and `steps` cycles and return the
        recommendation record for `case` (rrtl_design_autotune_recommend)."""
        import json as _json

        n = c_size_t()
        buf = ctypes.create_string_buffer(2 * len(case.encode()) + 512)  # the record is the case name and five numbers
        check(lib().rrtl_design_autotune_recommend(self.h, case.encode(), lanes, steps, buf, len(buf), byref(n)))
        return _json.loads(buf.value.decode())

    def autotune_apply(self, table, case: str, lanes: int, steps: int, nearest: bool = False) -> int:
        """Make the recommendation for (case, lanes, steps) in `table` (a list
        of records or its JSON text) this design's choice for batches of
        `lanes` lanes; returns its tile width (0: the compiled gate kernel)."""
        import json as _json

        text = table if isinstance(table, str) else _json.dumps(table)
        raw = text.encode()
        w = c_uint32()
        check(lib().rrtl_design_autotune_apply(self.h, raw, len(raw), case.encode(), lanes, steps,
                                               AUTOTUNE_NEAREST if nearest else AUTOTUNE_EXACT, byref(w)))
        return w.value

    def word_jit(self):
        """Compile the design's word kernel if not yet tried: (active, compile ms, reason if inactive)."""
        act, ms = c_uint32(), c_float()
        check(lib().rrtl_design_word_jit(self.h, byref(act), byref(ms)))
        return bool(act.value), ms.value, ("" if act.value else lib().rrtl_last_error().decode())

    def memory(self, name: str):
        idx, depth, w = c_uint32(), c_uint64(), c_uint32()
        check(lib().rrtl_design_memory(self.h, name.encode(), byref(idx), byref(depth), byref(w)))
        return idx.value, depth.value, w.value

    def close(self):
        if self.h:
            lib().rrtl_design_destroy(self.h)
            self.h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SignalRef = Union[str, int, "_b.Signal"]


class GpuBatchSimulator:
    """`lanes` independent instances of one compiled design on the GPU."""

    def __init__(self, design: Union[CompiledDesign, _b.Design, str], top: Optional[str] = None, lanes: int = 1,
                 ctx: Optional[Context] = None):
        if not isinstance(design, CompiledDesign):
            design = CompiledDesign(design, top, ctx)
        self.design = design
        self._names = design._builder_names if hasattr(design, "_builder_names") else None
        self.h = c_void_p()
        check(lib().rrtl_batch_create(design.h, lanes, byref(self.h)))
        self.lanes = lanes
        self._keep = None

    # -- signal addressing
    def _sig(self, s: SignalRef):
        if isinstance(s, int):
            return s
        if isinstance(s, str):
            return self.design.signal(s)[0]
        raise TypeError("signals are addressed by name or packed index")

    def _limbs(self, idx: int) -> int:
        return None

    def signal_width(self, s: SignalRef) -> int:
        if isinstance(s, str):
            return self.design.signal(s)[1]
        raise TypeError("use a name")

    # -- I/O (crates/rrtl-gpu-sim/src/lib.rs:820-951)
    def set_input(self, s: SignalRef, lane_values: Sequence[int]):
        name = s
        w = self.design.signal(name)[1] if isinstance(name, str) else 32
        if w > 32:
            raise RrtlError(1, "E_GPU_WIDE_SIGNAL: use set_input_limbs for signals wider than 32 bits")
        a = np.ascontiguousarray(np.asarray(lane_values, dtype=np.uint64).astype(np.uint32))
        check(lib().rrtl_batch_set_input_limbs(self.h, self._sig(s), _u32p(a), a.size))

    def set_input_limbs(self, s: SignalRef, limbs_by_lane: np.ndarray):
        """limbs_by_lane: [limbs][lanes] uint32."""
        a = np.ascontiguousarray(limbs_by_lane, dtype=np.uint32)
        check(lib().rrtl_batch_set_input_limbs(self.h, self._sig(s), _u32p(a), a.size))

    def get_signal_limbs(self, s: SignalRef) -> np.ndarray:
        name = s
        w = self.design.signal(name)[1] if isinstance(name, str) else None
        if w is None:
            raise TypeError("use a name")
        limbs = max(1, (w + 31) // 32)
        out = np.zeros((limbs, self.lanes), dtype=np.uint32)
        check(lib().rrtl_batch_get_signal_limbs(self.h, self._sig(s), _u32p(out), out.size))
        return out

    def get_signal(self, s: SignalRef) -> np.ndarray:
        if isinstance(s, str) and self.design.signal(s)[1] > 32:
            raise RrtlError(1, "E_GPU_WIDE_SIGNAL: use get_signal_limbs for signals wider than 32 bits")
        return self.get_signal_limbs(s)[0]

    def set_input_bits(self, s: SignalRef, words: np.ndarray):
        a = np.ascontiguousarray(words, dtype=np.uint32)
        check(lib().rrtl_batch_set_input_bits(self.h, self._sig(s), _u32p(a), a.size))

    def get_signal_bits(self, s: SignalRef) -> np.ndarray:
        out = np.zeros((self.lanes + 31) // 32, dtype=np.uint32)
        check(lib().rrtl_batch_get_signal_bits(self.h, self._sig(s), _u32p(out), out.size))
        return out

    def get_signals_bits(self, signals) -> np.ndarray:
        """[n][ceil(lanes/32)] bit-packed values of several 1-bit signals."""
        idx = np.asarray([self._sig(s) for s in signals], dtype=np.uint32)
        words = (self.lanes + 31) // 32
        out = np.zeros((len(idx), words), dtype=np.uint32)
        check(lib().rrtl_batch_get_signals_bits(self.h, _u32p(idx), len(idx), _u32p(out), out.size))
        return out

    def set_memory_limbs(self, mem: str, data: np.ndarray):
        """data: [depth][limbs][lanes] uint32."""
        idx = self.design.memory(mem)[0]
        a = np.ascontiguousarray(data, dtype=np.uint32)
        check(lib().rrtl_batch_set_memory_limbs(self.h, idx, _u32p(a), a.size))

    def get_memory_limbs(self, mem: str) -> np.ndarray:
        idx, depth, w = self.design.memory(mem)
        limbs = max(1, (w + 31) // 32)
        out = np.zeros((depth, limbs, self.lanes), dtype=np.uint32)
        check(lib().rrtl_batch_get_memory_limbs(self.h, idx, _u32p(out), out.size))
        return out

    def set_memory(self, mem: str, lane_words: np.ndarray):
        """lane_words: [lanes][depth] values (<= 32 bits)."""
        a = np.asarray(lane_words, dtype=np.uint64)
        data = np.ascontiguousarray(a.T.astype(np.uint32)[:, None, :])
        self.set_memory_limbs(mem, data)

    def get_memory(self, mem: str) -> np.ndarray:
        return self.get_memory_limbs(mem)[:, 0, :].T.copy()

    # -- stepping (crates/rrtl-gpu-sim/src/lib.rs:953-987)
    def eval_combinational(self):
        check(lib().rrtl_batch_eval(self.h))

    def eval_combinational_many(self, iterations: int):
        """`iterations` settles in a row (GpuBatchSimulator::eval_combinational_many,
        crates/rrtl-gpu-sim/src/lib.rs:958-964); 0 does nothing."""
        for _ in range(iterations):
            check(lib().rrtl_batch_eval(self.h))

    def tick(self):
        check(lib().rrtl_batch_tick(self.h))

    def tick_many(self, steps: int):
        check(lib().rrtl_batch_tick_many(self.h, steps))
        self.synchronize()

    def tick_many_async(self, steps: int):
        check(lib().rrtl_batch_tick_many(self.h, steps))

    def synchronize(self):
        check(lib().rrtl_batch_synchronize(self.h))

    def set_path(self, path: int):
        check(lib().rrtl_batch_set_path(self.h, path))

    def set_tile_words(self, words: int):
        """Gate engine, fused path: 32-lane words per tile (8, 4, 2, 1; 0 = automatic)."""
        check(lib().rrtl_batch_set_tile_words(self.h, words))

    @property
    def tile_words(self) -> int:
        """Tile width of the last fused run (0 after a plain-path run)."""
        v = c_uint32()
        check(lib().rrtl_batch_tile_words(self.h, byref(v)))
        return v.value

    @property
    def last_kernel_ms(self) -> float:
        f = c_float()
        check(lib().rrtl_batch_last_kernel_ms(self.h, byref(f)))
        return f.value

    # -- per-cycle runs
    def make_run(self, cycles: int, seed: int = 0, stim: Iterable = (), record: Iterable = (), mode: int = 0,
                 input_trace: Optional[np.ndarray] = None, out_trace=None, out_hash=None, detect=None,
                 lane_base: int = 0) -> Run:
        st = [(self._sig(s), k, p) for (s, k, p) in stim]
        arr = (Stim * max(1, len(st)))(*[Stim(a, b, c) for a, b, c in st])
        rec = np.asarray([self._sig(r) for r in record], dtype=np.uint32)
        r = Run()
        r.cycles = cycles
        r.seed = seed
        r.n_stim = len(st)
        r.stim = ctypes.cast(arr, POINTER(Stim))
        r.n_record = len(rec)
        r.record = _u32p(rec) if len(rec) else None
        r.record_mode = mode
        if input_trace is not None:
            input_trace = np.ascontiguousarray(input_trace, dtype=np.uint32)
            r.n_trace_cols = input_trace.shape[1]
            r.input_trace = _u32p(input_trace)
        r.out_trace = _u32p(out_trace) if out_trace is not None else None
        r.out_hash = out_hash.ctypes.data_as(POINTER(c_uint64)) if out_hash is not None else None
        r.detect = _u32p(detect) if detect is not None else None
        r.lane_base = lane_base
        r._keep = (arr, rec, input_trace, out_trace, out_hash, detect)
        return r

    def alloc_outputs(self, cycles: int, record: list, mode: int) -> dict:
        """Host arrays for a run's recorded outputs (None where not requested)."""
        engine = self.design.info.engine
        words = (self.lanes + 31) // 32
        out_trace = out_hash = detect = None
        if mode & REC_TRACE:
            if engine == ENGINE_GATE:
                out_trace = np.zeros((cycles, len(record), words), dtype=np.uint32)
            else:
                limbs = sum(max(1, (self.design.signal(r)[1] + 31) // 32) for r in record)
                out_trace = np.zeros((cycles, limbs, self.lanes), dtype=np.uint32)
        if mode & REC_HASH:
            out_hash = np.zeros(cycles, dtype=np.uint64)
        if mode & REC_DETECT:
            detect = np.zeros(self.lanes, dtype=np.uint32)
        return {"trace": out_trace, "hash": out_hash, "detect": detect}

    def run(self, cycles: int, seed: int = 0, stim: Iterable = (), record: Iterable = (), mode: int = 0,
            input_trace: Optional[np.ndarray] = None, lane_base: int = 0):
        """Run `cycles` cycles; returns dict(trace=..., hash=..., detect=...) for the requested records.
        lane_base: global index of this batch's lane 0 (a multiple of 32) when the batch is one shard of a
        larger run (random stimulus and hash terms follow global lanes)."""
        record = list(record)
        out = self.alloc_outputs(cycles, record, mode)
        r = self.make_run(cycles, seed, stim, record, mode, input_trace, out["trace"], out["hash"], out["detect"],
                          lane_base)
        check(lib().rrtl_batch_run(self.h, byref(r)))
        return out

    def replay_trace(self, steps: int, inputs: Sequence[tuple] = (), checks: Sequence[tuple] = (),
                     max_mismatches: int = 1024):
        """Trace replay (GpuBatchSimulator::replay_lane_trace). inputs: (step, signal, limb, values[lanes]);
        checks: (step, check_index, signal, limb, expected[lanes]). Returns (count, mismatches) with
        mismatches as (step, check_index, lane, limb, expected, actual) tuples (at most max_mismatches)."""
        keep = []
        ins = (TraceInput * max(1, len(inputs)))()
        for i, (st, sig, limb, vals) in enumerate(inputs):
            a = np.ascontiguousarray(vals, dtype=np.uint32)
            keep.append(a)
            ins[i] = TraceInput(st, self._sig(sig), limb, _u32p(a))
        chs = (TraceCheck * max(1, len(checks)))()
        for i, (st, ci, sig, limb, exp) in enumerate(checks):
            a = np.ascontiguousarray(exp, dtype=np.uint32)
            keep.append(a)
            chs[i] = TraceCheck(st, ci, self._sig(sig), limb, 0, _u32p(a))
        t = Trace(steps, len(inputs), ctypes.cast(ins, POINTER(TraceInput)), len(checks),
                  ctypes.cast(chs, POINTER(TraceCheck)))
        cap = max(1, max_mismatches)
        log = np.zeros(1 + 6 * cap, dtype=np.uint32)
        n = c_uint64()
        check(lib().rrtl_batch_replay_trace(self.h, byref(t), cap, _u32p(log), byref(n)))
        kept = min(n.value, cap)
        rows = log[1:1 + 6 * kept].reshape(kept, 6)
        return n.value, [tuple(int(x) for x in r) for r in rows]

    def set_faults(self, faults: Sequence[tuple]):
        """faults: (lane, signal, value) triples; signal by name or index."""
        arr = (Fault * max(1, len(faults)))(*[Fault(l, self._sig(s), v) for l, s, v in faults])
        check(lib().rrtl_batch_set_faults(self.h, arr, len(faults)))

    # -- snapshots (crates/rrtl-gpu-sim/src/lib.rs:1363-1408)
    def snapshot_storage(self):
        info = self.design.info
        v = np.zeros(info.total_signal_words * self.lanes, dtype=np.uint32)
        m = np.zeros(max(1, info.total_memory_words_per_lane * self.lanes), dtype=np.uint32)
        check(lib().rrtl_batch_snapshot(self.h, _u32p(v), v.size, _u32p(m), info.total_memory_words_per_lane * self.lanes))
        return v, m[: info.total_memory_words_per_lane * self.lanes]

    def restore_storage(self, values: np.ndarray, memories: np.ndarray):
        v = np.ascontiguousarray(values, dtype=np.uint32)
        m = np.ascontiguousarray(memories, dtype=np.uint32)
        if m.size == 0:
            m = np.zeros(1, dtype=np.uint32)
            nm = 0
        else:
            nm = m.size
        check(lib().rrtl_batch_restore(self.h, _u32p(v), v.size, _u32p(m), nm))

    def close(self):
        if self.h:
            lib().rrtl_batch_destroy(self.h)
            self.h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- serving --
class MemInit(ctypes.Structure):
    _fields_ = [("memory", c_uint32), ("data", POINTER(c_uint32)), ("n", c_size_t)]


class Request(ctypes.Structure):
    _fields_ = [("design", c_void_p), ("lanes", c_uint32), ("n_faults", c_uint32), ("faults", POINTER(Fault)),
                ("n_mem_init", c_uint32), ("mem_init", POINTER(MemInit)), ("run", Run)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("status", c_uint32), ("submit_ns", c_uint64), ("admit_ns", c_uint64), ("done_ns", c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("rounds", c_uint64), ("completed", c_uint64), ("failed", c_uint64), ("lane_cycles", c_uint64),
                ("busy_ns", c_uint64), ("pending", c_uint64)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("hbm_budget", c_uint64), ("chunk_cycles", c_uint32), ("max_active", c_uint32),
                ("round_us", c_uint32), ("policy", c_uint32)]


class _RunShape:
    """A design and a lane count: enough to build a run without a batch."""

    def __init__(self, design: CompiledDesign, lanes: int):
        self.design, self.lanes = design, lanes

    _sig = GpuBatchSimulator._sig
    make_run = GpuBatchSimulator.make_run
    alloc_outputs = GpuBatchSimulator.alloc_outputs


class ServedRequest:
    """A request submitted to a Server; `outputs` fills in when it finishes."""

    def __init__(self, server: "Server", rid: int, outputs: dict, keep):
        self.server, self.id, self.outputs, self._keep = server, rid, outputs, keep

    def info(self) -> dict:
        return self.server.info(self.id)

    def wait(self, timeout_ms: int = 0):
        self.server.wait(self.id, timeout_ms)
        return self.outputs


class Server:
    """The serving loop (rrtl_server_*): continuous batching of requests on one GPU."""

    def __init__(self, ctx: Optional[Context] = None, hbm_budget: int = 0, chunk_cycles: int = 0, max_active: int = 0,
                 round_us: int = 0, policy: int = 0):
        """policy: SERVE_FAIR (every active request shares each round) or
        SERVE_SHORTEST_FIRST (requests with the least work left go first)."""
        self.ctx = ctx or default_context()
        o = ServerOpts(hbm_budget, chunk_cycles, max_active, round_us, policy)
        self.h = c_void_p()
        check(lib().rrtl_server_create(self.ctx.h, byref(o), byref(self.h)))

    def submit(self, design: CompiledDesign, lanes: int, cycles: int, seed: int = 0, stim: Iterable = (),
               record: Iterable = (), mode: int = 0, faults: Sequence[tuple] = (),
               input_trace: Optional[np.ndarray] = None, memories: Optional[dict] = None) -> ServedRequest:
        """memories: {name: [addr][limb][lane] array} loaded before the run (word engine)."""
        shape = _RunShape(design, lanes)
        record = list(record)
        out = shape.alloc_outputs(cycles, record, mode)
        r = shape.make_run(cycles, seed, stim, record, mode, input_trace, out["trace"], out["hash"], out["detect"])
        fa = (Fault * max(1, len(faults)))(*[Fault(l, shape._sig(s), v) for l, s, v in faults])
        q = Request()
        q.design = design.h
        q.lanes = lanes
        q.n_faults = len(faults)
        q.faults = ctypes.cast(fa, POINTER(Fault))
        mems = [(design.memory(n)[0], np.ascontiguousarray(a, dtype=np.uint32).ravel()) for n, a in (memories or {}).items()]
        mi = (MemInit * max(1, len(mems)))(*[MemInit(i, _u32p(a), a.size) for i, a in mems])
        q.n_mem_init = len(mems)
        q.mem_init = ctypes.cast(mi, POINTER(MemInit))
        q.run = r
        rid = c_uint64()
        check(lib().rrtl_server_submit(self.h, byref(q), byref(rid)))
        return ServedRequest(self, rid.value, out, (r, fa, mi, mems, design))

    def info(self, rid: int) -> dict:
        i = RequestInfo()
        check(lib().rrtl_server_info(self.h, rid, byref(i)))
        return {"status": i.status, "submit_ns": i.submit_ns, "admit_ns": i.admit_ns, "done_ns": i.done_ns}

    def wait(self, rid: int, timeout_ms: int = 0):
        check(lib().rrtl_server_wait(self.h, rid, timeout_ms))

    def drain(self):
        check(lib().rrtl_server_drain(self.h))

    def release(self, rid: int):
        check(lib().rrtl_server_release(self.h, rid))

    @property
    def stats(self) -> dict:
        s = ServerStats()
        check(lib().rrtl_server_stats_get(self.h, byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self):
        if self.h:
            check(lib().rrtl_server_destroy(self.h))
            self.h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def instance_fold_plan(design: Union[_b.Design, str], top: str) -> dict:
    """The instance-fold plan of `top` (no device needed); raises RrtlError
    (code E_INSTANCE_FOLD) when the design does not fold."""
    text = design.to_json() if isinstance(design, _b.Design) else design
    raw = text.encode()
    n = c_size_t()
    check(lib().rrtl_instance_fold_plan(raw, len(raw), top.encode(), None, 0, byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    check(lib().rrtl_instance_fold_plan(raw, len(raw), top.encode(), buf, n.value + 1, byref(n)))
    return json.loads(buf.value.decode())


class InstanceFoldSimulator:
    """N independent instances of one module folded into the lane axis: the
    child module simulated over N x base_lanes lanes, instance i on lanes
    [i*base_lanes, (i+1)*base_lanes). Mirrors InstanceFoldSimulator
    (crates/rrtl-gpu-sim/src/instance_fold.rs): set_port / get_port address
    the child's ports over all lanes; set_top_input / get_top_output address
    the wrapper's own signals over base_lanes lanes, demultiplexed by lane
    block through the plan's connections."""

    def __init__(self, design: Union[_b.Design, str], top: str, base_lanes: int, ctx: Optional[Context] = None):
        text = design.to_json() if isinstance(design, _b.Design) else design
        self.plan = instance_fold_plan(text, top)
        self.n = len(self.plan["instances"])
        self.base_lanes = base_lanes
        self.sim = GpuBatchSimulator(text, self.plan["child"], self.n * base_lanes, ctx)
        self._in, self._out = {}, {}
        for tsig, inst, port, d in self.plan["connections"]:
            (self._out if d == "out" else self._in).setdefault(tsig, []).append((inst, port))

    @property
    def num_instances(self) -> int:
        return self.n

    @property
    def total_lanes(self) -> int:
        return self.n * self.base_lanes

    def instance_lane(self, inst: int, local: int) -> int:
        return inst * self.base_lanes + local

    def port_offset(self, port: str) -> Optional[int]:
        """Handle of a child input or output port (its packed signal index, what
        the C ABI's signal calls take), None when the child has no such port
        (InstanceFoldPlan::port_offset, crates/rrtl-gpu-sim/src/instance_fold.rs:45-55,
        which returns the storage offset the reference's own calls take)."""
        try:
            idx, _, kind = self.sim.design.signal(port)
        except RrtlError:
            return None
        return idx if kind in (0, 1) else None

    def synchronize(self):
        self.sim.synchronize()

    def set_port(self, port: str, limbs_by_lane: np.ndarray):
        """A child port over all lanes: [limbs][total_lanes]."""
        self.sim.set_input_limbs(port, limbs_by_lane)

    def get_port(self, port: str) -> np.ndarray:
        return self.sim.get_signal_limbs(port)

    def set_top_input(self, name: str, limbs_by_lane: np.ndarray):
        """A wrapper input over base_lanes lanes ([limbs][base_lanes]), written to
        the lane block of every instance port it drives."""
        vals = np.atleast_2d(np.asarray(limbs_by_lane, dtype=np.uint32))
        by_port = {}
        for inst, port in self._in.get(name, []):
            by_port.setdefault(port, []).append(inst)
        for port, insts in by_port.items():
            cur = self.get_port(port)
            for i in insts:
                cur[:, i * self.base_lanes:(i + 1) * self.base_lanes] = vals
            self.set_port(port, cur)

    def get_top_output(self, name: str) -> np.ndarray:
        """A wrapper signal driven by an instance output: [limbs][base_lanes]."""
        (inst, port), = self._out[name]
        return self.get_port(port)[:, inst * self.base_lanes:(inst + 1) * self.base_lanes]

    def tick(self):
        self.sim.tick()

    def tick_many(self, steps: int):
        self.sim.tick_many(steps)

    def eval_combinational(self):
        self.sim.eval_combinational()


def bitslice_json(design: Union[_b.Design, str], top: str) -> str:
    """The plane design (1-bit signals "<signal>[p]") of a multi-bit design,
    as design JSON (no device needed)."""
    text = design.to_json() if isinstance(design, _b.Design) else design
    raw = text.encode()
    n = c_size_t()
    check(lib().rrtl_bitslice_json(raw, len(raw), top.encode(), None, 0, byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    check(lib().rrtl_bitslice_json(raw, len(raw), top.encode(), buf, n.value + 1, byref(n)))
    return buf.value.decode()


class BitSliceSimulator:
    """A multi-bit design simulated bit-sliced on the gate engine (the
    reference's BitSliceSimulator, crates/rrtl-sim-ir/src/bitslice.rs): a
    W-bit signal is W plane signals "<name>[p]"; set_signal / get_signal move
    per-lane values (Python ints, up to any width) in and out of the planes."""

    def __init__(self, design: Union[_b.Design, str], top: str, lanes: int, ctx: Optional[Context] = None):
        self.design = CompiledDesign(design, top, ctx, bitslice=True)
        self.sim = GpuBatchSimulator(self.design, lanes=lanes)
        self.lanes = lanes
        self._width = {}

    def width(self, name: str) -> int:
        if name not in self._width:
            w = 0
            while True:
                try:
                    self.design.signal(f"{name}[{w}]")
                except RrtlError:
                    break
                w += 1
            if w == 0:
                raise RrtlError(3, f"E_GPU_SIGNAL: no signal `{name}`")
            self._width[name] = w
        return self._width[name]

    def planes(self, name: str):
        return [f"{name}[{p}]" for p in range(self.width(name))]

    def set_signal(self, name: str, lane_values: Sequence[int]):
        vals = [int(v) for v in lane_values]
        words = (self.lanes + 31) // 32
        for p, plane in enumerate(self.planes(name)):
            bits = np.array([(v >> p) & 1 for v in vals], dtype=np.uint32)
            packed = np.zeros(words, dtype=np.uint32)
            idx = np.nonzero(bits)[0]
            np.bitwise_or.at(packed, idx // 32, (np.uint32(1) << (idx % 32).astype(np.uint32)))
            self.sim.set_input_bits(plane, packed)

    def get_signal(self, name: str) -> list:
        out = [0] * self.lanes
        for p, plane in enumerate(self.planes(name)):
            words = self.sim.get_signal_bits(plane)
            bits = (words[np.arange(self.lanes) // 32] >> (np.arange(self.lanes) % 32).astype(np.uint32)) & 1
            for l in np.nonzero(bits)[0]:
                out[l] |= 1 << p
        return out

    def eval_combinational(self):
        self.sim.eval_combinational()

    def tick(self):
        self.sim.tick()

    def tick_many(self, steps: int):
        self.sim.tick_many(steps)


def shard_plan(total_lanes: int, shards: int) -> list:
    """Contiguous lane shards [(worker, start_lane, lanes)], each starting on a 32-lane word."""
    arr = (ShardInfo * shards)()
    check(lib().rrtl_shard_plan(total_lanes, shards, arr))
    return [(x.worker, x.start_lane, x.lanes) for x in arr]


class Runtime:
    """Lane-shard runtime (rrtl_runtime_*): the reference's DistributedRuntime
    shard plan on one GPU, one lane batch per shard; runs and outputs use
    global lanes."""

    def __init__(self, design: "CompiledDesign", total_lanes: int, shards: int):
        self.design = design
        self.lanes = total_lanes
        self.h = c_void_p()
        check(lib().rrtl_runtime_create(design.h, total_lanes, shards, byref(self.h)))
        self.n = shards
        self._shape = _RunShape(design, total_lanes)

    def shard(self, k: int):
        info = ShardInfo()
        check(lib().rrtl_runtime_shard(self.h, k, byref(info), None))
        return info.worker, info.start_lane, info.lanes

    def set_faults(self, faults: Sequence[tuple]):
        arr = (Fault * max(1, len(faults)))(*[Fault(l, self._shape._sig(s), v) for l, s, v in faults])
        check(lib().rrtl_runtime_set_faults(self.h, arr, len(faults)))

    def run(self, cycles: int, seed: int = 0, stim: Iterable = (), record: Iterable = (), mode: int = 0,
            input_trace: Optional[np.ndarray] = None, lane_base: int = 0):
        record = list(record)
        out = self._shape.alloc_outputs(cycles, record, mode)
        r = self._shape.make_run(cycles, seed, stim, record, mode, input_trace, out["trace"], out["hash"],
                                 out["detect"], lane_base)
        check(lib().rrtl_runtime_run(self.h, byref(r)))
        return out

    def close(self):
        if self.h:
            lib().rrtl_runtime_destroy(self.h)
            self.h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
