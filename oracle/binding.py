"""ctypes binding of the CPU oracle (test infrastructure only).

Only the tests, the smoke check and the benchmark's CPU-baseline leg import
this module; the product path never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_char_p, c_int, c_size_t, c_uint32, c_uint64, c_void_p

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


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


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_last_error.restype = c_char_p
        L.orc_design_load.restype = c_void_p
        L.orc_design_load.argtypes = [c_char_p, c_size_t, c_char_p]
        L.orc_design_free.argtypes = [c_void_p]
        for n in ("orc_signal_index", "orc_memory_index"):
            getattr(L, n).argtypes = [c_void_p, c_char_p]
            getattr(L, n).restype = c_int
        for n in ("orc_signal_width", "orc_signal_kind"):
            getattr(L, n).argtypes = [c_void_p, c_uint32]
            getattr(L, n).restype = c_uint32
        L.orc_signal_top_id.argtypes = [c_void_p, c_uint32]
        L.orc_signal_top_id.restype = c_int
        for n in ("orc_num_signals", "orc_num_comb_packets", "orc_num_levels"):
            getattr(L, n).argtypes = [c_void_p]
            getattr(L, n).restype = c_uint32
        for n in ("orc_total_signal_words", "orc_total_memory_words", "orc_num_instrs"):
            getattr(L, n).argtypes = [c_void_p]
            getattr(L, n).restype = c_uint64
        L.orc_stim_word.argtypes = [c_uint64, c_uint64, c_uint64, c_uint64]
        L.orc_stim_word.restype = c_uint32
        L.orc_hash_term.argtypes = [c_uint64, c_uint32, c_uint64, c_uint32]
        L.orc_hash_term.restype = c_uint64
        L.orc_packed_new.argtypes = [c_void_p, c_uint32]
        L.orc_packed_new.restype = c_void_p
        L.orc_simd_new.argtypes = [c_void_p, c_uint32]
        L.orc_simd_new.restype = c_void_p
        L.orc_bs_new.argtypes = [c_void_p, c_uint32]
        L.orc_bs_new.restype = c_void_p
        L.orc_bs_free.argtypes = [c_void_p]
        L.orc_bs_set_signal.argtypes = [c_void_p, c_uint32, c_void_p]
        L.orc_bs_get_signal.argtypes = [c_void_p, c_uint32, c_void_p]
        L.orc_bs_tick.argtypes = [c_void_p]
        L.orc_packed_free.argtypes = [c_void_p]
        L.orc_packed_set_signal.argtypes = [c_void_p, c_uint32, POINTER(c_uint32), c_int]
        L.orc_packed_get_signal.argtypes = [c_void_p, c_uint32, POINTER(c_uint32)]
        L.orc_packed_set_memory.argtypes = [c_void_p, c_uint32, POINTER(c_uint32), c_int]
        L.orc_packed_get_memory.argtypes = [c_void_p, c_uint32, POINTER(c_uint32)]
        for n in ("orc_packed_eval", "orc_packed_tick", "orc_packed_tick_from_evaluated"):
            getattr(L, n).argtypes = [c_void_p]
        L.orc_packed_tick_many.argtypes = [c_void_p, c_uint64]
        L.orc_packed_snapshot.argtypes = [c_void_p, POINTER(c_uint32), POINTER(c_uint32)]
        L.orc_packed_run.argtypes = [c_void_p, POINTER(Run)]
        L.orc_packed_run.restype = c_int
        L.orc_bp_new.argtypes = [c_void_p, c_uint32]
        L.orc_bp_new.restype = c_void_p
        L.orc_bp_free.argtypes = [c_void_p]
        L.orc_bp_set_force.argtypes = [c_void_p, c_uint32, c_uint32, c_int]
        L.orc_bp_set.argtypes = [c_void_p, c_uint32, c_uint32, c_int]
        L.orc_bp_set_all.argtypes = [c_void_p, c_uint32, c_int]
        L.orc_bp_get.argtypes = [c_void_p, c_uint32, c_uint32]
        L.orc_bp_get.restype = c_int
        L.orc_bp_tick.argtypes = [c_void_p]
        L.orc_bp_settle.argtypes = [c_void_p]
        L.orc_bp_get_bits.argtypes = [c_void_p, c_uint32, POINTER(c_uint32)]
        L.orc_bp_set_bits.argtypes = [c_void_p, c_uint32, POINTER(c_uint32)]
        L.orc_bp_run.argtypes = [c_void_p, POINTER(Run)]
        L.orc_bp_run.restype = c_int
        L.orc_bp_run_parallel.argtypes = [c_void_p, c_uint32, POINTER(Run), c_uint32]
        L.orc_bp_run_parallel.restype = c_int
        L.orc_bp_emit_c.argtypes = [c_void_p, POINTER(Stim), c_uint32, POINTER(c_uint32), c_uint32, ctypes.c_char_p,
                                    ctypes.c_size_t, POINTER(ctypes.c_size_t)]
        L.orc_bp_emit_c.restype = c_int
        L.orc_scalar_new.argtypes = [c_void_p]
        L.orc_scalar_new.restype = c_void_p
        L.orc_scalar_free.argtypes = [c_void_p]
        L.orc_scalar_id.argtypes = [c_void_p, c_char_p]
        L.orc_scalar_id.restype = c_int
        L.orc_scalar_set.argtypes = [c_void_p, c_uint32, c_uint64, c_uint64, c_int]
        L.orc_scalar_get.argtypes = [c_void_p, c_uint32, POINTER(c_uint64)]
        L.orc_scalar_get.restype = c_uint64
        L.orc_scalar_tick.argtypes = [c_void_p]
        L.orc_scalar_eval.argtypes = [c_void_p]
        L.orc_scalar_peek_mem.argtypes = [c_void_p, c_uint32, c_uint64]
        L.orc_scalar_peek_mem.restype = c_uint64
        L.orc_scalar_poke_mem.argtypes = [c_void_p, c_uint32, c_uint64, c_uint64]
        _lib = L
    return _lib


def _u32p(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_uint32))


def _u64p(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_uint64))


class OracleError(RuntimeError):
    pass


class OracleDesign:
    def __init__(self, design_json: str, top: str):
        L = lib()
        raw = design_json.encode()
        self.h = L.orc_design_load(raw, len(raw), top.encode())
        if not self.h:
            raise OracleError(L.orc_last_error().decode())
        self.top = top

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_design_free(self.h)
            self.h = None

    def signal(self, name: str) -> int:
        i = lib().orc_signal_index(self.h, name.encode())
        if i < 0:
            raise KeyError(name)
        return i

    def memory(self, name: str) -> int:
        i = lib().orc_memory_index(self.h, name.encode())
        if i < 0:
            raise KeyError(name)
        return i

    def width(self, sig: int) -> int:
        return lib().orc_signal_width(self.h, sig)

    def kind(self, sig: int) -> int:
        return lib().orc_signal_kind(self.h, sig)

    @property
    def num_signals(self) -> int:
        return lib().orc_num_signals(self.h)

    @property
    def total_signal_words(self) -> int:
        return lib().orc_total_signal_words(self.h)

    @property
    def total_memory_words(self) -> int:
        return lib().orc_total_memory_words(self.h)

    @property
    def num_instrs(self) -> int:
        return lib().orc_num_instrs(self.h)

    @property
    def num_levels(self) -> int:
        return lib().orc_num_levels(self.h)


def make_run(cycles, seed, stim, record, mode, input_trace=None, n_trace_cols=0, out_trace=None, out_hash=None,
             detect=None, lane_base=0):
    """Build an rrtl_run structure; keeps the numpy buffers alive on the object."""
    st = (Stim * max(1, len(stim)))(*[Stim(s, k, p) for (s, k, p) in stim])
    rec = np.asarray(record, dtype=np.uint32)
    r = Run()
    r.cycles = cycles
    r.seed = seed
    r.n_stim = len(stim)
    r.stim = ctypes.cast(st, POINTER(Stim))
    r.n_record = len(rec)
    r.record = _u32p(rec)
    r.record_mode = mode
    r.n_trace_cols = n_trace_cols
    r.input_trace = _u32p(input_trace) if input_trace is not None else None
    r.out_trace = _u32p(out_trace) if out_trace is not None else None
    r.out_hash = _u64p(out_hash) if out_hash is not None else None
    r.detect = _u32p(detect) if detect is not None else None
    r.lane_base = lane_base
    r._keep = (st, rec, input_trace, out_trace, out_hash, detect)
    return r


class PackedSim:
    """Restated `PackedSimulator` (word-level, any width)."""

    def __init__(self, design: OracleDesign, lanes: int):
        self.d = design
        self.lanes = lanes
        self.h = lib().orc_packed_new(design.h, lanes)
        if not self.h:
            raise OracleError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_packed_free(self.h)
            self.h = None

    def _limbs(self, sig):
        return (self.d.width(sig) + 31) // 32

    def set_signal(self, sig: int, values, settle: bool = True):
        a = np.ascontiguousarray(np.asarray(values, dtype=np.uint32).reshape(self._limbs(sig), self.lanes))
        lib().orc_packed_set_signal(self.h, sig, _u32p(a), 1 if settle else 0)

    def get_signal(self, sig: int) -> np.ndarray:
        out = np.zeros((self._limbs(sig), self.lanes), dtype=np.uint32)
        lib().orc_packed_get_signal(self.h, sig, _u32p(out))
        return out

    def set_memory(self, mem: int, data: np.ndarray, settle: bool = True):
        a = np.ascontiguousarray(data, dtype=np.uint32)
        lib().orc_packed_set_memory(self.h, mem, _u32p(a), 1 if settle else 0)

    def get_memory(self, mem: int, depth: int, limbs: int) -> np.ndarray:
        out = np.zeros((depth, limbs, self.lanes), dtype=np.uint32)
        lib().orc_packed_get_memory(self.h, mem, _u32p(out))
        return out

    def eval(self):
        lib().orc_packed_eval(self.h)

    def tick(self):
        lib().orc_packed_tick(self.h)

    def tick_many(self, n: int):
        lib().orc_packed_tick_many(self.h, n)

    def tick_from_evaluated(self):
        lib().orc_packed_tick_from_evaluated(self.h)

    def snapshot(self):
        v = np.zeros(self.d.total_signal_words * self.lanes, dtype=np.uint32)
        m = np.zeros(max(1, self.d.total_memory_words * self.lanes), dtype=np.uint32)
        lib().orc_packed_snapshot(self.h, _u32p(v), _u32p(m))
        return v, m[: self.d.total_memory_words * self.lanes]

    def run(self, run: Run):
        rc = lib().orc_packed_run(self.h, ctypes.byref(run))
        if rc:
            raise OracleError(lib().orc_last_error().decode())


class SimdSim(PackedSim):
    """Restated `SimdCpuSimulator` (crates/rrtl-sim-ir/src/lib.rs:5375-7457):
    PackedSim's cycle evaluated instruction by instruction across all lanes
    on u64 lanes (designs whose values are at most 64 bits). Same storage and
    entry points as PackedSim."""

    def __init__(self, design: OracleDesign, lanes: int):
        self.d = design
        self.lanes = lanes
        self.h = lib().orc_simd_new(design.h, lanes)
        if not self.h:
            raise OracleError(lib().orc_last_error().decode())


def simd_run_parallel(design: OracleDesign, lanes: int, cycles: int, seed: int, stim, record, mode: int = 2,
                      memories=None, threads: int = 0, snapshot: bool = False):
    """The SIMD engine over `lanes` lanes split into disjoint lane ranges, one
    engine per host thread (lanes never interact; the reference's parallel
    CPU engines split the same way). Each range runs with lane_base = its
    first lane, so per-cycle hashes add up to the whole batch's.
    memories: {memory index: [addr][limb][lanes] array}. Returns the per-cycle
    hash (mode & 2), and with `snapshot` the final PackedSimulatorStorage
    (values [word][lanes], memories [lanes][word] flattened)."""
    from concurrent.futures import ThreadPoolExecutor

    threads = threads or (os.cpu_count() or 1)
    chunks = max(1, min(threads, (lanes + 31) // 32))
    unit = ((lanes + 31) // 32 + chunks - 1) // chunks * 32  # lane ranges start on 32-lane words
    bounds = [min(lanes, i * unit) for i in range(chunks + 1)]
    bounds[-1] = lanes
    hashes = [np.zeros(max(cycles, 1), dtype=np.uint64) for _ in range(chunks)]
    tsw, tmw = design.total_signal_words, design.total_memory_words
    vals = np.zeros((tsw, lanes), dtype=np.uint32) if snapshot else None
    mems = np.zeros((lanes, tmw), dtype=np.uint32) if snapshot else None

    def work(i):
        a, b = bounds[i], bounds[i + 1]
        if b <= a:
            return
        s = SimdSim(design, b - a)
        for mi, data in (memories or {}).items():
            s.set_memory(mi, np.ascontiguousarray(np.asarray(data)[:, :, a:b]), settle=False)
        s.eval()
        r = make_run(cycles, seed, stim, record, mode, out_hash=hashes[i] if mode & 2 else None, lane_base=a)
        s.run(r)
        if snapshot:
            v, m = s.snapshot()
            vals[:, a:b] = v.reshape(tsw, b - a)
            if tmw:
                mems[a:b, :] = m.reshape(b - a, tmw)

    with ThreadPoolExecutor(max_workers=chunks) as ex:
        list(ex.map(work, range(chunks)))
    total = np.zeros(max(cycles, 1), dtype=np.uint64)
    for h in hashes:
        total += h
    total = total[:cycles]
    if snapshot:
        return total, vals.reshape(-1), mems.reshape(-1)
    return total


class BitSlice:
    """Restated `BitSliceSimulator` (multi-bit signals as bit-planes, 64 lanes
    per u64; crates/rrtl-sim-ir/src/bitslice.rs). Signals move as
    [limbs][lanes] u32, like PackedSim."""

    def __init__(self, design: OracleDesign, lanes: int):
        self.d = design
        self.lanes = lanes
        self.h = lib().orc_bs_new(design.h, lanes)
        if not self.h:
            raise OracleError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_bs_free(self.h)
            self.h = None

    def _limbs(self, sig):
        return max(1, (lib().orc_signal_width(self.d.h, sig) + 31) // 32)

    def set_signal(self, sig: int, values):
        a = np.ascontiguousarray(np.asarray(values, dtype=np.uint32).reshape(self._limbs(sig), self.lanes))
        lib().orc_bs_set_signal(self.h, sig, a.ctypes.data)

    def get_signal(self, sig: int) -> np.ndarray:
        out = np.zeros((self._limbs(sig), self.lanes), dtype=np.uint32)
        lib().orc_bs_get_signal(self.h, sig, out.ctypes.data)
        return out

    def tick(self):
        lib().orc_bs_tick(self.h)


class BitParallel:
    """Restated `BitParallelSimulator` (1-bit gate-level, per-lane stuck-at forces)."""

    def __init__(self, design: OracleDesign, lanes: int):
        self.d = design
        self.lanes = lanes
        self.h = lib().orc_bp_new(design.h, lanes)
        if not self.h:
            raise OracleError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_bp_free(self.h)
            self.h = None

    def set_force(self, sig, lane, value):
        lib().orc_bp_set_force(self.h, sig, lane, int(value))

    def set(self, sig, lane, v):
        lib().orc_bp_set(self.h, sig, lane, int(v))

    def set_all(self, sig, v):
        lib().orc_bp_set_all(self.h, sig, int(v))

    def get(self, sig, lane) -> int:
        return lib().orc_bp_get(self.h, sig, lane)

    def tick(self):
        lib().orc_bp_tick(self.h)

    def settle(self):
        lib().orc_bp_settle(self.h)

    def get_bits(self, sig) -> np.ndarray:
        out = np.zeros((self.lanes + 31) // 32, dtype=np.uint32)
        lib().orc_bp_get_bits(self.h, sig, _u32p(out))
        return out

    def set_bits(self, sig, words):
        a = np.ascontiguousarray(words, dtype=np.uint32)
        lib().orc_bp_set_bits(self.h, sig, _u32p(a))

    def run(self, run: Run):
        rc = lib().orc_bp_run(self.h, ctypes.byref(run))
        if rc:
            raise OracleError(lib().orc_last_error().decode())


def bp_run_parallel(design: OracleDesign, lanes: int, run: Run, threads: int):
    rc = lib().orc_bp_run_parallel(design.h, lanes, ctypes.byref(run), threads)
    if rc:
        raise OracleError(lib().orc_last_error().decode())


class ScalarSim:
    """Restated `rrtl_core::Simulator` (single instance, top-module signal names)."""

    def __init__(self, design: OracleDesign):
        self.h = lib().orc_scalar_new(design.h)
        if not self.h:
            raise OracleError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_scalar_free(self.h)
            self.h = None

    def id(self, name: str) -> int:
        i = lib().orc_scalar_id(self.h, name.encode())
        if i < 0:
            raise KeyError(name)
        return i

    def set(self, name_or_id, value: int, settle: bool = True):
        i = self.id(name_or_id) if isinstance(name_or_id, str) else name_or_id
        lib().orc_scalar_set(self.h, i, value & (2**64 - 1), (value >> 64) & (2**64 - 1), 1 if settle else 0)

    def get(self, name_or_id) -> int:
        i = self.id(name_or_id) if isinstance(name_or_id, str) else name_or_id
        hi = c_uint64(0)
        lo = lib().orc_scalar_get(self.h, i, ctypes.byref(hi))
        return (hi.value << 64) | lo

    def tick(self):
        lib().orc_scalar_tick(self.h)

    def eval(self):
        lib().orc_scalar_eval(self.h)

    def peek_mem(self, name_or_id, addr) -> int:
        i = self.id(name_or_id) if isinstance(name_or_id, str) else name_or_id
        return lib().orc_scalar_peek_mem(self.h, i, addr)

    def poke_mem(self, name_or_id, addr, value):
        i = self.id(name_or_id) if isinstance(name_or_id, str) else name_or_id
        lib().orc_scalar_poke_mem(self.h, i, addr, value)


def crc_step(c: int, din: int) -> int:
    """CRC-32 byte step, MSB-first, polynomial 0x04C11DB7
    (crates/rrtl-sim-ir/examples/netlist_crc32.rs:26-33)."""
    for i in range(8):
        bit = ((c >> 31) & 1) ^ ((din >> i) & 1)
        c = ((c << 1) & 0xFFFFFFFF) ^ (0x04C11DB7 if bit else 0)
    return c


class BitParallelAot:
    """The reference's AOT bit-parallel engine restated (BitParallelAot,
    crates/rrtl-sim-ir/src/bitparallel.rs:348-528): the design emitted as
    straight-line u64 C (orc_bp_emit_c), compiled with the host C compiler at
    -O3 and run over disjoint 64-lane group ranges on all host threads
    (tick_many_parallel, :513-523). Stimulus and output hash follow this
    library's run protocol, so its per-cycle hash equals the GPU engines'."""

    def __init__(self, design: "OracleDesign", stim, record, cc: str = "gcc", opt: str = "-O3", native: bool = False):
        import hashlib
        import subprocess

        st = (Stim * max(1, len(stim)))(*[Stim(a, b, c) for a, b, c in stim])
        rec = np.asarray(record, dtype=np.uint32)
        need = ctypes.c_size_t()
        rp = rec.ctypes.data_as(POINTER(c_uint32))
        if lib().orc_bp_emit_c(design.h, st, len(stim), rp, len(rec), None, 0, ctypes.byref(need)):
            raise OracleError(lib().orc_last_error().decode())
        buf = ctypes.create_string_buffer(need.value)
        if lib().orc_bp_emit_c(design.h, st, len(stim), rp, len(rec), buf, need.value, ctypes.byref(need)):
            raise OracleError(lib().orc_last_error().decode())
        src = buf.value
        flags = [opt]
        if native:
            # tuned for the host it runs on (the emitted C is built where it runs, like the reference's
            # clang -O3 build of its AOT source)
            import platform

            flags.append("-mcpu=native" if platform.machine() in ("aarch64", "arm64") else "-march=native")
        self.flags = flags
        tag = hashlib.sha1(src + " ".join(flags).encode()).hexdigest()[:16]
        d = os.path.join(_HERE, "_build", "aot")
        os.makedirs(d, exist_ok=True)
        so = os.path.join(d, f"bp_{tag}.so")
        if not os.path.exists(so):
            # the source comes as translation units; compile them in parallel, then link
            parts = src.split(b"\n//@@PART@@\n")
            objs, procs = [], []
            for i, part in enumerate(parts):
                cpath = os.path.join(d, f"bp_{tag}_{i}.c")
                with open(cpath, "wb") as f:
                    f.write(part)
                obj = cpath[:-2] + f".{os.getpid()}.o"
                objs.append(obj)
                procs.append(subprocess.Popen([cc] + flags + ["-fPIC", "-c", "-o", obj, cpath],
                                              stdout=subprocess.PIPE, stderr=subprocess.PIPE))
            for p in procs:
                _, err = p.communicate()
                if p.returncode:
                    raise RuntimeError(f"{cc} failed: {err.decode()[-2000:]}")
            tmp = so + f".{os.getpid()}.tmp"
            r = subprocess.run([cc, "-shared", "-o", tmp] + objs, capture_output=True, text=True)
            if r.returncode:
                raise RuntimeError(f"{cc} link failed: {r.stderr[-2000:]}")
            os.replace(tmp, so)
            for o in objs:
                os.remove(o)
        self.lib = ctypes.CDLL(so)
        self.lib.run_bp.argtypes = [POINTER(ctypes.c_uint64), ctypes.c_long, ctypes.c_long, ctypes.c_long,
                                    ctypes.c_long, ctypes.c_uint64, POINTER(ctypes.c_uint64)]
        self.lib.run_bp.restype = None
        self.ns = design.num_signals

    def run(self, lanes: int, cycles: int, seed: int, threads: int = 0, lane_base: int = 0, signals=None):
        """`cycles` cycles of `lanes` lanes (a multiple of 64) from the zero
        state, global lanes [lane_base, lane_base + lanes) (lane_base a
        multiple of 64); returns the per-cycle hash summed over all lanes, and
        with `signals` (signal indices) also their final values as 32-lane
        words [len(signals)][lanes / 32] (bit k of word w = lane 32w + k)."""
        from concurrent.futures import ThreadPoolExecutor

        assert lanes % 64 == 0 and lane_base % 64 == 0
        groups = lanes // 64
        threads = threads or (os.cpu_count() or 1)
        chunks = max(1, min(groups, threads * 4))
        bounds = [groups * i // chunks for i in range(chunks + 1)]
        hashes = [np.zeros(cycles, dtype=np.uint64) for _ in range(chunks)]
        sig = None if signals is None else np.asarray(signals, dtype=np.int64)
        final = None if sig is None else np.zeros((len(sig), groups), dtype=np.uint64)

        def work(i):
            g0, g1 = bounds[i], bounds[i + 1]
            if g1 == g0:
                return
            st = np.zeros((g1 - g0) * self.ns, dtype=np.uint64)
            self.lib.run_bp(st.ctypes.data_as(POINTER(ctypes.c_uint64)), g1 - g0, lane_base // 64 + g0, 0, cycles,
                            seed, hashes[i].ctypes.data_as(POINTER(ctypes.c_uint64)))
            if final is not None:
                final[:, g0:g1] = st.reshape(g1 - g0, self.ns)[:, sig].T

        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(work, range(chunks)))
        total = np.zeros(cycles, dtype=np.uint64)
        for h in hashes:
            total += h
        if final is None:
            return total
        words = np.zeros((len(sig), 2 * groups), dtype=np.uint32)
        words[:, 0::2] = (final & 0xFFFFFFFF).astype(np.uint32)
        words[:, 1::2] = (final >> 32).astype(np.uint32)
        return total, words
