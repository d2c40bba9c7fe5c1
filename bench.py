"""Benchmark of the batched cycle-simulation hot path on GB300.

Workload (default): the synthetic gate-level netlist — 50,000 gates uniform
over {AND, OR, XOR, NAND, NOR, XNOR, NOT, MUX2}, 2,048 flip-flops with a
synchronous reset, 64 primary inputs, 64 primary outputs, depth 40, fanins
from the previous 1-3 levels inside a 4,096-net window — at 65,536 lanes per
GPU x 1,000 cycles per step. Primary inputs take fresh uniform bits every
cycle (counter hash of seed, input, cycle, word); reset is held for cycle 0.
Each step produces a per-cycle output hash over all lanes' outputs and the
final flip-flop state.

Metric: lane-cycles/s (gate-evals/s = gates x lane-cycles/s), whole job over
all ranks. `value` is timed with CUDA events on the engine's stream with the
design and lane state resident in HBM; `e2e` runs the same steps through the
C ABI with pinned host buffers (stimulus spec in, per-cycle hash and final
flop state out) inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: one process per GPU (torchrun); every rank simulates its own
65,536 lanes (weak scaling), no data-path collective; the time is the max
over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GATES, FFS, PIS, POS, DEPTH, WINDOW, SEED = 50_000, 2048, 64, 64, 40, 4096, 2
LANES, CYCLES = 65_536, 1000
METRIC = "lane-cycles/s (gate-evals/s) batched vs plain CUDA on 1 GB300; p99 job latency"


def dist_setup():
    """Host-side process group over gloo: it only carries barriers and the
    max of the ranks' timings (lanes shard with no data-path exchange). A
    rank that fails or never arrives makes the others' next collective fail
    within RRTL_DIST_TIMEOUT_S seconds (default 600) instead of hanging."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        from datetime import timedelta

        import torch.distributed as dist

        timeout = timedelta(seconds=float(os.environ.get("RRTL_DIST_TIMEOUT_S", "600")))
        dist.init_process_group("gloo", init_method="env://", timeout=timeout)
        return ws, rank, local, dist
    return 1, 0, 0, None


def reduce_max(dist, value: float) -> float:
    """Max of a host-side timing over all ranks (gloo); identity when single-process."""
    if not dist:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def throughput(ws: int, lanes_per_rank: int, cycles: int, steps: int, ms: float) -> float:
    """Whole-job lane-cycles/s: every rank's lanes over the slowest rank's time."""
    return ws * lanes_per_rank * cycles * steps / (ms / 1000.0)


def lane_shard(total_lanes: int, rank: int, ws: int, align: int = 1):
    """Global lane range [first, last) of a rank: contiguous, disjoint shards
    (the reference's shard plan, crates/rrtl-runtime/src/lib.rs:168-175),
    each starting on a multiple of `align` lanes (32: a whole 32-lane word,
    the unit the engines key stimulus and hashes on)."""
    units = (total_lanes + align - 1) // align

    def edge(r):
        return min(total_lanes, units * r // ws * align)

    return edge(rank), edge(rank + 1)


def sum_hashes(dist, h):
    """Per-cycle hashes of every rank's lane shard added up (wrapping u64), on
    every rank: the shards' hashes compose into the hash of the whole run.
    Identity when single-process."""
    h = np.asarray(h, dtype=np.uint64)
    if not dist:
        return h
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, h)
    total = np.zeros_like(h)
    for p in parts:
        total += p
    return total


def net_stream_bytes_per_lane_cycle(meta_fanins, n_ff, n_pi, n_po):
    """Net-streaming model: every gate reads its fanins and writes its output,
    each flop's D is read and Q written, inputs written and outputs read, one
    4-byte word per 32 lanes each."""
    words = sum(f + 1 for f in meta_fanins) + 2 * n_ff + n_pi + n_po
    return 4.0 * words / 32.0


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_issue(name):
    """Issue-slot figures of the top kernel from a committed ncu summary
    (lines 'issue_<key>: value')."""
    p = os.path.join(ROOT, "profiles", name)
    out = {}
    if os.path.exists(p):
        with open(p) as f:
            for line in f:
                ln = line.strip()
                if ln.startswith("issue_") and ":" in ln:
                    k, v = ln.split(":", 1)
                    try:
                        out[k[len("issue_"):]] = float(v)
                    except ValueError:
                        out[k[len("issue_"):]] = v.strip()
    return out or None


def profiled_traffic(name):
    """Per-launch DRAM bytes from a committed ncu summary (line 'traffic_bytes_per_launch: N')."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None, None
    lanes = None
    traffic = None
    with open(p) as f:
        for line in f:
            s = line.strip()
            if s.startswith("traffic_bytes_per_launch:"):
                traffic = float(s.split(":", 1)[1])
            elif s.startswith("traffic_lanes:"):
                lanes = int(s.split(":", 1)[1])
    if traffic is None or not lanes:
        return None, None
    return traffic, lanes


def cpu_baseline(od, aot, compile_s, stim_idx, rec_idx, budget_s=12.0):
    """The reference's fastest CPU engine for this path restated: the AOT
    bit-parallel engine (BitParallelAot, crates/rrtl-sim-ir/src/bitparallel.rs:348-528:
    the design as straight-line u64 C, compiled -O3 for the host, 64 lanes per
    word, group ranges over all host threads), on a bounded sample of the same
    netlist and stimulus. The bit-parallel interpreter is timed beside it, and
    for the word-level configuration the SIMD-shaped packed engine
    (SimdCpuSimulator restated) on all threads and the scalar packed
    simulator on one."""
    from oracle import binding as ob

    threads = os.cpu_count() or 1
    lanes = 64 * threads * 8
    aot.run(lanes, 2, SEED)
    t = time.perf_counter()
    aot.run(lanes, 8, SEED)
    dt = max(time.perf_counter() - t, 1e-3)
    cycles = max(8, int(budget_s / dt * 8))
    t = time.perf_counter()
    aot.run(lanes, cycles, SEED)
    dt = time.perf_counter() - t
    value = lanes * cycles / dt
    # one core, on a quarter of the budget
    l1 = 64 * 8
    t = time.perf_counter()
    aot.run(l1, 8, SEED, threads=1)
    d1 = max(time.perf_counter() - t, 1e-3)
    c1 = max(8, int(budget_s / 4 / d1 * 8))
    t = time.perf_counter()
    aot.run(l1, c1, SEED, threads=1)
    one_core = l1 * c1 / (time.perf_counter() - t)
    # the interpreter on a shorter sample
    ilanes, icycles = 64 * threads * 4, 4
    run = ob.make_run(icycles, SEED, stim_idx, rec_idx, 2, out_hash=np.zeros(icycles, dtype=np.uint64))
    t = time.perf_counter()
    ob.bp_run_parallel(od, ilanes, run, threads)
    idt = time.perf_counter() - t
    # the word-level configuration: the SIMD-shaped packed engine (all host
    # threads) and the scalar packed simulator (one thread) on the pipelined
    # CPU with per-lane hashed ROMs
    from rrtl_gb300 import sim as _sim
    from rrtl_gb300.workloads import cpu_rom_hashed, pipelined_cpu

    cod = ob.OracleDesign(pipelined_cpu().to_json(), "Cpu8")
    cstim = [(cod.signal("clk"), _sim.STIM_CONST, 1), (cod.signal("rst"), _sim.STIM_PULSE, 1)]
    crec = [cod.signal("out_pc"), cod.signal("out_acc")]
    rom_mi = cod.memory("rom")
    slanes = 512 * threads
    srom = cpu_rom_hashed(slanes, seed=3)
    t = time.perf_counter()
    ob.simd_run_parallel(cod, slanes, 50, 0, cstim, crec, 2, memories={rom_mi: srom}, threads=threads)
    sdt = max(time.perf_counter() - t, 1e-3)
    scyc = max(50, int(budget_s / 3 / sdt * 50))
    t = time.perf_counter()
    ob.simd_run_parallel(cod, slanes, scyc, 0, cstim, crec, 2, memories={rom_mi: srom}, threads=threads)
    simd = slanes * scyc / (time.perf_counter() - t)
    plane, pcyc = 64, 16

    def packed_run(cycles):
        ps = ob.PackedSim(cod, plane)
        ps.set_memory(rom_mi, cpu_rom_hashed(plane, seed=3))
        r = ob.make_run(cycles, 0, cstim, crec, 2, out_hash=np.zeros(cycles, dtype=np.uint64))
        t0 = time.perf_counter()
        ps.run(r)
        return time.perf_counter() - t0

    pdt = max(packed_run(pcyc), 1e-4)
    pcyc = max(16, int(budget_s / 8 / pdt * pcyc))
    packed = plane * pcyc / packed_run(pcyc)
    # the bit-slice engine restated (planes of 64 lanes, one core) on the
    # 16-bit ALU of the bit-slice leg without its compare (outside the
    # reference engine's scope)
    bitslice = None
    try:
        from rrtl_gb300.workloads import narrow_alu

        aod = ob.OracleDesign(narrow_alu(16, compare=False).to_json(), "Alu")
        blanes = 64 * 64
        bsim = ob.BitSlice(aod, blanes)
        rng = np.random.default_rng(1)
        t0 = time.perf_counter()
        bcyc = 0
        while time.perf_counter() - t0 < budget_s / 8:
            for name, w in (("din", 16), ("sel", 2)):
                bsim.set_signal(aod.signal(name), rng.integers(0, 1 << w, size=(1, blanes), dtype=np.uint32))
            bsim.tick()
            bcyc += 1
        bitslice = {"value": blanes * bcyc / (time.perf_counter() - t0), "cores": 1,
                    "sample": f"16-bit ALU without compare, {blanes} lanes x {bcyc} cycles, bit-slice engine "
                              "restated, 1 thread"}
    except Exception as e:  # the baseline is reported, not required
        bitslice = {"unavailable": str(e)[:200]}
    return {"value": value, "unit": "lane-cycles/s", "cores": threads, "kind": "port",
            "packed_cpu8": {"value": simd, "cores": threads,
                            "sample": f"pipelined CPU, {slanes} lanes x {scyc} cycles, SIMD-shaped packed engine "
                                      f"(SimdCpuSimulator restated), {threads} threads"},
            "packed_cpu8_scalar": {"value": packed, "cores": 1,
                                   "sample": f"pipelined CPU, {plane} lanes x {pcyc} cycles, scalar packed "
                                             "simulator restated, 1 thread"},
            "bitslice_alu16": bitslice,
            "sample": f"{lanes} lanes x {cycles} cycles of the same netlist and stimulus (bit-parallel AOT: "
                      f"emitted C, gcc {' '.join(aot.flags)}, {threads} threads)", "seconds": round(dt, 3),
            "compile_s": round(compile_s, 1),
            "one_core": {"value": one_core, "sample": f"{l1} lanes x {c1} cycles, 1 thread"},
            "interpreter": {"value": ilanes * icycles / idt, "sample": f"{ilanes} lanes x {icycles} cycles"}}


AOT_OPT = "-O3"  # the emitted C is built where it runs, tuned for that host (the reference builds with clang -O3)


def aot_engine(od, stim_idx, rec_idx):
    """The bit-parallel AOT engine (oracle) for the headline netlist and run."""
    from oracle import binding as ob

    t = time.perf_counter()
    aot = ob.BitParallelAot(od, stim_idx, rec_idx, opt=AOT_OPT, native=True)
    return aot, time.perf_counter() - t


def c2_parity(sim, cd, meta, stim, rec, aot, od, lanes, cycles, lane_base):
    """The headline run at its full size against the oracle: a fresh batch of
    `lanes` lanes (global lanes from lane_base) runs `cycles` cycles from reset
    on the default fused path; its per-cycle output hash and final flip-flop
    state must equal the bit-parallel AOT engine's (emitted C on every host
    thread) on the same seed and lanes."""
    g = sim.GpuBatchSimulator(cd, lanes=lanes)
    r = g.run(cycles, seed=SEED, stim=stim, record=rec, mode=sim.REC_HASH, lane_base=lane_base)
    q_gpu = g.get_signals_bits(meta.regs)
    tile_words = g.tile_words
    del g
    t = time.perf_counter()
    h_or, q_or = aot.run(lanes, cycles, SEED, lane_base=lane_base, signals=[od.signal(q) for q in meta.regs])
    dt = time.perf_counter() - t
    hash_ok = bool(np.array_equal(r["hash"], h_or))
    state_ok = bool(np.array_equal(q_gpu, q_or[:, : q_gpu.shape[1]]))
    return {"equal": hash_ok and state_ok, "hash_equal": hash_ok, "state_equal": state_ok, "lanes": lanes,
            "cycles": cycles, "lane_base": lane_base, "tile_words": tile_words,
            "checked": f"per-cycle output hash ({cycles} cycles) and final state of {len(meta.regs)} flip-flops "
                       f"on all {lanes} lanes",
            "oracle": f"bit-parallel AOT engine (emitted C, {AOT_OPT} host-tuned), {os.cpu_count()} host threads",
            "oracle_s": round(dt, 2)}


def build_workload():
    from rrtl_gb300.workloads import gate_netlist, netlist_run_spec

    d, meta = gate_netlist(n_gates=GATES, n_ff=FFS, n_pi=PIS, n_po=POS, depth=DEPTH, window=WINDOW, seed=SEED)
    js = d.to_json()
    stim, rec = netlist_run_spec(meta)
    return d, meta, js, stim, rec


def gate_fanins(js):
    """Fanin count of each gate assignment (1 NOT, 3 MUX2, 2 otherwise)."""
    obj = json.loads(js)
    out = []
    for a in obj["modules"][0]["assignments"]:
        e = a["expr"]
        tag = next(iter(e))
        if tag == "Signal":
            continue  # output buffers are counted as outputs
        if tag == "Not" and next(iter(e["Not"])) == "Signal":
            out.append(1)
        elif tag == "Mux":
            out.append(3)
        else:
            out.append(2)
    return out


def job_stream_leg(ctx, sim, n_jobs, n_designs, plain=True, plain_jobs=12, graph_jobs=8, cycles=(100, 50_000)):
    """Uneven job stream (C4): `n_jobs` jobs on netlists of the 50k-gate
    family with gate counts log-uniform 5k-200k (a pool of `n_designs`
    netlists of distinct seeds; each job takes one at random), lanes
    log-uniform 32-65,536, cycles log-uniform in `cycles` (the stated range
    is 100-50,000), 30% fault jobs
    (one stuck-at fault per lane, lane-uniform stimulus so every fault-free
    lane equals the golden lane). All jobs run in one launch of the
    persistent job-queue kernel. The plain one-launch-per-cycle path runs a
    seeded subset of `plain_jobs` jobs (every n/plain_jobs-th), which also
    runs alone on the persistent queue, so the speed-up compares the same
    jobs; the subset's hashes and detection vectors must equal the full
    stream's. Graph capture of the plain path is timed on `graph_jobs` of them."""
    from rrtl_gb300.workloads import job_faults, job_stream, job_stream_designs, netlist_run_spec

    t0 = time.perf_counter()
    designs = job_stream_designs(n_designs)
    cds = []
    for d, meta in designs:
        cds.append((meta, sim.CompiledDesign(d.to_json(), meta.top, ctx), netlist_run_spec(meta),
                    netlist_run_spec(meta, uniform=True)))
    del designs
    jobs = job_stream(n_jobs, len(cds), cycles_lo=cycles[0], cycles_hi=cycles[1])
    setup_s = time.perf_counter() - t0

    def make(j, path):
        meta, cd, _, _ = cds[j.design]
        g = sim.GpuBatchSimulator(cd, lanes=j.lanes)
        g.set_path(path)
        if j.fault:
            g.set_faults(job_faults(meta, j.lanes, j.seed))
        return g

    def spec(j):
        stim, rec = cds[j.design][3] if j.fault else cds[j.design][2]
        return stim, rec, sim.REC_HASH | (sim.REC_DETECT if j.fault else 0)

    def queue_run(sub):
        batches = [make(j, sim.PATH_FUSED) for j in sub]
        ctx.synchronize()
        t = time.perf_counter()
        q = []
        for g, j in zip(batches, sub):
            stim, rec, mode = spec(j)
            q.append(ctx.submit(g, j.cycles, seed=j.seed, stim=stim, record=rec, mode=mode))
        ctx.launch()
        ctx.wait()
        wall = time.perf_counter() - t
        outs = [jq.outputs for jq in q]
        widths = sorted({g.tile_words for g in batches})
        return wall, ctx.queue_ms, outs, widths

    lane_cycles = sum(j.lanes * j.cycles for j in jobs)
    gate_evals = sum(j.lanes * j.cycles * cds[j.design][1].info.n_gates for j in jobs)
    persist_s, persist_dev_ms, results, widths = queue_run(jobs)
    # fault coverage: faulted lanes (all but lane 0 of each word) that detected
    fl = fd = 0
    for j, r in zip(jobs, results):
        if j.fault:
            det = r["detect"]
            faulted = np.arange(j.lanes) % 32 != 0
            fl += int(faulted.sum())
            fd += int((det[faulted] != 0xFFFFFFFF).sum())
    fault_free_quiet = all((r["detect"][::32] == 0xFFFFFFFF).all() for j, r in zip(jobs, results) if j.fault)
    out = {"jobs": n_jobs, "design_pool": n_designs, "designs_gates": [m.n_gates for m, _, _, _ in cds],
           "fault_jobs": sum(j.fault for j in jobs), "lane_cycles": lane_cycles, "gate_evals": gate_evals,
           "lanes": "log-uniform 32-65536", "cycles": f"log-uniform {cycles[0]}-{cycles[1]}",
           "persistent": {"value": lane_cycles / persist_s, "unit": "lane-cycles/s", "wall_s": persist_s,
                          "device_ms": persist_dev_ms, "device_value": lane_cycles / (persist_dev_ms / 1e3),
                          "gate_evals_per_s": gate_evals / persist_s, "tile_words": widths, "launches": 1},
           "fault_coverage": {"faulted_lanes": fl, "detected": fd, "frac": fd / max(fl, 1),
                              "fault_free_lanes_quiet": bool(fault_free_quiet),
                              "protocol": "one stuck-at fault per lane, lane-uniform random inputs, detection = first "
                                          "cycle a lane's outputs differ from the fault-free lane 0 of its word"},
           "setup_s": setup_s}
    if plain and plain_jobs:
        step = max(1, len(jobs) // plain_jobs)
        idx = list(range(0, len(jobs), step))[:plain_jobs]
        sub = [jobs[i] for i in idx]
        sub_lc = sum(j.lanes * j.cycles for j in sub)
        q_s, q_ms, q_out, _ = queue_run(sub)
        same = all(np.array_equal(q_out[k]["hash"], results[i]["hash"]) and
                   (q_out[k]["detect"] is None or np.array_equal(q_out[k]["detect"], results[i]["detect"]))
                   for k, i in enumerate(idx))
        per_job = {}
        for name, path, n in (("plain", sim.PATH_PLAIN, len(sub)), ("plain_graph", sim.PATH_PLAIN_GRAPH, graph_jobs)):
            times = []
            for j, i in zip(sub[:n], idx[:n]):
                g = make(j, path)
                stim, rec, mode = spec(j)
                ctx.synchronize()
                t = time.perf_counter()
                r = g.run(j.cycles, seed=j.seed, stim=stim, record=rec, mode=mode)
                times.append(time.perf_counter() - t)
                same = same and np.array_equal(r["hash"], results[i]["hash"]) and (
                    r["detect"] is None or np.array_equal(r["detect"], results[i]["detect"]))
                del g
            per_job[name] = times
        tot = sum(per_job["plain"])
        rates = sorted(j.lanes * j.cycles / t for j, t in zip(sub, per_job["plain"]))
        out["subset"] = {"jobs": len(sub), "indices": f"every {step}th job from 0", "lane_cycles": sub_lc,
                         "persistent": {"value": sub_lc / q_s, "wall_s": q_s, "device_ms": q_ms},
                         "plain": {"value": sub_lc / tot, "wall_s": tot, "launches": sum(j.cycles + 1 for j in sub),
                                   "per_job_rate_min": rates[0], "per_job_rate_median": rates[len(rates) // 2],
                                   "per_job_rate_max": rates[-1]},
                         "unit": "lane-cycles/s"}
        out["speedup_vs_plain"] = out["subset"]["persistent"]["value"] / out["subset"]["plain"]["value"]
        gsum = sum(per_job["plain_graph"])
        out["subset"]["plain_graph"] = {"jobs": graph_jobs, "wall_s": gsum,
                                        "speedup_vs_plain_same_jobs": sum(per_job["plain"][:graph_jobs]) / gsum}
        out["bitexact_across_paths"] = bool(same)
    return out


def serving_leg(ctx, sim, c2, loads, rates, duration_s, cycle_div=50, chunk=128, big=(500_000, 20_000),
                round_us=5_000, policy=None, burst=64):
    """Serving loop (C5): Poisson arrivals over three resident designs (the
    50k-gate netlist, the 8-stage CPU on the word engine, a 500k-gate /
    20k-FF netlist of the same family); lanes log-uniform 64-16,384, cycles
    log-uniform 1,000-50,000 divided by `cycle_div`, stimulus from a
    per-request seed (CPU requests: a per-request window of a hashed ROM).
    First the capacity: a burst of `burst` requests submitted at once, in
    requests/s and lane-cycles/s; then arrivals at each fraction of that
    capacity in `loads` and at each absolute rate in `rates`, each for
    `duration_s` seconds of arrivals (shorter above twice the capacity, so
    the backlog stays at twice what the capacity serves in `duration_s`:
    such a rate measures the overloaded loop, not the length of its queue).
    Reports throughput and p50/p99 latency
    overall and per design; a sample of requests is re-run alone and must
    match bit for bit."""
    from rrtl_gb300.workloads import Rng, cpu_rom_hashed, gate_netlist, log_uniform_int, netlist_run_spec, pipelined_cpu

    policy = sim.SERVE_SHORTEST_FIRST if policy is None else policy
    t0 = time.perf_counter()
    d_big, m_big = gate_netlist(n_gates=big[0], n_ff=big[1], depth=40, seed=5)
    s_big, r_big = netlist_run_spec(m_big)
    cd_big = sim.CompiledDesign(d_big.to_json(), m_big.top, ctx)
    del d_big
    cd_cpu = sim.CompiledDesign(pipelined_cpu(), "Cpu8", ctx)
    rom_pool = cpu_rom_hashed(32768, seed=9)
    cd_c2, s_c2, r_c2 = c2
    designs = [("c2", cd_c2, s_c2, r_c2), ("cpu", cd_cpu, [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)],
                                          ["out_pc", "out_acc"]), ("big", cd_big, s_big, r_big)]
    setup_s = time.perf_counter() - t0
    out = {"designs": {"c2": cd_c2.info.n_gates, "cpu": "8-stage CPU (word engine)", "big": cd_big.info.n_gates},
           "lanes": "log-uniform 64-16384", "cycles": f"log-uniform 1000-50000 / {cycle_div}",
           "chunk_cycles": chunk, "round_us": round_us,
           "policy": "shortest remaining first" if policy == sim.SERVE_SHORTEST_FIRST else "fair share",
           "duration_s": duration_s, "setup_s": setup_s, "rates": []}

    def spec(rng, i):
        k = rng.below(3)
        lanes = log_uniform_int(rng, 64, 16384)
        cycles = max(1, log_uniform_int(rng, 1000, 50000) // cycle_div)
        return k, lanes, cycles, 7000 + i

    def submit(server, k, lanes, cycles, seed):
        name, cd, stim, rec = designs[k]
        mems = None
        if name == "cpu":
            off = seed % (rom_pool.shape[2] - lanes + 1)
            mems = {"rom": rom_pool[:, :, off:off + lanes]}
        return server.submit(cd, lanes, cycles, seed=seed, stim=stim, record=rec, mode=sim.REC_HASH, memories=mems)

    def summarize(handles, t_start, t_end, server, check_sample):
        infos = [h.info() for _, h in handles]
        lat = np.array([(x["done_ns"] - x["submit_ns"]) / 1e6 for x in infos])
        queue = np.array([(x["admit_ns"] - x["submit_ns"]) / 1e6 for x in infos])
        lc = sum(sp[1] * sp[2] for sp, _ in handles)
        st = server.stats
        per = {}
        for k, (name, _, _, _) in enumerate(designs):
            l = np.array([lat[i] for i, (sp, _) in enumerate(handles) if sp[0] == k])
            if len(l):
                per[name] = {"requests": len(l), "p50_ms": float(np.percentile(l, 50)),
                             "p99_ms": float(np.percentile(l, 99))}
        same = True
        if check_sample:
            for sp, h in handles[:: max(1, len(handles) // 4)][:4]:
                k, lanes, cycles, seed = sp
                name, cd, stim, rec = designs[k]
                g = sim.GpuBatchSimulator(cd, lanes=lanes)
                if name == "cpu":
                    off = seed % (rom_pool.shape[2] - lanes + 1)
                    g.set_memory_limbs("rom", rom_pool[:, :, off:off + lanes])
                ref = g.run(cycles, seed=seed, stim=stim, record=rec, mode=sim.REC_HASH)
                same = same and np.array_equal(ref["hash"], h.outputs["hash"])
                del g
        return {"requests": len(handles), "failed": st["failed"], "throughput": lc / (t_end - t_start),
                "unit": "lane-cycles/s", "wall_s": t_end - t_start,
                "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
                "p50_queue_ms": float(np.percentile(queue, 50)) if len(queue) else None,
                "per_design": per, "rounds": st["rounds"], "gpu_busy_frac": st["busy_ns"] / 1e9 / (t_end - t_start),
                "bitexact_sample": bool(same)}

    # capacity: a burst of requests submitted at once
    server = sim.Server(ctx, chunk_cycles=chunk, round_us=round_us, policy=policy)
    rng = Rng(424242)
    handles = []
    t_start = time.perf_counter()
    for i in range(burst):
        sp = spec(rng, i)
        handles.append((sp, submit(server, *sp)))
    server.drain()
    t_end = time.perf_counter()
    cap = summarize(handles, t_start, t_end, server, False)
    server.close()
    capacity = burst / (t_end - t_start)
    out["capacity"] = {"requests_per_s": capacity, "lane_cycles_per_s": cap["throughput"], "burst": burst,
                       "wall_s": cap["wall_s"], "p99_ms": cap["p99_ms"], "per_design": cap["per_design"]}
    plan = [("load", f, f * capacity) for f in loads] + [("rate", r, r) for r in rates]
    for kind, tag, rate in plan:
        server = sim.Server(ctx, chunk_cycles=chunk, round_us=round_us, policy=policy)
        rng = Rng(int(rate * 1000) + 1)
        handles = []
        # above twice the capacity the backlog grows without bound: arrivals
        # stop once they hold twice what the capacity serves in `duration_s`
        window = min(duration_s, duration_s * 2.0 * capacity / rate)
        t_start = time.perf_counter()
        t_next = t_start
        i = 0
        while True:
            t_next += -math.log(1.0 - rng.uniform()) / rate
            if t_next - t_start > window:
                break
            sp = spec(rng, i)
            i += 1
            wait = t_next - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            handles.append((sp, submit(server, *sp)))
        server.drain()
        t_end = time.perf_counter()
        row = summarize(handles, t_start, t_end, server, True)
        row["rate_per_s"] = rate
        row["arrival_window_s"] = round(window, 3)
        if kind == "load":
            row["load_of_capacity"] = tag
        out["rates"].append(row)
        server.close()
    return out


def word_configs_leg(ctx, sim, cpu8_cycles=20_000, counter=True, parity_lanes=16384):
    """The word-engine configs: the README Counter (1,024 lanes x 10,000
    cycles, full output trace recorded) and the 8-stage pipelined CPU
    (16,384 lanes x 20,000 cycles, per-lane hashed ROMs). The fused path runs
    the design's compiled kernel; each config is also timed on the
    interpreted word kernel (whole run, one launch) and on the plain
    one-launch-per-cycle path (200 cycles of the same batch shape). Parity at
    the stated sizes: the Counter's full trace, and the CPU's per-cycle hash
    over all 20,000 cycles plus the final register file, PC, pipeline
    registers and data memory of the first `parity_lanes` lanes (all of them
    by default; 0 skips it), against the SIMD-shaped packed engine (oracle)
    on every host thread. The CPU run is timed three ways: CUDA events inside
    the library around its kernels, CUDA events on the stream around the
    whole call (table uploads and output copies included), and the host
    clock."""
    from oracle import binding as ob
    from rrtl_gb300.workloads import counter as counter_design, cpu_rom_hashed, pipelined_cpu

    out = {}
    if counter:
        cjs = counter_design().to_json()
        cd = sim.CompiledDesign(cjs, "Counter", ctx)
        jit, jit_ms, why = cd.word_jit()
        stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1), ("en", sim.STIM_RANDOM, 1)]
        for path, cyc, key in ((sim.PATH_FUSED, 10_000, "value"), (sim.PATH_WORD_INTERP, 10_000, "interpreted"),
                               (sim.PATH_PLAIN, 200, "plain")):
            g = sim.GpuBatchSimulator(cd, lanes=1024)
            g.set_path(path)
            r = g.run(cyc, seed=1, stim=stim, record=["out"], mode=sim.REC_TRACE)
            v = 1024 * cyc / (g.last_kernel_ms / 1e3)
            if key == "value":
                out["counter"] = {"lanes": 1024, "cycles": cyc, "value": v, "unit": "lane-cycles/s",
                                  "kernel_ms": g.last_kernel_ms, "trace_bytes": 1024 * cyc * 4, "compiled": jit,
                                  "compile_ms": jit_ms}
                if parity_lanes:
                    od = ob.OracleDesign(cjs, "Counter")
                    ps = ob.SimdSim(od, 1024)
                    tr = np.zeros((cyc, 1, 1024), dtype=np.uint32)
                    ps.run(ob.make_run(cyc, 1, [(od.signal(n), k, p) for n, k, p in stim], [od.signal("out")], 1,
                                       out_trace=tr))
                    out["counter"]["parity"] = {"equal": bool(np.array_equal(tr, r["trace"])),
                                                "checked": "full out trace, 1,024 lanes x 10,000 cycles",
                                                "oracle": "SIMD-shaped packed engine"}
            else:
                out["counter"][key] = v
    cjs = pipelined_cpu().to_json()
    cd = sim.CompiledDesign(cjs, "Cpu8", ctx)
    jit, jit_ms, why = cd.word_jit()
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)]
    rom = cpu_rom_hashed(16384, seed=3)
    res = {}
    for path, cyc in ((sim.PATH_FUSED, cpu8_cycles), (sim.PATH_WORD_INTERP, 2_000), (sim.PATH_PLAIN, 200)):
        g = sim.GpuBatchSimulator(cd, lanes=16384)
        g.set_path(path)
        g.set_memory_limbs("rom", rom)
        r = g.run(cyc, stim=stim, record=["out_pc", "out_acc"], mode=sim.REC_HASH)
        res[path] = (1.0e3 * 16384 * cyc / g.last_kernel_ms, r["hash"], g)
    h = res[sim.PATH_FUSED][1]
    n = min(2000, cpu8_cycles)
    same = bool(np.array_equal(h[:200], res[sim.PATH_PLAIN][1][:200]) and
                np.array_equal(h[:n], res[sim.PATH_WORD_INTERP][1][:n]))
    gf = res[sim.PATH_FUSED][2]
    # the same run again on a fresh batch, timed three ways
    g2 = sim.GpuBatchSimulator(cd, lanes=16384)
    g2.set_memory_limbs("rom", rom)
    ctx.synchronize()
    t0 = time.perf_counter()
    ctx.record(6)
    g2.run(cpu8_cycles, stim=stim, record=["out_pc", "out_acc"], mode=sim.REC_HASH)
    ctx.record(7)
    stream_ms = ctx.elapsed_ms(6, 7)
    wall_ms = (time.perf_counter() - t0) * 1e3
    kernel_ms = g2.last_kernel_ms
    del g2
    timing = {"kernel_events_ms": kernel_ms, "stream_events_ms": stream_ms, "wall_ms": wall_ms,
              "kernel_events_value": 16384 * cpu8_cycles / (kernel_ms / 1e3),
              "stream_events_value": 16384 * cpu8_cycles / (stream_ms / 1e3),
              "wall_value": 16384 * cpu8_cycles / (wall_ms / 1e3)}
    out["cpu8"] = {"lanes": 16384, "cycles": cpu8_cycles, "value": res[sim.PATH_FUSED][0], "unit": "lane-cycles/s",
                   "interpreted": res[sim.PATH_WORD_INTERP][0], "interpreted_cycles": 2_000,
                   "plain": res[sim.PATH_PLAIN][0], "hash_prefix_equal_all_paths": same, "compiled": jit,
                   "compile_ms": jit_ms, "timing": timing,
                   "note": "one thread per lane: 16,384 lanes are 512 warps, under one per warp scheduler, so "
                           "the run is bound by one warp's dependent-instruction latency"}
    if parity_lanes:
        # parity against the SIMD-shaped packed engine at the stated size
        od = ob.OracleDesign(cjs, "Cpu8")
        pl = min(parity_lanes, 16384)
        t = time.perf_counter()
        h_or, v_or, m_or = ob.simd_run_parallel(od, pl, cpu8_cycles, 0, [(od.signal(nm), k, p) for nm, k, p in stim],
                                                [od.signal("out_pc"), od.signal("out_acc")], 2,
                                                memories={od.memory("rom"): rom[:, :, :pl]}, snapshot=True)
        odt = time.perf_counter() - t
        v_gpu, m_gpu = gf.snapshot_storage()
        tsw, tmw = od.total_signal_words, od.total_memory_words
        v_gpu = v_gpu.reshape(tsw, 16384)[:, :pl].reshape(-1)
        m_gpu = m_gpu.reshape(16384, tmw)[:pl].reshape(-1)
        parity = {"state_equal": bool(np.array_equal(v_gpu, v_or) and np.array_equal(m_gpu, m_or)),
                  "lanes": pl, "cycles": cpu8_cycles,
                  "oracle": f"SIMD-shaped packed engine, {os.cpu_count()} host threads", "oracle_s": round(odt, 2),
                  "checked": "final signal words (register-file read ports, PC, pipeline registers, accumulator) and "
                             "all memory words (register file, data memory, ROM) of every checked lane"}
        if pl == 16384:
            parity["hash_equal"] = bool(np.array_equal(h, h_or))
            parity["checked"] += f", and the per-cycle hash of out_pc/out_acc over all {cpu8_cycles} cycles"
        parity["equal"] = parity["state_equal"] and parity.get("hash_equal", True)
        out["cpu8"]["parity"] = parity
    return out


def crc32_netlist():
    """The reference's crc32 gate netlist (bench/sv/crc32_gates.json), from the
    committed compact fixture."""
    from rrtl_gb300.netlist import import_yosys_netlist

    c = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                                    "crc32_gates.compact.json")))
    y = {"modules": {c["top"]: {
        "ports": {k: {"direction": d, "bits": b} for k, (d, b) in c["ports"].items()},
        "cells": {f"c{i:04d}": {"type": t, "connections": conns} for i, (t, conns) in enumerate(c["cells"])}}}}
    return import_yosys_netlist(y, c["top"])


def crc32_leg(ctx, sim, cycles=2000):
    """The reference's headline GPU workload: its per-design compiled gate
    kernel on the crc32 netlist (docs/rrtl-optimizations.md:1725-1734, M3 /
    OpenCL: 4,182 / 4,719 / 19,315 / 17,129 M lane-cycles/s at 16K / 65K /
    256K / 1M lanes). Random din per lane per cycle, reset on cycle 0; the
    compiled gate kernel with no per-cycle recording (state only, like the
    reference's run) and with a per-cycle hash of the 32 crc outputs, the
    fused kernel (tile width 8) beside it; per-cycle hashes compared."""
    cd = sim.CompiledDesign(crc32_netlist(), "crc32", ctx)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)] + [(f"din_{i}", sim.STIM_RANDOM, i) for i in range(8)]
    rec = [f"crc_{i}" for i in range(32)]
    rows = []
    for lanes in (16384, 65536, 262144, 1048576):
        row = {"lanes": lanes}
        hashes = {}
        for key, words, mode in (("compiled", 0, 0), ("compiled_hash", 0, sim.REC_HASH), ("fused_hash", 8, sim.REC_HASH)):
            g = sim.GpuBatchSimulator(cd, lanes=lanes)
            if words:
                g.set_tile_words(words)
            g.run(10, stim=stim, record=rec, mode=mode)
            best = float("inf")
            for _ in range(3):
                r = g.run(cycles, stim=stim, record=rec, mode=mode)
                best = min(best, g.last_kernel_ms)
            row[key] = lanes * cycles / (best / 1e3)
            if mode:
                hashes[key] = r["hash"]
        row["hash_equal"] = bool(np.array_equal(hashes["compiled_hash"], hashes["fused_hash"]))
        rows.append(row)
    return {"cycles": cycles, "unit": "lane-cycles/s", "cells": cd.info.n_gates, "rows": rows,
            "reference_m3_opencl": {"16384": 4.182e9, "65536": 4.719e9, "262144": 1.9315e10, "1048576": 1.7129e10,
                                    "note": "published Apple M3 numbers, unavailable on this box (OpenCL.framework)"}}


def bitslice_leg(ctx, sim, cycles=1000):
    """Bit-sliced multi-bit evaluation: a 16-bit ALU datapath (add, sub, xor,
    compare, mux; no multiply or memory) run as bit-planes on the gate engine
    against the word engine's compiled kernel, random inputs, no recording."""
    from rrtl_gb300.workloads import narrow_alu

    js = narrow_alu(16).to_json()
    planes = sim.CompiledDesign(js, "Alu", ctx, bitslice=True)
    words = sim.CompiledDesign(js, "Alu", ctx)
    rows = []
    for lanes in (65536, 1048576):
        row = {"lanes": lanes}
        for key, cd, stim in (
                ("bitsliced", planes, [("__bitslice_clk", sim.STIM_CONST, 1), ("rst[0]", sim.STIM_PULSE, 1)] +
                 [(f"din[{p}]", sim.STIM_RANDOM, p) for p in range(16)] + [(f"sel[{p}]", sim.STIM_RANDOM, 20 + p)
                                                                          for p in range(2)]),
                ("word", words, [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1), ("din", sim.STIM_RANDOM, 1),
                                 ("sel", sim.STIM_RANDOM, 2)])):
            g = sim.GpuBatchSimulator(cd, lanes=lanes)
            g.run(10, stim=stim)
            best = float("inf")
            for _ in range(3):
                g.run(cycles, stim=stim)
                best = min(best, g.last_kernel_ms)
            row[key] = lanes * cycles / (best / 1e3)
        rows.append(row)
    return {"design": "16-bit ALU datapath", "cycles": cycles, "unit": "lane-cycles/s",
            "plane_cells": planes.info.n_gates, "word_instrs": words.info.n_gates, "rows": rows}


def instance_fold_leg(ctx, sim, cycles=2000):
    """Instance folding: a wrapper of 64 independent 32-bit datapaths,
    flattened (one program with 64 copies, `base` lanes) against folded (the
    datapath once, 64 x `base` lanes), in datapath-cycles/s (instances x base
    lanes x cycles per second, the same total work both ways), at the base
    lane counts of the reference's table (docs/rrtl-optimizations.md:544-572).
    Outputs of every instance are compared between the two."""
    from rrtl_gb300.workloads import replicated_datapath

    n = 64
    js = replicated_datapath(n).to_json()
    flat_d = sim.CompiledDesign(js, "Top", ctx)
    plan = sim.instance_fold_plan(js, "Top")
    fold_d = sim.CompiledDesign(js, plan["child"], ctx)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 2)]
    rows = []
    for base in (64, 1024, 4096):
        rng = np.random.default_rng(base)
        din = rng.integers(0, 2**32, size=(cycles, n, base), dtype=np.uint64).astype(np.uint32)
        gf = sim.GpuBatchSimulator(flat_d, lanes=base)
        rf = gf.run(cycles, stim=stim + [(f"din{i}", sim.STIM_TRACE, i) for i in range(n)],
                    record=[f"o{i}" for i in range(n)], mode=sim.REC_TRACE, input_trace=din)
        flat_ms = gf.last_kernel_ms
        gc = sim.GpuBatchSimulator(fold_d, lanes=n * base)
        rc = gc.run(cycles, stim=stim + [("din", sim.STIM_TRACE, 0)], record=["o"], mode=sim.REC_TRACE,
                    input_trace=din.reshape(cycles, 1, n * base))
        fold_ms = gc.last_kernel_ms
        same = bool(np.array_equal(rc["trace"][:, 0, :].reshape(cycles, n, base), rf["trace"]))
        work = n * base * cycles
        rows.append({"base_lanes": base, "flattened": work / (flat_ms / 1e3), "folded": work / (fold_ms / 1e3),
                     "speedup": flat_ms / fold_ms, "bitexact": same})
    return {"instances": n, "cycles": cycles, "unit": "datapath-cycles/s",
            "program_instrs": {"flattened": flat_d.info.n_gates, "folded": fold_d.info.n_gates}, "rows": rows}


def run_reference(args, ws, rank):
    """The reference's CPU implementation of the path on the host cores: the
    AOT bit-parallel engine restated (see cpu_baseline: the same emitted C,
    flags and threads), each step a bounded sample of the same workload long
    enough (at least half a second) that thread start-up is noise."""
    if rank != 0:
        return
    d, meta, js, stim, rec = build_workload()
    from oracle import binding as ob

    od = ob.OracleDesign(js, meta.top)
    stim_idx = [(od.signal(n), k, p) for n, k, p in stim]
    rec_idx = [od.signal(r) for r in rec]
    threads = os.cpu_count() or 1
    aot, _ = aot_engine(od, stim_idx, rec_idx)
    lanes = 64 * threads * 8
    # step length: at least 0.6 s of simulation, so thread start-up is noise
    # (the probe's per-cycle time includes that start-up, so grow until a
    # probe of the chosen length itself lasts long enough)
    cycles = 32
    for _ in range(6):
        t = time.perf_counter()
        aot.run(lanes, cycles, SEED)
        dt = time.perf_counter() - t
        if dt >= 0.6:
            break
        cycles = max(cycles + 1, int(cycles * 0.7 / max(dt, 1e-4)))
    vals = []
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        aot.run(lanes, cycles, SEED)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            vals.append(dt)
    tot = sum(vals)
    value = lanes * cycles * len(vals) / tot
    line = {
        "metric": METRIC, "value": value, "unit": "lane-cycles/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * tot / len(vals), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64 bit-sliced", "data": "synthetic (seeded netlist and stimulus)",
        "impl": "reference",
        "config": {"workload": f"gate netlist {GATES} gates / {FFS} FF / {PIS} PI / {POS} PO / depth {DEPTH}",
                   "lanes_per_step": lanes, "cycles_per_step": cycles, "parallelism": f"{threads} host threads"},
        "cpu_baseline": {"value": value, "unit": "lane-cycles/s", "cores": threads, "kind": "port",
                         "sample": f"{lanes} lanes x {cycles} cycles per step (bit-parallel AOT restated from "
                                   f"crates/rrtl-sim-ir/src/bitparallel.rs:348-528, gcc {' '.join(aot.flags)})"},
        "e2e": {"value": value, "unit": "lane-cycles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e-trace", action="store_true", help="skip the e2e leg with a host-resident input trace")
    ap.add_argument("--lanes", type=int, default=LANES, help="lanes per GPU (profiling cases)")
    ap.add_argument("--cycles", type=int, default=CYCLES, help="cycles per step (profiling cases)")
    ap.add_argument("--tile-words", type=int, default=0, help="fused tile width in 32-lane words (0 = automatic)")
    ap.add_argument("--jobs", type=int, default=2048, help="jobs in the uneven job-stream leg (0 = skip it)")
    ap.add_argument("--job-designs", type=int, default=16, help="netlists of distinct seeds in the job stream's pool")
    ap.add_argument("--plain-jobs", type=int, default=12, help="job stream: jobs of the subset timed on the plain path")
    ap.add_argument("--job-cycles", default="10,5000",
                    help="job stream: cycle range lo,hi (the stated range 100,50000 takes about 6 minutes of GPU "
                         "time; the default divides it by 10)")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle checks of the benchmarked runs")
    ap.add_argument("--cpu8-parity-lanes", type=int, default=16384,
                    help="pipelined CPU: lanes checked against the oracle after the full run")
    ap.add_argument("--no-plain-jobs", action="store_true", help="job stream: skip the plain-path comparison")
    ap.add_argument("--serve-loads", default="0.5,0.9",
                    help="serving leg: arrival rates as fractions of the measured capacity ('' = none)")
    ap.add_argument("--serve-rates", default="50,2000", help="serving leg: absolute arrival rates per second ('' = none)")
    ap.add_argument("--serve-cycle-div", type=int, default=50, help="serving leg: request cycles divided by this")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-word-configs", action="store_true", help="skip the Counter and pipelined-CPU legs")
    ap.add_argument("--serve-seconds", type=float, default=5.0, help="serving leg arrival window per rate")
    ap.add_argument("--serve-round-us", type=int, default=5_000, help="serving loop target round time")
    ap.add_argument("--word-only", action="store_true",
                    help="profiling case: only the pipelined-CPU word config (its compiled run is the second "
                         "rrtl_word_jit launch, after the batch's creation settle)")
    ap.add_argument("--cpu8-cycles", type=int, default=20_000, help="cycles of the pipelined-CPU compiled run")
    ap.add_argument("--no-fold", action="store_true", help="skip the instance-folding leg")
    ap.add_argument("--no-crc32", action="store_true", help="skip the crc32 compiled-gate-kernel leg")
    ap.add_argument("--no-bitslice", action="store_true", help="skip the bit-slice leg")
    ap.add_argument("--crc32-only", action="store_true", help="only the crc32 leg")
    ap.add_argument("--fold-only", action="store_true", help="only the instance-folding leg")
    args = ap.parse_args()
    globals()["LANES"], globals()["CYCLES"] = args.lanes, args.cycles
    args.warmup = max(args.warmup, 3)
    ws, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        if dist:
            dist.barrier()
        return

    import torch

    from rrtl_gb300 import sim

    if args.word_only:
        ctx = sim.Context(local)
        if rank == 0:
            print(json.dumps({"word_configs": word_configs_leg(ctx, sim, args.cpu8_cycles, counter=False)}))
        return
    if args.fold_only:
        ctx = sim.Context(local)
        if rank == 0:
            print(json.dumps({"instance_fold": instance_fold_leg(ctx, sim)}))
        return
    if args.crc32_only:
        ctx = sim.Context(local)
        if rank == 0:
            print(json.dumps({"crc32": crc32_leg(ctx, sim), "bitslice": bitslice_leg(ctx, sim)}))
        return
    d, meta, js, stim, rec = build_workload()
    ctx = sim.Context(local)
    cd = sim.CompiledDesign(js, meta.top, ctx)
    info = cd.info
    g = sim.GpuBatchSimulator(cd, lanes=LANES)
    g.set_tile_words(args.tile_words)
    dev = torch.device("cuda", local)
    hash_dev = [torch.zeros(CYCLES, dtype=torch.int64, device=dev) for _ in range(args.steps + args.warmup)]

    # rank r simulates global lanes [r*L, (r+1)*L) of one run: stimulus and
    # hashes follow global lanes, so the ranks' shards compose into one job
    lane_base = rank * LANES

    def device_run(i, path=sim.PATH_FUSED, cycles=CYCLES):
        g.set_path(path)
        r = g.make_run(cycles, seed=SEED + i, stim=stim, record=rec, mode=sim.REC_HASH, lane_base=lane_base)
        r.out_hash = ctypes_u64(hash_dev[i].data_ptr())
        sim.check(sim.lib().rrtl_batch_run_device(g.h, sim.byref(r)))

    # warm-up, then K timed steps back to back on the engine's stream
    for i in range(args.warmup):
        device_run(i)
    ctx.synchronize()
    tile_words = g.tile_words
    if dist:
        dist.barrier()
    with ClockSampler(local) as clocks:
        ctx.record(0)
        for i in range(args.steps):
            device_run(args.warmup + i)
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1)
    ms = reduce_max(dist, ms)
    lane_cycles = ws * LANES * CYCLES * args.steps
    value = throughput(ws, LANES, CYCLES, args.steps, ms)
    ms_step = ms / args.steps

    # e2e: same steps through the C ABI with pinned host buffers
    hash_host = torch.zeros(CYCLES, dtype=torch.int64, pin_memory=True)
    words = (LANES + 31) // 32
    regs_host = torch.zeros((FFS, words), dtype=torch.int32, pin_memory=True)
    reg_idx = np.asarray([cd.signal(q)[0] for q in meta.regs], dtype=np.uint32)
    h2d = len(stim) * 16 + len(rec) * 4
    d2h = CYCLES * 8 + FFS * words * 4
    ctx.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    ctx.record(2)
    for i in range(args.steps):
        g.set_path(sim.PATH_FUSED)
        r = g.make_run(CYCLES, seed=SEED + i, stim=stim, record=rec, mode=sim.REC_HASH, lane_base=lane_base)
        r.out_hash = ctypes_u64(hash_host.data_ptr())
        sim.check(sim.lib().rrtl_batch_run(g.h, sim.byref(r)))
        sim.check(sim.lib().rrtl_batch_get_signals_bits(g.h, reg_idx.ctypes.data_as(sim.POINTER(sim.c_uint32)),
                                                        len(reg_idx), ctypes_u32(regs_host.data_ptr()), FFS * words))
    ctx.record(3)
    e2e_ms = ctx.elapsed_ms(2, 3)
    e2e_ms = reduce_max(dist, e2e_ms)
    e2e_value = throughput(ws, LANES, CYCLES, args.steps, e2e_ms)

    # e2e with host stimulus: the primary inputs as a host-resident (pinned)
    # input trace, copied to the device inside every step, as a caller with
    # its own stimulus would drive the batch. The trace holds the bits the
    # on-device generator gives for seed SEED, so the run's per-cycle hash
    # must equal the first warm-up step's from cycle 1 on (cycle 0's outputs
    # depend on the state the previous run left; the reset pulse clears
    # every register at the end of cycle 0).
    e2e_trace = None
    if not args.no_e2e_trace:
        pis = [n for n, k, p in stim if k == sim.STIM_RANDOM]
        tr = torch.empty((CYCLES, len(pis), words), dtype=torch.int32, pin_memory=True)
        trn = tr.numpy().view(np.uint32)
        g.set_path(sim.PATH_FUSED)
        r = g.make_run(CYCLES, seed=SEED, stim=stim, record=pis, mode=sim.REC_TRACE, out_trace=trn, lane_base=lane_base)
        sim.check(sim.lib().rrtl_batch_run(g.h, sim.byref(r)))
        tstim = [(n, k, p) for n, k, p in stim if k != sim.STIM_RANDOM] + [(n, sim.STIM_TRACE, i) for i, n in enumerate(pis)]
        ctx.synchronize()
        if dist:
            dist.barrier()
        ctx.record(2)
        for i in range(args.steps):
            r = g.make_run(CYCLES, seed=SEED, stim=tstim, record=rec, mode=sim.REC_HASH, input_trace=trn,
                           lane_base=lane_base)
            r.out_hash = ctypes_u64(hash_host.data_ptr())
            sim.check(sim.lib().rrtl_batch_run(g.h, sim.byref(r)))
            sim.check(sim.lib().rrtl_batch_get_signals_bits(g.h, reg_idx.ctypes.data_as(sim.POINTER(sim.c_uint32)),
                                                            len(reg_idx), ctypes_u32(regs_host.data_ptr()), FFS * words))
        ctx.record(3)
        t_ms = reduce_max(dist, ctx.elapsed_ms(2, 3))
        same = bool(torch.equal(hash_host[1:], hash_dev[0].cpu()[1:]))
        e2e_trace = {"value": throughput(ws, LANES, CYCLES, args.steps, t_ms), "unit": "lane-cycles/s",
                     "h2d_bytes_per_step": int(trn.nbytes) + len(tstim) * 16 + len(rec) * 4, "d2h_bytes_per_step": d2h,
                     "input_trace": f"{len(pis)} inputs x {words} words x {CYCLES} cycles, pinned host memory",
                     "hash_equal_to_device_stimulus": same, "hash_cycles_compared": f"1-{CYCLES - 1}"}
        del tr, trn

    # plain one-launch-per-cycle path on the same workload (fewer cycles; same per-cycle work)
    plain = None
    if not args.no_plain:
        pc = 100
        device_run(0, sim.PATH_PLAIN, pc)
        ctx.synchronize()
        ctx.record(4)
        device_run(0, sim.PATH_PLAIN, pc)
        ctx.record(5)
        pms = ctx.elapsed_ms(4, 5)
        plain = {"value": LANES * pc / (pms / 1000.0) * ws, "unit": "lane-cycles/s", "cycles_timed": pc,
                 "launches": pc + 1}

    del g
    clock_summary = clocks.summary()
    # the headline run at its full size against the oracle (rank 0's shard)
    parity = {}
    aot = aot_compile_s = od = None
    if rank == 0 and not args.no_parity:
        from oracle import binding as ob

        od = ob.OracleDesign(js, meta.top)
        aot, aot_compile_s = aot_engine(od, [(od.signal(n), k, p) for n, k, p in stim], [od.signal(r) for r in rec])
        parity["c2"] = c2_parity(sim, cd, meta, stim, rec, aot, od, LANES, CYCLES, lane_base)

    peak, peak_kind = load_peaks()
    bpl = net_stream_bytes_per_lane_cycle(gate_fanins(js), FFS, PIS, POS)
    algo_bytes = bpl * LANES * CYCLES
    achieved = algo_bytes / (ms_step / 1000.0) / 1e9
    # the roof that binds: every cell-word evaluation reads its fanin rows and
    # writes its output row in shared memory, so the net-streaming bytes are
    # the kernel's shared-memory traffic; the nominal shared-memory bandwidth
    # is 128 bytes per clock per SM
    sm_mhz = clock_summary.get("sm_mhz") or 2070.0
    smem_peak = ctx.sm_count * 128.0 * sm_mhz * 1e6 / 1e9
    issue = profiled_issue("gate_fused_kernel_c2.md")
    # DRAM traffic of one launch grows with lanes (closing write-back of every
    # net), not with cycles (per-cycle work stays in shared memory and L2)
    traffic, tlanes = profiled_traffic("gate_fused_kernel_c2.md")
    if traffic is not None:
        traffic = traffic * LANES / tlanes
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback", "bytes_per_lane_cycle": bpl,
                "model": "net-streaming bytes per lane-cycle (fanin reads + output write per gate, D read + Q write "
                         "per flop, inputs and outputs), 4 bytes per 32 lanes",
                "note": "nets stay in shared memory for all cycles of a tile, so measured DRAM traffic per launch "
                        "(traffic) is far below the streamed bytes (achieved*time): HBM does not bind this kernel; "
                        "the shared-memory roof below does",
                "smem": {"bound": "smem", "achieved": achieved, "peak": smem_peak, "unit": "GB/s",
                         "frac": achieved / smem_peak,
                         "peak_kind": f"nominal: {ctx.sm_count} SMs x 128 B/clock x {sm_mhz:.0f} MHz (sampled SM clock)",
                         "model": "the net-streaming bytes are the cell evaluations' shared-memory row reads and "
                                  "writes"},
                "issue": issue}
    out = {
        "metric": METRIC, "value": value, "unit": "lane-cycles/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 bit-sliced (32 lanes per word)", "data": "synthetic (seeded netlist and stimulus)",
        "config": {"workload": f"gate netlist {GATES} gates / {FFS} FF / {PIS} PI / {POS} PO / depth {DEPTH} / "
                               f"window {WINDOW}", "lanes_per_gpu": LANES, "cycles_per_step": CYCLES,
                   "global_lanes": LANES * ws, "parallelism": f"lane shards x{ws} (no collective; rank r simulates "
                                                     f"global lanes [r*{LANES}, (r+1)*{LANES}) of one run)",
                   "l2": "lane state 428 MB > 129 MB L2 (no flush)", "path": ("fused persistent kernel (generic: RRTL_FUSED_JIT=0)" if os.environ.get("RRTL_FUSED_JIT", "1")[:1] == "0"
                            else "fused persistent kernel compiled for the design's truth-table classes (NVRTC)"),
                   "tile_words": tile_words},
        "gate_evals_per_s": value * info.n_gates,
        "design": {"gates": info.n_gates, "levels": info.n_levels, "nets": info.n_nets, "slots": info.n_slots,
                   "flops": info.n_regs},
        "e2e": {"value": e2e_value, "unit": "lane-cycles/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "e2e_host_trace": e2e_trace,
        "plain_path": plain,
        "roofline": roofline,
        "gpu_launches": args.steps,
        "clocks": clock_summary,
        "parity": parity,
    }
    if not args.no_word_configs:
        out["word_configs"] = word_configs_leg(ctx, sim, args.cpu8_cycles,
                                               parity_lanes=0 if rank != 0 or args.no_parity else args.cpu8_parity_lanes)
        wc = out["word_configs"]
        if "counter" in wc and "parity" in wc["counter"]:
            parity["c1"] = wc["counter"]["parity"]
        if "parity" in wc["cpu8"]:
            parity["c3"] = wc["cpu8"]["parity"]
    if not args.no_fold:
        out["instance_fold"] = instance_fold_leg(ctx, sim)
    if not args.no_crc32:
        out["crc32"] = crc32_leg(ctx, sim)
    if not args.no_bitslice:
        out["bitslice"] = bitslice_leg(ctx, sim)
    if args.jobs > 0:
        lo, hi = (int(x) for x in args.job_cycles.split(","))
        out["job_stream"] = job_stream_leg(ctx, sim, args.jobs, args.job_designs, plain=not args.no_plain_jobs,
                                           plain_jobs=args.plain_jobs, cycles=(lo, hi))
    if not args.no_serving:
        loads = [float(x) for x in args.serve_loads.split(",") if x]
        rates = [float(x) for x in args.serve_rates.split(",") if x]
        out["serving"] = serving_leg(ctx, sim, (cd, stim, rec), loads, rates, args.serve_seconds,
                                     cycle_div=args.serve_cycle_div, round_us=args.serve_round_us)
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import binding as ob

        od = od or ob.OracleDesign(js, meta.top)
        si, ri = [(od.signal(n), k, p) for n, k, p in stim], [od.signal(r) for r in rec]
        if aot is None:
            aot, aot_compile_s = aot_engine(od, si, ri)
        out["cpu_baseline"] = cpu_baseline(od, aot, aot_compile_s, si, ri)
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.barrier()


def ctypes_u64(ptr):
    import ctypes

    return ctypes.cast(ctypes.c_void_p(ptr), ctypes.POINTER(ctypes.c_uint64))


def ctypes_u32(ptr):
    import ctypes

    return ctypes.cast(ctypes.c_void_p(ptr), ctypes.POINTER(ctypes.c_uint32))


if __name__ == "__main__":
    main()
