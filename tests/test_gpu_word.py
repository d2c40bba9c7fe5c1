"""GPU parity of the lane-per-thread word engine against the packed oracle."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.builder import Design, lit_u, mux, uint
from rrtl_gb300.workloads import counter

from .helpers import oracle_packed_run

pytestmark = pytest.mark.gpu


def test_counter_known_answer(engine):
    """crates/rrtl-gpu-sim/src/lib.rs:5763-5787: rst=[1,0,0,0], en=[1,0,1,1]; tick; rst=0; tick -> [1,0,2,2]."""
    d = Design()
    m = d.module("Counter")
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    en = m.input("en", uint(1))
    count = m.reg("count", uint(8))
    m.clock(count, clk)
    m.reset(count, rst, 0)
    m.next(count, mux(en, count + lit_u(1, 8), count))
    g = sim.GpuBatchSimulator(d, "Counter", 4)
    assert g.design.info.engine == sim.ENGINE_WORD
    g.set_input("rst", [1, 0, 0, 0])
    g.set_input("en", [1, 0, 1, 1])
    g.tick()
    g.set_input("rst", [0, 0, 0, 0])
    g.tick()
    assert list(g.get_signal("count")) == [1, 0, 2, 2]


@pytest.mark.parametrize("path", [sim.PATH_FUSED, sim.PATH_PLAIN])
def test_counter_1024_lanes_10k_cycles(engine, path):
    """Counter, 1,024 lanes x 10,000 cycles, rst on cycle 0, en ~ Bernoulli(0.5): full out trace."""
    d = counter()
    g = sim.GpuBatchSimulator(d, "Counter", 1024)
    g.set_path(path)
    cycles = 10_000
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1), ("en", sim.STIM_RANDOM, 0)]
    res = g.run(cycles, seed=1, stim=stim, record=["out"], mode=sim.REC_TRACE | sim.REC_HASH)
    tr = res["trace"][:, 0, :]
    # closed form of the design: count' = rst ? 0 : count + en (mod 256); out samples count before the edge
    from rrtl_gb300.workloads import stim_word

    lanes = np.arange(1024)
    cnt = np.zeros(1024, dtype=np.int64)
    for c in range(cycles):
        assert np.array_equal(tr[c], cnt), c
        words = np.array([stim_word(1, 0, c, w) for w in range(32)], dtype=np.uint64)
        en = (words[lanes // 32] >> (lanes % 32).astype(np.uint64)) & 1
        cnt = np.zeros(1024, dtype=np.int64) if c < 1 else (cnt + en.astype(np.int64)) % 256
    od = ob.OracleDesign(d.to_json(), "Counter")
    small = 96
    gs = sim.GpuBatchSimulator(d, "Counter", small)
    r2 = gs.run(400, seed=1, stim=stim, record=["out"], mode=sim.REC_TRACE | sim.REC_HASH)
    ref = oracle_packed_run(od, small, 400, 1, [(od.signal(n), k, p) for n, k, p in stim], [od.signal("out")], 3)
    assert np.array_equal(r2["trace"], ref["trace"])
    assert np.array_equal(r2["hash"], ref["hash"])


@pytest.mark.parametrize("seed", range(16))
def test_random_designs_match_packed_oracle(engine, seed):
    """Random word-level designs (every expression kind, memories with a write
    port, synchronous and asynchronous resets): trace, per-cycle hash and the
    final storage snapshot are bit-exact against PackedSimulator."""
    from .designs import random_word_design

    d, meta = random_word_design(seed, n_wires=16, depth=3)
    js = d.to_json()
    lanes, cycles = 70, 24
    g = sim.GpuBatchSimulator(js, meta["top"], lanes)
    assert g.design.info.engine == sim.ENGINE_WORD
    od = ob.OracleDesign(js, meta["top"])
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 2)]
    stim += [(n, sim.STIM_RANDOM, i + 7) for i, (n, w) in enumerate(meta["inputs"])]
    rec = [n for n, w in meta["outputs"]]
    res = g.run(cycles, seed=seed, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH)
    ref = oracle_packed_run(od, lanes, cycles, seed, [(od.signal(n), k, p) for n, k, p in stim],
                            [od.signal(r) for r in rec], 3)
    assert np.array_equal(res["trace"], ref["trace"])
    assert np.array_equal(res["hash"], ref["hash"])
    v, m = g.snapshot_storage()
    rv, rm = ref["sim"].snapshot()
    assert np.array_equal(v, rv)
    assert np.array_equal(m, rm)


@pytest.mark.parametrize("path", [sim.PATH_FUSED, sim.PATH_PLAIN, sim.PATH_WORD_INTERP])
def test_pipelined_cpu_matches_oracle(engine, path):
    """8-stage pipelined CPU with per-lane random ROMs: PC/accumulator trace,
    register file and data memory bit-exact against PackedSimulator."""
    from rrtl_gb300.workloads import cpu_rom, pipelined_cpu

    d = pipelined_cpu()
    js = d.to_json()
    lanes, cycles = 48, 300
    rom = cpu_rom(lanes, seed=11)
    g = sim.GpuBatchSimulator(js, "Cpu8", lanes)
    g.set_path(path)
    g.set_memory_limbs("rom", rom)
    od = ob.OracleDesign(js, "Cpu8")
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)]
    rec = ["out_pc", "out_acc"]
    res = g.run(cycles, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH)
    ps = ob.PackedSim(od, lanes)
    ps.set_memory(od.memory("rom"), rom)
    r = ob.make_run(cycles, 0, [(od.signal(n), k, p) for n, k, p in stim], [od.signal(x) for x in rec], 3,
                    out_trace=np.zeros((cycles, 3, lanes), dtype=np.uint32), out_hash=np.zeros(cycles, dtype=np.uint64))
    ps.run(r)
    assert np.array_equal(res["trace"], r._keep[3])
    assert np.array_equal(res["hash"], r._keep[4])
    for mem in ("rf", "dmem"):
        depth = 16 if mem == "rf" else 1024
        assert np.array_equal(g.get_memory_limbs(mem), ps.get_memory(od.memory(mem), depth, 1)), mem
    # the programs do real work: stores happened and the pipeline retired instructions
    assert g.get_memory_limbs("dmem").any()
    assert len(set(res["trace"][-1, 0, :].tolist())) > 4


def test_word_tick_many_matches_oracle(engine):
    """tick_many with held inputs equals the oracle's comb-fused tick_many
    (crates/rrtl-sim-ir/src/lib.rs:9295-9307)."""
    from .designs import random_word_design

    d, meta = random_word_design(99, n_wires=12)
    js = d.to_json()
    lanes = 40
    g = sim.GpuBatchSimulator(js, meta["top"], lanes)
    od = ob.OracleDesign(js, meta["top"])
    ps = ob.PackedSim(od, lanes)
    from rrtl_gb300.workloads import Rng

    rng = Rng(3)
    for name, w in meta["inputs"] + [("clk", 1)]:
        limbs = max(1, (w + 31) // 32)
        arr = np.array([[rng.next() & 0xFFFFFFFF for _ in range(lanes)] for _ in range(limbs)], dtype=np.uint32)
        if w % 32:
            arr[-1] &= np.uint32((1 << (w % 32)) - 1)
        g.set_input_limbs(name, arr)
        ps.set_signal(od.signal(name), arr)
    g.tick_many(37)
    ps.tick_many(37)
    v, m = g.snapshot_storage()
    rv, rm = ps.snapshot()
    assert np.array_equal(v, rv) and np.array_equal(m, rm)
