"""The SIMD-shaped packed engine (SimdCpuSimulator restated,
crates/rrtl-sim-ir/src/lib.rs:5375-7457) against the packed simulator: every
signal word and memory word after every tick, on random designs of every
expression kind up to 64 bits (memories, synchronous and asynchronous
resets) and on the pipelined CPU; and its lane-parallel runner against one
engine over all lanes."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300.workloads import Rng, cpu_rom_hashed, pipelined_cpu

from .designs import random_word_design


@pytest.mark.parametrize("seed", range(24))
def test_simd_engine_matches_packed_simulator(oracle_lib, seed):
    d, meta = random_word_design(500 + seed, n_wires=16, n_mems=2, depth=4)
    od = ob.OracleDesign(d.to_json(), meta["top"])
    lanes = 37
    ps, ss = ob.PackedSim(od, lanes), ob.SimdSim(od, lanes)
    rng = Rng(seed)
    for mem, aw, dw, depth in meta["mems"]:
        mi = od.memory(mem)
        limbs = (dw + 31) // 32
        data = np.array([[[rng.next() & ((1 << min(32, dw - 32 * k)) - 1) for _ in range(lanes)] for k in range(limbs)]
                         for _ in range(depth)], dtype=np.uint32)
        for s in (ps, ss):
            s.set_memory(mi, data)
    for cyc in range(12):
        for name, w in meta["inputs"] + [("rst", 1), ("clk", 1)]:
            if name == "clk":
                vals = [1] * lanes
            elif name == "rst":
                vals = [int(cyc < 2 and l % 3 == 0) for l in range(lanes)]
            else:
                vals = [rng.next() & ((1 << w) - 1) for _ in range(lanes)]
            limbs = max(1, (w + 31) // 32)
            arr = np.array([[(v >> (32 * k)) & 0xFFFFFFFF for v in vals] for k in range(limbs)], dtype=np.uint32)
            for s in (ps, ss):
                s.set_signal(od.signal(name), arr)
        for s in (ps, ss):
            s.tick()
        vp, mp = ps.snapshot()
        vs, ms = ss.snapshot()
        assert np.array_equal(vp, vs), (seed, cyc)
        assert np.array_equal(mp, ms), (seed, cyc)
    assert vp.any()


def test_simd_parallel_runner_matches_one_engine_on_the_cpu(oracle_lib):
    od = ob.OracleDesign(pipelined_cpu().to_json(), "Cpu8")
    lanes, cycles = 200, 150
    rom = cpu_rom_hashed(lanes, seed=4)
    stim = [(od.signal("clk"), 3, 1), (od.signal("rst"), 2, 1)]
    rec = [od.signal("out_pc"), od.signal("out_acc")]
    ps = ob.PackedSim(od, lanes)
    ps.set_memory(od.memory("rom"), rom)
    h = np.zeros(cycles, dtype=np.uint64)
    ps.run(ob.make_run(cycles, 0, stim, rec, 2, out_hash=h))
    vp, mp = ps.snapshot()
    hs, vs, ms = ob.simd_run_parallel(od, lanes, cycles, 0, stim, rec, 2, memories={od.memory("rom"): rom}, threads=3,
                                      snapshot=True)
    assert np.array_equal(h, hs)
    assert np.array_equal(vp, vs)
    assert np.array_equal(mp, ms)
