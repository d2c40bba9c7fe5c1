"""The per-design compiled word kernel against the interpreted word kernel
and the packed oracle.

The default (fused) path of a word-engine batch runs the compiled kernel, so
every word-engine oracle test elsewhere already checks it; these tests pin
what is specific to it: that it is the kernel that runs, that it equals the
interpreter bit for bit under every shared-memory placement (signals and
memories staged or left in HBM, memories past the eighth addressed directly),
and that runs split over several calls continue exactly.
"""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.workloads import counter, cpu_rom, pipelined_cpu

from .designs import random_word_design
from .helpers import oracle_packed_run

pytestmark = pytest.mark.gpu


def _run_both(js, top, lanes, cycles, stim, rec, setup=None, seed=5):
    out = {}
    for path in (sim.PATH_FUSED, sim.PATH_WORD_INTERP):
        g = sim.GpuBatchSimulator(js, top, lanes)
        g.set_path(path)
        if setup:
            setup(g)
        res = g.run(cycles, seed=seed, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH)
        out[path] = (res, g.snapshot_storage())
    return out[sim.PATH_FUSED], out[sim.PATH_WORD_INTERP]


def _assert_same(a, b):
    (ra, (va, ma)), (rb, (vb, mb)) = a, b
    assert np.array_equal(ra["trace"], rb["trace"])
    assert np.array_equal(ra["hash"], rb["hash"])
    assert np.array_equal(va, vb)
    assert np.array_equal(ma, mb)


def test_compiled_kernel_is_active(engine):
    for d, top in ((counter(), "Counter"), (pipelined_cpu(), "Cpu8")):
        cd = sim.CompiledDesign(d, top)
        active, ms, why = cd.word_jit()
        assert active, why
        assert ms > 0


@pytest.mark.parametrize("lanes,cycles", [(48, 300), (2048, 300), (65536, 12)])
def test_cpu_compiled_equals_interpreted(engine, lanes, cycles):
    """2,048 lanes x 300 cycles stage the signals, register file and ROM in
    shared memory (the data memory stays in HBM); 65,536 lanes x 12 cycles
    split the SM between four blocks and leave the ROM in HBM."""
    js = pipelined_cpu().to_json()
    rom = cpu_rom(lanes, seed=lanes)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)]
    a, b = _run_both(js, "Cpu8", lanes, cycles, stim, ["out_pc", "out_acc"],
                     setup=lambda g: g.set_memory_limbs("rom", rom))
    _assert_same(a, b)
    assert a[1][1].any()


@pytest.mark.parametrize("seed", range(6))
def test_random_designs_many_memories(engine, seed):
    """Ten memories per design: the first eight go through the placement
    table, the rest are addressed in HBM directly."""
    d, meta = random_word_design(500 + seed, n_wires=18, depth=3, n_mems=10)
    js = d.to_json()
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 2)]
    stim += [(n, sim.STIM_RANDOM, i + 7) for i, (n, w) in enumerate(meta["inputs"])]
    rec = [n for n, w in meta["outputs"]]
    for lanes, cycles in ((37, 40), (3000, 9)):
        a, b = _run_both(js, meta["top"], lanes, cycles, stim, rec)
        _assert_same(a, b)
    od = ob.OracleDesign(js, meta["top"])
    g = sim.GpuBatchSimulator(js, meta["top"], 37)
    res = g.run(40, seed=5, stim=stim, record=rec, mode=sim.REC_TRACE | sim.REC_HASH)
    ref = oracle_packed_run(od, 37, 40, 5, [(od.signal(n), k, p) for n, k, p in stim], [od.signal(r) for r in rec], 3)
    assert np.array_equal(res["trace"], ref["trace"])
    assert np.array_equal(res["hash"], ref["hash"])


def test_split_runs_continue_exactly(engine):
    """eval, single ticks, tick_many and runs of a few cycles, one after the
    other, leave the same state as the interpreter doing the same calls."""
    js = pipelined_cpu().to_json()
    lanes = 300
    rom = cpu_rom(lanes, seed=2)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)]
    snaps = {}
    for path in (sim.PATH_FUSED, sim.PATH_WORD_INTERP):
        g = sim.GpuBatchSimulator(js, "Cpu8", lanes)
        g.set_path(path)
        g.set_memory_limbs("rom", rom)
        g.set_input("clk", [1] * lanes)
        g.set_input("rst", [1] * lanes)
        g.eval_combinational()
        g.tick()
        g.set_input("rst", [0] * lanes)
        g.tick_many(25)
        hs = []
        for k in range(4):
            hs.append(g.run(7 + k, seed=k, stim=stim[:1], record=["out_pc", "out_acc"], mode=sim.REC_HASH)["hash"])
        snaps[path] = (g.snapshot_storage(), np.concatenate(hs))
    (va, ma), ha = snaps[sim.PATH_FUSED]
    (vb, mb), hb = snaps[sim.PATH_WORD_INTERP]
    assert np.array_equal(ha, hb)
    assert np.array_equal(va, vb) and np.array_equal(ma, mb)


def test_counter_trace_and_detect(engine):
    """Record modes through the compiled kernel: detection against lane 0 of
    each warp and the full trace of a 1,024-lane counter."""
    js = counter().to_json()
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1), ("en", sim.STIM_RANDOM, 3)]
    out = {}
    for path in (sim.PATH_FUSED, sim.PATH_WORD_INTERP):
        g = sim.GpuBatchSimulator(js, "Counter", 1024)
        g.set_path(path)
        out[path] = g.run(500, seed=9, stim=stim, record=["out"],
                          mode=sim.REC_TRACE | sim.REC_HASH | sim.REC_DETECT)
    for k in ("trace", "hash", "detect"):
        assert np.array_equal(out[sim.PATH_FUSED][k], out[sim.PATH_WORD_INTERP][k]), k
    assert (out[sim.PATH_FUSED]["detect"] != 0xFFFFFFFF).any()


def test_run_specialised_equals_general_kernel(engine, monkeypatch):
    """The fused path compiles a kernel for each run's tables; with that off
    (RRTL_WORD_JIT_RUNS=0) it runs the general compiled kernel. Both equal
    the interpreter, for every record mode and a multi-limb trace stimulus."""
    d, meta = random_word_design(777, n_wires=16, depth=3, n_mems=2)
    js = d.to_json()
    lanes, cycles = 200, 30
    rng = np.random.default_rng(5)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 2)]
    stim += [(n, sim.STIM_RANDOM, i + 3) for i, (n, w) in enumerate(meta["inputs"][1:])]
    name0, w0 = meta["inputs"][0]
    limbs0 = max(1, (w0 + 31) // 32)
    trace = rng.integers(0, 2**32, size=(cycles, limbs0, lanes), dtype=np.uint64).astype(np.uint32)
    if w0 % 32:
        trace[:, -1, :] &= np.uint32((1 << (w0 % 32)) - 1)
    stim += [(name0, sim.STIM_TRACE, 0)]
    rec = [n for n, w in meta["outputs"]]
    mode = sim.REC_TRACE | sim.REC_HASH | sim.REC_DETECT
    out = {}
    for key, path, env in (("spec", sim.PATH_FUSED, "1"), ("general", sim.PATH_FUSED, "0"),
                           ("interp", sim.PATH_WORD_INTERP, "1")):
        monkeypatch.setenv("RRTL_WORD_JIT_RUNS", env)
        g = sim.GpuBatchSimulator(js, meta["top"], lanes)
        g.set_path(path)
        res = g.run(cycles, seed=11, stim=stim, record=rec, mode=mode, input_trace=trace)
        out[key] = (res, g.snapshot_storage())
    for key in ("general", "interp"):
        for k in ("trace", "hash", "detect"):
            assert np.array_equal(out["spec"][0][k], out[key][0][k]), (key, k)
        assert np.array_equal(out["spec"][1][0], out[key][1][0])
        assert np.array_equal(out["spec"][1][1], out[key][1][1])


def _split_vs_unsplit(monkeypatch, js, top, lanes, cycles, stim, rec, mode, setup=None, input_trace=None):
    out = {}
    for key, env in (("split", "2"), ("unsplit", "0")):
        monkeypatch.setenv("RRTL_WORD_JIT_SPLIT", env)
        g = sim.GpuBatchSimulator(js, top, lanes)
        if setup:
            setup(g)
        res = g.run(cycles, seed=4, stim=stim, record=rec, mode=mode, input_trace=input_trace)
        out[key] = (res, g.snapshot_storage())
    for k in ("trace", "hash", "detect"):
        if out["split"][0][k] is not None:
            assert np.array_equal(out["split"][0][k], out["unsplit"][0][k]), k
    assert np.array_equal(out["split"][1][0], out["unsplit"][1][0])
    assert np.array_equal(out["split"][1][1], out["unsplit"][1][1])


@pytest.mark.parametrize("lanes,cycles", [(64, 200), (2048, 300), (16384, 40)])
def test_cpu_two_warp_split_equals_one_warp(engine, monkeypatch, lanes, cycles):
    """Two warps per 32 lanes (each the cones of its share of the registers and
    memory writes, registers exchanged at the edge) against one warp per 32
    lanes, on the pipelined CPU: hashes, register file, data memory, state."""
    js = pipelined_cpu().to_json()
    rom = cpu_rom(lanes, seed=lanes + 1)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 1)]
    _split_vs_unsplit(monkeypatch, js, "Cpu8", lanes, cycles, stim, ["out_pc", "out_acc"],
                      sim.REC_HASH | sim.REC_TRACE | sim.REC_DETECT, setup=lambda g: g.set_memory_limbs("rom", rom))


@pytest.mark.parametrize("seed", range(8))
def test_random_designs_two_warp_split(engine, monkeypatch, seed):
    d, meta = random_word_design(900 + seed, n_wires=20, depth=3, n_mems=2, async_resets=False)
    stim = [("clk", sim.STIM_CONST, 1), ("rst", sim.STIM_PULSE, 2)]
    stim += [(n, sim.STIM_RANDOM, i + 7) for i, (n, w) in enumerate(meta["inputs"])]
    rec = [n for n, w in meta["outputs"]]
    _split_vs_unsplit(monkeypatch, d.to_json(), meta["top"], 100, 30, stim, rec, sim.REC_TRACE | sim.REC_HASH)
