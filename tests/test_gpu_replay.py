"""GPU trace replay (GpuBatchSimulator::replay_lane_trace,
crates/rrtl-gpu-sim/src/lib.rs:989-1357): expected values taken from the
oracle replay with no mismatch, and planted wrong expectations reported
exactly (step, check index, lane, limb, expected, actual)."""
import numpy as np
import pytest

from oracle import binding as ob
from rrtl_gb300 import sim
from rrtl_gb300.workloads import Rng, counter, gate_netlist

from .designs import random_word_design
from .helpers import oracle_packed_run, oracle_bp_run

pytestmark = pytest.mark.gpu


def _sparse_inputs(rng, names_widths, lanes, steps):
    """Input ops: every input fully set at step 0, then sparse updates."""
    ops = []
    for name, w in names_widths:
        limbs = (w + 31) // 32
        for s in range(steps):
            if s == 0 or rng.below(3) == 0:
                for limb in range(limbs):
                    bits = 32 if limb + 1 < limbs or w % 32 == 0 else w % 32
                    ops.append((s, name, limb, np.array([rng.next() & ((1 << bits) - 1) for _ in range(lanes)],
                                                        dtype=np.uint32)))
    return ops


def _dense(ops, names_widths, lanes, steps, unit_fn):
    """[step][col][unit] columns with carry-forward, as the engine builds them."""
    cols, base = {}, 0
    for name, w in names_widths:
        cols[name] = base
        base += (w + 31) // 32
    cur = np.zeros((base, lanes), dtype=np.uint32)
    out = np.zeros((steps, base, lanes), dtype=np.uint32)
    by_step = {}
    for s, name, limb, vals in ops:
        by_step.setdefault(s, []).append((name, limb, vals))
    for s in range(steps):
        for name, limb, vals in by_step.get(s, []):
            cur[cols[name] + limb] = vals
        out[s] = cur
    return out, cols


def _pack(trace):  # [step][col][lanes] bits -> [step][col][words]
    steps, cols, lanes = trace.shape
    words = (lanes + 31) // 32
    out = np.zeros((steps, cols, words), dtype=np.uint32)
    for l in range(lanes):
        out[:, :, l // 32] |= ((trace[:, :, l] & 1) << (l % 32)).astype(np.uint32)
    return out


def test_word_engine_replay_matches_oracle_and_logs_planted_mismatches(engine):
    d, info = random_word_design(31, n_inputs=3, max_width=64, wire_every_node=True)
    js = d.to_json()
    od = ob.OracleDesign(js, info["top"])
    lanes, steps = 70, 24
    rng = Rng(5)
    ins = [("rst", 1)] + info["inputs"]
    ops = _sparse_inputs(rng, ins, lanes, steps)
    dense, cols = _dense(ops, ins, lanes, steps, None)
    stim = [(od.signal("clk"), sim.STIM_CONST, 1)] + [(od.signal(n), sim.STIM_TRACE, cols[n]) for n, _ in ins]
    outs = info["outputs"]
    ref = oracle_packed_run(od, lanes, steps, 0, stim, [od.signal(n) for n, _ in outs], 1, input_trace=dense)
    # checks: every limb of every output at every step, from the oracle's trace
    checks, row, ci = [], 0, 0
    for name, w in outs:
        for limb in range((w + 31) // 32):
            for s in range(steps):
                checks.append((s, ci, name, limb, ref["trace"][s, row + limb]))
                ci += 1
        row += (w + 31) // 32
    g = sim.GpuBatchSimulator(js, info["top"], lanes)
    g.set_input("clk", [1] * lanes)
    n, log = g.replay_trace(steps, inputs=ops, checks=checks)
    assert n == 0 and log == []
    # plant wrong expectations
    g2 = sim.GpuBatchSimulator(js, info["top"], lanes)
    g2.set_input("clk", [1] * lanes)
    bad = []
    planted = set()
    for k in range(0, len(checks), 37):
        s, c, name, limb, exp = checks[k]
        exp = exp.copy()
        lane = (k * 7) % lanes
        exp[lane] ^= 1
        planted.add((s, c, lane, limb, int(exp[lane]), int(exp[lane] ^ 1)))
        bad.append(k)
        checks[k] = (s, c, name, limb, exp)
    n, log = g2.replay_trace(steps, inputs=ops, checks=checks, max_mismatches=4096)
    assert n == len(planted) and set(log) == planted
    # a small log keeps the full count
    g3 = sim.GpuBatchSimulator(js, info["top"], lanes)
    g3.set_input("clk", [1] * lanes)
    n3, log3 = g3.replay_trace(steps, inputs=ops, checks=checks, max_mismatches=3)
    assert n3 == len(planted) and len(log3) == 3 and set(log3) <= planted


@pytest.mark.parametrize("path", [sim.PATH_FUSED, sim.PATH_PLAIN, "compiled"])
def test_gate_engine_replay_matches_oracle(engine, path, monkeypatch):
    if path == "compiled":  # the compiled gate kernel's check stage
        monkeypatch.setenv("RRTL_GATE_JIT", "2")
        path = sim.PATH_FUSED
    d, meta = gate_netlist(n_gates=1500, n_ff=80, n_pi=12, n_po=16, depth=8, seed=44)
    js = d.to_json()
    od = ob.OracleDesign(js, meta.top)
    lanes, steps = 100, 20
    rng = Rng(9)
    ins = [(meta.rst, 1)] + [(p, 1) for p in meta.inputs]
    ops = _sparse_inputs(rng, ins, lanes, steps)
    dense, cols = _dense(ops, ins, lanes, steps, None)
    packed = _pack(dense)
    stim = [(od.signal(meta.clk), sim.STIM_CONST, 1)] + [(od.signal(n), sim.STIM_TRACE, cols[n]) for n, _ in ins]
    ref = oracle_bp_run(od, lanes, steps, 0, stim, [od.signal(o) for o in meta.outputs], 1, input_trace=packed)
    checks, ci = [], 0
    for k, o in enumerate(meta.outputs):
        for s in range(steps):
            bits = np.array([(ref["trace"][s, k, l // 32] >> (l % 32)) & 1 for l in range(lanes)], dtype=np.uint32)
            checks.append((s, ci, o, 0, bits))
            ci += 1
    g = sim.GpuBatchSimulator(js, meta.top, lanes)
    g.set_path(path)
    g.set_input(meta.clk, [1] * lanes)
    n, log = g.replay_trace(steps, inputs=ops, checks=checks)
    assert n == 0, log[:5]
    s, c, o, limb, exp = checks[41]
    exp = exp.copy()
    exp[63] ^= 1
    checks[41] = (s, c, o, limb, exp)
    g = sim.GpuBatchSimulator(js, meta.top, lanes)
    g.set_path(path)
    g.set_input(meta.clk, [1] * lanes)
    n, log = g.replay_trace(steps, inputs=ops, checks=checks)
    assert n == 1 and log == [(s, c, 63, 0, int(exp[63]), int(exp[63] ^ 1))]


def test_replay_errors(engine):
    g = sim.GpuBatchSimulator(counter(), "Counter", lanes=8)
    with pytest.raises(sim.RrtlError) as e:
        g.replay_trace(4, inputs=[(9, "en", 0, [1] * 8)])
    assert e.value.code == "E_GPU_TRACE_INPUTS"
    with pytest.raises(sim.RrtlError) as e:
        g.replay_trace(4, checks=[(0, 0, "count", 1, [0] * 8)])
    assert e.value.code == "E_GPU_TRACE_CHECKS"
