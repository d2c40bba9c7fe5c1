"""Seeded synthetic designs and stimulus for the batched simulation workloads.

Every random choice comes from a SplitMix64 stream (Steele, Lea, Flood,
OOPSLA 2014), so a (generator, seed) pair names the same design on any host.

Workloads:
  counter()          the 8-bit Counter (README.md:33-50 of the reference): inputs clk, rst, en;
                     count <= en ? count + 1 : count; synchronous reset.
  gate_netlist()     synthetic levelized gate netlist: gates uniform over
                     {AND, OR, XOR, NAND, NOR, XNOR, NOT, MUX2}, D flip-flops with a
                     synchronous reset, primary inputs/outputs; each gate's fanins come
                     from the previous 1-3 levels inside a locality window of nets.
  pipelined_cpu()    word-level 8-stage pipelined 32-bit accumulator CPU (see its docstring).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List

from .builder import Design, concat, lit_u, mem_read, mux, uint

MASK64 = (1 << 64) - 1


def smix64(z: int) -> int:
    z = (z + 0x9E3779B97F4A7C15) & MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def stim_word(seed: int, stream: int, cycle: int, idx: int) -> int:
    """Python copy of the engines' stimulus hash (rrtl_gb300/csrc/stim.h)."""
    k = smix64((seed ^ ((stream * 0xD6E8FEB86659FD93) & MASK64)) & MASK64)
    return smix64(k ^ ((cycle * 0xA0761D6478BD642F) & MASK64) ^ ((idx * 0xE7037ED1A0B428DB) & MASK64)) & 0xFFFFFFFF


class Rng:
    """SplitMix64 sequence."""

    def __init__(self, seed: int):
        self.s = seed & MASK64

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & MASK64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def below(self, n: int) -> int:
        return self.next() % n

    def uniform(self) -> float:
        return (self.next() >> 11) / float(1 << 53)

    def perm(self, n: int) -> List[int]:
        p = list(range(n))
        for i in range(n - 1, 0, -1):
            j = self.below(i + 1)
            p[i], p[j] = p[j], p[i]
        return p


# ---------------------------------------------------------------- counter --
def counter() -> Design:
    d = Design()
    m = d.module("Counter")
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    en = m.input("en", uint(1))
    count = m.reg("count", uint(8))
    m.clock(count, clk)
    m.reset(count, rst, 0)
    m.next(count, mux(en, count + lit_u(1, 8), count))
    out = m.output("out", uint(8))
    m.assign(out, count)
    return d


# ----------------------------------------------------------- gate netlist --
GATE_TYPES = ("AND", "OR", "XOR", "NAND", "NOR", "XNOR", "NOT", "MUX2")


@dataclass
class NetlistMeta:
    top: str
    inputs: List[str]
    outputs: List[str]
    regs: List[str]
    rst: str = "rst"
    clk: str = "clk"
    n_gates: int = 0
    depth: int = 0
    gate_names: List[str] = field(default_factory=list)


def gate_netlist(n_gates: int = 50_000, n_ff: int = 2048, n_pi: int = 64, n_po: int = 64, depth: int = 40,
                 window: int = 4096, seed: int = 2, top: str = "netlist"):
    """Levelized random gate netlist. Returns (Design, NetlistMeta).

    Level 0 holds the primary inputs and flip-flop outputs. Level L >= 1 has
    n_gates/depth gates; fanin 0 walks a permutation of level L-1 (so every
    gate of a level drives at least one gate of the next) and the other fanins
    are drawn from levels L-3..L-1 restricted to the `window` most recent nets.
    Flip-flop D inputs and primary outputs sample the last three levels, with
    D inputs covering every last-level gate first.
    """
    rng = Rng(seed)
    d = Design()
    m = d.module(top)
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    pis = [m.input(f"pi_{i}", uint(1)) for i in range(n_pi)]
    regs = [m.reg(f"q_{i}", uint(1)) for i in range(n_ff)]
    nets = list(pis) + list(regs)  # creation order
    level_start = [0]
    level_end = [len(nets)]
    per_level = [n_gates // depth + (1 if i < n_gates % depth else 0) for i in range(depth)]
    names = []
    for L in range(1, depth + 1):
        prev_b, prev_e = level_start[L - 1], level_end[L - 1]
        lo = max(level_start[max(0, L - 3)], level_end[L - 1] - window)
        hi = level_end[L - 1]
        start = len(nets)
        order = rng.perm(prev_e - prev_b)
        for i in range(per_level[L - 1]):
            t = GATE_TYPES[rng.below(len(GATE_TYPES))]
            a = nets[prev_b + order[i % len(order)]]
            b = nets[lo + rng.below(hi - lo)]
            c = nets[lo + rng.below(hi - lo)]
            if t == "AND":
                e = a & b
            elif t == "OR":
                e = a | b
            elif t == "XOR":
                e = a ^ b
            elif t == "NAND":
                e = ~(a & b)
            elif t == "NOR":
                e = ~(a | b)
            elif t == "XNOR":
                e = ~(a ^ b)
            elif t == "NOT":
                e = ~a.value()
            else:
                e = mux(b, a, c)
            name = f"g{L}_{i}"
            w = m.wire(name, uint(1))
            m.assign(w, e)
            nets.append(w)
            names.append(name)
        level_start.append(start)
        level_end.append(len(nets))
    tail_b = level_start[max(1, depth - 2)]
    tail_e = level_end[depth]
    last_b, last_e = level_start[depth], level_end[depth]
    last_order = rng.perm(last_e - last_b)
    for i, q in enumerate(regs):
        m.clock(q, clk)
        m.reset(q, rst, 0)
        if i < len(last_order):
            src = nets[last_b + last_order[i]]
        else:
            src = nets[tail_b + rng.below(tail_e - tail_b)]
        m.next(q, src)
    outs = []
    for j in range(n_po):
        o = m.output(f"po_{j}", uint(1))
        m.assign(o, nets[tail_b + rng.below(tail_e - tail_b)])
        outs.append(f"po_{j}")
    meta = NetlistMeta(top, [f"pi_{i}" for i in range(n_pi)], outs, [f"q_{i}" for i in range(n_ff)],
                       n_gates=n_gates, depth=depth, gate_names=names)
    return d, meta


def netlist_run_spec(meta: NetlistMeta, reset_cycles: int = 1):
    """Stimulus for a netlist run: rst pulses for `reset_cycles`, every
    primary input takes fresh uniform bits each cycle (stream = input index),
    clk is held at 1. Returns (stim, record) in name form."""
    from .sim import STIM_CONST, STIM_PULSE, STIM_RANDOM

    stim = [(meta.clk, STIM_CONST, 1), (meta.rst, STIM_PULSE, reset_cycles)]
    stim += [(p, STIM_RANDOM, i) for i, p in enumerate(meta.inputs)]
    return stim, list(meta.outputs)
