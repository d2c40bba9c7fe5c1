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

import math
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


def netlist_run_spec(meta: NetlistMeta, reset_cycles: int = 1, uniform: bool = False):
    """Stimulus for a netlist run: rst pulses for `reset_cycles`, every
    primary input takes fresh uniform bits each cycle (stream = input index),
    clk is held at 1. Returns (stim, record) in name form.

    uniform: every lane sees the same input sequence (RANDOM_UNIFORM), the
    fault-simulation protocol of the reference (set_signal_all before each
    tick, crates/rrtl-sim-ir/examples/fault_sim.rs:66-76): lanes then differ
    only through their injected faults."""
    from .sim import STIM_CONST, STIM_PULSE, STIM_RANDOM, STIM_RANDOM_UNIFORM

    kind = STIM_RANDOM_UNIFORM if uniform else STIM_RANDOM
    stim = [(meta.clk, STIM_CONST, 1), (meta.rst, STIM_PULSE, reset_cycles)]
    stim += [(p, kind, i) for i, p in enumerate(meta.inputs)]
    return stim, list(meta.outputs)


# --------------------------------------------------------- pipelined CPU --
CPU_OPS = ("add", "sub", "and", "or", "xor", "sll", "srl", "sra", "slt", "sltu",
           "addi", "lw", "sw", "beq", "bne", "jal")


def _shift_barrel(x, amt, kind):
    """32-bit shift by a 5-bit amount as a mux barrel over the amount bits:
    `<<k` = concat(slice, 0_k), `>>k` = zext(slice), `>>>k` = sext(slice)."""
    for i in range(5):
        k = 1 << i
        if kind == "sll":
            sh = concat([x.slice(0, 32 - k), lit_u(0, k)])
        elif kind == "srl":
            sh = x.slice(k, 32 - k).zext(32)
        else:
            sh = x.slice(k, 32 - k).sext(32).as_uint()
        x = mux(amt.slice(i, 1), sh, x)
    return x


def pipelined_cpu(top: str = "Cpu8"):
    """8-stage pipelined 32-bit accumulator CPU (IF1 IF2 ID RR EX1 EX2 MEM WB).

    Per lane: 16 x 32-bit register file, 1,024 x 32-bit data memory and a
    256 x 32-bit instruction ROM (all memories), an 8-bit PC and a 64-bit
    accumulator that sums every written-back result. Instruction word:
    op[3:0] rd[7:4] rs1[11:8] rs2[15:12] imm[31:16]; ops are
    add sub and or xor sll srl sra slt sltu (register-register), addi, lw, sw,
    beq, bne (target = imm[7:0]) and jal (rd = pc + 1, jump to imm[7:0]).
    Branches resolve in EX1 and squash the three younger instructions; there
    is no forwarding, so a register read sees the register file as of the read.
    """
    d = Design()
    m = d.module(top)
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    rom = m.mem("rom", 8, uint(32), 256)
    dmem = m.mem("dmem", 10, uint(32), 1024)
    rf = m.mem("rf", 4, uint(32), 16)

    def reg(name, w, reset=True):
        r = m.reg(name, uint(w))
        m.clock(r, clk)
        if reset:
            m.reset(r, rst, 0)
        return r

    def wire(name, w, e):
        x = m.wire(name, uint(w))
        m.assign(x, e)
        return x

    pc = reg("pc", 8)
    v1, pc1 = reg("v1", 1), reg("pc1", 8)
    v2, pc2, ins2 = reg("v2", 1), reg("pc2", 8), reg("ins2", 32)
    v3, pc3, op3, rd3, rs13, rs23, imm3 = (reg("v3", 1), reg("pc3", 8), reg("op3", 4), reg("rd3", 4),
                                          reg("rs1_3", 4), reg("rs2_3", 4), reg("imm3", 16))
    v4, pc4, op4, rd4, a4, b4, imm4 = (reg("v4", 1), reg("pc4", 8), reg("op4", 4), reg("rd4", 4),
                                      reg("a4", 32), reg("b4", 32), reg("imm4", 16))
    v5, op5, rd5, res5, addr5, sd5 = (reg("v5", 1), reg("op5", 4), reg("rd5", 4), reg("res5", 32),
                                      reg("addr5", 10), reg("sd5", 32))
    v6, op6, rd6, res6, addr6, sd6 = (reg("v6", 1), reg("op6", 4), reg("rd6", 4), reg("res6", 32),
                                      reg("addr6", 10), reg("sd6", 32))
    v7, op7, rd7, res7 = reg("v7", 1), reg("op7", 4), reg("rd7", 4), reg("res7", 32)
    acc = reg("acc", 64)

    def is_op(o, name):
        return o.eq_expr(lit_u(CPU_OPS.index(name), 4))

    # EX1: ALU and branch resolution from the RR stage registers
    simm4 = wire("simm4", 32, imm4.sext(32).as_uint())
    amt = wire("amt", 5, b4.slice(0, 5))
    alu = {
        "add": a4 + b4,
        "sub": a4 - b4,
        "and": a4 & b4,
        "or": a4 | b4,
        "xor": a4 ^ b4,
        "sll": _shift_barrel(a4.value(), amt, "sll"),
        "srl": _shift_barrel(a4.value(), amt, "srl"),
        "sra": _shift_barrel(a4.value(), amt, "sra"),
        "slt": a4.as_sint().lt_expr(b4.as_sint()).zext(32),
        "sltu": a4.lt_expr(b4).zext(32),
        "addi": a4 + simm4,
        "jal": pc4.zext(32) + lit_u(1, 32),
    }
    res = lit_u(0, 32)
    for name, e in alu.items():
        res = mux(is_op(op4, name), wire(f"alu_{name}", 32, e), res)
    res_w = wire("alu_res", 32, res)
    eq = wire("eq4", 1, a4.eq_expr(b4))
    taken = wire("taken", 1, v4 & ((is_op(op4, "beq") & eq) | (is_op(op4, "bne") & ~eq.value()) | is_op(op4, "jal")))
    flush = taken
    nflush = wire("nflush", 1, ~flush.value())

    # IF1 / IF2 / ID / RR
    m.next(pc, mux(flush, imm4.slice(0, 8), pc + lit_u(1, 8)))
    m.next(v1, nflush)
    m.next(pc1, pc)
    m.next(v2, v1 & nflush)
    m.next(pc2, pc1)
    m.next(ins2, mem_read(rom, pc1))
    m.next(v3, v2 & nflush)
    m.next(pc3, pc2)
    m.next(op3, ins2.slice(0, 4))
    m.next(rd3, ins2.slice(4, 4))
    m.next(rs13, ins2.slice(8, 4))
    m.next(rs23, ins2.slice(12, 4))
    m.next(imm3, ins2.slice(16, 16))
    m.next(v4, v3 & nflush)
    m.next(pc4, pc3)
    m.next(op4, op3)
    m.next(rd4, rd3)
    m.next(a4, mem_read(rf, rs13))
    m.next(b4, mem_read(rf, rs23))
    m.next(imm4, imm3)
    # EX1 -> EX2 -> MEM -> WB
    m.next(v5, v4)
    m.next(op5, op4)
    m.next(rd5, rd4)
    m.next(res5, res_w)
    m.next(addr5, (a4 + simm4).slice(0, 10))
    m.next(sd5, b4)
    m.next(v6, v5)
    m.next(op6, op5)
    m.next(rd6, rd5)
    m.next(res6, res5)
    m.next(addr6, addr5)
    m.next(sd6, sd5)
    m.next(v7, v6)
    m.next(op7, op6)
    m.next(rd7, rd6)
    m.next(res7, mux(is_op(op6, "lw"), mem_read(dmem, addr6), res6))
    m.mem_write(dmem, clk, v6 & is_op(op6, "sw"), addr6, sd6)
    writes = wire("wb_en", 1, v7 & ~(is_op(op7, "sw") | is_op(op7, "beq") | is_op(op7, "bne")))
    m.mem_write(rf, clk, writes, rd7, res7)
    m.next(acc, mux(writes, acc + res7.zext(64), acc))
    out_pc = m.output("out_pc", uint(8))
    m.assign(out_pc, pc)
    out_acc = m.output("out_acc", uint(64))
    m.assign(out_acc, acc)
    return d


def cpu_rom(lanes: int, seed: int = 3):
    """[256][1][lanes] instruction words: random valid instructions per lane,
    branch and jump targets uniform over the ROM."""
    import numpy as np

    rng = Rng(seed)
    rom = np.zeros((256, 1, lanes), dtype=np.uint32)
    for lane in range(lanes):
        for a in range(256):
            op = rng.below(16)
            rd, rs1, rs2 = rng.below(16), rng.below(16), rng.below(16)
            imm = rng.below(256) if op in (13, 14, 15) else rng.below(1 << 16)
            rom[a, 0, lane] = op | (rd << 4) | (rs1 << 8) | (rs2 << 12) | (imm << 16)
    return rom


def _smix64_np(z):
    import numpy as np

    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def cpu_rom_hashed(lanes: int, seed: int = 3):
    """Same instruction format and distribution as cpu_rom, drawn from a
    counter hash of (seed, lane, address) so large batches build fast."""
    import numpy as np

    with np.errstate(over="ignore"):
        idx = np.arange(256 * lanes, dtype=np.uint64).reshape(256, lanes)
        base = _smix64_np(idx ^ np.uint64((seed * 0xD1B54A32D192ED03) & MASK64))
        f = [_smix64_np(base + np.uint64(k)) for k in range(5)]
    op = (f[0] % np.uint64(16)).astype(np.uint32)
    rd, rs1, rs2 = [(x % np.uint64(16)).astype(np.uint32) for x in f[1:4]]
    imm_small = (f[4] % np.uint64(256)).astype(np.uint32)
    imm_big = (f[4] % np.uint64(1 << 16)).astype(np.uint32)
    imm = np.where(op >= 13, imm_small, imm_big)
    rom = op | (rd << 4) | (rs1 << 8) | (rs2 << 12) | (imm << 16)
    return rom.reshape(256, 1, lanes).astype(np.uint32)


# --------------------------------------------------------------- job stream --
@dataclass
class JobSpec:
    """One job of the uneven job stream: a run on a fresh batch of a design."""
    design: int        # index into the stream's design list
    lanes: int
    cycles: int
    seed: int          # stimulus seed
    fault: bool        # one stuck-at fault per lane (lanes 32k are the fault-free references)


def log_uniform_int(rng: Rng, lo: int, hi: int) -> int:
    return int(round(math.exp(math.log(lo) + rng.uniform() * (math.log(hi) - math.log(lo)))))


def job_stream_designs(n_designs: int = 8, gates_lo: int = 5_000, gates_hi: int = 200_000, seed: int = 40):
    """Netlists of the 50k-gate family with gate counts log-uniform in [lo, hi]:
    flip-flops scale with gates (2,048 per 50k), 64 PIs, 64 POs, depth 40."""
    rng = Rng(seed)
    out = []
    for i in range(n_designs):
        g = log_uniform_int(rng, gates_lo, gates_hi)
        out.append(gate_netlist(n_gates=g, n_ff=max(64, g * 2048 // 50_000), depth=40, seed=seed * 1000 + i))
    return out


def job_stream(n_jobs: int, n_designs: int, lanes_lo: int = 32, lanes_hi: int = 65_536, cycles_lo: int = 100,
               cycles_hi: int = 50_000, fault_frac: float = 0.3, seed: int = 41) -> List[JobSpec]:
    """Jobs with log-uniform lanes and cycles over `n_designs` designs; a
    `fault_frac` share are fault-simulation jobs."""
    rng = Rng(seed)
    jobs = []
    for i in range(n_jobs):
        jobs.append(JobSpec(design=rng.below(n_designs), lanes=log_uniform_int(rng, lanes_lo, lanes_hi),
                            cycles=log_uniform_int(rng, cycles_lo, cycles_hi), seed=seed * 100_000 + i,
                            fault=rng.uniform() < fault_frac))
    return jobs


def job_faults(meta: NetlistMeta, lanes: int, seed: int):
    """One stuck-at fault per lane at a seeded random net (wires, flops,
    outputs); lane 0 of every 32-lane word stays fault-free as the reference.
    Run fault jobs with lane-uniform stimulus (netlist_run_spec(uniform=True)):
    every fault-free lane then equals the reference's golden lane 0, so the
    per-word comparison is the reference's comparison with lane 0."""
    rng = Rng(seed ^ 0xFA17)
    sites = meta.gate_names + meta.regs + meta.outputs
    return [(l, sites[rng.below(len(sites))], rng.below(2)) for l in range(lanes) if l % 32]


# ------------------------------------------------------- instance folding --
def replicated_datapath(n_instances: int, top: str = "Top", child: str = "Lane") -> Design:
    """A flat wrapper of `n_instances` independent copies of one 32-bit
    datapath (the shape the reference folds into the lane axis: shared clk
    and reset, a data input and an output per instance). The datapath: a
    multiply-accumulate register, a rotate-xor mixer and a small history of
    its inputs, reset synchronously."""
    d = Design()
    m = d.module(child)
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    din = m.input("din", uint(32))
    acc = m.reg("acc", uint(32))
    mix = m.reg("mix", uint(32))
    h0 = m.reg("h0", uint(32))
    h1 = m.reg("h1", uint(32))
    for r in (acc, mix, h0, h1):
        m.clock(r, clk)
        m.reset(r, rst, 0)
    m.next(acc, acc * lit_u(0x9E3779B9, 32) + din)
    rot = concat([mix.slice(0, 7), mix.slice(7, 25)])
    m.next(mix, (rot ^ acc) + (h0 ^ h1))
    m.next(h0, din)
    m.next(h1, h0 + lit_u(0x7F4A7C15, 32))
    o = m.output("o", uint(32))
    m.assign(o, mix ^ acc)
    t = d.module(top)
    tclk = t.input("clk", uint(1))
    trst = t.input("rst", uint(1))
    for i in range(n_instances):
        di = t.input(f"din{i}", uint(32))
        oi = t.output(f"o{i}", uint(32))
        t.instance(f"u{i}", child, [("clk", tclk), ("rst", trst), ("din", di), ("o", oi)])
    return d


def narrow_alu(width: int = 16, top: str = "Alu", compare: bool = True) -> Design:
    """A small multi-bit datapath inside the bit-slice scope (no memory, no
    multiply): two operand registers loaded from inputs, an accumulator that
    adds, subtracts, xors or keeps the larger operand by a 2-bit select, and
    a flag output; synchronous reset. With compare=False the larger operand
    becomes their xor (the reference's bit-slice engine has no compare)."""
    d = Design()
    m = d.module(top)
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    din = m.input("din", uint(width))
    sel = m.input("sel", uint(2))
    a = m.reg("a", uint(width))
    b = m.reg("b", uint(width))
    acc = m.reg("acc", uint(width))
    for r in (a, b, acc):
        m.clock(r, clk)
        m.reset(r, rst, 0)
    m.next(a, din)
    m.next(b, a ^ acc)
    s0, s1 = sel.slice(0, 1), sel.slice(1, 1)
    larger = mux(a.lt_expr(b), b, a) if compare else a ^ b
    m.next(acc, mux(s1, mux(s0, acc + a, acc - b), mux(s0, acc ^ larger, acc + larger)))
    flag = m.output("flag", uint(1))
    m.assign(flag, acc.eq_expr(a))
    out = m.output("out", uint(width))
    m.assign(out, acc)
    return d
