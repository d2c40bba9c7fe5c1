"""Seeded random RTL designs for differential tests.

Every IR expression kind appears (Not, And, Or, Xor, Add, Sub, Mul, Eq, Ne,
Lt signed/unsigned, Mux, Slice, Zext, Sext, Trunc, Cast, Concat, MemRead),
over widths 1..max_width, with registers (optionally reset, synchronously or
asynchronously) and memories with a write port. With `wire_every_node`
every operation result is assigned to a wire first, so the scalar simulator's
unmasked intermediates (crates/rrtl-core/src/lib.rs:6401-6469) never reach a
mux condition, comparison or address.
"""
from rrtl_gb300.builder import Design, concat, lit_u, mem_read, mux, uint
from rrtl_gb300.workloads import Rng


def random_word_design(seed, n_inputs=4, n_regs=5, n_wires=14, n_mems=1, max_width=64, depth=3,
                       wire_every_node=False, async_resets=True, top="Rand", no_mul=False):
    rng = Rng(seed)
    d = Design()
    m = d.module(top)
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    widths = [1, 2, 3, 5, 8, 13, 16, 31, 32, 33, 47, 63, 64]
    widths = [w for w in widths if w <= max_width]
    sigs = []  # (signal, width)
    inputs = []
    for i in range(n_inputs):
        w = widths[rng.below(len(widths))]
        s = m.input(f"in{i}", uint(w))
        sigs.append((s, w))
        inputs.append((f"in{i}", w))
    regs = []
    for i in range(n_regs):
        w = widths[rng.below(len(widths))]
        r = m.reg(f"r{i}", uint(w))
        m.clock(r, clk)
        k = rng.below(4)
        if k == 1:
            m.reset(r, rst, rng.next() & ((1 << w) - 1))
        elif k == 2 and async_resets:
            m.async_reset(r, rst, rng.next() & ((1 << w) - 1))
        elif k == 3:
            m.reset_low(r, rst, rng.next() & ((1 << w) - 1))
        regs.append((r, w))
        sigs.append((r, w))
    mems = []
    for i in range(n_mems):
        aw = 1 + rng.below(5)
        dw = widths[rng.below(len(widths))]
        depth_m = (1 << aw) - rng.below(2)  # sometimes not a power of two: out-of-range addresses read 0
        mm = m.mem(f"mem{i}", aw, uint(dw), depth_m)
        mems.append((mm, aw, dw))
    counter = [0]

    def as_wire(e, w):
        if not wire_every_node:
            return e
        counter[0] += 1
        x = m.wire(f"t{counter[0]}", uint(w))
        m.assign(x, e)
        return x.value()

    def leaf(w):
        cands = [s for s, sw in sigs if sw == w]
        r = rng.below(4)
        if cands and r < 3:
            return cands[rng.below(len(cands))].value()
        if r == 3 or not sigs:
            return lit_u(rng.next() & ((1 << w) - 1), w)
        s, sw = sigs[rng.below(len(sigs))]
        if sw > w:
            lsb = rng.below(sw - w + 1)
            return as_wire(s.slice(lsb, w), w)
        if sw < w:
            return as_wire(s.zext(w) if rng.below(2) else s.sext(w).as_uint(), w)
        return s.value()

    def expr(w, dep):
        if dep == 0:
            return leaf(w)
        k = rng.below(15)
        if k == 0:
            e = ~expr(w, dep - 1)
        elif k in (1, 2, 3):
            a, b = expr(w, dep - 1), expr(w, dep - 1)
            e = a & b if k == 1 else a | b if k == 2 else a ^ b
        elif k in (4, 5, 6):
            a, b = expr(w, dep - 1), expr(w, dep - 1)
            e = a + b if k == 4 else a - b if k == 5 else (a ^ b if no_mul else a * b)
        elif k == 7 and w == 1:
            v = widths[rng.below(len(widths))]
            a, b = expr(v, dep - 1), expr(v, dep - 1)
            j = rng.below(4)
            if j == 0:
                e = a.eq_expr(b)
            elif j == 1:
                e = a.ne_expr(b)
            elif j == 2:
                e = a.lt_expr(b)
            else:
                e = a.as_sint().lt_expr(b.as_sint())
        elif k == 8:
            c = expr(1, dep - 1)
            e = mux(c, expr(w, dep - 1), expr(w, dep - 1))
        elif k == 9 and w < max_width:
            v = w + 1 + rng.below(max_width - w)
            lsb = rng.below(v - w + 1)
            e = expr(v, dep - 1).slice(lsb, w)
        elif k == 10 and w > 1:
            v = 1 + rng.below(w - 1)
            e = expr(v, dep - 1).zext(w) if rng.below(2) else expr(v, dep - 1).sext(w).as_uint()
        elif k == 11 and w < max_width:
            v = w + 1 + rng.below(max_width - w)
            e = expr(v, dep - 1).trunc(w)
        elif k == 12 and w > 1:
            parts, left = [], w
            while left > 0:
                pw = 1 + rng.below(left)
                parts.append(expr(pw, dep - 1))
                left -= pw
            e = concat(parts)
        elif k == 13 and mems:
            cands = [(mm, aw, dw) for mm, aw, dw in mems if dw == w]
            if cands:
                mm, aw, dw = cands[rng.below(len(cands))]
                e = mem_read(mm, expr(aw, dep - 1))
            else:
                e = leaf(w)
        elif k == 14:
            e = expr(w, dep - 1).as_sint().as_uint()
        else:
            e = leaf(w)
        return as_wire(e, w)

    wires = []
    for i in range(n_wires):
        w = widths[rng.below(len(widths))]
        x = m.wire(f"w{i}", uint(w))
        m.assign(x, expr(w, depth))
        wires.append((x, w))
        sigs.append((x, w))
    for r, w in regs:
        m.next(r, expr(w, depth))
    for mm, aw, dw in mems:
        m.mem_write(mm, clk, expr(1, depth - 1), expr(aw, depth - 1), expr(dw, depth - 1))
    outs = []
    for i, (x, w) in enumerate(wires[-4:] + regs[:2]):
        o = m.output(f"out{i}", uint(w))
        m.assign(o, x)
        outs.append((f"out{i}", w))
    return d, {"inputs": inputs, "outputs": outs, "regs": [(f"r{i}", w) for i, (_, w) in enumerate(regs)],
               "mems": [(f"mem{i}", aw, dw, (1 << aw)) for i, (_, aw, dw) in enumerate(mems)], "top": top}


def wide_ops_design(w, top="WideOps"):
    """Registers of every operation class at width `w` (up to 128 bits):
    add, sub, mul, unsigned and signed lt, eq, sext, concat, slice, trunc,
    zext, mux, an accumulator and a 16-entry memory written and read each
    cycle. Inputs a, b, din (w bits), sel, we (1 bit), addr (4 bits)."""
    from rrtl_gb300.builder import sint

    d = Design()
    m = d.module(top)
    clk = m.input("clk", uint(1))
    rst = m.input("rst", uint(1))
    a = m.input("a", uint(w))
    b = m.input("b", uint(w))
    din = m.input("din", uint(w))
    sel = m.input("sel", uint(1))
    we = m.input("we", uint(1))
    addr = m.input("addr", uint(4))
    mem = m.mem("mem", 4, uint(w), 16)
    m.mem_write(mem, clk, we, addr, din)
    ext = min(128, w + 37)
    half = w // 2
    exprs = {
        "r_add": (a + b, w),
        "r_sub": (a - b, w),
        "r_mul": (a * b, w),
        "r_ltu": (a.lt_expr(b), 1),
        "r_lts": (a.as_sint().lt_expr(b.as_sint()), 1),
        "r_eq": (a.eq_expr(b), 1),
        "r_sext": (a.sext(ext).as_uint(), ext),
        "r_zext": (b.slice(0, min(w, 40)).zext(ext), ext),
        "r_cat": (concat([a.slice(0, half), sel, b.slice(w - (w - half - 1), w - half - 1)]), w),
        "r_slice": (a.slice(w // 3, w - w // 3), w - w // 3),
        "r_trunc": (b.trunc(max(1, w - 70)), max(1, w - 70)),
        "r_mux": (mux(sel, a, b), w),
        "r_mem": (mem_read(mem, addr), w),
    }
    regs = []
    for name, (e, ew) in exprs.items():
        r = m.reg(name, uint(ew))
        m.clock(r, clk)
        m.reset(r, rst, (1 << ew) - 3 if ew > 2 else 0)
        m.next(r, e)
        regs.append((name, ew))
    acc = m.reg("r_acc", uint(w))
    m.clock(acc, clk)
    m.reset(acc, rst, 0)
    m.next(acc, (acc + (a ^ b)) * lit_u(3, w))
    regs.append(("r_acc", w))
    o = m.output("o", uint(w))
    m.assign(o, acc.value() ^ mem_read(mem, addr))
    inputs = [("a", w), ("b", w), ("din", w), ("sel", 1), ("we", 1), ("addr", 4)]
    return d, {"top": top, "inputs": inputs, "regs": regs, "outputs": [("o", w)]}
