"""RTL design builder that emits the design interchange JSON.

Mirrors the reference's typed builder `rrtl_core::Design` / `ModuleBuilder`
(crates/rrtl-core/src/lib.rs:980-1035, 1080-2583) and expression helpers
(crates/rrtl-ir/src/lib.rs:256-430). `Design.to_json()` produces the serde-JSON
encoding of `rrtl_ir::Design` (crates/rrtl-ir/src/lib.rs:651-658): the exact
bytes a Rust caller gets from `serde_json::to_string(design.ir())`, and what
`rrtl_design_load_json` accepts.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from typing import Iterable, List, Optional, Sequence, Union


@dataclass(frozen=True)
class BitType:
    width: int
    signed: bool = False

    def to_json(self):
        return {"width": self.width, "signedness": "Signed" if self.signed else "Unsigned"}


def uint(width: int) -> BitType:
    return BitType(width, False)


def sint(width: int) -> BitType:
    return BitType(width, True)


class Expr:
    """Expression tree node; operators build the reference's `Expr` variants."""

    __slots__ = ("tag", "body")

    def __init__(self, tag: str, body):
        self.tag = tag
        self.body = body

    def to_json(self):
        t, b = self.tag, self.body
        if t == "Lit":
            return {"Lit": {"value": b[0], "ty": b[1].to_json()}}
        if t == "Signal":
            return {"Signal": {"module": b.module, "id": b.id}}
        if t == "Not":
            return {"Not": b.to_json()}
        if t in ("And", "Or", "Xor", "Add", "Sub", "Mul", "Eq", "Ne", "Lt"):
            return {t: [b[0].to_json(), b[1].to_json()]}
        if t == "Mux":
            return {"Mux": {"cond": b[0].to_json(), "then_expr": b[1].to_json(), "else_expr": b[2].to_json()}}
        if t == "Slice":
            return {"Slice": {"expr": b[0].to_json(), "lsb": b[1], "width": b[2]}}
        if t in ("Zext", "Sext", "Trunc"):
            return {t: {"expr": b[0].to_json(), "width": b[1]}}
        if t == "Cast":
            return {"Cast": {"expr": b[0].to_json(), "signedness": "Signed" if b[1] else "Unsigned"}}
        if t == "Concat":
            return {"Concat": [p.to_json() for p in b]}
        if t == "MemRead":
            return {"MemRead": {"mem": {"module": b[0].module, "id": b[0].id}, "addr": b[1].to_json()}}
        raise ValueError(t)

    # operator sugar (crates/rrtl-ir/src/lib.rs:384-430)
    def __invert__(self):
        return Expr("Not", self)

    def __and__(self, o):
        return Expr("And", (self, to_expr(o)))

    def __or__(self, o):
        return Expr("Or", (self, to_expr(o)))

    def __xor__(self, o):
        return Expr("Xor", (self, to_expr(o)))

    def __add__(self, o):
        return Expr("Add", (self, to_expr(o)))

    def __sub__(self, o):
        return Expr("Sub", (self, to_expr(o)))

    def __mul__(self, o):
        return Expr("Mul", (self, to_expr(o)))

    def eq_expr(self, o):
        return Expr("Eq", (self, to_expr(o)))

    def ne_expr(self, o):
        return Expr("Ne", (self, to_expr(o)))

    def lt_expr(self, o):
        return Expr("Lt", (self, to_expr(o)))

    def slice(self, lsb: int, width: int):
        return Expr("Slice", (self, lsb, width))

    def zext(self, width: int):
        return Expr("Zext", (self, width))

    def sext(self, width: int):
        return Expr("Sext", (self, width))

    def trunc(self, width: int):
        return Expr("Trunc", (self, width))

    def as_uint(self):
        return Expr("Cast", (self, False))

    def as_sint(self):
        return Expr("Cast", (self, True))


@dataclass(frozen=True)
class Signal:
    module: int
    id: int

    def value(self) -> Expr:
        return Expr("Signal", self)

    # let a Signal stand in for its value like the Rust `impl Into<Expr>`
    def __invert__(self):
        return ~self.value()

    def __and__(self, o):
        return self.value() & o

    def __or__(self, o):
        return self.value() | o

    def __xor__(self, o):
        return self.value() ^ o

    def __add__(self, o):
        return self.value() + o

    def __sub__(self, o):
        return self.value() - o

    def __mul__(self, o):
        return self.value() * o

    def eq_expr(self, o):
        return self.value().eq_expr(o)

    def ne_expr(self, o):
        return self.value().ne_expr(o)

    def lt_expr(self, o):
        return self.value().lt_expr(o)

    def slice(self, lsb, width):
        return self.value().slice(lsb, width)

    def zext(self, w):
        return self.value().zext(w)

    def sext(self, w):
        return self.value().sext(w)

    def trunc(self, w):
        return self.value().trunc(w)

    def as_uint(self):
        return self.value().as_uint()

    def as_sint(self):
        return self.value().as_sint()


ExprLike = Union[Expr, Signal]


def to_expr(x: ExprLike) -> Expr:
    if isinstance(x, Signal):
        return x.value()
    if isinstance(x, Expr):
        return x
    raise TypeError(f"not an expression: {x!r}")


def lit(value: int, width: int) -> Expr:
    return lit_u(value, width)


def lit_u(value: int, width: int) -> Expr:
    v = value & ((1 << 128) - 1)
    if v >= 1 << 127:  # Rust `value as i128`
        v -= 1 << 128
    return Expr("Lit", (v, uint(width)))


def lit_s(value: int, width: int) -> Expr:
    return Expr("Lit", (value, sint(width)))


def mux(cond: ExprLike, then_expr: ExprLike, else_expr: ExprLike) -> Expr:
    return Expr("Mux", (to_expr(cond), to_expr(then_expr), to_expr(else_expr)))


def concat(parts: Iterable[ExprLike]) -> Expr:
    return Expr("Concat", [to_expr(p) for p in parts])


def mem_read(mem: Signal, addr: ExprLike) -> Expr:
    return Expr("MemRead", (mem, to_expr(addr)))


@dataclass
class _SignalInfo:
    handle: Signal
    name: str
    ty: BitType
    kind: str  # Input/Output/Inout/Wire/Reg/Mem
    clock: Optional[Signal] = None
    reset: Optional[dict] = None
    next: Optional[Expr] = None
    addr_width: int = 0
    depth: int = 0


@dataclass
class _Module:
    id: int
    name: str
    is_external: bool = False
    signals: List[_SignalInfo] = field(default_factory=list)
    assignments: List[tuple] = field(default_factory=list)
    memory_writes: List[tuple] = field(default_factory=list)
    initial_register_values: List[tuple] = field(default_factory=list)
    initial_memory_values: List[tuple] = field(default_factory=list)
    instances: List[tuple] = field(default_factory=list)


class ModuleBuilder:
    """Mirror of `ModuleBuilder` (crates/rrtl-core/src/lib.rs:1069-2985)."""

    def __init__(self, design: "Design", module: _Module):
        self._d = design
        self._m = module

    def _add(self, name: str, ty: BitType, kind: str, **kw) -> Signal:
        h = Signal(self._m.id, len(self._m.signals))
        self._m.signals.append(_SignalInfo(h, name, ty, kind, **kw))
        return h

    def input(self, name: str, ty: BitType) -> Signal:
        return self._add(name, ty, "Input")

    def output(self, name: str, ty: BitType) -> Signal:
        return self._add(name, ty, "Output")

    def wire(self, name: str, ty: BitType) -> Signal:
        return self._add(name, ty, "Wire")

    def reg(self, name: str, ty: BitType) -> Signal:
        return self._add(name, ty, "Reg")

    def mem(self, name: str, addr_width: int, data_ty: BitType, depth: int) -> Signal:
        return self._add(name, data_ty, "Mem", addr_width=addr_width, depth=depth)

    def assign(self, dst: Signal, expr: ExprLike) -> None:
        self._m.assignments.append((dst, to_expr(expr)))

    def clock(self, reg: Signal, clk: Signal) -> None:
        self._m.signals[reg.id].clock = clk

    def next(self, reg: Signal, expr: ExprLike) -> None:
        self._m.signals[reg.id].next = to_expr(expr)

    def _reset(self, reg, sig, value, kind, polarity):
        self._m.signals[reg.id].reset = {
            "signal": {"module": sig.module, "id": sig.id},
            "value": value,
            "kind": kind,
            "polarity": polarity,
        }

    def reset(self, reg: Signal, rst: Signal, value: int) -> None:
        self._reset(reg, rst, value, "Sync", "ActiveHigh")

    def reset_low(self, reg: Signal, rst: Signal, value: int) -> None:
        self._reset(reg, rst, value, "Sync", "ActiveLow")

    def async_reset(self, reg: Signal, rst: Signal, value: int) -> None:
        self._reset(reg, rst, value, "Async", "ActiveHigh")

    def async_reset_low(self, reg: Signal, rst: Signal, value: int) -> None:
        self._reset(reg, rst, value, "Async", "ActiveLow")

    def mem_write(self, mem: Signal, clk: Signal, enable: ExprLike, addr: ExprLike, data: ExprLike) -> None:
        self._m.memory_writes.append((mem, clk, to_expr(enable), to_expr(addr), to_expr(data)))

    def initial(self, reg: Signal, value: int) -> None:
        self._m.initial_register_values.append((reg, value))

    def mem_init(self, mem: Signal, addr: int, value: int) -> None:
        self._m.initial_memory_values.append((mem, addr, value))

    def instance(self, name: str, module: str, connections: Sequence[tuple]) -> None:
        self._m.instances.append((name, module, list(connections)))

    def mem_read(self, mem: Signal, addr: ExprLike) -> Expr:
        return mem_read(mem, addr)

    def signal_name(self, s: Signal) -> str:
        return self._m.signals[s.id].name


class Design:
    """Mirror of `rrtl_core::Design` (crates/rrtl-core/src/lib.rs:980-1033)."""

    def __init__(self):
        self._modules: List[_Module] = []

    def module(self, name: str) -> ModuleBuilder:
        m = _Module(len(self._modules), name)
        self._modules.append(m)
        return ModuleBuilder(self, m)

    def find_signal(self, module: str, name: str) -> Optional[Signal]:
        for m in self._modules:
            if m.name == module:
                for s in m.signals:
                    if s.name == name:
                        return s.handle
        return None

    def to_obj(self):
        mods = []
        for m in self._modules:
            sigs = []
            for s in m.signals:
                if s.kind == "Reg":
                    kind = {
                        "Reg": {
                            "clock": None if s.clock is None else {"module": s.clock.module, "id": s.clock.id},
                            "reset": s.reset,
                            "next": None if s.next is None else s.next.to_json(),
                        }
                    }
                elif s.kind == "Mem":
                    kind = {"Mem": {"addr_width": s.addr_width, "data_width": s.ty.width, "depth": s.depth}}
                else:
                    kind = s.kind
                sigs.append(
                    {
                        "handle": {"module": s.handle.module, "id": s.handle.id},
                        "name": s.name,
                        "width": s.ty.width,
                        "ty": s.ty.to_json(),
                        "kind": kind,
                    }
                )
            mods.append(
                {
                    "id": m.id,
                    "name": m.name,
                    "is_external": m.is_external,
                    "signals": sigs,
                    "assignments": [
                        {"dst": {"module": d.module, "id": d.id}, "expr": e.to_json()} for d, e in m.assignments
                    ],
                    "memory_writes": [
                        {
                            "mem": {"module": mm.module, "id": mm.id},
                            "clock": {"module": c.module, "id": c.id},
                            "enable": en.to_json(),
                            "addr": a.to_json(),
                            "data": dt.to_json(),
                        }
                        for mm, c, en, a, dt in m.memory_writes
                    ],
                    "initial_register_values": [
                        {"signal": {"module": r.module, "id": r.id}, "value": v} for r, v in m.initial_register_values
                    ],
                    "initial_memory_values": [
                        {"mem": {"module": r.module, "id": r.id}, "addr": a, "value": v}
                        for r, a, v in m.initial_memory_values
                    ],
                    "assertions": [],
                    "cover_points": [],
                    "instances": [
                        {
                            "name": n,
                            "module": mod,
                            "connections": [[p, {"module": s.module, "id": s.id}] for p, s in conns],
                        }
                        for n, mod, conns in m.instances
                    ],
                    "state_types": [],
                    "state_signals": [],
                    "bundle_types": [],
                    "bundle_signals": [],
                    "interface_types": [],
                    "interface_signals": [],
                    "builder_diagnostics": [],
                }
            )
        return {"modules": mods}

    def to_json(self) -> str:
        return json.dumps(self.to_obj(), separators=(",", ":"))
