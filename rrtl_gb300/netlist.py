"""Gate-level netlist import (Yosys `write_json` format) into a Design.

Restates `import_yosys_netlist` (crates/rrtl-sv-frontend/src/netlist.rs:49-198):
every net becomes a 1-bit signal (input port bit, flop output register, or
wire), every cell becomes an assignment or a register next-state, and output
port bits become output signals. Supported cells: $_NOT_ $_AND_ $_OR_ $_XOR_
$_NAND_ $_NOR_ $_XNOR_ $_ANDNOT_ $_ORNOT_ $_MUX_ (Y = S ? B : A) and $_DFF*
(posedge; $_DFFE* adds an active-high enable). Unknown cells are rejected.
"""
from __future__ import annotations

import json
from typing import Union

from .builder import Design, lit_u, mux, uint


class NetlistError(ValueError):
    pass


def _net(v):
    if isinstance(v, int):
        return ("id", v)
    if isinstance(v, str):
        return ("const", v == "1")  # "0"/"x"/"z" -> 0 (netlist.rs:27-34)
    raise NetlistError(f"unexpected net value: {v!r}")


def _conn1(cell, port):
    arr = cell.get("connections", {}).get(port)
    if not isinstance(arr, list):
        raise NetlistError(f"cell missing connection `{port}`")
    if len(arr) != 1:
        raise NetlistError(f"gate cell port `{port}` is not 1-bit")
    return _net(arr[0])


def import_yosys_netlist(netlist: Union[str, dict], top: str) -> Design:
    v = json.loads(netlist) if isinstance(netlist, str) else netlist
    module = v.get("modules", {}).get(top)
    if module is None:
        raise NetlistError(f"module `{top}` not found")
    # serde_json's default map is ordered by key; iterate the same way.
    cells = dict(sorted(module.get("cells", {}).items()))
    ports = dict(sorted(module.get("ports", {}).items()))

    input_nets, reg_nets, all_nets = set(), set(), set()
    input_name = {}
    output_port_bits = []
    for pname, p in ports.items():
        direction = p.get("direction", "")
        bits = p.get("bits", [])
        multi = len(bits) > 1
        for i, b in enumerate(bits):
            n = _net(b)
            if n[0] == "id":
                all_nets.add(n[1])
                if direction == "input":
                    input_nets.add(n[1])
                    input_name[n[1]] = f"{pname}_{i}" if multi else pname
            if direction == "output":
                output_port_bits.append((pname, i, n, multi))
    for cell in cells.values():
        ty = cell.get("type", "")
        for arr in cell.get("connections", {}).values():
            for b in arr:
                n = _net(b)
                if n[0] == "id":
                    all_nets.add(n[1])
        if ty.startswith("$_DFF"):
            q = _conn1(cell, "Q")
            if q[0] == "id":
                reg_nets.add(q[1])

    d = Design()
    m = d.module(top)
    sig = {}
    for nid in sorted(all_nets):
        if nid in input_nets:
            sig[nid] = m.input(input_name[nid], uint(1))
        elif nid in reg_nets:
            sig[nid] = m.reg(f"n{nid}", uint(1))
        else:
            sig[nid] = m.wire(f"n{nid}", uint(1))

    def val(n):
        return sig[n[1]].value() if n[0] == "id" else lit_u(1 if n[1] else 0, 1)

    for cname, cell in cells.items():
        ty = cell.get("type", "")

        def a(p):
            return val(_conn1(cell, p))

        if ty.startswith("$_DFF"):
            q = _conn1(cell, "Q")
            if q[0] != "id":
                raise NetlistError(f"DFF `{cname}` Q is constant")
            c = _conn1(cell, "C")
            if c[0] != "id":
                raise NetlistError(f"DFF `{cname}` clock is constant")
            qs = sig[q[1]]
            m.clock(qs, sig[c[1]])
            dn = a("D")
            m.next(qs, mux(a("E"), dn, qs.value()) if ty.startswith("$_DFFE") else dn)
            continue
        y = _conn1(cell, "Y")
        if y[0] != "id":
            raise NetlistError(f"cell `{cname}` output is constant")
        if ty == "$_NOT_":
            e = ~a("A")
        elif ty == "$_AND_":
            e = a("A") & a("B")
        elif ty == "$_OR_":
            e = a("A") | a("B")
        elif ty == "$_XOR_":
            e = a("A") ^ a("B")
        elif ty == "$_NAND_":
            e = ~(a("A") & a("B"))
        elif ty == "$_NOR_":
            e = ~(a("A") | a("B"))
        elif ty == "$_XNOR_":
            e = ~(a("A") ^ a("B"))
        elif ty == "$_ANDNOT_":
            e = a("A") & ~a("B")
        elif ty == "$_ORNOT_":
            e = a("A") | ~a("B")
        elif ty == "$_MUX_":
            e = mux(a("S"), a("B"), a("A"))
        else:
            raise NetlistError(f"unsupported gate cell `{ty}` (cell `{cname}`)")
        m.assign(sig[y[1]], e)

    for pname, i, n, multi in output_port_bits:
        o = m.output(f"{pname}_{i}" if multi else pname, uint(1))
        m.assign(o, val(n))
    return d
