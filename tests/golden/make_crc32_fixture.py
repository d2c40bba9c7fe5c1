"""Regenerate tests/golden/crc32_gates.compact.json.

Source: the reference's Yosys-synthesised CRC-32 gate netlist
(bench/sv/crc32_gates.json: `synth; dfflegalize; abc -g AND,OR,XOR,MUX` of
bench/sv/crc32.sv, 195 cells). The fixture keeps only what the netlist
importer reads (port bit lists, cell types and connections), with cells
renamed to their index in key order so the file stays small.

Usage (the argument is the netlist inside a checkout of the reference):
    python tests/golden/make_crc32_fixture.py <reference>/bench/sv/crc32_gates.json
"""
import json
import os
import sys


def main(src):
    v = json.load(open(src))
    m = v["modules"]["crc32"]
    ports = {k: [p["direction"], p["bits"]] for k, p in sorted(m["ports"].items())}
    cells = []
    for _, c in sorted(m["cells"].items()):
        cells.append([c["type"], {k: c["connections"][k] for k in sorted(c["connections"])}])
    out = {"top": "crc32", "ports": ports, "cells": cells}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "crc32_gates.compact.json")
    with open(dst, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"wrote {dst}: {len(cells)} cells")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_crc32_fixture.py <reference>/bench/sv/crc32_gates.json")
    main(sys.argv[1])
