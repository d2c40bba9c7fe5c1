"""Shared helpers for the parity tests (designs and oracle runs)."""
import json
import os

import numpy as np

from oracle import binding as ob
from rrtl_gb300.netlist import import_yosys_netlist

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def crc32_netlist_json():
    """The reference's crc32 gate netlist, re-expanded from the compact fixture."""
    c = json.load(open(os.path.join(GOLDEN, "crc32_gates.compact.json")))
    y = {
        "modules": {
            c["top"]: {
                "ports": {k: {"direction": d, "bits": b} for k, (d, b) in c["ports"].items()},
                "cells": {f"c{i:04d}": {"type": t, "connections": conns} for i, (t, conns) in enumerate(c["cells"])},
            }
        }
    }
    return import_yosys_netlist(y, c["top"])


def oracle_bp_run(od, lanes, cycles, seed, stim, record, mode, faults=(), input_trace=None, lane_base=0):
    """Run the bit-parallel oracle; stim/record use packed indices."""
    bp = ob.BitParallel(od, lanes)
    for lane, sig, v in faults:
        bp.set_force(sig, lane, v)
    words = (lanes + 31) // 32
    out_trace = np.zeros((cycles, len(record), words), dtype=np.uint32) if mode & 1 else None
    out_hash = np.zeros(cycles, dtype=np.uint64) if mode & 2 else None
    detect = np.zeros(lanes, dtype=np.uint32) if mode & 4 else None
    cols = 0
    if input_trace is not None:
        input_trace = np.ascontiguousarray(input_trace, dtype=np.uint32)
        cols = input_trace.shape[1]
    r = ob.make_run(cycles, seed, stim, record, mode, input_trace, cols, out_trace, out_hash, detect, lane_base)
    bp.run(r)
    return {"trace": out_trace, "hash": out_hash, "detect": detect, "sim": bp}


def oracle_packed_run(od, lanes, cycles, seed, stim, record, mode, input_trace=None):
    ps = ob.PackedSim(od, lanes)
    limbs = sum(max(1, (od.width(r) + 31) // 32) for r in record)
    out_trace = np.zeros((cycles, limbs, lanes), dtype=np.uint32) if mode & 1 else None
    out_hash = np.zeros(cycles, dtype=np.uint64) if mode & 2 else None
    cols = 0
    if input_trace is not None:
        input_trace = np.ascontiguousarray(input_trace, dtype=np.uint32)
        cols = input_trace.shape[1]
    r = ob.make_run(cycles, seed, stim, record, mode, input_trace, cols, out_trace, out_hash, None)
    ps.run(r)
    return {"trace": out_trace, "hash": out_hash, "sim": ps}
