"""The allocation-free tick_many entry point against the regular one.

rrtl_word_tick_many_noalloc is for callers that may not allocate device
memory (a serving process whose device memory is divided up front, or a loop
that cannot afford the device synchronisation cudaFree can cause). Here it
runs on device buffers the test owns; the regular batch runs the same design
from the same state, and both must agree bit-exactly after each of two calls
in a row. Collected last so a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

from rrtl_gb300 import sim

from .designs import random_word_design

pytestmark = pytest.mark.gpu


def _pad(lanes):
    return (lanes + 127) // 128 * 128


def _to_device_layout(values, memories, tsw, tmw, lanes):
    """PackedSimulatorStorage order -> the engine's [word][lanes_pad] device order."""
    lp = _pad(lanes)
    v = np.zeros((tsw, lp), dtype=np.uint32)
    v[:, :lanes] = values.reshape(tsw, lanes)
    m = np.zeros((max(tmw, 1), lp), dtype=np.uint32)
    if tmw:
        m[:tmw, :lanes] = memories.reshape(lanes, tmw).T
    return v, m


def _from_device_layout(v, m, tsw, tmw, lanes):
    values = np.ascontiguousarray(v[:, :lanes]).reshape(-1)
    memories = np.ascontiguousarray(m[:tmw, :lanes].T).reshape(-1) if tmw else np.zeros(0, dtype=np.uint32)
    return values, memories


@pytest.mark.parametrize("seed,n_mems", [(1234, 2), (4321, 0)])
def test_noalloc_tick_many_matches_batch_tick_many(engine, seed, n_mems):
    """Two calls in a row (and a zero-step call between them) equal the
    regular batch; the memory-free design passes memories=None."""
    torch = pytest.importorskip("torch")
    d, meta = random_word_design(seed, n_wires=14, n_mems=n_mems, depth=3)
    js = d.to_json()
    lanes = 300
    g = sim.GpuBatchSimulator(js, meta["top"], lanes)
    cd = g.design
    info = cd.info
    tsw, tmw = info.total_signal_words, info.total_memory_words_per_lane
    rng = np.random.default_rng(5)
    for name, w in meta["inputs"] + [("clk", 1)]:
        limbs = max(1, (w + 31) // 32)
        a = rng.integers(0, 1 << 32, size=(limbs, lanes), dtype=np.uint64).astype(np.uint32)
        if w % 32:
            a[-1] &= np.uint32((1 << (w % 32)) - 1)
        g.set_input_limbs(name, a)
    for mem, aw, dw, depth in meta["mems"]:
        idx, depth_real, width = cd.memory(mem)
        limbs = max(1, (width + 31) // 32)
        data = rng.integers(0, 1 << 32, size=(depth_real, limbs, lanes), dtype=np.uint64).astype(np.uint32)
        if width % 32:
            data[:, -1, :] &= np.uint32((1 << (width % 32)) - 1)
        g.set_memory_limbs(mem, data)
    v0, m0 = g.snapshot_storage()
    hv, hm = _to_device_layout(v0, m0, tsw, tmw, lanes)
    dev = torch.device("cuda", 0)
    dv = torch.from_numpy(hv.view(np.int32)).to(dev)
    dm = torch.from_numpy(hm.view(np.int32)).to(dev)
    torch.cuda.synchronize()
    fn = sim.lib().rrtl_word_tick_many_noalloc
    mem_arg = ctypes.c_void_p(dm.data_ptr()) if tmw else None
    for steps in (17, 0, 5):  # calls in a row, each compared with the regular path (0: no launch)
        g.tick_many(steps)
        sim.check(fn(cd.h, ctypes.c_void_p(dv.data_ptr()), mem_arg, lanes, steps))
        want_v, want_m = g.snapshot_storage()
        got_v, got_m = _from_device_layout(dv.cpu().numpy().view(np.uint32), dm.cpu().numpy().view(np.uint32),
                                           tsw, tmw, lanes)
        assert np.array_equal(got_v, want_v)
        assert np.array_equal(got_m, want_m)
    assert want_v.any()


def test_noalloc_rejects_requests_beyond_its_scratch(engine):
    d, meta = random_word_design(77, n_regs=8)
    g = sim.GpuBatchSimulator(d.to_json(), meta["top"], 1)
    fn = sim.lib().rrtl_word_tick_many_noalloc
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check fails first
    rc = fn(g.design.h, dummy, dummy, 1 << 30, 1)
    assert rc == 1
    assert b"E_NOALLOC_SIZE" in sim.lib().rrtl_last_error()


def test_noalloc_rejects_host_memory_before_launching(engine):
    """Host buffers would be dereferenced by the kernel: they are refused on
    the host, before any launch, with RRTL_E_ARG."""
    d, meta = random_word_design(99, n_mems=1)
    g = sim.GpuBatchSimulator(d.to_json(), meta["top"], 64)
    info = g.design.info
    host_v = np.zeros((info.total_signal_words, 128), dtype=np.uint32)
    host_m = np.zeros((max(info.total_memory_words_per_lane, 1), 128), dtype=np.uint32)
    fn = sim.lib().rrtl_word_tick_many_noalloc
    rc = fn(g.design.h, host_v.ctypes.data_as(ctypes.c_void_p), host_m.ctypes.data_as(ctypes.c_void_p), 64, 3)
    assert rc == 1
    assert b"not device memory" in sim.lib().rrtl_last_error()
    assert not host_v.any()  # nothing ran on it
