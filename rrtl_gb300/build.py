"""Build the engine's shared library in-tree.

Host C++ translation units compile with g++, CUDA ones with nvcc for sm_103a
only; objects go to rrtl_gb300/_build/ and the library to
rrtl_gb300/_lib/librrtl_gb300.so. Translation units compile in parallel and
are skipped when their object is newer than every source and header.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "librrtl_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h"))


# Headers the per-design compiled word kernels include (word_jit.cpp hands
# them to NVRTC by these names), plus minimal <stdint.h>/<stddef.h>: NVRTC
# has no system headers and predefines size_t itself.
JIT_HEADERS = [
    ("word_lane.h", "word_lane.h"),
    ("word_dev.h", "word_dev.h"),
    ("stim.h", "stim.h"),
    ("check_log.h", "check_log.h"),
    ("gate_dev.h", "gate_dev.h"),
    ("gate_common.h", "gate_common.h"),
    ("gate_fused.h", "gate_fused.h"),
    ("lut_classes.h", "lut_classes.h"),
    ("../../include/rrtl_cuda.h", os.path.join("..", "..", "include", "rrtl_cuda.h")),
]
JIT_STUBS = [
    ("stdint.h", "#pragma once\ntypedef signed char int8_t; typedef short int16_t; typedef int int32_t;\n"
                 "typedef long long int64_t; typedef unsigned char uint8_t; typedef unsigned short uint16_t;\n"
                 "typedef unsigned int uint32_t; typedef unsigned long long uint64_t;\n"),
    ("stddef.h", "#pragma once\n"),
]
GEN = os.path.join(BUILD, "gen")


def _c_string(text: str) -> str:
    delim = "rrtljit"
    assert ")" + delim + '"' not in text
    return 'R"' + delim + "(" + text + ")" + delim + '"'


def write_jit_headers() -> str:
    """Write _build/gen/word_jit_headers.inc (only when its content changes)."""
    os.makedirs(GEN, exist_ok=True)
    names, texts = [], []
    for name, rel in JIT_HEADERS:
        with open(os.path.join(CSRC, rel)) as f:
            names.append(name)
            texts.append(f.read())
    for name, text in JIT_STUBS:
        names.append(name)
        texts.append(text)
    out = ["// Generated by rrtl_gb300/build.py from the package headers; do not edit.",
           f"static const int kJitHeaderCount = {len(names)};",
           "static const char* const kJitHeaderNames[] = {" + ", ".join('"' + n + '"' for n in names) + "};",
           "static const char* const kJitHeaderTexts[] = {"]
    out += ["    " + _c_string(t) + "," for t in texts]
    out.append("};")
    content = "\n".join(out) + "\n"
    path = os.path.join(GEN, "word_jit_headers.inc")
    if not os.path.exists(path) or open(path).read() != content:
        with open(path, "w") as f:
            f.write(content)
    return path


def _stale(obj: str, src: str, hdr_mtime: float) -> bool:
    if not os.path.exists(obj):
        return True
    m = os.path.getmtime(obj)
    return m < os.path.getmtime(src) or m < hdr_mtime


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    cuda_home = os.path.dirname(os.path.dirname(nvcc))
    inc = write_jit_headers()
    hdr_mtime = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__), os.path.getmtime(inc)])
    jobs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp")) + glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        if src.endswith(".cu"):
            cmd = [nvcc, *NVCC_FLAGS, "-c", src, "-o", obj]
        else:
            cmd = ["g++", *CXX_FLAGS, f"-I{cuda_home}/include", f"-I{GEN}",
                   f'-DRRTL_CUDA_LIB_DIR="{cuda_home}/lib64"', "-c", src, "-o", obj]
        jobs.append((src, obj, cmd))
    todo = [j for j in jobs if force or _stale(j[1], j[0], hdr_mtime)]

    def run(job):
        src, obj, cmd = job
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        if verbose and (p.stdout or p.stderr):
            print(p.stdout, p.stderr, file=sys.stderr)
        return src

    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            for src in ex.map(run, todo):
                if verbose:
                    print("compiled", os.path.basename(src), file=sys.stderr)
    objs = [j[1] for j in jobs]
    if force or todo or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-lpthread", "-ldl"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
