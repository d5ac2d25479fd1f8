"""Builds the in-tree shared library cupss_gb300/libcupss.so for sm_103a.

All CUDA and host C++ sources under cupss_gb300/csrc are compiled by nvcc in
parallel (one -gencode, sm_103a) and linked into one shared library exporting
the C-ABI of include/cupss_gb300.h and the drop-in C++ classes of
include/cupss.h.  Objects go to cupss_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcupss.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = [
    "k_line_1024.cu", "k_line_512.cu", "k_line_256.cu", "k_line_128.cu", "k_line_small.cu", "k_line_r3.cu",
    "k_row.cu", "k_plane.cu", "k_misc.cu", "noalloc.cu",
    "engine.cpp", "engine_batch.cpp", "engine_multi.cpp", "capi.cpp", "jit.cpp",
    "host_parser.cpp", "host_evolver.cpp", "host_field_term.cpp", "host_init.cpp", "host_utils.cpp",
    "host_ir.cpp", "host_ensemble.cpp", "host_server.cpp", "host_output.cpp", "tune_cache.cpp",
]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


JIT_HEADERS = ["engine_types.h", "twiddle32.h", "fft.cuh", "philox.cuh", "point_math.cuh",
               "line_geom.cuh", "turn.cuh", "kernels.cuh"]


def write_jit_headers():
    """Embeds the device headers the runtime-compiled kernels include (jit_headers.inc)."""
    names, bodies = [], []
    for h in JIT_HEADERS:
        with open(os.path.join(CSRC, h)) as fh:
            body = fh.read()
        assert ")CUPSSJIT" not in body
        names.append('"%s"' % h)
        bodies.append('R"CUPSSJIT(%s)CUPSSJIT"' % body)
    text = ("// Generated by cupss_gb300/build.py from the device headers -- do not edit.\n"
            "static const int kJitNumHeaders = %d;\n"
            "static const char* const kJitHeaderNames[] = {%s};\n"
            "static const char* const kJitHeaderSources[] = {\n%s};\n") % (
        len(names), ", ".join(names), ",\n".join(bodies))
    out = os.path.join(CSRC, "jit_headers.inc")
    old = open(out).read() if os.path.exists(out) else None
    if old != text:
        with open(out, "w") as fh:
            fh.write(text)


def _deps_mtime():
    m = 0.0
    for d in (CSRC, os.path.join(HERE, "..", "include"), os.path.join(HERE, "..", "include", "cupss")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".inc")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _compile(src, nvcc, hdr_mtime):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) > max(os.path.getmtime(path), hdr_mtime):
        return obj, ""
    cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
           "-I", os.path.join(HERE, "..", "include"), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    write_jit_headers()
    nvcc = nvcc_path()
    hdr = _deps_mtime()
    jobs = jobs or min(len(SOURCES), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_compile, s, nvcc, hdr) for s in SOURCES]
        objs = []
        for f in futs:
            obj, log = f.result()
            objs.append(obj)
            if verbose and log.strip():
                print(log)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc, "-shared", *ARCH, "-o", LIB + ".tmp", *objs, "-lcudart", "-lnvrtc"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
