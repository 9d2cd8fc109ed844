"""In-tree build of libaarambam_gpu.so for sm_103a.

Compiles each CUDA translation unit of aarambam_gb300/csrc with nvcc in
parallel (one -gencode, sm_103a only) and links them into
aarambam_gb300/_build/libaarambam_gpu.so (CUDA runtime linked statically,
cuFFT dynamically with an rpath into the toolkit).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libaarambam_gpu.so")
SOURCES = ["noise.cu", "fused.cu", "capi.cu", "plain64.cu", "adjoint.cu", "jit.cu", "decomp.cu", "gram_tc.cu", "slab.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libaarambam_gpu.so")
    return cand


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "aarambam.h"))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _embed_headers() -> None:
    """_build/jit_embed.h: the device headers the run-time specialised row
    and accumulation kernels are compiled from (jit.cu), as raw string
    literals."""
    out = os.path.join(OUT, "jit_embed.h")
    parts = ["// generated by build.py from csrc/fft.cuh, csrc/rows.cuh and csrc/cells.cuh\n#pragma once\n"]
    for var, name in (("kEmbedFft", "fft.cuh"), ("kEmbedRows", "rows.cuh"), ("kEmbedCells", "cells.cuh")):
        with open(os.path.join(CSRC, name)) as f:
            text = f.read()
        if ")AARJIT\"" in text:
            raise RuntimeError(name + " contains the raw-string delimiter")
        parts.append("static const char* " + var + " = R\"AARJIT(" + text + ")AARJIT\";\n")
    new = "".join(parts)
    old = open(out).read() if os.path.exists(out) else None
    if new != old:
        with open(out, "w") as f:
            f.write(new)


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    _embed_headers()
    flags = ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
             "-I" + os.path.join(os.path.dirname(HERE), "include"), "-I" + OUT] + ARCH
    procs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, s):
            cmd = [nvcc()] + flags + ["-c", s, "-o", o]
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, pr in procs:
        out, _ = pr.communicate()
        if pr.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + out.decode(errors="replace"))
        if verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    libdir = os.path.join(cuda_home(), "lib64")
    if not os.path.isdir(libdir):
        libdir = os.path.join(cuda_home(), "lib")
    if procs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-L" + libdir, "-lcufft", "-lnvrtc",
                                                                  "-Xlinker", "-rpath=" + libdir]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
