"""Build libcudasirecon.so and the cudasirecon executable in-tree with nvcc.

All CUDA code is compiled for sm_103a only.  Translation units are compiled
in parallel into cudasirecon_gb300/_build/; outputs:
  cudasirecon_gb300/libcudasirecon.so
  cudasirecon_gb300/bin/cudasirecon
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcudasirecon.so")
CLI = os.path.join(HERE, "bin", "cudasirecon")
SOURCES = ["fft_plan.cu", "k_selftest.cu", "k_ingest.cu", "k_fit.cu", "k_assemble.cu", "reconstructor.cu",
           "params.cpp", "image_io.cpp", "capi.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _flags():
    return ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
            "-I", CSRC] + ARCH


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "cudasirecon.h"))
    newest_header = max(os.path.getmtime(h) for h in headers)
    procs, objs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if not force and os.path.exists(o) and os.path.getmtime(o) >= max(os.path.getmtime(s), newest_header):
            continue
        lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
        cmd = [nvcc()] + lang + ["-c", s, "-o", o] + _flags()
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append(" ".join(cmd) + "\n" + text[-6000:])
        elif verbose and text.strip():
            sys.stderr.write(text)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    if force or procs or not os.path.exists(LIB):
        link = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-Xlinker", "--no-undefined"]
        r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    cli_src = os.path.join(CSRC, "cli_main.cpp")
    if force or not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(LIB),
                                                                         os.path.getmtime(cli_src)):
        cmd = [nvcc(), "-x", "c++", cli_src, "-o", CLI, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
               "-L", HERE, "-lcudasirecon", "-Xlinker", "-rpath=$ORIGIN/.."]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("CLI build failed:\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
