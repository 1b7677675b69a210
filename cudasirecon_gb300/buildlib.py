"""Build libcudasirecon.so and the cudasirecon executable in-tree with nvcc.

All CUDA code is compiled for sm_103a only.  Translation units are compiled
in parallel into cudasirecon_gb300/_build/; outputs:
  cudasirecon_gb300/libcudasirecon.so
  cudasirecon_gb300/bin/cudasirecon
  cudasirecon_gb300/bin/makeotf
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
MAKEOTF = os.path.join(HERE, "bin", "makeotf")
SOURCES = ["fft_plan.cu", "k_selftest.cu", "k_ingest.cu", "k_fit.cu", "k_search.cu", "k_assemble.cu", "reconstructor.cu",
           "makeotf.cu", "params.cpp", "image_io.cpp", "makeotf_io.cpp", "server.cpp", "capi.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _flags():
    # host code: no contraction into FMA, so float decisions (makeotf's radial
    # bins, the filter radii) round the same on x86-64 and aarch64 hosts
    return ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC] + ARCH


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
    for exe, main_src in ((CLI, "cli_main.cpp"), (MAKEOTF, "makeotf_main.cpp")):
        src = os.path.join(CSRC, main_src)
        if force or not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(LIB),
                                                                             os.path.getmtime(src)):
            cmd = [nvcc(), "-x", "c++", src, "-o", exe, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                   "-L", HERE, "-lcudasirecon", "-Xlinker", "-rpath=$ORIGIN/.."]
            r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
            if r.returncode != 0:
                raise RuntimeError(main_src + " build failed:\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
