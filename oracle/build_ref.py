"""Build recipe for the reference harness (test infrastructure only).

Stages the reference's own GPU sources -- src/cudaSirecon/gpuFunctionsImpl.cu,
gpuFunctionsImpl_hh.cu, gpuFunctions.h, cudaSireconImpl.h, the vendored
CImg.h, src/Buffers/*.cpp|h and src/cutilSafeCall.h -- from the reference
checkout into ``oracle/_ref/src`` (git-ignored, never committed), writes a
three-line include shim for CImg.h (libtiff is absent: ``cimg_use_tiff`` is
undefined and an opaque ``TIFF`` type is declared for the two prototypes in
cudaSireconImpl.h:345-346), and compiles them unmodified together with
``oracle/ref_harness/refharness.cu`` into ``oracle/_ref/librefsirecon.so``
for sm_103a, with the reference's Release flags (-O3 -DNDEBUG,
-Dcimg_display=0; src/CMakeLists.txt:48, build.sh:17) and cuFFT.

Where the reference checkout is absent (the GPU host), the previously staged
copy under ``oracle/_ref/src`` is used.  Nothing here is imported by the
product; only tests, ``bench.py --impl reference`` and the golden-fixture
generator load the resulting library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("SIRECON_REFERENCE_ROOT", "/root/reference")
OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "librefsirecon.so")

STAGED_FILES = [
    "src/cudaSirecon/gpuFunctionsImpl.cu",
    "src/cudaSirecon/gpuFunctionsImpl_hh.cu",
    "src/cudaSirecon/gpuFunctions.h",
    "src/cudaSirecon/cudaSireconImpl.h",
    "src/cudaSirecon/CImg.h",
    "src/cutilSafeCall.h",
    "src/Buffers/Buffer.h",
    "src/Buffers/Buffer.cpp",
    "src/Buffers/CPUBuffer.h",
    "src/Buffers/CPUBuffer.cpp",
    "src/Buffers/GPUBuffer.h",
    "src/Buffers/GPUBuffer.cpp",
    "src/Buffers/PinnedCPUBuffer.h",
    "src/Buffers/PinnedCPUBuffer.cpp",
]

SHIM = """// include shim: the real CImg.h without libtiff
#undef cimg_use_tiff
typedef struct tiff TIFF;
#include "../src/src/cudaSirecon/CImg.h"
"""


def stage() -> bool:
    """Copy the reference's GPU sources into oracle/_ref/src (if the checkout exists)."""
    if not os.path.isdir(REF_ROOT):
        return all(os.path.exists(os.path.join(STAGE, f)) for f in STAGED_FILES)
    for rel in STAGED_FILES:
        src = os.path.join(REF_ROOT, rel)
        dst = os.path.join(STAGE, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src):
            shutil.copyfile(src, dst)
    shim_dir = os.path.join(OUT, "shim")
    os.makedirs(shim_dir, exist_ok=True)
    with open(os.path.join(shim_dir, "CImg.h"), "w") as f:
        f.write(SHIM)
    return True


def build(force: bool = False, verbose: bool = False) -> str | None:
    """Compile the harness; returns the library path, or None if it cannot be built."""
    if not stage():
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        return None
    harness = os.path.join(HERE, "ref_harness", "refharness.cu")
    srcs = [harness, os.path.join(STAGE, "src/cudaSirecon/gpuFunctionsImpl.cu")] + [
        os.path.join(STAGE, f) for f in STAGED_FILES if f.endswith(".cpp")
    ]
    if os.path.exists(LIB) and not force:
        newest = max(os.path.getmtime(s) for s in srcs)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    flags = [
        "-std=c++17", "-O3", "-DNDEBUG", "-Dcimg_display=0", "-Dcimg_use_openmp=0",
        "-gencode", "arch=compute_103a,code=sm_103a",
        "-Xcompiler", "-fPIC", "-w",
        "-I", os.path.join(OUT, "shim"),
        "-I", os.path.join(STAGE, "src/cudaSirecon"),
        "-I", os.path.join(STAGE, "src/Buffers"),
    ]
    procs = []
    objs = []
    for s in srcs:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        cmd = [nvcc, "-x", "cu", "-c", s, "-o", o] + flags
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    ok = True
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            ok = False
            sys.stderr.write(" ".join(cmd) + "\n" + out.decode(errors="replace")[-4000:] + "\n")
        elif verbose:
            sys.stderr.write(out.decode(errors="replace"))
    if not ok:
        return None
    link = [nvcc, "-shared", "-o", LIB] + objs + ["-lcufft", "-gencode", "arch=compute_103a,code=sm_103a",
                                                   "-Xlinker", "--no-undefined"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        sys.stderr.write(r.stdout.decode(errors="replace")[-4000:])
        return None
    return LIB


if __name__ == "__main__":
    lib = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(lib if lib else "reference harness not built")
    sys.exit(0 if lib else 1)
