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
        "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp", "-w",
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
    link = [nvcc, "-shared", "-o", LIB] + objs + ["-lcufft", "-lgomp", "-gencode", "arch=compute_103a,code=sm_103a",
                                                   "-Xlinker", "--no-undefined"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        sys.stderr.write(r.stdout.decode(errors="replace")[-4000:])
        return None
    return LIB


# ---------------------------------------------------------------------------
# makeotf (src/otf/radialft.cpp) reference program, host only
# ---------------------------------------------------------------------------
MO_LIB = os.path.join(OUT, "libmakeotf_ref.so")
MO_STAGED = ["src/otf/radialft.cpp", "src/cudaSirecon/CImg.h"]

MO_CIMG_SHIM = """// include shim for radialft.cpp: the real CImg.h without libtiff; the TIFF
// calls radialft.cpp makes itself are declared here and defined by the
// harness, and CImg's save_tiff is routed to its own raw .cimg writer
#undef cimg_use_tiff
#include "tiffio_stub.h"
#include "../src/src/cudaSirecon/CImg.h"
#define save_tiff save_cimg
"""

MO_TIFF_STUB = """#pragma once
#include <cstdarg>
typedef struct tiff TIFF;
typedef void (*TIFFErrorHandler)(const char*, const char*, va_list);
extern "C" {
TIFFErrorHandler TIFFSetWarningHandler(TIFFErrorHandler);
TIFFErrorHandler TIFFSetErrorHandler(TIFFErrorHandler);
TIFF* TIFFOpen(const char*, const char*);
void TIFFClose(TIFF*);
}
"""

MO_FFTW_SHIM = """// the four FFTW3f declarations radialft.cpp uses (radialft.cpp:339-348)
#pragma once
typedef float fftwf_complex[2];
typedef struct fftwf_plan_s* fftwf_plan;
#define FFTW_ESTIMATE (1U << 6)
extern "C" {
void fftwf_plan_with_nthreads(int nthreads);
fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float* in, fftwf_complex* out, unsigned flags);
void fftwf_execute_dft_r2c(const fftwf_plan p, float* in, fftwf_complex* out);
void fftwf_destroy_plan(fftwf_plan p);
}
"""


def build_makeotf(force: bool = False) -> str | None:
    """Compile the reference makeotf program with the harness into
    oracle/_ref/libmakeotf_ref.so (g++, the reference's Release flags)."""
    if os.path.isdir(REF_ROOT):
        for rel in MO_STAGED:
            src = os.path.join(REF_ROOT, rel)
            dst = os.path.join(STAGE, rel)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src):
                shutil.copyfile(src, dst)
    if not all(os.path.exists(os.path.join(STAGE, f)) for f in MO_STAGED):
        return None
    shim = os.path.join(OUT, "mo_shim")
    os.makedirs(shim, exist_ok=True)
    for name, text in (("CImg.h", MO_CIMG_SHIM), ("tiffio_stub.h", MO_TIFF_STUB), ("fftw3.h", MO_FFTW_SHIM)):
        path = os.path.join(shim, name)
        if not os.path.exists(path) or open(path).read() != text:
            with open(path, "w") as f:
                f.write(text)
    harness = os.path.join(HERE, "ref_harness", "makeotf_harness.cpp")
    srcs = [os.path.join(STAGE, "src/otf/radialft.cpp"), harness]
    if os.path.exists(MO_LIB) and not force:
        if os.path.getmtime(MO_LIB) >= max(os.path.getmtime(s) for s in srcs):
            return MO_LIB
    gxx = shutil.which("g++")
    if not gxx:
        return None
    cmd = [gxx, "-std=c++17", "-O3", "-DNDEBUG", "-Dcimg_display=0", "-Dmain=radialft_reference_main",
           "-fPIC", "-shared", "-w", "-I", shim, "-o", MO_LIB] + srcs + ["-lpthread", "-Wl,--no-undefined"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout.decode(errors="replace")[-4000:] + "\n")
        return None
    return MO_LIB


if __name__ == "__main__":
    lib = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(lib if lib else "reference harness not built")
    mo = build_makeotf(force="--force" in sys.argv)
    print(mo if mo else "reference makeotf not built")
    sys.exit(0 if lib and mo else 1)
