"""Build recipe of the CUDA library: libvsc.so, in-tree, for sm_103a only
(and, where ONNX Runtime headers exist, the custom-op library libvsc_ort.so).

Each translation unit is compiled by nvcc in parallel and linked into a
shared library next to this file.  Flags that matter for results:
  -fmad=false   products and sums are rounded separately, as the reference's
                expressions read (explicit fmaf calls stay fused);
  -gencode arch=compute_103a,code=sm_103a   GB300 only, no other targets.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libvsc.so"
INCLUDE = PKG.parent / "include"

SOURCES = ["vsc_ops.cu", "vsc_stab.cu", "vsc_solver.cu", "vsc_flow.cu", "vsc_corr_tc.cu", "vsc_upsampler.cu",
           "vsc_upsampler_tc.cu", "vsc_api.cpp", "vsc_files.cpp", "vsc_jpeg.cpp"]
HEADERS = ["vsc_internal.h", "vsc_math.cuh", "vsc_ptx.cuh"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler",
          "-fvisibility=hidden", "-Xcompiler", "-Wall"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _newest_input() -> float:
    files = [CSRC / s for s in SOURCES] + [CSRC / h for h in HEADERS] + [INCLUDE / "vsc.h", Path(__file__)]
    return max(f.stat().st_mtime for f in files)


def _compile(src: str, verbose: bool) -> Path:
    obj = BUILD / (src + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link libvsc.so unless it is newer than every input."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= _newest_input():
        return LIB
    BUILD.mkdir(exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_ort(ort_include: str, out: Path | None = None, extra_sources=()) -> Path:
    """Build the ONNX Runtime custom-op library (csrc/ort/vsc_ort_ops.cpp)
    against the ONNX Runtime headers in ort_include, linked to libvsc.so.
    extra_sources are compiled into the same library (the tests add a
    stand-in runtime)."""
    lib = build()
    out = Path(out) if out else PKG / "libvsc_ort.so"
    srcs = [str(CSRC / "ort" / "vsc_ort_ops.cpp"), *map(str, extra_sources)]
    cmd = [nvcc(), *ARCH, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-I", str(INCLUDE),
           "-I", str(ort_include), *srcs, "-o", str(out), "-L", str(PKG), "-lvsc", f"-Xlinker=-rpath={PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ORT adapter build failed:\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
