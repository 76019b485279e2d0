"""Build the engine's shared library (and the anne-compatible CLI) for sm_103a.

    python -m vedo_gb300.build          # -> vedo_gb300/_build/libvedogpu.so, vedo_gb300/_build/anne-gpu

Every translation unit with physics is compiled with -fmad=false and the host compiler
with -ffp-contract=off, so that no multiply-add is contracted behind the source's back:
the plain-FP64 form then evaluates the reference's IEEE operation sequence exactly, and
the mixed form's fused multiply-adds are the explicit fma/fmaf calls of its source.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libvedogpu.so")
CLI = os.path.join(OUT, "anne-gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc() -> str:
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the engine has no CPU fallback and must be built with CUDA")
    return p


# source -> (compiler, extra flags)
SOURCES = {
    "engine.cu": ("nvcc", ["-fmad=false"]),
    "mixed.cu": ("nvcc", ["-fmad=false"]),
    "sort_scan.cu": ("nvcc", []),
    "noalloc.cu": ("nvcc", []),
    "coordination.cu": ("nvcc", ["-fmad=false"]),
    "vtk_io.cpp": ("cxx", []),
    "scene_host.cpp": ("cxx", []),
    "capi.cpp": ("cxx", []),
    "xml_io.cpp": ("cxx", []),
    "serve.cpp": ("cxx", ["-pthread"]),
    "scene_gen.cpp": ("cxx", []),
}


def _compile(src: str, kind: str, extra, verbose: bool) -> str:
    obj = os.path.join(OUT, src + ".o")
    path = os.path.join(CSRC, src)
    if kind == "nvcc":
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC,-ffp-contract=off", *extra, "-c", path, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
               "-I", os.path.join(CUDA_HOME, "include"), *extra, "-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = {k: v for k, v in SOURCES.items() if os.path.exists(os.path.join(CSRC, k))}
    newest = max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC))
    hdr = os.path.join(HERE, "..", "include", "vedo_gpu.h")
    newest = max(newest, os.path.getmtime(hdr), os.path.getmtime(__file__))
    if not force and os.path.exists(LIB) and os.path.exists(CLI) and os.path.getmtime(LIB) >= newest:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1][0], kv[1][1], verbose), srcs.items()))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC,-pthread", "-Xlinker", "--no-undefined"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "anne_gpu.cpp")
    if os.path.exists(cli_src):
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off", cli_src, "-o", CLI,
               "-L", OUT, "-lvedogpu", f"-Wl,-rpath,{OUT}", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
