"""Build recipe for the native library ``genpk_gb300/_lib/libgenpk_gb300.so``.

CUDA sources are compiled for sm_103a only (GB300); the host translation units
with g++.  ``tables.cpp`` is compiled with the reference's floating-point
flags (-O2 -ffast-math) because it evaluates the reference's bin expression,
whose rounding decides bin edges.  Objects go to ``genpk_gb300/_build``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libgenpk_gb300.so")
COMPAT_LIB = os.path.join(LIBDIR, "libgenpk_compat.so")
CLI = os.path.join(LIBDIR, "gen-pk-gb300")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["deposit.cu", "deposit_window.cu", "spectrum.cu", "xfft.cu", "adjoint.cu",
              "noalloc.cu"]
CXX_SOURCES = {"genpk.cpp": ["-O2"], "tables.cpp": ["-O2", "-ffast-math"]}
COMPAT_SOURCE = "compat.cpp"
# The gen-pk command line (format-II reader + driver) over the C ABI.
CLI_SOURCES = ["gadget2.cpp", "bigfile.cpp", "gen_pk_gb300.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    """Compile every translation unit (in parallel) and link the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "genpk_gb300.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src, flags in CXX_SOURCES.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", *flags, "-std=c++17", "-fPIC", "-Wall",
                         f"-I{CUDA_HOME}/include", "-c", s, "-o", o])
    cobj = os.path.join(BUILD, COMPAT_SOURCE + ".o")
    csrc = os.path.join(CSRC, COMPAT_SOURCE)
    if force or _stale(cobj, [csrc] + headers):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", f"-I{CUDA_HOME}/include",
                     "-c", csrc, "-o", cobj])
    cli_dir = os.path.join(PKG, "cli")
    cli_objs = []
    for src in CLI_SOURCES:
        s = os.path.join(cli_dir, src)
        o = os.path.join(BUILD, "cli_" + src + ".o")
        cli_objs.append(o)
        if force or _stale(o, [s, os.path.join(cli_dir, "gadget2.h"),
                               os.path.join(cli_dir, "bigfile.h"),
                               os.path.join(ROOT, "include", "genpk_gb300.h")]):
            jobs.append(["g++", "-O2", "-std=c++17", "-Wall", f"-I{ROOT}/include", "-c", s,
                         "-o", o])
    out = []
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for text in ex.map(_run, jobs):
            out.append(text)
    if jobs or not os.path.exists(LIB):
        out.append(_run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcufft",
                         f"-L{CUDA_HOME}/lib64", "-Xlinker", f"-rpath,{CUDA_HOME}/lib64"]))
    if jobs or not os.path.exists(COMPAT_LIB):
        out.append(_run(["g++", "-shared", "-o", COMPAT_LIB, cobj, f"-L{LIBDIR}", "-lgenpk_gb300",
                         "-Wl,-rpath,$ORIGIN"]))
    if jobs or not os.path.exists(CLI):
        out.append(_run(["g++", "-o", CLI, *cli_objs, f"-L{LIBDIR}", "-lgenpk_gb300",
                         "-Wl,-rpath,$ORIGIN"]))
    text = "".join(out)
    if verbose and text:
        print(text, file=sys.stderr)
    return LIB


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)
    shutil.rmtree(LIBDIR, ignore_errors=True)


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
