"""Build recipe for libpump.so and the ``pump`` command-line program.

Every CUDA translation unit is compiled for sm_103a only, in parallel, with
``-fmad=false`` (no multiply-add contraction; see include/pump.h) and host
code with ``-ffp-contract=off`` (GCC contracts by default on aarch64).  The
outputs go to ``pump_gb300/_build/`` (not tracked); ``build()`` skips work
whose inputs are older than its outputs.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libpump.so")
CLI = os.path.join(OUT, "pump")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# translation units compiled with multiply-add contraction: the precision
# mode and the refinement (not bound to the reference's roundings), and the
# pair BVP in the reference GPU kernel's own arithmetic (contracted as nvcc
# contracts the reference)
FMAD_TRUE = {os.path.join(CSRC, "bvp_precise.cu"), os.path.join(CSRC, "refine.cu"),
             os.path.join(CSRC, "bvp_refgpu.cu")}
HOST_FLAGS = "-fPIC,-ffp-contract=off,-fno-fast-math,-Wall,-Wno-unused-function"
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", HOST_FLAGS,
          "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    lib_srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    lib_srcs = [s for s in lib_srcs if os.path.basename(s) != "cli.cpp"]
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return lib_srcs, headers


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile libpump.so and the CLI; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    lib_srcs, headers = _sources()
    nv = nvcc()
    objs = []
    jobs = []
    for src in lib_srcs:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        if ptxas_info or _stale(obj, [src] + headers + [__file__]):
            cmd = [nv, "-c", src, "-o", obj] + ARCH + COMMON
            if src in FMAD_TRUE:
                cmd = [c if c != "-fmad=false" else "-fmad=true" for c in cmd]
            if ptxas_info and src.endswith(".cu"):
                cmd += ["-Xptxas", "-v"]
            if src.endswith(".cpp"):
                cmd = [nv, "-x", "cu", "-c", src, "-o", obj] + ARCH + COMMON
            jobs.append(cmd)
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if verbose or ptxas_info:
        for log in logs:
            if log.strip():
                sys.stdout.write(log)
    if _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([nv, "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "static"])
        os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB] + headers):
        tmp = CLI + ".tmp%d" % os.getpid()
        _run([nv, "-x", "cu", cli_src, "-o", tmp, "-L", OUT, "-lpump",
              "-Xlinker", "-rpath,$ORIGIN"] + ARCH + COMMON)
        os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
