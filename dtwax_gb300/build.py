"""In-tree build of libdtwx.so (and the `dtwx_main` CLI) for sm_103a.

nvcc compiles every translation unit in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo`` and links a shared
library next to this file.  Rebuilds only when a source is newer than the
library.  No cmake; nvcc and a host C++ compiler are all it needs.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libdtwx.so")
BIN = os.path.join(PKG, "bin", "dtwx_main")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["sdtw.cu", "refdel.cu", "prep.cu", "api.cpp", "host_util.cpp", "static_scratch.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _flags(extra=()):
    return ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-O3",
            "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr", *extra]


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def _deps():
    return (glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(INCLUDE, "*.h"))
            + [os.path.abspath(__file__)])


def _run_parallel(cmds, verbose=False):
    procs = []
    for c in cmds:
        if verbose:
            print(" ".join(c), flush=True)
        procs.append((c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out))
        elif verbose and out.strip():
            print(out, flush=True)
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + out for c, out in failed)
        raise RuntimeError("nvcc failed:\n" + msg)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile libdtwx.so and the CLI; returns the library path."""
    deps = _deps()
    if (not force and os.path.exists(LIB) and os.path.exists(BIN)
            and os.path.getmtime(LIB) >= _newest(deps) and os.path.getmtime(BIN) >= _newest(deps)):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    cmds, objs = [], []
    for src in LIB_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        extra = ["-Xptxas", "-v"] if (ptxas_info and src.endswith(".cu")) else []
        cmds.append([nvcc(), *_flags(extra), "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    _run_parallel(cmds, verbose=verbose or ptxas_info)
    tmp = LIB + ".tmp"
    _run_parallel([[nvcc(), *ARCH, "-shared", "-o", tmp, *objs]], verbose)
    os.replace(tmp, LIB)
    main_obj = os.path.join(BUILD, "main.cpp.o")
    _run_parallel([[nvcc(), *_flags(), "-c", os.path.join(CSRC, "main.cpp"), "-o", main_obj]], verbose)
    _run_parallel([[nvcc(), *ARCH, "-o", BIN + ".tmp", main_obj, "-L", PKG, "-ldtwx",
                    "-Xlinker", "-rpath,$ORIGIN/.."]], verbose)
    os.replace(BIN + ".tmp", BIN)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
