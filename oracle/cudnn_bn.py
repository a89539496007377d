"""cuDNN batch normalisation as the reference's normaliser calls it.

TEST INFRASTRUCTURE ONLY: the checker for the library's normalize_kernel.
Only tests/ may import this module; the product never does.

The reference z-scores its reads with cudnnBatchNormalizationForwardTraining
(src/include/normalizer.cu:71-113).  cuDNN is a closed library, so the
library's normaliser is restated from cuDNN's documented formula (per read:
(x - mean) / sqrt(biased variance + 1e-4)).  This module pins that
restatement to cuDNN's own output: ``build()`` compiles oracle/cudnn_bn.cpp
(the reference's call, restated) against the cuDNN headers and libraries it
finds -- the nvidia-cudnn Python package that PyTorch depends on, or a system
install -- into oracle/libcudnn_bn.so; ``normalize()`` runs it on device
buffers.  Where no cuDNN with headers is found, ``available()`` is False and
``why_unavailable()`` says what was missing.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cudnn_bn.cpp")
LIB = os.path.join(HERE, "libcudnn_bn.so")

_lib = None
_why = None


def _cudnn_dirs():
    """(include dir, lib dir) of a cuDNN 9 with headers, or None."""
    cands = []
    try:
        import nvidia.cudnn as nc  # the package PyTorch's CUDA wheels depend on
        for root in list(nc.__path__):
            cands.append((os.path.join(root, "include"), os.path.join(root, "lib")))
    except ImportError:
        pass
    for inc, lib in (("/usr/include", "/usr/lib/aarch64-linux-gnu"), ("/usr/include", "/usr/lib/x86_64-linux-gnu"),
                     ("/usr/local/cuda/include", "/usr/local/cuda/lib64")):
        cands.append((inc, lib))
    for inc, lib in cands:
        if os.path.exists(os.path.join(inc, "cudnn.h")) and glob.glob(os.path.join(lib, "libcudnn.so*")):
            return inc, lib
    return None


def build(force: bool = False) -> bool:
    """Compile libcudnn_bn.so; False (and why_unavailable()) without cuDNN."""
    global _why
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return True
    dirs = _cudnn_dirs()
    if dirs is None:
        _why = "no cuDNN with headers found (nvidia-cudnn package or system install)"
        return False
    inc, lib = dirs
    so = sorted(glob.glob(os.path.join(lib, "libcudnn.so*")))[0]
    cuda_inc = "/usr/local/cuda/include"
    cmd = ["g++", "-O2", "-shared", "-fPIC", "-I", inc, "-I", cuda_inc, SRC, "-o", LIB + ".tmp", so,
           f"-Wl,-rpath,{lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        _why = "building against cuDNN failed: " + r.stderr.strip()[-300:]
        return False
    os.replace(LIB + ".tmp", LIB)
    return True


def available() -> bool:
    return build()


def why_unavailable() -> str:
    build()
    return _why or ""


def lib():
    global _lib
    if _lib is None:
        if not build():
            raise RuntimeError(_why)
        L = ctypes.CDLL(LIB)
        L.cudnn_bn_normalize.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_double]
        L.cudnn_bn_normalize.restype = ctypes.c_int
        L.cudnn_bn_last_error.restype = ctypes.c_char_p
        L.cudnn_bn_version.restype = ctypes.c_int
        _lib = L
    return _lib


def version() -> int:
    return int(lib().cudnn_bn_version())


def normalize(d_x: int, reads: int, length: int, d_scale: int, d_bias: int, epsilon: float = 1e-4):
    """In place on the device buffer d_x (reads x length floats)."""
    rc = lib().cudnn_bn_normalize(ctypes.c_void_p(d_x), reads, length, ctypes.c_void_p(d_scale),
                                  ctypes.c_void_p(d_bias), float(epsilon))
    if rc != 0:
        raise RuntimeError(f"cudnnBatchNormalizationForwardTraining: {lib().cudnn_bn_last_error().decode()}")
