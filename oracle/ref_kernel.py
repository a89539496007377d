"""The reference's own sDTW GPU kernel, built from its sources and run as a second oracle.

TEST INFRASTRUCTURE ONLY.  Like the CPU oracle next to it, this module is a
test oracle: only tests/ and bench.py's reference arm may import it, and the
product package (dtwax_gb300) never does.

* ``build()`` compiles oracle/ref_dtw_harness.cu, which includes the
  reference's unmodified src/include/DTW.hpp + DTW.cu (FullDTW::DTW,
  DTW.cu:151-572, with -DNO_REF_DEL as src/Makefile:8 sets it, or without it
  for the REF_DEL recurrence), into one device-only cubin per reference
  geometry under oracle/_ref/.  It needs the
  reference's sources, so it runs only where they are present;
  the cubins travel with the repository and nothing else of the reference does.
* ``RefKernel`` loads a cubin through the CUDA driver API (ctypes on
  libcuda), lays out the reference and the queries the way the reference's
  host does (main.cu:93-109 tile interleave, main.cu:165-178 query broadcast
  with a 32-entry tail) and launches the kernel the way its launcher does
  (DTW.hpp:287-295: one 32-thread block per read), either all reads in one
  launch or BLOCK_NUM = 10 reads per launch as main.cu:217-271 does.

One launch detail differs from the reference's launcher: 256 bytes of dynamic
shared memory are requested.  The kernel's lane 0 reads penalty_last_col[wave]
for wave up to NUM_WAVES = 1,055 (DTW.cu:384, :516) from a 1,024-entry shared
array (DTW.cu:155); the padding keeps those 31 reads inside the block's shared
window.  The values read there are never used (lane 0 computes no cell after
wave 1,024), so results are unchanged.

Every other access was checked against the buffers this module allocates:
queries are read up to index n_reads*2048 + 31 (the reference allocates the
same 32-entry tail), reference tiles up to (REF_LEN/832)*832 - 1, the row
state up to n_reads*REF_LEN - 1, and dist[block] per block.  The kernel has no
waits and no data-dependent loop bounds.

The row state is indexed as block_id * REF_LEN + column in 32-bit int
(DTW.cu:208, :293, :325, :419-456, :546), which overflows once
n_reads * REF_LEN passes 2^31 - 1: 2,147 reads per launch for the 1 Mb
geometry, 429 for the 5 Mb one.  launch() refuses more reads per launch than
that (max_reads_per_launch), so the kernel never indexes out of bounds.

The reference's sources are found through the DTWAX_REFERENCE environment
variable (the reference project's root); oracle/Makefile sets it.  Without it
build() keeps the prebuilt cubins.
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
HARNESS = os.path.join(HERE, "ref_dtw_harness.cu")
INT32_MAX = 2 ** 31 - 1


def reference_include():
    """src/include of the reference project named by DTWAX_REFERENCE, or None."""
    root = os.environ.get("DTWAX_REFERENCE")
    return os.path.join(root, "src", "include") if root else None

TILE = 832            # SEGMENT_SIZE 26 x WARP_SIZE 32 (common.hpp:88)
QUERY_LEN = 2048      # common.hpp:58
BLOCK_NUM = 10        # reads per launch in main.cu (common.hpp:68)
DYN_SMEM = 256

# name -> (precision, REF_LEN, ref_del).  FP16: REF_LEN columns per strand (fwd
# in .x, rev in .y of one half2); FP32: fwd then rev concatenated
# (load_reference.hpp:36-37).  ref_del: built without -DNO_REF_DEL, i.e. with
# the left predecessor of DTW.cu:23-29 (names ending in _rd).
GEOMETRIES = {
    "fp16_4160": ("fp16", 4160, False),          # 5 tiles per strand
    "fp16_48128": ("fp16", 48128, False),        # the shipped FP16 shape, 47*1024 (57 tiles scored)
    "fp16_1000064": ("fp16", 1000064, False),    # 1,202 tiles: a 1 Mb genome (999,995 columns per strand)
    "fp32_8320": ("fp32", 8320, False),          # 2 x 4,160 concatenated
    "fp32_94848": ("fp32", 94848, False),        # 2 x 47,424 concatenated (114 tiles)
    "fp32_2000128": ("fp32", 2000128, False),    # 2 x 1,000,064 concatenated: a 1 Mb genome (2,404 tiles)
    "fp16_5000320": ("fp16", 5000320, False),    # 6,010 tiles: a 5 Mb genome (4,999,995 columns per strand)
    "fp32_10000640": ("fp32", 10000640, False),  # 2 x 5,000,320 concatenated: a 5 Mb genome (12,020 tiles)
    "fp16_4160_rd": ("fp16", 4160, True),
    "fp16_48128_rd": ("fp16", 48128, True),
    "fp32_8320_rd": ("fp32", 8320, True),
}

# Kernel symbols of the two instantiations (as ptxas -v reports them when the
# harness is compiled).
KERNEL_NAMES = {
    "fp16": b"_ZN7FullDTW3DTWIi7__half2EEvP16ref_coefficientsPT0_S5_T_S4_S5_",
    "fp32": b"_ZN7FullDTW3DTWIifEEvP16ref_coefficientsPT0_S4_T_S3_S4_",
}


def cubin_path(name: str) -> str:
    return os.path.join(OUT_DIR, f"dtw_{name}.cubin")


def available(name: str) -> bool:
    return os.path.exists(cubin_path(name))


def sources_present() -> bool:
    inc = reference_include()
    return bool(inc) and os.path.exists(os.path.join(inc, "DTW.cu"))


def _compile(name: str) -> str:
    prec, ref_len, ref_del = GEOMETRIES[name]
    out = cubin_path(name)
    cmd = ["nvcc", "-cubin", "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
           f"-DHARNESS_REF_LEN={ref_len}", "-I", reference_include()]
    if not ref_del:
        cmd.append("-DNO_REF_DEL")
    if prec == "fp16":
        cmd.append("-DFP16")
    cmd += [HARNESS, "-o", out + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def build(force: bool = False) -> list:
    """Compile the cubins that are missing or older than the harness.  Without
    the reference's sources this is a no-op (prebuilt cubins are used)."""
    if not sources_present():
        return [cubin_path(n) for n in GEOMETRIES if available(n)]
    os.makedirs(OUT_DIR, exist_ok=True)
    todo = [n for n in GEOMETRIES
            if force or not available(n) or os.path.getmtime(cubin_path(n)) < os.path.getmtime(HARNESS)]
    with cf.ThreadPoolExecutor(max_workers=max(1, len(todo))) as ex:
        list(ex.map(_compile, todo))
    return [cubin_path(n) for n in GEOMETRIES]


# ------------------------------------------------------------- driver API

class _Driver:
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            L = ctypes.CDLL("libcuda.so.1")
            vp = ctypes.c_void_p
            L.cuInit.argtypes = [ctypes.c_uint]
            L.cuCtxGetCurrent.argtypes = [ctypes.POINTER(vp)]
            L.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
            L.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
            L.cuModuleUnload.argtypes = [vp]
            L.cuLaunchKernel.argtypes = [vp, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                         ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, vp,
                                         ctypes.POINTER(vp), ctypes.POINTER(vp)]
            L.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
            cls._lib = L
        return cls._lib

    @classmethod
    def check(cls, rc: int, what: str):
        if rc != 0:
            s = ctypes.c_char_p()
            cls.lib().cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} ({s.value.decode() if s.value else '?'})")


def _half2_bits(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """uint32 words of __half2 values (.x = a, .y = b), round to nearest even."""
    lo = np.asarray(a, np.float32).astype(np.float16).view(np.uint16).astype(np.uint32)
    hi = np.asarray(b, np.float32).astype(np.float16).view(np.uint16).astype(np.uint32)
    return lo | (hi << np.uint32(16))


def tile_interleave(cols: np.ndarray, tiles: int) -> np.ndarray:
    """main.cu:93-109: within each 832-column tile, lane j's 26 consecutive
    columns are stored at stride 32 (h[l*832 + i*32 + j] = cols[l*832 + j*26 + i])."""
    head = cols[: tiles * TILE].reshape(tiles, 32, 26)
    out = cols.copy()
    out[: tiles * TILE] = head.transpose(0, 2, 1).reshape(-1)
    return out


class RefKernel:
    """One reference-kernel geometry loaded on the current CUDA device."""

    def __init__(self, name: str):
        import torch
        if name not in GEOMETRIES:
            raise KeyError(name)
        if not available(name):
            raise FileNotFoundError(f"{cubin_path(name)} not built (needs the reference's sources at build time)")
        self.name = name
        self.precision, self.ref_len, self.ref_del = GEOMETRIES[name]
        self.tiles = self.ref_len // TILE
        self.scored = self.tiles * TILE
        torch.zeros(1, device="cuda")  # make the primary context current
        L = _Driver.lib()
        _Driver.check(L.cuInit(0), "cuInit")
        ctx = ctypes.c_void_p()
        _Driver.check(L.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self._mod = ctypes.c_void_p()
        _Driver.check(L.cuModuleLoad(ctypes.byref(self._mod), cubin_path(name).encode()), "cuModuleLoad")
        self._fn = ctypes.c_void_p()
        _Driver.check(L.cuModuleGetFunction(ctypes.byref(self._fn), self._mod, KERNEL_NAMES[self.precision]),
                      "cuModuleGetFunction")
        self.launches = 0

    def close(self):
        if getattr(self, "_mod", None) is not None and self._mod.value:
            _Driver.lib().cuModuleUnload(self._mod)
            self._mod = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---------------------------------------------------------- layouts
    @property
    def strand_columns(self) -> int:
        """Columns per strand the kernel scores (FP16: the scored tiles; FP32: half the buffer)."""
        return self.scored if self.precision == "fp16" else self.ref_len // 2

    def reference(self, fwd: np.ndarray, rev: np.ndarray):
        """Device reference buffer from z-scored per-strand levels.  Columns
        past the strand's length are +inf (never the minimum)."""
        import torch
        fwd = np.asarray(fwd, np.float32)
        rev = np.asarray(rev, np.float32)
        if fwd.size != rev.size:
            raise ValueError("strands differ in length")
        if self.precision == "fp16":
            if fwd.size > self.scored:
                raise ValueError(f"{fwd.size} columns per strand > {self.scored} scored by {self.name}")
            a = np.full(self.ref_len, np.inf, np.float32)
            b = np.full(self.ref_len, np.inf, np.float32)
            a[: fwd.size] = fwd
            b[: rev.size] = rev
            cols = _half2_bits(a, b)
        else:
            half = self.ref_len // 2
            if fwd.size > half:
                raise ValueError(f"{fwd.size} columns per strand > {half} for {self.name}")
            cols = np.full(self.ref_len, np.inf, np.float32)
            cols[: fwd.size] = fwd
            cols[half: half + rev.size] = rev
            cols = cols.view(np.uint32)
        host = tile_interleave(cols, self.tiles)
        return torch.from_numpy(host.view(np.int32).copy()).cuda()

    def queries(self, z: np.ndarray):
        """Device query buffer from z-scored reads (n, 2048): half2 broadcast
        (FP16) or floats, plus the 32-entry zero tail."""
        import torch
        z = np.asarray(z, np.float32)
        if z.ndim != 2 or z.shape[1] != QUERY_LEN:
            raise ValueError(f"queries must be (n, {QUERY_LEN})")
        flat = np.concatenate([z.reshape(-1), np.zeros(32, np.float32)])
        words = _half2_bits(flat, flat) if self.precision == "fp16" else flat.view(np.uint32)
        return torch.from_numpy(words.view(np.int32).copy()).cuda()

    # ---------------------------------------------------------- launches
    def max_reads_per_launch(self) -> int:
        """Most reads one launch may hold: the kernel's 32-bit row-state index
        block_id * REF_LEN + column must stay below 2^31."""
        return INT32_MAX // self.ref_len

    def launch(self, d_ref, d_query, d_dist, d_last, n_reads: int, first_read: int = 0, stream: int = 0):
        """One launch of FullDTW::DTW over reads [first_read, first_read + n_reads)
        of d_query; results to d_dist[0:n_reads], row state in d_last."""
        if n_reads <= 0:
            return
        if n_reads > self.max_reads_per_launch():
            raise ValueError(f"{n_reads} reads per launch overflow the kernel's 32-bit row-state index "
                             f"(at most {self.max_reads_per_launch()} for REF_LEN {self.ref_len})")
        if d_ref.numel() < self.ref_len:
            raise ValueError("reference buffer too small")
        if d_query.numel() < (first_read + n_reads) * QUERY_LEN + 32:
            raise ValueError("query buffer too small")
        if d_last.numel() < n_reads * self.ref_len or d_dist.numel() < n_reads:
            raise ValueError("row-state or result buffer too small")
        vp = ctypes.c_void_p
        a_ref = vp(d_ref.data_ptr())
        a_q = vp(d_query.data_ptr() + first_read * QUERY_LEN * 4)
        a_dist = vp(d_dist.data_ptr())
        a_n = ctypes.c_int(n_reads)
        a_th = ctypes.c_uint32(0)     # thresh: FLOAT2HALF2(0) / 0.0f, unused by the kernel
        a_last = vp(d_last.data_ptr())
        args = [a_ref, a_q, a_dist, a_n, a_th, a_last]
        params = (vp * len(args))(*[ctypes.addressof(x) for x in args])
        rc = _Driver.lib().cuLaunchKernel(self._fn, n_reads, 1, 1, 32, 1, 1, DYN_SMEM, vp(stream), params, None)
        _Driver.check(rc, "cuLaunchKernel(FullDTW::DTW)")
        self.launches += 1

    def run(self, d_ref, z: np.ndarray, reads_per_launch: int = 0):
        """Scores of each read: (fwd, rev) float arrays for FP16, one array for
        FP32 (the min over the concatenated strands).  reads_per_launch 0 puts
        every read in one launch; BLOCK_NUM reproduces main.cu's batching."""
        import torch
        n = int(np.asarray(z).shape[0])
        d_q = self.queries(z)
        per = n if reads_per_launch <= 0 else min(reads_per_launch, n)
        per = min(per, self.max_reads_per_launch())
        d_last = torch.empty(max(per, 1) * self.ref_len, dtype=torch.int32, device="cuda")
        d_dist = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        for s in range(0, n, per):
            k = min(per, n - s)
            self.launch(d_ref, d_q, d_dist[s:], d_last, k, first_read=s, stream=stream)
        torch.cuda.synchronize()
        out = d_dist[:n].cpu().numpy().view(np.uint32)
        if self.precision == "fp16":
            lo = (out & 0xFFFF).astype(np.uint16).view(np.float16).astype(np.float32)
            hi = (out >> 16).astype(np.uint16).view(np.float16).astype(np.float32)
            return lo, hi
        return out.view(np.float32).copy()
