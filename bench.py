"""Benchmark of the sDTW classification path on the batched uneven-read workload.

Workload (one step, default C3): 8,192 reads of U[1000, 8000] samples (50/50
target / non-target) against a seeded random 5 Mb genome (4,999,995 k-mer
columns per strand, both strands), about 3.7e14 DP cells in one persistent
launch: raw pA samples resident in HBM -> window + z-score kernel -> sDTW sweep
(FP16 half2 cells, FP32 offsets) -> min/argmin finalize, replayed as a captured
CUDA graph with the autotuned launch shape.  --workload C2 runs the
precision-study shape (2,048 x 2,000 samples vs 1 Mb).  Metric: sDTW GCUPS =
sum over reads of samples x columns x 2 strands / s / 1e9.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU implementation of the path (the OpenMP FP64
restatement of the reference's scripts/sdtw.py `sdtw_default`; the Python
original needs numba, which is not installed) on a bounded read sample with
every host thread, and prints the same metric.  Beside it, under
"reference_gpu_kernel", it times the reference's own FP16 CUDA kernel
(compiled from its sources into oracle/_ref/) on this GPU, with main.cu's
10-reads-per-launch pattern and with every read in one launch.

Multi-GPU: reads are independent, each rank runs its own copy of the
workload (weak scaling, no collective on the data path); the timed region is
bracketed by a barrier and the max over ranks is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "C3"
WORKLOAD_DESC = {
    "C2": ("precision-study shape: seeded random 1 Mb genome (999,995 k-mer columns per strand, both strands), "
           "2,048 reads x 2,000 samples (1,024 target / 1,024 non-target), dwell geometric mean 9, noise sd 1.8 pA"),
    "C3": ("batched uneven reads: seeded random 5 Mb genome (4,999,995 k-mer columns per strand, both strands), "
           "8,192 reads of U[1000, 8000] samples (50/50 target / non-target), one persistent launch, "
           "CUDA-graph replay, autotuned launch shape"),
}
CPU_TARGET_S = 15.0


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        loaded = [v for v in sm if mx and v > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def measured_hbm_gbs():
    """Copy bandwidth measured on this machine's GPUs, when the file is present."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def traffic_per_launch(precision: str, workload: str):
    """DRAM bytes per sweep launch of this precision and workload from
    profiles/traffic.json (ncu dram__bytes_read.sum + dram__bytes_write.sum,
    written beside the summary each figure comes from), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        rec = json.load(open(path)).get(f"sdtw_{precision}_{workload}")
    except (OSError, ValueError):
        return None
    return float(rec["dram_bytes_per_launch"]) if rec else None


def cpu_baseline(workload, n_steps: int = 1, target_s: float = CPU_TARGET_S):
    """FP64 OpenMP oracle (restatement of sdtw.py `sdtw_default`) on a
    bounded sample of the same workload, all host threads.  The sample is one
    read per thread (more when they are short), each aligned over a prefix of
    its samples against both strands of the whole reference, the prefix
    sized so that a pass takes about target_s.  Returns the record."""
    from oracle import oracle as O

    O.build()
    fwd, rev = O.build_levels(workload.genome, workload.table.astype(np.float64))
    m = fwd.size
    reads = workload.reads
    cores = O.max_threads()
    lens = np.diff(reads.offsets)
    zs = {}

    def z(i):
        if i not in zs:
            zs[i] = O.zscore(reads.read(i).astype(np.float64), 1e-4)
        return zs[i]

    def run(idx, prefix):
        qs = [z(i)[:prefix] for i in idx]
        q = np.concatenate(qs)
        offs = np.concatenate([[0], np.cumsum([x.size for x in qs])]).astype(np.int64)
        t = time.perf_counter()
        O.sdtw_batch(fwd, rev, q, offs)
        dt = time.perf_counter() - t
        return float(q.size) * m * 2, dt

    # calibrate on one read per thread over a short prefix, then size the
    # sample (reads x prefix) to about target_s per pass
    idx = list(range(min(cores, reads.n)))
    c0, t0 = run(idx, 64)
    rate = c0 / t0
    want = target_s * rate / (m * 2)              # samples per pass
    n = len(idx)
    prefix = int(min(lens[idx].min(), max(64, want / n)))
    if prefix >= lens[idx].min() and want > n * prefix:  # whole reads: take more of them
        n = int(min(reads.n, max(n, round(want / lens.mean() / cores) * cores)))
        idx = list(range(n))
        prefix = int(lens.max())
    total_c, total_t = 0.0, 0.0
    for _ in range(n_steps):
        c, t = run(idx, prefix)
        total_c += c
        total_t += t
    # the reference's Python sDTW (scripts/sdtw.py sdtw_default) needs numba; its
    # row-vectorised numpy restatement runs one read prefix on one core instead
    try:
        import numba  # noqa: F401
        numba_state = "installed but not timed (the oracle port is the timed baseline)"
    except ImportError:
        numba_state = "unavailable: numba is not installed"
    q1 = z(0)[:200]
    t = time.perf_counter()
    O.np_sdtw(fwd, q1)
    np_dt = time.perf_counter() - t
    whole = prefix >= lens[idx].max()
    shape = "whole reads" if whole else f"the first {prefix} samples of each"
    return {"value": total_c / total_t / 1e9, "unit": "GCUPS", "cores": cores, "kind": "port",
            "sample": f"{n} of {reads.n} reads ({shape}) against both strands of the full "
                      f"{m}-column reference, FP64, {n_steps} pass(es)",
            "seconds": total_t,
            # reads/s of whole reads of the workload's mean length at the measured cell rate
            "reads_per_s": total_c / total_t / (float(lens.mean()) * m * 2),
            "numpy_restatement_1core_gcups": float(q1.size) * m / np_dt / 1e9,
            "numba_original": numba_state}


SERVING = {
    # Read Until: 1,600-sample chunks every 0.4 s per channel, Poisson read
    # starts at 1/s per channel, decision after at most 3 chunks
    "C4": dict(genome_len=5_000_000, channels=512, budget_gb=40.0),
    # memory-admitted stress: 3,000 channels, 12 Mb genome (96 MB FP32 row per read)
    "C5": dict(genome_len=12_000_000, channels=3000, budget_gb=100.0),
}


def run_serving(name: str, precision: int, device: int, duration_s: float, batches: int = 0,
                state: str = "fp32"):
    import dtwax_gb300 as d
    from dtwax_gb300 import readuntil, synth

    spec = SERVING[name]
    g = synth.random_genome(spec["genome_len"], synth.GENOME_SEED)
    o = synth.random_genome(spec["genome_len"], synth.OTHER_SEED)
    tab = synth.level_table()
    cfg = readuntil.ServeConfig(channels=spec["channels"], duration_s=duration_s, warmup_s=2.0)
    reads = readuntil.make_pool(g, o, tab, cfg)
    # accept / reject rates from reads that are never served: the call
    # accuracy of the run is held out
    held = readuntil.make_pool(g, o, tab, cfg, held_out=True, n=256)
    state_precision = d.STATE_FP16 if state == "fp16" and precision == d.FP16 else d.STATE_FP32
    with d.Classifier(sequence=g, level_table=tab, precision=precision, device=device,
                      serve_batches=batches, state_precision=state_precision) as clf:
        accept, reject = readuntil.calibrate(clf, held, cfg)
        rec = readuntil.run(clf, reads, cfg, accept, reject, state_budget_bytes=spec["budget_gb"] * 1e9)
    # row-state traffic of the resumed sweeps: a slot holds both strands' last
    # DP row (8 B per column pair in FP32, about 4 B with FP16 rows); each
    # chunk-step reads it (except a read's first chunk) and writes it back
    slot_bytes = (4 if state_precision == d.STATE_FP16 else 8) * (spec["genome_len"] - 5)
    rec["row_state_gbs"] = rec["chunks_processed_per_s"] * 2 * slot_bytes / 1e9
    rec["row_state_bytes_per_chunk_step"] = 2 * slot_bytes
    rec["calibration"] = "accept/reject rates from the first chunks of 256 held-out reads (not served)"
    rec["workload"] = (f"{name}: {spec['channels']} channels, 1,600-sample chunks every 0.4 s, Poisson read "
                       f"starts 1/s/channel, <= 3 chunks per decision, {spec['genome_len'] // 1_000_000} Mb "
                       f"seeded genome ({2 * (spec['genome_len'] - 5)} columns), row-state budget "
                       f"{spec['budget_gb']:.0f} GB, {'FP16' if state_precision == d.STATE_FP16 else 'FP32'} "
                       f"row state")
    return rec


REF_GPU_GEOMETRY = {"C2": "fp16_1000064", "C3": "fp16_5000320"}
REF_GPU_GEOMETRY_FP32 = {"C2": "fp32_2000128", "C3": "fp32_10000640"}
REF_FP32_READS = {"C2": 4, "C3": 2}  # one read per launch: about 1 s (C2) and 10 s (C3) per read


def reference_gpu_kernel(workload, n_reads: int = 2048, shipped_launches: int = 2, fp32_reads: int = 0):
    """The reference's own FP16 kernel (FullDTW::DTW, src/include/DTW.cu,
    compiled from its sources into oracle/_ref) on this GPU, on the workload's
    genome: reads of the kernel's fixed 2,048-sample query from the same
    generator, levels from the oracle's restatement of the reference's builder.
    Two launch patterns: main.cu's (BLOCK_NUM = 10 reads per launch, one
    stream, `shipped_launches` launches timed) and every read in one launch.
    Beside it the reference's FP32 build of the same kernel (strands
    concatenated, load_reference.hpp:36-37) with one read per launch: the
    plain one-read-per-launch FP32 sDTW, timed on `fp32_reads` reads.
    Returns the record, or {"unavailable": why}."""
    import torch
    from dtwax_gb300 import synth
    from oracle import oracle as O
    from oracle import ref_kernel as RK

    fp32_reads = fp32_reads or REF_FP32_READS.get(workload.name, 2)
    name = REF_GPU_GEOMETRY.get(workload.name)
    if name is None:
        return {"unavailable": f"no reference-kernel geometry for {workload.name} (its query length is fixed "
                               "at 2,048 samples)"}
    if not RK.available(name):
        return {"unavailable": f"{os.path.relpath(RK.cubin_path(name), ROOT)} not built (needs the reference's "
                               "sources at build time)"}
    if not torch.cuda.is_available():
        return {"unavailable": "no CUDA device"}
    fwd, rev = O.build_levels(workload.genome, workload.table.astype(np.float64))
    m = fwd.size
    mask = (np.arange(n_reads) % 2 == 0).astype(np.int8)
    reads = synth.simulate_reads(workload.genome, workload.other, workload.table, [RK.QUERY_LEN] * n_reads, mask,
                                 seed=synth.READ_SEED)
    z = np.stack([O.zscore(reads.read(i).astype(np.float64), 1e-4) for i in range(n_reads)]).astype(np.float32)
    cells_per_read = float(RK.QUERY_LEN) * m * 2
    out = {"kernel": "FullDTW::DTW<int, __half2> (src/include/DTW.cu:151-572, -DFP16 -DNO_REF_DEL), "
                     f"cubin {name}: {m} columns per strand in {-(-m // RK.TILE)} tiles",
           "query_samples": RK.QUERY_LEN, "unit": "GCUPS"}
    with RK.RefKernel(name) as k:
        d_ref = k.reference(fwd.astype(np.float32), rev.astype(np.float32))
        d_q = k.queries(z)
        d_dist = torch.empty(n_reads, dtype=torch.int32, device="cuda")
        d_last = torch.empty(min(n_reads, k.max_reads_per_launch()) * k.ref_len, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream()
        sh = stream.cuda_stream
        # warm-up: one small launch
        k.launch(d_ref, d_q, d_dist, d_last, 2, stream=sh)
        torch.cuda.synchronize()
        # main.cu's pattern: 10 reads per launch, launches in sequence
        b, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b.record(stream)
        for i in range(shipped_launches):
            k.launch(d_ref, d_q, d_dist[i * RK.BLOCK_NUM:], d_last, RK.BLOCK_NUM, first_read=i * RK.BLOCK_NUM,
                     stream=sh)
        e.record(stream)
        torch.cuda.synchronize()
        ms = b.elapsed_time(e)
        nr = shipped_launches * RK.BLOCK_NUM
        out["as_shipped"] = {"value": nr * cells_per_read / (ms * 1e-3) / 1e9, "reads_per_s": nr / (ms * 1e-3),
                             "ms": ms, "launches": shipped_launches, "reads_per_launch": RK.BLOCK_NUM}
        # every read in one launch (one warp per read), or as many per launch
        # as the kernel's 32-bit row-state index allows (429 on the 5 Mb genome)
        per = min(n_reads, k.max_reads_per_launch())
        b.record(stream)
        for s0 in range(0, n_reads, per):
            k.launch(d_ref, d_q, d_dist[s0:], d_last, min(per, n_reads - s0), first_read=s0, stream=sh)
        e.record(stream)
        torch.cuda.synchronize()
        ms = b.elapsed_time(e)
        out["one_launch"] = {"value": n_reads * cells_per_read / (ms * 1e-3) / 1e9,
                             "reads_per_s": n_reads / (ms * 1e-3), "ms": ms, "reads": n_reads,
                             "reads_per_launch": per, "launches": -(-n_reads // per)}
    name32 = REF_GPU_GEOMETRY_FP32.get(workload.name)
    if name32 is None or not RK.available(name32):
        out["fp32_one_read_per_launch"] = {"unavailable": f"no FP32 reference-kernel cubin for {workload.name}"}
        return out
    with RK.RefKernel(name32) as k:
        d_ref = k.reference(fwd.astype(np.float32), rev.astype(np.float32))
        d_q = k.queries(z[:fp32_reads])
        d_dist = torch.empty(fp32_reads, dtype=torch.float32, device="cuda")
        d_last = torch.empty(k.ref_len, dtype=torch.float32, device="cuda")
        stream = torch.cuda.current_stream()
        sh = stream.cuda_stream
        k.launch(d_ref, d_q, d_dist, d_last, 1, stream=sh)  # warm-up
        torch.cuda.synchronize()
        b, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b.record(stream)
        for i in range(fp32_reads):
            k.launch(d_ref, d_q, d_dist[i:], d_last, 1, first_read=i, stream=sh)
        e.record(stream)
        torch.cuda.synchronize()
        ms = b.elapsed_time(e)
        out["fp32_one_read_per_launch"] = {
            "kernel": f"FullDTW::DTW<int, float> (-DNO_REF_DEL), cubin {name32}: fwd and rev concatenated, "
                      f"{-(-2 * m // RK.TILE)} tiles",
            "value": fp32_reads * cells_per_read / (ms * 1e-3) / 1e9, "reads_per_s": fp32_reads / (ms * 1e-3),
            "ms": ms, "reads": fp32_reads, "launches": fp32_reads,
            # the same cell rate in reads of the workload's own mean length
            "reads_per_s_at_workload_mean_length": fp32_reads * cells_per_read / (ms * 1e-3)
            / (float(np.diff(workload.reads.offsets).mean()) * m * 2),
            "score_min": float(d_dist.min().item()), "score_max": float(d_dist.max().item())}
    return out


def run_reference(args, rank, world):
    from dtwax_gb300 import synth
    if rank != 0:
        return 0
    w = synth.make_workload(args.workload)
    # each step is one pass over the bounded sample; warm-up passes are shorter
    cpu_baseline(w, 1, target_s=min(2.0, args.cpu_seconds)) if args.warmup > 0 else None
    rec = cpu_baseline(w, n_steps=max(args.steps, 1),
                       target_s=max(min(4.0, args.cpu_seconds), args.cpu_seconds / max(args.steps, 1)))
    line = {"metric": "sDTW GCUPS", "value": rec["value"], "unit": "GCUPS", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rec["seconds"] * 1e3 / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"{args.workload}: {WORKLOAD_DESC[args.workload]}", "implementation":
                       "oracle/sdtw_oracle.c: OpenMP FP64 restatement of scripts/sdtw.py sdtw_default "
                       "(numba original not installed); bounded read sample"},
            "cpu_baseline": {k: rec[k] for k in ("value", "unit", "cores", "kind", "sample",
                                                 "numpy_restatement_1core_gcups", "numba_original")},
            "e2e": {"value": rec["value"], "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reads_per_s": rec["reads_per_s"]}
    if not args.skip_ref_gpu:
        try:
            line["reference_gpu_kernel"] = reference_gpu_kernel(w)
        except Exception as exc:  # a failed reference-kernel run must not hide the CPU line
            line["reference_gpu_kernel"] = {"unavailable": f"{type(exc).__name__}: {exc}"}
    print(json.dumps(line), flush=True)
    return 0


def c2_subrecord(device: int, precision: int, peak_cells_s: float, steps: int = 5, warmup: int = 3):
    """The precision-study shape (C2: 2,048 x 2,000 samples vs 1 Mb) beside a
    C3 line: the same device-resident step, timed the same way."""
    import torch
    import dtwax_gb300 as d
    from dtwax_gb300 import synth

    w = synth.make_workload("C2")
    cells = w.cells()
    with d.Classifier(sequence=w.genome, level_table=w.table, precision=precision, device=device) as clf:
        stream = torch.cuda.Stream()
        d_raw = torch.tensor(w.reads.raw, device="cuda")
        d_out = torch.zeros(32 * w.reads.n, dtype=torch.uint8, device="cuda")
        flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
        step_ms, sweep_ms = [], []
        with torch.cuda.stream(stream):
            for i in range(warmup + steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                clf.classify_device(d_raw.data_ptr(), w.reads.offsets, d_out.data_ptr(), stream.cuda_stream)
                e1.record(stream)
                stream.synchronize()
                if i >= warmup:
                    step_ms.append(e0.elapsed_time(e1))
                    sweep_ms.append(clf.last_sweep_ms())
        clf.sync()
        tuning = clf.tuning()
    sweep = cells / (float(np.mean(sweep_ms)) / 1e3) / 1e9
    return {"workload": f"C2: {WORKLOAD_DESC['C2']}", "steps": steps, "warmup": warmup,
            "value": cells * steps / (sum(step_ms) / 1e3) / 1e9, "unit": "GCUPS",
            "reads_per_s": w.reads.n * steps / (sum(step_ms) / 1e3), "ms_per_step": sum(step_ms) / steps,
            "sweep_gcups": sweep, "sweep_frac_of_probe": sweep / (peak_cells_s / 1e9),
            "traffic": traffic_per_launch({d.FP16: "fp16", d.FP32: "fp32", d.MIXED: "mixed"}[precision], "C2"),
            "tuning": tuning}


def run_ours(args, rank, world, local):
    import torch
    import dtwax_gb300 as d
    from dtwax_gb300 import synth

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(v: float) -> float:
        if dist is None:
            return v
        t = torch.tensor([v], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    precision = {"fp16": d.FP16, "fp32": d.FP32, "mixed": d.MIXED}[args.precision]
    ref_del = args.recurrence == "ref_del"
    if ref_del and precision == d.MIXED:
        raise SystemExit("--recurrence ref_del runs FP16 or FP32 cells")
    w = synth.make_workload(args.workload, n_reads=args.reads or None)
    cells = w.cells()
    n_reads = w.reads.n
    peak = d.peak_probe(local, precision, 400.0)
    use_graphs = 1 if (args.graphs or args.workload == "C3") and not args.no_graphs else 0
    clf = d.Classifier(sequence=w.genome, level_table=w.table, precision=precision, device=local,
                       cells_per_thread=args.cells, chunk_strips=args.strips, warps_per_cta=args.warps,
                       use_graphs=use_graphs, recurrence=d.REF_DEL if ref_del else d.NO_REF_DEL)
    if (args.autotune or args.workload == "C3") and not args.no_autotune:
        clf.autotune(n_reads, int(np.diff(w.reads.offsets).mean()))
    stream = torch.cuda.Stream()
    d_raw = torch.tensor(w.reads.raw, device="cuda")
    d_out = torch.zeros(32 * n_reads, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB of L2

    def step():
        clf.classify_device(d_raw.data_ptr(), w.reads.offsets, d_out.data_ptr(), stream.cuda_stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        stream.synchronize()
    launches_per_step = clf.last_launch_count

    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    time.sleep(0.3)
    step_ms, sweep_ms = [], []
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between timed steps, outside the events
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.nvtx.range_push("timed_step")  # lets ncu pick a timed launch (--nvtx-include)
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.nvtx.range_pop()
            stream.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            sweep_ms.append(clf.last_sweep_ms())
    barrier()
    clock_rec = clocks.stop()
    clf.sync()  # raises if a kernel of the timed steps reported a device-side error
    tuning = clf.tuning()
    total_ms = max_over_ranks(sum(step_ms))
    res = np.frombuffer(d_out.cpu().numpy().tobytes(), d.RESULT_DTYPE)
    if (res["call"] < 0).any():
        raise SystemExit(f"{int((res['call'] < 0).sum())} reads have no valid result")

    # end to end through the public host API: host samples in, results out
    e2e_ms = []
    for _ in range(1 if args.workload == "C3" else max(2, min(args.steps, 5))):
        t = time.perf_counter()
        host_res = clf.classify(raw=w.reads.raw, offsets=w.reads.offsets)
        e2e_ms.append((time.perf_counter() - t) * 1e3)
    e2e_total = max_over_ranks(sum(e2e_ms))
    h2d = int(w.reads.raw.nbytes + n_reads * 60)  # samples + per-read task/window metadata
    d2h = int(host_res.nbytes)

    # plain comparator: FP32, one sweep launch per read, on a read sample, with
    # the launch shape the autotuner picks for one-read FP32 batches
    n_plain = min(64, n_reads)
    with d.Classifier(sequence=w.genome, level_table=w.table, precision=d.FP32, device=local) as pclf:
        pclf.autotune(1, int(np.diff(w.reads.offsets[: n_plain + 1]).mean()))
        pclf.classify_plain_fp32(raw=w.reads.raw[: w.reads.offsets[2]], offsets=w.reads.offsets[:3])  # warm-up
        t = time.perf_counter()
        plain = pclf.classify_plain_fp32(raw=w.reads.raw[: w.reads.offsets[n_plain]],
                                         offsets=w.reads.offsets[: n_plain + 1])
        plain_s = time.perf_counter() - t
        plain_shape = pclf.tuning()
    plain_rps = n_plain / plain_s
    plain_gcups = float(w.reads.offsets[n_plain]) * w.ref_len * 2 / plain_s / 1e9

    value = world * cells * args.steps / (total_ms / 1e3) / 1e9
    reads_per_s = world * n_reads * args.steps / (total_ms / 1e3)
    mean_sweep_s = float(np.mean(sweep_ms)) / 1e3
    achieved = cells / mean_sweep_s / 1e9
    # pipe-bound ceiling from the SM count and the measured SM clock: FP16 cell
    # pairs cost 2 FMA-pipe instructions that hold the pipe 2 cycles each
    # (64 cells/SM/cycle); FP32 cells cost 3 issue slots (42.7 cells/SM/cycle);
    # MIXED cells cost 2.5 issue slots (half an HSUB2, one FMA, one FMNMX: 51.2)
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clock_rec.get("sm_mhz") or 2070.0
    per_sm_cycle = {d.FP16: 64.0, d.FP32: 128.0 / 3.0, d.MIXED: 128.0 / 2.5}[precision]
    if ref_del:
        # REF_DEL (anti-diagonal sweeps): a FP32 cell takes 4 issue slots (sub,
        # two mins, FMA); a FP16 pair takes the same 4 (HSUB2, two HMNMX2,
        # HFMA2), its HSUB2 and HFMA2 holding the FMA pipe 2 cycles each
        per_sm_cycle = 128.0 / 4.0 if precision == d.FP32 else 64.0
    theoretical = sms * per_sm_cycle * mhz * 1e6 / 1e9
    traffic = traffic_per_launch(args.precision, args.workload) if not ref_del else None
    # the roofline peak: the measured probe of the cell's instruction mix where
    # it is a ceiling (FP16 and MIXED cells); the FP32 probe runs below the
    # sweep itself and REF_DEL has a different mix, so those use the bound
    if ref_del or precision == d.FP32 or peak / 1e9 < achieved:
        roof_peak = theoretical
        peak_source = ("issue/pipe bound from the SM count and the SM clock measured in this run "
                       "(the probe of this mix is not a ceiling for it)")
    else:
        roof_peak = peak / 1e9
        peak_source = ("dtwx_peak_probe: the per-cell instruction mix (sub, min, fma) on register-resident "
                       "cells, all SMs, measured in this run")
    t_mask = w.reads.target == 1
    line = {
        "metric": "sDTW GCUPS", "value": value, "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {d.FP16: "f16x2", d.FP32: "f32", d.MIXED: "f16-diff/f32"}[precision],
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: {WORKLOAD_DESC[args.workload]}", "cells_per_step": cells,
                   "reads_per_step": n_reads, "ref_columns_per_strand": w.ref_len,
                   "precision": args.precision, "recurrence": args.recurrence, "step": "window+z-score kernel, sDTW sweep, min/argmin finalize; "
                   "raw samples resident in HBM", "l2": "flushed between timed steps (256 MB write)",
                   "tuning": tuning, "seeds": w.meta["seeds"], "parallelism": f"replicas x{world}"},
        "reads_per_s": reads_per_s,
        # the reference's own secondary figure (hpc_helpers.hpp:93-100): samples
        # per microsecond / 10, i.e. Mbases/s at 10 samples per base
        "mbps": float(np.diff(w.reads.offsets).sum()) * world * args.steps / (total_ms * 1e3) / 10,
        "roofline": {"bound": "alu", "achieved": achieved, "peak": roof_peak, "unit": "Gcell/s",
                     "frac": achieved / roof_peak, "traffic": traffic,
                     "peak_theoretical": theoretical, "frac_of_theoretical": achieved / theoretical,
                     "peak_probe": peak / 1e9, "peak_source": peak_source,
                     "kernel": "dtwx::sdtw_kernel, mean of CUDA events around each launch",
                     # the HBM roofline, for contrast: the sweep's measured DRAM traffic per
                     # launch over its duration, against the measured copy bandwidth
                     "hbm_achieved_gbs": (traffic / mean_sweep_s / 1e9) if traffic else None,
                     "hbm_peak_gbs": measured_hbm_gbs()},
        "e2e": {"value": world * cells * len(e2e_ms) / (e2e_total / 1e3) / 1e9, "unit": "GCUPS",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "dtwx_classify_batch (host raw samples -> host results)"},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clock_rec,
        "plain_fp32": {"reads_per_s": plain_rps, "gcups": plain_gcups, "sample_reads": n_plain,
                       "sample_mean_samples": float(w.reads.offsets[n_plain]) / n_plain, "tuning": plain_shape,
                       "path": "dtwx_classify_plain_fp32: this library's FP32 kernel, one launch per read, "
                               "shape autotuned for one-read batches",
                       "speedup_reads_per_s": reads_per_s / world / plain_rps,
                       "speedup_gcups": value / world / plain_gcups},
        "check": {"target_score_per_sample_max": float((res["score"] / res["n_samples"])[t_mask].max()),
                  "other_score_per_sample_min": float((res["score"] / res["n_samples"])[~t_mask].min())},
    }
    # the serving run and the CPU baseline belong to the one-GPU line only: with
    # N ranks every GPU would be held while rank 0 alone ran them
    if args.workload == "C3" and not args.no_c2 and not ref_del and not args.reads and rank == 0 and world == 1:
        line["c2"] = c2_subrecord(local, precision, peak)
    if args.serving != "none" and rank == 0 and world == 1:
        line["serving"] = run_serving(args.serving, precision, local, args.serving_seconds, args.serve_batches,
                                      args.state)
    if args.reads:
        line["config"]["workload"] += f" (first {n_reads} reads only)"
    if rank == 0:
        line["cpu_baseline"] = None if (args.skip_cpu or world > 1) else {
            k: v for k, v in cpu_baseline(w).items()
            if k in ("value", "unit", "cores", "kind", "sample", "numpy_restatement_1core_gcups", "numba_original")}
        print(json.dumps(line), flush=True)
    clf.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skip-ref-gpu", action="store_true",
                    help="reference arm: do not time the reference's own GPU kernel beside the CPU line")
    ap.add_argument("--precision", choices=["fp16", "fp32", "mixed"], default="fp16")
    ap.add_argument("--state", choices=["fp32", "fp16"], default="fp32",
                    help="serving row state: FP32 values or FP16 cells with frame offsets (FP16 cells only)")
    ap.add_argument("--recurrence", choices=["no_ref_del", "ref_del"], default="no_ref_del",
                    help="ref_del: the left predecessor of DTW.cu:23-29 (FP16 or FP32 cells)")
    ap.add_argument("--reads", type=int, default=0,
                    help="use only the first N reads of the workload (small cases for profiling)")
    ap.add_argument("--skip-cpu", action="store_true", help="do not time the CPU baseline")
    ap.add_argument("--cpu-seconds", type=float, default=60.0,
                    help="reference arm: CPU seconds over all timed steps (each step is a bounded read sample)")
    ap.add_argument("--serving", choices=["none", "C4", "C5"], default="C4",
                    help="Read Until serving simulation reported beside the batch metric")
    ap.add_argument("--serving-seconds", type=float, default=30.0)
    ap.add_argument("--serve-batches", type=int, default=0, help="serving batches in flight (0 = library default)")
    ap.add_argument("--cells", type=int, default=0, help="cells per thread (0 = tuned)")
    ap.add_argument("--strips", type=int, default=0, help="strips per work item (0 = tuned)")
    ap.add_argument("--warps", type=int, default=0, help="warps per CTA (0 = tuned)")
    ap.add_argument("--autotune", action="store_true", help="time candidate launch shapes before measuring")
    ap.add_argument("--graphs", action="store_true", help="replay the step as a captured CUDA graph")
    ap.add_argument("--no-autotune", action="store_true",
                    help="C3: keep the given or default launch shape (profiling a fixed launch)")
    ap.add_argument("--no-graphs", action="store_true", help="C3: launch the kernels directly, no graph replay")
    ap.add_argument("--workload", choices=["C2", "C3"], default=WORKLOAD,
                    help="C3: 8,192 uneven reads vs 5 Mb (default); C2: 2,048 x 2,000 samples vs 1 Mb")
    ap.add_argument("--no-c2", action="store_true", help="do not add the C2 sub-record to a C3 line")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
