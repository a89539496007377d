"""Generate the FP64 answers of the precision-study (C2) and batched-uneven
(C3) workloads for the GPU parity tests.

The GPU tests regenerate the same seeded inputs with dtwax_gb300.synth and
compare the library's results with the FP64 scores and end columns stored
here, so the oracle does not have to run on the GPU host.  Inputs are checked
first: each fixture stores SHA-256 digests of the raw samples and of the
oracle's levels (rounded to FP32, the precision the library stores its
reference in), and a test fails with a clear message if the generator gives
different inputs on the machine it runs on.

  python tests/golden/make_precision_fixtures.py [--only c2|c3] [--threads N]

What is computed (the oracle's restatement of scripts/sdtw.py:86-116 and
:205-225 and of load_reference.hpp:33-128, oracle/sdtw_oracle.c):
  levels  = z-scored 6-mer levels of both strands, FP64, rounded to FP32;
  queries = each read z-scored in FP64 with eps 1e-4 (normalizer.cu:397-399),
            rounded to FP32 (the library's query buffer is FP32);
  answers = FP64 sDTW of every query against each strand: the best score and
            its end column per strand.

C2: all 2,048 reads x 2,000 samples against the seeded 1 Mb genome
    (8.19e12 cells; about 15 minutes on 8 x86 cores).
C3: 48 of the 8,192 reads of U[1000, 8000] samples against the seeded 5 Mb
    genome: the shortest and the longest read and 46 drawn with seed 7
    (about 2e12 cells).
C4: six reads served in 1,600-sample chunks against the seeded 5 Mb genome
    of the Read Until simulation (3, 3, 3, 3, 2 and 1 chunks; targets and
    non-targets): the best (score, end column, strand) after each chunk,
    each chunk z-scored with its own statistics and resumed from the
    previous chunk's last DP row in FP64, as the serving path does (one
    process per read).
C5: the same for four reads (3, 3, 2, 1 chunks) against the seeded 12 Mb
    genome of the memory-admitted stress run.
C2R: the first 32 C2 reads with the REF_DEL recurrence (the left
    predecessor of src/include/DTW.cu:23-29) against the 1 Mb genome.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

C2_PATH = os.path.join(HERE, "precision_c2.npz")
C3_PATH = os.path.join(HERE, "uneven_c3.npz")
C4_PATH = os.path.join(HERE, "serving_c4.npz")
C4_READ_SEED = 12
C4_CHUNK = 1600
C4_CHUNKS = [3, 3, 3, 3, 2, 1]
C4_TARGET = [1, 0, 1, 0, 1, 0]
C5_PATH = os.path.join(HERE, "serving_c5.npz")
C2R_PATH = os.path.join(HERE, "refdel_c2.npz")
C2R_READS = 32
C5_CHUNKS = [3, 3, 2, 1]
C5_TARGET = [1, 0, 1, 0]
C3_SAMPLE_SEED = 7
C3_SAMPLE = 48


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def c3_sample(lengths: np.ndarray) -> np.ndarray:
    """Indices of the C3 reads the fixture covers: shortest, longest, and a
    seeded draw of the rest, in ascending order."""
    rng = np.random.default_rng(C3_SAMPLE_SEED)
    lo, hi = int(np.argmin(lengths)), int(np.argmax(lengths))
    rest = np.setdiff1d(np.arange(lengths.size), [lo, hi])
    pick = rng.choice(rest, C3_SAMPLE - 2, replace=False)
    return np.sort(np.concatenate([[lo, hi], pick])).astype(np.int64)


def oracle_inputs(O, w, idx):
    """FP32-rounded oracle levels and z-scored queries of reads idx."""
    fwd, rev = O.build_levels(w.genome, w.table.astype(np.float64))
    fwd32, rev32 = fwd.astype(np.float32), rev.astype(np.float32)
    qs, offs = [], [0]
    for i in idx:
        z = O.zscore(w.reads.read(int(i)).astype(np.float64), 1e-4).astype(np.float32)
        qs.append(z)
        offs.append(offs[-1] + z.size)
    return fwd32, rev32, np.concatenate(qs), np.asarray(offs, np.int64)


def make(name: str, threads: int):
    from dtwax_gb300 import synth
    from oracle import oracle as O

    O.build()
    ref_del = name == "C2R"
    w = synth.make_workload("C2" if ref_del else name)
    lengths = np.diff(w.reads.offsets)
    if ref_del:
        idx = np.arange(C2R_READS, dtype=np.int64)
    else:
        idx = np.arange(w.reads.n, dtype=np.int64) if name == "C2" else c3_sample(lengths)
    fwd32, rev32, q, offs = oracle_inputs(O, w, idx)
    t = time.time()
    sf, ef, sr, er = O.sdtw_batch(fwd32.astype(np.float64), rev32.astype(np.float64), q.astype(np.float64), offs,
                                  n_threads=threads, ref_del=ref_del)
    dt = time.time() - t
    cells = float(lengths[idx].sum()) * fwd32.size * 2
    print(f"{name}: {idx.size} reads, {cells:.3e} cells in {dt:.0f} s ({cells / dt / 1e9:.1f} GCUPS)", flush=True)
    out = dict(read_index=idx, score_fwd=sf, end_fwd=ef, score_rev=sr, end_rev=er,
               target=w.reads.target[idx], n_samples=lengths[idx].astype(np.int32),
               ref_columns=np.int64(fwd32.size),
               raw_sha256=np.array(sha(w.reads.raw)), levels_sha256=np.array(sha(np.stack([fwd32, rev32]))),
               query_sha256=np.array(sha(q)), numpy_version=np.array(np.__version__))
    np.savez_compressed({"C2": C2_PATH, "C3": C3_PATH, "C2R": C2R_PATH}[name], **out)


def c4_reads(genome_len=5_000_000, chunks=C4_CHUNKS, target=C4_TARGET):
    """The serving genome pair and the served reads (seeded)."""
    from dtwax_gb300 import synth
    g = synth.random_genome(genome_len, synth.GENOME_SEED)
    o = synth.random_genome(genome_len, synth.OTHER_SEED)
    tab = synth.level_table()
    reads = synth.simulate_reads(g, o, tab, [C4_CHUNK * k for k in chunks], target, seed=C4_READ_SEED)
    return g, o, tab, reads


def _c4_one(args):
    """FP64 decisions after each chunk of one read (runs in its own process)."""
    i, fwd32, rev32, x = args
    from oracle import oracle as O
    fwd, rev = fwd32.astype(np.float64), rev32.astype(np.float64)
    rf = rr = None
    out = []
    for c in range(0, x.size, C4_CHUNK):
        z = O.zscore(x[c:c + C4_CHUNK].astype(np.float64), 1e-4).astype(np.float32).astype(np.float64)
        sf, ef, rf = O.sdtw(fwd, z, init_row=rf, want_row=True)
        sr, er, rr = O.sdtw(rev, z, init_row=rr, want_row=True)
        out.append((i, sf, ef, sr, er))
    return out


def make_c4(name="C4"):
    import multiprocessing as mp
    from oracle import oracle as O
    O.build()
    if name == "C4":
        path, chunks_, target_ = C4_PATH, C4_CHUNKS, C4_TARGET
        g, o, tab, reads = c4_reads()
    else:
        path, chunks_, target_ = C5_PATH, C5_CHUNKS, C5_TARGET
        g, o, tab, reads = c4_reads(12_000_000, C5_CHUNKS, C5_TARGET)
    fwd, rev = O.build_levels(g, tab.astype(np.float64))
    fwd32, rev32 = fwd.astype(np.float32), rev.astype(np.float32)
    t = time.time()
    with mp.get_context("spawn").Pool(len(chunks_)) as pool:
        rows = pool.map(_c4_one, [(i, fwd32, rev32, reads.read(i)) for i in range(reads.n)])
    print(f"{name}: {reads.n} reads, {sum(chunks_)} chunk-steps in {time.time() - t:.0f} s", flush=True)
    flat = [r for per in rows for r in per]
    np.savez_compressed(path, read=np.array([r[0] for r in flat], np.int32),
                        score_fwd=np.array([r[1] for r in flat]), end_fwd=np.array([r[2] for r in flat], np.int64),
                        score_rev=np.array([r[3] for r in flat]), end_rev=np.array([r[4] for r in flat], np.int64),
                        chunks=np.array(chunks_, np.int32), target=np.array(target_, np.int8),
                        raw_sha256=np.array(sha(reads.raw)), levels_sha256=np.array(sha(np.stack([fwd32, rev32]))),
                        numpy_version=np.array(np.__version__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["c2", "c3", "c4", "c5", "c2r"])
    ap.add_argument("--threads", type=int, default=0)
    a = ap.parse_args()
    for name in ("C2R", "C5", "C4", "C3", "C2"):
        if a.only and a.only != name.lower():
            continue
        if name in ("C4", "C5"):
            make_c4(name)
        else:
            make(name, a.threads)


if __name__ == "__main__":
    main()
