"""Seeded synthetic nanopore squiggles of the benchmark shapes.

The reference's datasets (lambda / COVID / human FAST5 fetched by
download_datasets.sh) are not available, so reads are simulated:

* genomes: uniform i.i.d. ACGT, seed 1 (target) and seed 2 (non-target);
* 6-mer level table: the k-mer model file when given, else 4096 means drawn
  from N(90, 12) pA with seed 3 (the shipped R9.4 model has mean 90.2, sd 12.9);
* reads (seed 4): a random strand and start on the source genome; each k-mer
  is held for a geometric dwell (p = 1/9, mean 9 samples, >= 1) and Gaussian
  noise of sd 1.8 pA is added.  Samples are pA floats; the classifier z-scores
  them.

Workload shapes (one per benchmark configuration):
  C1  48,502 bp genome, 512 reads x 2,000 samples (256 target / 256 other)
  C2  1 Mb genome, 2,048 reads x 2,000 samples
  C3  5 Mb genome, 8,192 reads of U[1000, 8000] samples, 50/50
  C4  5 Mb genome, Read Until: 512 channels, 1,600-sample chunks
  C5  12 Mb genome, Read Until: 3,000 channels, 1,600-sample chunks
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

GENOME_SEED, OTHER_SEED, TABLE_SEED, READ_SEED = 1, 2, 3, 4
DWELL_MEAN, NOISE_SD = 9.0, 1.8

_LUT = np.full(256, -1, np.int64)
for _c, _v in zip(b"ACGT", range(4)):
    _LUT[_c] = _v


def random_genome(length: int, seed: int) -> bytes:
    rng = np.random.default_rng(seed)
    return np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, length)].tobytes()


def level_table(seed: int = TABLE_SEED) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.normal(90.0, 12.0, 4096).astype(np.float32)


def revcomp(seq: bytes) -> bytes:
    return seq.translate(bytes.maketrans(b"ACGTacgt", b"TGCAtgca"))[::-1]


def kmer_codes(seq: bytes) -> np.ndarray:
    b = _LUT[np.frombuffer(seq, np.uint8)]
    m = len(seq) - 5
    code = np.zeros(max(m, 0), np.int64)
    for k in range(6):
        code = code * 4 + b[k:k + m]
    return code


@dataclass
class Reads:
    raw: np.ndarray            # float32 samples, reads back to back
    offsets: np.ndarray        # int64 [n+1]
    target: np.ndarray         # 1 = drawn from the target genome
    strand: np.ndarray         # 0 forward, 1 reverse complement
    start: np.ndarray          # first k-mer position on that strand
    kmers: np.ndarray          # k-mers the read traverses

    @property
    def n(self) -> int:
        return self.offsets.size - 1

    def read(self, i: int) -> np.ndarray:
        return self.raw[self.offsets[i]:self.offsets[i + 1]]


def _simulate_one(rng, lv, length: int):
    m = lv.size
    need = int(length / DWELL_MEAN * 1.6) + 32
    dw = rng.geometric(1.0 / DWELL_MEAN, need)
    while dw.sum() < length:
        dw = np.concatenate([dw, rng.geometric(1.0 / DWELL_MEAN, need)])
    nk = int(np.searchsorted(np.cumsum(dw), length) + 1)
    nk = min(nk, m)
    start = int(rng.integers(0, max(m - nk, 0) + 1))
    sig = np.repeat(lv[start:start + nk], dw[:nk])[:length]
    if sig.size < length:  # source shorter than the read: pad by holding the last level
        sig = np.concatenate([sig, np.full(length - sig.size, sig[-1] if sig.size else 0.0)])
    sig = sig + rng.normal(0.0, NOISE_SD, length)
    return sig.astype(np.float32), start, nk


def simulate_reads(target_genome: bytes, other_genome: bytes, table, lengths, target_mask,
                   seed: int = READ_SEED) -> Reads:
    """One read per entry of `lengths`; target_mask[i] picks the source genome."""
    rng = np.random.default_rng(seed)
    table = np.asarray(table, np.float64)
    levels = {}
    for tag, g in ((1, target_genome), (0, other_genome)):
        levels[(tag, 0)] = table[kmer_codes(g)]
        levels[(tag, 1)] = table[kmer_codes(revcomp(g))]
    n = len(lengths)
    sigs = []
    strand = np.zeros(n, np.int8)
    start = np.zeros(n, np.int64)
    kmers = np.zeros(n, np.int64)
    for i in range(n):
        s = int(rng.integers(0, 2))
        sig, st, nk = _simulate_one(rng, levels[(int(target_mask[i]), s)], int(lengths[i]))
        sigs.append(sig)
        strand[i], start[i], kmers[i] = s, st, nk
    offsets = np.zeros(n + 1, np.int64)
    offsets[1:] = np.cumsum([x.size for x in sigs])
    raw = np.concatenate(sigs) if sigs else np.zeros(0, np.float32)
    return Reads(raw, offsets, np.asarray(target_mask, np.int8), strand, start, kmers)


@dataclass
class Workload:
    name: str
    genome: bytes
    other: bytes
    table: np.ndarray
    reads: Reads
    meta: dict = field(default_factory=dict)

    @property
    def ref_len(self) -> int:
        return len(self.genome) - 5

    def cells(self) -> float:
        """Algorithmic DP cells: sum over reads of samples x columns x 2 strands."""
        lens = np.diff(self.reads.offsets).astype(np.float64)
        return float(lens.sum() * self.ref_len * 2)


WORKLOADS = {
    "C1": dict(genome_len=48_502, n_reads=512, lengths=2000),
    "C2": dict(genome_len=1_000_000, n_reads=2048, lengths=2000),
    "C3": dict(genome_len=5_000_000, n_reads=8192, lengths=(1000, 8000)),
}


def make_workload(name: str, n_reads: int | None = None, genome_len: int | None = None,
                  table: np.ndarray | None = None, length=None) -> Workload:
    spec = dict(WORKLOADS[name])
    if n_reads is not None:
        spec["n_reads"] = n_reads
    if genome_len is not None:
        spec["genome_len"] = genome_len
    if length is not None:
        spec["lengths"] = length
    g = random_genome(spec["genome_len"], GENOME_SEED)
    o = random_genome(spec["genome_len"], OTHER_SEED)
    tab = level_table() if table is None else np.asarray(table, np.float32)
    n = spec["n_reads"]
    rng = np.random.default_rng(READ_SEED + 100)
    lens = spec["lengths"]
    if isinstance(lens, tuple):
        lengths = rng.integers(lens[0], lens[1] + 1, n)
    else:
        lengths = np.full(n, int(lens))
    mask = np.zeros(n, np.int8)
    mask[: n // 2] = 1
    rng.shuffle(mask)
    reads = simulate_reads(g, o, tab, lengths, mask)
    meta = dict(genome_len=spec["genome_len"], n_reads=n, seeds=dict(genome=GENOME_SEED, other=OTHER_SEED,
                table=TABLE_SEED, reads=READ_SEED), dwell_mean=DWELL_MEAN, noise_sd=NOISE_SD)
    return Workload(name, g, o, tab, reads, meta)
