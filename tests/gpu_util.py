"""Helpers shared by the GPU tests: classifiers on small seeded genomes, the
oracle's answer for the same inputs, and the committed FP64 fixtures of the
full-size workloads."""
import hashlib
import os

import numpy as np

from dtwax_gb300 import synth


def small_genome(length=20_000, seed=11):
    return synth.random_genome(length, seed)


def make_classifier(genome, table=None, **cfg):
    import dtwax_gb300 as d
    if table is None:
        table = synth.level_table()
    return d.Classifier(sequence=genome, level_table=table, **cfg)


def oracle_reference(oracle, genome, table, cap=0):
    return oracle.build_levels(genome, np.asarray(table, np.float64), cap=cap)


def oracle_classify(oracle, clf, raw, offsets, eps=1e-4, query_len=0, skip=0):
    """Oracle on the classifier's own (GPU-built, FP32) reference and the
    oracle's FP64 z-score of each read window: (score_fwd, end_fwd, score_rev,
    end_rev) per read."""
    fwd, rev = clf.reference()
    qs = []
    offs = [0]
    for r in range(offsets.size - 1):
        x = raw[offsets[r] + skip: offsets[r + 1]].astype(np.float64)
        if query_len:
            x = x[:query_len]
        z = oracle.zscore(x, eps) if x.size else x
        # the GPU writes the z-scored window as float32
        qs.append(z.astype(np.float32).astype(np.float64))
        offs.append(offs[-1] + z.size)
    q = np.concatenate(qs) if qs else np.zeros(0)
    return oracle.sdtw_batch(fwd.astype(np.float64), rev.astype(np.float64), q, np.asarray(offs, np.int64))


def reads_of_lengths(genome, other, table, lengths, seed=5):
    mask = np.arange(len(lengths)) % 2 == 0
    return synth.simulate_reads(genome, other, table, lengths, mask.astype(np.int8), seed=seed)


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load_fixture(path, workload):
    """An FP64 fixture of tests/golden/make_precision_fixtures.py, after
    checking that the seeded generator gives the same samples here."""
    fx = dict(np.load(path))
    assert sha(workload.reads.raw) == str(fx["raw_sha256"]), (
        f"the seeded generator gave other samples here than where {os.path.basename(path)} was made "
        f"(numpy {np.__version__} here, {fx['numpy_version']} there): regenerate the fixture")
    return fx
