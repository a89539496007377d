"""FP64-oracle parity on the batched uneven-read workload (C3): 8,192 reads of
U[1000, 8000] samples against the seeded 5 Mb genome (2 x 4,999,995 columns).

The FP16 path runs the whole 8,192-read batch in one persistent launch with
the autotuned shape, as the benchmark does, and the FP32 and MIXED paths run
the sampled reads; 48 of the reads (the shortest, the longest and 46 drawn
with a fixed seed) are compared with the FP64 oracle's scores and end
columns, committed as tests/golden/uneven_c3.npz by
tests/golden/make_precision_fixtures.py (the oracle's restatement of
scripts/sdtw.py:86-116,205-225; the reference's batch loop over every read is
src/main.cu:217-271).  Reads of up to 8,000 rows are where the FP16 cells'
running-minimum offset has to hold the most range.

Tolerances: FP32 1e-5 relative with exact end columns, MIXED 1e-3, FP16 1e-2
with the end columns of target reads within 2.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from dtwax_gb300 import synth
from gpu_util import load_fixture, sha

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(GOLDEN, "uneven_c3.npz")


@pytest.fixture(scope="module")
def c3(built_lib, oracle):
    w = synth.make_workload("C3")
    fx = load_fixture(FIXTURE, w)
    fwd, rev = oracle.build_levels(w.genome, w.table.astype(np.float64))
    assert sha(np.stack([fwd.astype(np.float32), rev.astype(np.float32)])) == str(fx["levels_sha256"])
    score, end, strand = oracle.combine(fx["score_fwd"], fx["end_fwd"], fx["score_rev"], fx["end_rev"])
    return w, fx, score, end, strand


def _sample(w, idx):
    reads = [w.reads.read(int(i)) for i in idx]
    offsets = np.concatenate([[0], np.cumsum([r.size for r in reads])]).astype(np.int64)
    return np.concatenate(reads), offsets


def _rel(a, b):
    return np.abs(a - b) / np.maximum(b, 1e-12)


def test_c3_fp16_full_batch_matches_fp64(c3, capsys):
    import dtwax_gb300 as d
    w, fx, score, end, strand = c3
    idx = fx["read_index"]
    lens = np.diff(w.reads.offsets)
    with d.Classifier(sequence=w.genome, level_table=w.table, precision=d.FP16) as clf:
        clf.autotune(w.reads.n, int(lens.mean()))
        res = clf.classify(raw=w.reads.raw, offsets=w.reads.offsets)  # all 8,192 reads, one launch
        tuning = clf.tuning()
    assert (res["call"] >= 0).all() and (res["n_samples"] == lens).all()
    got = res[idx]
    rel = np.maximum(_rel(got["score_fwd"], fx["score_fwd"]), _rel(got["score_rev"], fx["score_rev"]))
    t = fx["target"] == 1
    end_ok = (np.abs(got["end_pos"] - end) <= 2) & (got["strand"] == strand)
    with capsys.disabled():
        print(f"\nC3 FP16, {w.reads.n} reads in one launch ({tuning}); {idx.size} sampled reads of "
              f"{int(fx['n_samples'].min())}..{int(fx['n_samples'].max())} samples vs FP64: max rel {rel.max():.2e}, "
              f"end exact {float(((got['end_pos'] == end) & (got['strand'] == strand)).mean()):.3f}, "
              f"target ends within 2 {float(end_ok[t].mean()):.3f}")
    assert rel.max() <= 1e-2
    assert end_ok[t].all()


@pytest.mark.parametrize("name,rtol", [("fp32", 1e-5), ("mixed", 1e-3)])
def test_c3_sample_matches_fp64(c3, name, rtol):
    import dtwax_gb300 as d
    w, fx, score, end, strand = c3
    raw, offsets = _sample(w, fx["read_index"])
    prec = {"fp32": d.FP32, "mixed": d.MIXED}[name]
    with d.Classifier(sequence=w.genome, level_table=w.table, precision=prec) as clf:
        got = clf.classify(raw=raw, offsets=offsets)
    rel = np.maximum(_rel(got["score_fwd"], fx["score_fwd"]), _rel(got["score_rev"], fx["score_rev"]))
    assert rel.max() <= rtol, rel.max()
    if name == "fp32":
        np.testing.assert_array_equal(got["end_pos"], end)
        np.testing.assert_array_equal(got["strand"], strand)
