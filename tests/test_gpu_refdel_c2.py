"""The REF_DEL recurrence at the C2 size: the 2,048-read batch against the
seeded 1 Mb genome (977 strips of 1,024 columns per read), compared on its
first 32 reads with the FP64 REF_DEL oracle.

The FP16-pair kernel hands values between per-lane frames 31 times per row
in every strip, so a long genome is where its rounding could add up.  The
FP64 answers (the oracle's REF_DEL recurrence, src/include/DTW.cu:23-29
without -DNO_REF_DEL) are the committed fixture tests/golden/refdel_c2.npz
(tests/golden/make_precision_fixtures.py --only c2r).  FP32 cells within 1e-5
with exact end columns; FP16 pairs within 1e-2 with the end columns of target
reads within 2.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_util import load_fixture, sha
from dtwax_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2r(built_lib, oracle):
    w = synth.make_workload("C2")
    fx = load_fixture(os.path.join(GOLDEN, "refdel_c2.npz"), w)
    fwd, rev = oracle.build_levels(w.genome, w.table.astype(np.float64))
    assert sha(np.stack([fwd.astype(np.float32), rev.astype(np.float32)])) == str(fx["levels_sha256"])
    score, end, strand = oracle.combine(fx["score_fwd"], fx["end_fwd"], fx["score_rev"], fx["end_rev"])
    return w, fx, end, strand


@pytest.mark.parametrize("cells", ["fp16", "fp32"])
def test_ref_del_batch_matches_fp64(c2r, cells, capsys):
    import dtwax_gb300 as d
    w, fx, end, strand = c2r
    prec = d.FP16 if cells == "fp16" else d.FP32
    with d.Classifier(sequence=w.genome, level_table=w.table, precision=prec, recurrence=d.REF_DEL) as clf:
        res = clf.classify(raw=w.reads.raw, offsets=w.reads.offsets)  # the whole 2,048-read batch
        tuning = clf.tuning()
    idx = fx["read_index"]
    got = res[idx]
    rel = np.maximum(np.abs(got["score_fwd"] - fx["score_fwd"]) / fx["score_fwd"],
                     np.abs(got["score_rev"] - fx["score_rev"]) / fx["score_rev"])
    with capsys.disabled():
        print(f"\nREF_DEL {cells}, {w.reads.n} reads vs 2 x {w.ref_len:,} columns ({tuning}): "
              f"max rel {rel.max():.2e} on {idx.size} reads")
    if cells == "fp32":
        assert rel.max() <= 1e-5
        np.testing.assert_array_equal(got["end_pos"], end)
        np.testing.assert_array_equal(got["strand"], strand)
    else:
        assert rel.max() <= 1e-2
        t = fx["target"] == 1
        assert ((np.abs(got["end_pos"] - end) <= 2) & (got["strand"] == strand))[t].all()
