"""Read Until serving at the size of the C4 simulation: six reads served in
1,600-sample chunks against the seeded 5 Mb genome (two 4,999,995-column DP
rows per read kept on the device between chunks), compared after every chunk
with the FP64 oracle resumed row by row.

The oracle's decisions are the committed fixture tests/golden/serving_c4.npz
(tests/golden/make_precision_fixtures.py --only c4: each chunk z-scored with
its own statistics, as the serving path does, and resumed from the previous
chunk's last row; the reference itself has no per-read resume,
src/ru_main.cu:172-326 re-aligns fixed windows).  Served with FP32 cells
(1e-5 relative, the same end column and strand), FP16 cells with FP32 row
state and FP16 cells with FP16 row state (1e-2; the end columns of target
reads within 2).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_util import sha
from test_gpu_serving import serve_reads, split
from dtwax_gb300 import synth

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(GOLDEN, "serving_c4.npz")
CHUNK, CHUNKS, TARGET, READ_SEED = 1600, [3, 3, 3, 3, 2, 1], [1, 0, 1, 0, 1, 0], 12


@pytest.fixture(scope="module")
def c4(built_lib, oracle):
    fx = dict(np.load(FIXTURE))
    g = synth.random_genome(5_000_000, synth.GENOME_SEED)
    o = synth.random_genome(5_000_000, synth.OTHER_SEED)
    tab = synth.level_table()
    reads = synth.simulate_reads(g, o, tab, [CHUNK * k for k in CHUNKS], TARGET, seed=READ_SEED)
    assert sha(reads.raw) == str(fx["raw_sha256"]), "the seeded generator gave other samples: regenerate the fixture"
    assert list(fx["chunks"]) == CHUNKS
    score, end, strand = oracle.combine(fx["score_fwd"], fx["end_fwd"], fx["score_rev"], fx["end_rev"])
    want = {}
    for k, i in enumerate(fx["read"]):
        want.setdefault(int(i), []).append((float(score[k]), int(end[k]), int(strand[k])))
    return g, tab, reads, want


@pytest.mark.parametrize("cells,state", [("fp32", "fp32"), ("fp16", "fp32"), ("fp16", "fp16")])
def test_c4_served_chunks_match_fp64(c4, cells, state):
    import dtwax_gb300 as d
    g, tab, reads, want = c4
    prec = d.FP32 if cells == "fp32" else d.FP16
    sp = d.STATE_FP16 if state == "fp16" else d.STATE_FP32
    with d.Classifier(sequence=g, level_table=tab, precision=prec, state_precision=sp,
                      threshold=-1.0) as clf:  # never early: every chunk is aligned
        chunks = {i: split(reads.read(i), CHUNK) for i in range(reads.n)}
        got = serve_reads(clf, chunks, chunks_per_decision=3, budget=4e9)
    rtol = 1e-5 if cells == "fp32" else 1e-2
    for i in range(reads.n):
        ds = got[i]
        assert [x["chunks"] for x in ds] == list(range(1, CHUNKS[i] + 1))
        assert ds[-1]["decided"] == 1
        for x, (s, e, st) in zip(ds, want[i]):
            assert x["score"] == pytest.approx(s, rel=rtol)
            if cells == "fp32":
                assert (x["end_pos"], x["strand"]) == (e, st)
            elif TARGET[i]:
                assert x["strand"] == st and abs(x["end_pos"] - e) <= 2
