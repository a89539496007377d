"""Read Until serving at the sizes of the C4 and C5 simulations: reads served
in 1,600-sample chunks against the seeded 5 Mb genome (C4: two 4,999,995-column
DP rows per read kept on the device between chunks) and 12 Mb genome (C5: 96 MB
of FP32 row state per read), compared after every chunk with the FP64 oracle
resumed row by row.

The oracle's decisions are the committed fixtures tests/golden/serving_c4.npz
and serving_c5.npz (tests/golden/make_precision_fixtures.py --only c4 / c5:
each chunk z-scored with its own statistics, as the serving path does, and
resumed from the previous chunk's last row; the reference itself has no
per-read resume, src/ru_main.cu:172-326 re-aligns fixed windows).  Served with
FP32 cells (1e-5 relative, the same end column and strand), FP16 cells with
FP32 row state and FP16 cells with FP16 row state (1e-2; the end columns of
target reads within 2).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_util import sha
from test_gpu_serving import serve_reads, split
from dtwax_gb300 import synth

pytestmark = pytest.mark.gpu

CHUNK, READ_SEED = 1600, 12
SIZES = {"C4": (5_000_000, [3, 3, 3, 3, 2, 1], [1, 0, 1, 0, 1, 0]),
         "C5": (12_000_000, [3, 3, 2, 1], [1, 0, 1, 0])}


@pytest.fixture(scope="module", params=["C4", "C5"])
def served(request, built_lib, oracle):
    name = request.param
    genome_len, chunks, target = SIZES[name]
    fx = dict(np.load(os.path.join(GOLDEN, f"serving_{name.lower()}.npz")))
    g = synth.random_genome(genome_len, synth.GENOME_SEED)
    o = synth.random_genome(genome_len, synth.OTHER_SEED)
    tab = synth.level_table()
    reads = synth.simulate_reads(g, o, tab, [CHUNK * k for k in chunks], target, seed=READ_SEED)
    assert sha(reads.raw) == str(fx["raw_sha256"]), "the seeded generator gave other samples: regenerate the fixture"
    assert list(fx["chunks"]) == chunks
    score, end, strand = oracle.combine(fx["score_fwd"], fx["end_fwd"], fx["score_rev"], fx["end_rev"])
    want = {}
    for k, i in enumerate(fx["read"]):
        want.setdefault(int(i), []).append((float(score[k]), int(end[k]), int(strand[k])))
    return name, g, tab, reads, chunks, target, want


@pytest.mark.parametrize("cells,state", [("fp32", "fp32"), ("fp16", "fp32"), ("fp16", "fp16")])
def test_served_chunks_match_fp64(served, cells, state):
    import dtwax_gb300 as d
    name, g, tab, reads, nchunks, target, want = served
    prec = d.FP32 if cells == "fp32" else d.FP16
    sp = d.STATE_FP16 if state == "fp16" else d.STATE_FP32
    with d.Classifier(sequence=g, level_table=tab, precision=prec, state_precision=sp,
                      threshold=-1.0) as clf:  # never early: every chunk is aligned
        chunks = {i: split(reads.read(i), CHUNK) for i in range(reads.n)}
        got = serve_reads(clf, chunks, chunks_per_decision=3, budget=4e9)
    rtol = 1e-5 if cells == "fp32" else 1e-2
    for i in range(reads.n):
        ds = got[i]
        assert [x["chunks"] for x in ds] == list(range(1, nchunks[i] + 1))
        assert ds[-1]["decided"] == 1
        for x, (s, e, st) in zip(ds, want[i]):
            assert x["score"] == pytest.approx(s, rel=rtol), (name, i)
            if cells == "fp32":
                assert (x["end_pos"], x["strand"]) == (e, st)
            elif target[i]:
                assert x["strand"] == st and abs(x["end_pos"] - e) <= 2
