"""The committed FP64 fixtures of the full-size workloads (no GPU).

tests/golden/precision_c2.npz (all 2,048 C2 reads), uneven_c3.npz (48 of
the 8,192 C3 reads) and refdel_c2.npz (32 C2 reads, REF_DEL recurrence) hold
the oracle's scores and end columns for seeded inputs; the GPU parity tests compare the library with them.  Checked here:
the generator still gives the inputs the fixtures were made from (digests of
the samples and of the FP32-rounded levels), and the oracle recomputes the
stored answers of a few reads bit for bit.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from dtwax_gb300 import synth

FIXTURES = {"C2": "precision_c2.npz", "C3": "uneven_c3.npz", "C2R": "refdel_c2.npz"}


@pytest.mark.parametrize("name", ["C2", "C3", "C2R"])
def test_fixture_inputs_and_answers(oracle, name):
    import hashlib
    path = os.path.join(GOLDEN, FIXTURES[name])
    if name == "C2" and not os.path.exists(path):
        pytest.skip("precision_c2.npz not generated yet")
    fx = dict(np.load(path))
    w = synth.make_workload("C2" if name == "C2R" else name)

    def sha(a):
        return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()

    assert sha(w.reads.raw) == str(fx["raw_sha256"])
    fwd, rev = oracle.build_levels(w.genome, w.table.astype(np.float64))
    fwd32, rev32 = fwd.astype(np.float32), rev.astype(np.float32)
    assert sha(np.stack([fwd32, rev32])) == str(fx["levels_sha256"])
    assert int(fx["ref_columns"]) == fwd.size == w.ref_len
    lens = np.diff(w.reads.offsets)
    assert (fx["n_samples"] == lens[fx["read_index"]]).all()
    assert (fx["target"] == w.reads.target[fx["read_index"]]).all()
    # recompute the two shortest reads of the fixture
    pos = np.argsort(fx["n_samples"], kind="stable")[:2]
    qs = [oracle.zscore(w.reads.read(int(fx["read_index"][p])).astype(np.float64), 1e-4).astype(np.float32)
          for p in pos]
    offs = np.concatenate([[0], np.cumsum([q.size for q in qs])]).astype(np.int64)
    sf, ef, sr, er = oracle.sdtw_batch(fwd32.astype(np.float64), rev32.astype(np.float64),
                                       np.concatenate(qs).astype(np.float64), offs, ref_del=name == "C2R")
    np.testing.assert_array_equal(sf, fx["score_fwd"][pos])
    np.testing.assert_array_equal(sr, fx["score_rev"][pos])
    np.testing.assert_array_equal(ef, fx["end_fwd"][pos])
    np.testing.assert_array_equal(er, fx["end_rev"][pos])


@pytest.mark.parametrize("name,genome_len", [("c4", 5_000_000), ("c5", 12_000_000)])
def test_serving_fixture_inputs(oracle, name, genome_len):
    """tests/golden/serving_c4.npz and serving_c5.npz: the served reads and
    the genome's levels are still what the generator gives, and the fixture
    holds one decision per chunk of every read."""
    import hashlib
    fx = dict(np.load(os.path.join(GOLDEN, f"serving_{name}.npz")))
    chunks = [int(c) for c in fx["chunks"]]
    g = synth.random_genome(genome_len, synth.GENOME_SEED)
    o = synth.random_genome(genome_len, synth.OTHER_SEED)
    tab = synth.level_table()
    reads = synth.simulate_reads(g, o, tab, [1600 * k for k in chunks], fx["target"], seed=12)

    def sha(a):
        return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()

    assert sha(reads.raw) == str(fx["raw_sha256"])
    fwd, rev = oracle.build_levels(g, tab.astype(np.float64))
    assert sha(np.stack([fwd.astype(np.float32), rev.astype(np.float32)])) == str(fx["levels_sha256"])
    assert np.bincount(fx["read"]).tolist() == chunks
    assert (np.diff(fx["score_fwd"][fx["read"] == 0]) > 0).all()  # the path cost grows chunk by chunk
