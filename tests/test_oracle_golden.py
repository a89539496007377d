"""The CPU oracle pinned against the reference's own golden outputs.

scripts/log of the reference holds the FP64 DP trace of `sdtw_default`
(scripts/sdtw.py:205-225) for one 4096-sample lambda read against the
96,256-sample lambda reference (fwd||rev, each strand cut to R//2 = 48,128
k-mers, sdtw.py:101-116 and :234).  The oracle must reproduce every logged
cell, the final minimum and (derived) its column.
"""
import numpy as np
import pytest


def kat_reference(oracle, kat, builder="c"):
    seq = kat["seq"].tobytes()
    R = int(kat["ref_cols"])
    fn = oracle.build_levels if builder == "c" else oracle.np_build_levels
    f, r = fn(seq, kat["model_means"], cap=R // 2)
    return np.concatenate([f, r])


def test_kat_trace_every_logged_cell(oracle, kat):
    ref = kat_reference(oracle, kat)
    assert ref.size == int(kat["ref_cols"]) == 96256
    score, end, trace = oracle.sdtw(ref, kat["query"], trace_cols=kat["trace_cols"])
    # all 4096 rows x 6 columns; the log prints 16-17 significant digits and the
    # z-score sums differ from numpy's pairwise order only in the last bits
    np.testing.assert_allclose(trace, kat["trace"], rtol=1e-11, atol=0)
    assert abs(score - float(kat["min_score"])) <= 5e-8  # log prints 10 significant digits
    assert end == 33305


def test_kat_numpy_and_c_builders_agree(oracle, kat):
    a = kat_reference(oracle, kat, "c")
    b = kat_reference(oracle, kat, "np")
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-12)


def test_numpy_sdtw_matches_c_oracle(oracle):
    rng = np.random.default_rng(0)
    for m, n in [(1, 1), (1, 7), (7, 1), (33, 40), (257, 129)]:
        ref = rng.normal(size=m)
        q = rng.normal(size=n)
        s, j = oracle.sdtw(ref, q)
        s2, j2, _ = oracle.np_sdtw(ref, q)
        assert s == pytest.approx(s2, rel=1e-13)
        assert j == j2


def test_resume_from_row_equals_one_pass(oracle):
    """The row-state resume used by serving: aligning q1 then q2 from the saved
    row equals aligning q1||q2 in one pass."""
    rng = np.random.default_rng(1)
    ref = rng.normal(size=500)
    q = rng.normal(size=300)
    s, j, row = oracle.sdtw(ref, q[:120], want_row=True)
    s2, j2, _ = oracle.sdtw(ref, q[120:], init_row=row, want_row=True)
    s3, j3 = oracle.sdtw(ref, q)
    assert s2 == s3 and j2 == j3


def test_batch_matches_single(oracle):
    rng = np.random.default_rng(2)
    fwd = rng.normal(size=400)
    rev = rng.normal(size=400)
    reads = [rng.normal(size=n) for n in (5, 50, 120)]
    offs = np.concatenate([[0], np.cumsum([r.size for r in reads])])
    sf, ef, sr, er = oracle.sdtw_batch(fwd, rev, np.concatenate(reads), offs, n_threads=2)
    for i, q in enumerate(reads):
        assert oracle.sdtw(fwd, q) == (sf[i], ef[i])
        assert oracle.sdtw(rev, q) == (sr[i], er[i])


def test_zscore_eps_semantics(oracle):
    x = np.random.default_rng(3).normal(50, 7, 2048)
    np.testing.assert_allclose(oracle.zscore(x, 0.0), oracle.np_zscore(x, 0.0), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(oracle.zscore(x, 1e-4), oracle.np_zscore(x, 1e-4), rtol=1e-12, atol=1e-12)


def test_threshold_tuner_reproduces_reference_script(oracle, score_logs):
    """calc_classification_threshold.py run on the reference's mapped/unmapped
    FP16 logs gives 194.0076 at 97.6237 %; the restatement must agree."""
    th, acc = oracle.np_best_threshold(score_logs["target"], score_logs["other"])
    assert th == pytest.approx(float(score_logs["ref_threshold"]), rel=1e-12)
    assert acc == pytest.approx(float(score_logs["ref_accuracy"]), rel=1e-12)


def test_tie_rule(oracle):
    score, end, strand = oracle.combine([1.0, 2.0, 3.0, 3.0], [5, 5, 7, 2], [1.0, 1.0, 3.0, 3.0], [4, 9, 7, 9])
    assert list(score) == [1.0, 1.0, 3.0, 3.0]
    assert list(end) == [4, 9, 7, 2]
    assert list(strand) == [1, 1, 0, 0]
