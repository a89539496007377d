"""Precision study on the C2 generator (1 Mb genome): FP16 half2 cells with the
per-strip running-minimum offset, MIXED (FP16 differences, FP32 path cost) and
FP32 cells, each against the FP64 oracle.

Reported per precision: relative error of the best score (max, p99, median),
exact end-position agreement, and agreement of the call at the threshold the
FP64 scores give: the sweep of calc_classification_threshold.py, reported both
with the reference's choice of the first best threshold (on the edge of the
target scores when the classes separate) and with the centre of the
best-accuracy plateau.  Targets: FP16 within 1e-2 relative, FP32 within 1e-5,
MIXED within 1e-3, calls agree on >= 99.9 % of reads at the plateau centre.
The FP64 oracle runs on a 256-read sample (5.1e11 cells on the host cores).
Run with -s to see the table.
"""
import numpy as np
import pytest

from gpu_util import make_classifier, oracle_classify
from dtwax_gb300 import synth, threshold

pytestmark = pytest.mark.gpu

N_READS = 256


@pytest.fixture(scope="module")
def study(built_lib, oracle):
    w = synth.make_workload("C2", n_reads=N_READS)
    out = {}
    for name, prec in (("fp16", 0), ("mixed", 2), ("fp32", 1)):
        with make_classifier(w.genome, w.table, precision=prec) as clf:
            out[name] = clf.classify(raw=w.reads.raw, offsets=w.reads.offsets)
            if name == "fp32":
                ora = oracle_classify(oracle, clf, w.reads.raw, w.reads.offsets)
    sf, ef, sr, er = ora
    score, end, strand = oracle.combine(sf, ef, sr, er)
    t = w.reads.target == 1
    th, acc = threshold.best_threshold(score[t], score[~t])
    thc, _ = threshold.best_threshold(score[t], score[~t], plateau="center")
    return w, out, score, end, strand, (th, thc), acc


def summarize(res, score, end, strand, ths):
    th, thc = ths
    rel = np.abs(res["score"] - score) / np.maximum(score, 1e-12)
    return {
        "max_rel": float(rel.max()), "p99_rel": float(np.percentile(rel, 99)),
        "median_rel": float(np.median(rel)),
        "end_agree": float(((res["end_pos"] == end) & (res["strand"] == strand)).mean()),
        "end_within_2": float(((np.abs(res["end_pos"] - end) <= 2) & (res["strand"] == strand)).mean()),
        "call_agree": float((threshold.call(res["score"], th) == threshold.call(score, th)).mean()),
        "call_agree_center": float((threshold.call(res["score"], thc) == threshold.call(score, thc)).mean()),
    }


def test_precision_table(study, capsys):
    w, out, score, end, strand, th, acc = study
    rows = {k: summarize(v, score, end, strand, th) for k, v in out.items()}
    with capsys.disabled():
        print(f"\nC2 precision study, {N_READS} reads x 2000 samples vs 2 x 999,995 columns; FP64 "
              f"thresholds: first best {th[0]:.3f}, plateau centre {th[1]:.3f} ({acc:.2f} % accuracy)")
        print(f"{'cells':6s} {'max rel':>10s} {'p99 rel':>10s} {'median rel':>11s} {'end exact':>10s} "
              f"{'end +-2':>8s} {'call (first)':>13s} {'call (centre)':>14s}")
        for k, r in rows.items():
            print(f"{k:6s} {r['max_rel']:10.2e} {r['p99_rel']:10.2e} {r['median_rel']:11.2e} "
                  f"{r['end_agree']:10.4f} {r['end_within_2']:8.4f} {r['call_agree']:13.4f} "
                  f"{r['call_agree_center']:14.4f}")
    assert rows["fp32"]["max_rel"] <= 1e-5
    assert rows["fp16"]["max_rel"] <= 1e-2
    assert rows["mixed"]["max_rel"] <= 1e-3
    for k in ("fp16", "mixed", "fp32"):
        assert rows[k]["call_agree_center"] >= 0.999
    assert rows["fp32"]["call_agree"] >= 0.999
    assert rows["fp32"]["end_agree"] >= 0.999
