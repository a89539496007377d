"""Threshold tuning and the score log, as the reference's Python tools use them.

* ``parse_log`` reads the 6-column log of the CLI (src/main.cu:289-297) the way
  src/ReadUntil/calc_classification_threshold.py:5-33 does: header lines
  (first token "Read_ID") are skipped and a read's score is min(fwd, rev).  It
  also reads the CLI's extended side file (idx, read id, score, end column,
  strand, call), whose fifth token is the strand sign; skipped reads are left
  out.
* ``best_threshold`` is the sweep of calc_classification_threshold.py:49-57:
  100,000 thresholds in linspace(0, max score); a target read is correct when
  its score < t, a non-target read when its score >= t; the first threshold of
  maximal accuracy wins.
* ``call`` is the online decision of src/ReadUntil/plot_realtime.py:42-43
  (score > t -> non-target; the offline tuner counts score == t as
  non-target, which is the rule used here).
* ``best_f1_threshold`` is the F1-optimal variant of src/test/find_threshold.py.
"""
from __future__ import annotations

import numpy as np


def parse_log(text_or_lines) -> np.ndarray:
    lines = text_or_lines.splitlines() if isinstance(text_or_lines, str) else list(text_or_lines)
    scores = []
    for line in lines:
        t = line.split()
        if not t or t[0] == "Read_ID":
            continue
        if t[4] in ("+", "-"):  # extended side file
            if t[5] != "skipped":
                scores.append(float(t[2]))
            continue
        scores.append(min(float(t[4]), float(t[5])))
    return np.asarray(scores, np.float64)


def best_threshold(target_scores, other_scores, num: int = 100000, plateau: str = "first"):
    """(threshold, accuracy %) maximising (#target < t + #other >= t) / total.

    plateau="first" keeps the reference's choice (the first threshold of
    maximal accuracy, which sits on the edge of the target scores when the
    classes separate); plateau="center" takes the middle of the run of
    maximal-accuracy thresholds that contains the first one, which leaves the
    same margin to both classes."""
    t_s = np.asarray(target_scores, np.float64)
    o_s = np.asarray(other_scores, np.float64)
    if t_s.size + o_s.size == 0:
        raise ValueError("no scores")
    hi = max(t_s.max() if t_s.size else 0.0, o_s.max() if o_s.size else 0.0)
    th = np.linspace(0, hi, num=num)
    ts = np.sort(t_s)
    os_ = np.sort(o_s)
    correct = np.searchsorted(ts, th, side="left") + (os_.size - np.searchsorted(os_, th, side="left"))
    acc = correct * 100.0 / (t_s.size + o_s.size)
    k = int(np.argmax(acc))
    if plateau == "center":
        e = k
        while e + 1 < acc.size and acc[e + 1] == acc[k]:
            e += 1
        return float(0.5 * (th[k] + th[e])), float(acc[k])
    return float(th[k]), float(acc[k])


def best_f1_threshold(target_scores, other_scores, num: int = 100000):
    """(threshold, F1) with targets as the positive class (score < t)."""
    t_s = np.sort(np.asarray(target_scores, np.float64))
    o_s = np.sort(np.asarray(other_scores, np.float64))
    hi = max(t_s.max(), o_s.max())
    th = np.linspace(0, hi, num=num)
    tp = np.searchsorted(t_s, th, side="left").astype(np.float64)
    fp = np.searchsorted(o_s, th, side="left").astype(np.float64)
    fn = t_s.size - tp
    f1 = np.where(tp > 0, 2 * tp / np.maximum(2 * tp + fp + fn, 1), 0.0)
    k = int(np.argmax(f1))
    return float(th[k]), float(f1[k])


def call(scores, threshold: float) -> np.ndarray:
    """1 = target (score < threshold), 0 = non-target."""
    return (np.asarray(scores) < threshold).astype(np.int8)


def main(argv=None) -> int:
    """`python -m dtwax_gb300.threshold <target_log> <other_log> [--plateau center]`:
    the command line of calc_classification_threshold.py (microbial = target
    log, human = other log), with the same three output lines."""
    import argparse
    ap = argparse.ArgumentParser(description="Calculate DTW classification accuracy thresholds")
    ap.add_argument("microbial_file", help="path to the target (microbial) classification log")
    ap.add_argument("human_file", help="path to the non-target (human) classification log")
    ap.add_argument("--plateau", choices=["first", "center"], default="first",
                    help="first: the reference's choice; center: the middle of the best-accuracy run")
    args = ap.parse_args(argv)
    with open(args.human_file) as f:
        human = parse_log(f.read())
    with open(args.microbial_file) as f:
        microbial = parse_log(f.read())
    print(len(microbial))
    print(len(human))
    th, acc = best_threshold(microbial, human, plateau=args.plateau)
    print(f"Best classification threshold: {th}, accuracy: {acc}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
