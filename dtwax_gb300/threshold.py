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
* ``f1_threshold`` is the F1 sweep of src/test/find_threshold.py:60-81:
  1,000 thresholds in linspace(min - 1, max + 1) over both classes; a read is
  kept when its score <= t; rates are counted against the non-zero scores of
  each class (np.count_nonzero); F1 = TPR / (TPR + (FNR + FPR) / 2) with
  those rates; the first maximum wins.  ``f1_main`` is that script's command
  line (``<32|16> <target> <other>``: FP32 score files, or FP16 .fwd/.rev
  pairs whose per-read minimum is taken); it also reads the CLI's logs.
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


def f1_threshold(target_scores, other_scores, num: int = 1000) -> dict:
    """find_threshold.py's sweep.  Returns the best threshold with the rates
    the script prints: the fraction of targets kept (score <= t), the
    fraction of others discarded (score > t) and F1; plus the sweep's range
    and the class means (its first two output lines)."""
    t_s = np.asarray(target_scores, np.float64)
    o_s = np.asarray(other_scores, np.float64)
    if t_s.size == 0 or o_s.size == 0:
        raise ValueError("both classes need scores")
    lo = min(t_s.min(), o_s.min()) - 1
    hi = max(t_s.max(), o_s.max()) + 1
    th = np.linspace(lo, hi, num=num)
    ts, os_ = np.sort(t_s), np.sort(o_s)
    # fraction discarded (score > t), over the non-zero scores of the class
    vd = (ts.size - np.searchsorted(ts, th, side="right")) / np.count_nonzero(t_s)
    od = (os_.size - np.searchsorted(os_, th, side="right")) / np.count_nonzero(o_s)
    f1 = (1 - vd) / ((1 - vd) + 0.5 * (1 + vd - od))
    k = int(np.argmax(f1))
    return {"threshold": float(th[k]), "target_kept": float(1 - vd[k]), "other_discarded": float(od[k]),
            "f1": float(f1[k]), "min": float(lo), "max": float(hi), "mean_target": float(t_s.mean()),
            "mean_other": float(o_s.mean())}


def _read_scores(path: str) -> np.ndarray:
    """One score per line (find_threshold.py's input), or a CLI log."""
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    if lines and (len(lines[0].split()) >= 6 or lines[0].split()[0] == "Read_ID"):
        return parse_log(lines)
    return np.asarray([float(ln.strip()) for ln in lines], np.float64)


def f1_main(argv=None) -> int:
    """`python -m dtwax_gb300.threshold f1 <32|16> <target> <other>`: the
    command line and output lines of src/test/find_threshold.py.  With 16 the
    scores come from <name>.fwd and <name>.rev and a read's score is their
    minimum; CLI logs (6-column or extended) are read directly."""
    import sys
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 3:
        print("usage: f1 <32|16> <target> <other>")
        return 2
    bits, tf, of = int(argv[0]), argv[1], argv[2]
    if bits == 32:
        t_s, o_s = _read_scores(tf), _read_scores(of)
    else:
        t_s = np.minimum(_read_scores(tf + ".fwd"), _read_scores(tf + ".rev"))
        o_s = np.minimum(_read_scores(of + ".fwd"), _read_scores(of + ".rev"))
    r = f1_threshold(t_s, o_s)
    print(r["min"], r["max"])
    print(r["mean_target"], r["mean_other"])
    print(r["target_kept"], r["other_discarded"], r["f1"])
    return 0


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
    import sys
    if len(sys.argv) > 1 and sys.argv[1] == "f1":
        raise SystemExit(f1_main(sys.argv[2:]))
    raise SystemExit(main())
