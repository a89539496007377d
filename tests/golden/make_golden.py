"""Generate the golden fixtures in this folder from the reference checkout.

Run once, in a container that has the reference (harisankarsadasivan/DTWax)
checked out; the outputs are committed so the tests never need the reference
at run time:

    python tests/golden/make_golden.py /path/to/DTWax

Outputs
-------
lambda_kat.npz
    The known-answer test of scripts/log: the lambda phage genome exactly as
    scripts/sdtw.py:60-63 `get_fasta` reads src/ref/reference.fasta, the
    6-mer model src/ref/dna_kmer_model.txt (means and stdevs by 2-bit code),
    the 4096 normalised query samples the log prints, the FP64 DP values the
    log prints at columns {0, 1, 31, 32, R-2, R-1} of every row, and the
    final minimum the log prints (286.8895631).
score_logs.npz
    min(fwd, rev) per read of the reference FP16 GPU runs src/mapped.log
    (targets) and src/unmapped.log (non-targets), plus the threshold and
    accuracy that the reference's own src/ReadUntil/calc_classification_threshold.py
    prints for those two logs (it runs here: it needs numpy only).
find_threshold.npz
    The three output lines of the reference's src/test/find_threshold.py
    (numpy only) on the same two logs: in its FP32 mode on min(fwd, rev) score
    files, and in its FP16 mode on the .fwd / .rev score-file pairs.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def kmer_code(k: str) -> int:
    c = 0
    for ch in k:
        c = c * 4 + "ACGT".index(ch)
    return c


def main(ref_root: str) -> None:
    fasta_fn = os.path.join(ref_root, "src/ref/reference.fasta")
    model_fn = os.path.join(ref_root, "src/ref/dna_kmer_model.txt")
    log_fn = os.path.join(ref_root, "scripts/log")

    with open(fasta_fn) as f:
        text = f.read()
    header = text.split("\n")[0]
    seq = "".join(text.split("\n")[1:])  # sdtw.py:63

    means = np.zeros(4096, np.float64)
    stdevs = np.zeros(4096, np.float64)
    seen = np.zeros(4096, bool)
    with open(model_fn) as f:
        for line in f:
            k, mu, sd = line.split()
            c = kmer_code(k)
            means[c] = float(mu)
            stdevs[c] = float(sd)
            seen[c] = True
    assert seen.all()

    pat = re.compile(r"i= (\d+) query= (\S+) val\[0\]= (\S+) val\[1\]= (\S+) val\[31\]= (\S+) "
                     r"val\[32\]= (\S+) val\[R-2\]= (\S+) val\[R-1\]= (\S+)")
    rows = {}
    min_score = None
    with open(log_fn) as f:
        for line in f:
            m = pat.match(line)
            if m:
                i = int(m.group(1))
                rows[i] = [float(x) for x in m.groups()[1:]]
            elif line.startswith("min scores="):
                min_score = float(re.search(r"array\(([^)]+)\)", line).group(1))
    n = len(rows)
    assert n == 4096 and sorted(rows) == list(range(n))
    arr = np.array([rows[i] for i in range(n)], np.float64)
    R = 47 * 1024 * 2  # sdtw.py:51
    np.savez_compressed(
        os.path.join(HERE, "lambda_kat.npz"),
        fasta_header=np.array(header),
        seq=np.frombuffer(seq.encode(), np.uint8),
        model_means=means,
        model_stdevs=stdevs,
        query=arr[:, 0],
        trace=arr[:, 1:],
        trace_cols=np.array([0, 1, 31, 32, R - 2, R - 1], np.int64),
        ref_cols=np.int64(R),
        min_score=np.float64(min_score),
    )

    def mins(fn):
        out = []
        with open(fn) as f:
            for line in f:
                t = line.split()
                if t[0] == "Read_ID":
                    continue
                out.append(min(float(t[4]), float(t[5])))
        return np.array(out, np.float64)

    mapped = os.path.join(ref_root, "src/mapped.log")
    unmapped = os.path.join(ref_root, "src/unmapped.log")
    script = os.path.join(ref_root, "src/ReadUntil/calc_classification_threshold.py")
    out = subprocess.run([sys.executable, script, mapped, unmapped], check=True,
                         capture_output=True, text=True).stdout
    m = re.search(r"Best classification threshold: (\S+), accuracy: (\S+)", out)
    np.savez_compressed(
        os.path.join(HERE, "score_logs.npz"),
        target=mins(mapped),
        other=mins(unmapped),
        ref_threshold=np.float64(float(m.group(1))),
        ref_accuracy=np.float64(float(m.group(2))),
    )
    print("threshold", m.group(1), "accuracy", m.group(2), "min", min_score)
    find_threshold_golden(ref_root)


def log_columns(fn):
    """(fwd, rev) score columns of a 6-column log."""
    fwd, rev = [], []
    with open(fn) as f:
        for line in f:
            t = line.split()
            if t[0] == "Read_ID":
                continue
            fwd.append(float(t[4]))
            rev.append(float(t[5]))
    return np.array(fwd, np.float64), np.array(rev, np.float64)


def find_threshold_golden(ref_root: str) -> None:
    import tempfile
    script = os.path.join(ref_root, "src/test/find_threshold.py")
    tf, tr = log_columns(os.path.join(ref_root, "src/mapped.log"))
    of, orr = log_columns(os.path.join(ref_root, "src/unmapped.log"))
    rec = {}
    with tempfile.TemporaryDirectory() as tmp:
        def write(name, values):
            with open(os.path.join(tmp, name), "w") as f:
                f.write("".join(f"{float(v)!r}\n" for v in values))
        write("t32", np.minimum(tf, tr))
        write("o32", np.minimum(of, orr))
        write("t16.fwd", tf)
        write("t16.rev", tr)
        write("o16.fwd", of)
        write("o16.rev", orr)
        for bits, t, o in (("32", "t32", "o32"), ("16", "t16", "o16")):
            out = subprocess.run([sys.executable, script, bits, os.path.join(tmp, t), os.path.join(tmp, o)],
                                 check=True, capture_output=True, text=True, cwd=tmp).stdout
            vals = [float(x) for line in out.splitlines()[:3] for x in line.split()]
            rec[f"mode{bits}"] = np.array(vals, np.float64)  # min max, mean_t mean_o, kept discarded f1
    rec["target_fwd"], rec["target_rev"], rec["other_fwd"], rec["other_rev"] = tf, tr, of, orr
    np.savez_compressed(os.path.join(HERE, "find_threshold.npz"), **rec)
    print("find_threshold", rec["mode32"], rec["mode16"])


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DTWAX_REFERENCE")
    if not root:
        sys.exit("usage: make_golden.py <root of the reference project> (or set DTWAX_REFERENCE)")
    main(root)
