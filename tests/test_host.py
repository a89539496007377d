"""Host-side logic that needs no GPU: the C ABI library and its exports, the
FASTA / k-mer model parsers (reference rules), windows, the threshold tuner,
the synthetic generator."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, write_kat_files


def header_functions():
    text = open(os.path.join(ROOT, "include", "dtwx.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dtwx_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_header_symbol(built_lib):
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(built_lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "dtwax_gb300", "libdtwx.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (dtwx_\w+)", out))
    assert set(names) <= exported


def test_python_binding_covers_header(built_lib):
    import dtwax_gb300
    assert set(header_functions()) <= set(dtwax_gb300._SIGNATURES)


def test_config_default(built_lib):
    import dtwax_gb300 as d
    c = d.default_config()
    assert c.abi_version == 2 and c.precision == d.FP16 and c.strand_mode == d.STRANDS_PAIRED
    assert c.norm_eps == pytest.approx(1e-4)
    assert ctypes.sizeof(d.Config) == 96  # same static_assert in api.cpp


def test_config_combinations_are_checked(built_lib, kat, tmp_path):
    """Invalid precision / recurrence / row-state combinations are refused
    before any device work (code -1, DTWX_E_ARG), with or without a GPU."""
    import dtwax_gb300 as d
    fasta, model = write_kat_files(kat, str(tmp_path))
    c = d.default_config()
    assert c.recurrence == d.NO_REF_DEL and c.state_precision == d.STATE_FP32
    bad = [dict(precision=3), dict(recurrence=2), dict(state_precision=2),
           dict(precision=d.FP16, recurrence=d.REF_DEL, state_precision=d.STATE_FP16),
           dict(precision=d.MIXED, recurrence=d.REF_DEL),
           dict(precision=d.FP32, state_precision=d.STATE_FP16),
           dict(precision=d.FP32, recurrence=d.REF_DEL, cells_per_thread=48),
           # 16-warp CTAs only for the FP16-pair REF_DEL kernel (128 registers a thread)
           dict(precision=d.FP16, warps_per_cta=16), dict(precision=d.FP32, recurrence=d.REF_DEL, warps_per_cta=16),
           dict(precision=d.FP16, recurrence=d.REF_DEL, warps_per_cta=17), dict(warps_per_cta=-1)]
    for kw in bad:
        with pytest.raises(d.DtwxError) as e:
            d.Classifier(fasta=fasta, kmer_model=model, **kw)
        assert e.value.code == -1, kw


def test_create_without_gpu_fails_loudly(built_lib, tmp_path, kat):
    """No CPU fallback: on a machine without a GPU creation must fail."""
    import dtwax_gb300 as d
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    fasta, model = write_kat_files(kat, str(tmp_path))
    with pytest.raises(d.DtwxError) as e:
        d.Classifier(fasta=fasta, kmer_model=model)
    assert e.value.code == -4


def test_fasta_and_model_roundtrip(built_lib, tmp_path, kat):
    import dtwax_gb300 as d
    fasta, model = write_kat_files(kat, str(tmp_path))
    assert d.load_fasta(fasta) == kat["seq"].tobytes()
    t = d.load_kmer_model(model)
    np.testing.assert_allclose(t, kat["model_means"].astype(np.float32), rtol=0, atol=0)


@pytest.mark.parametrize("text,expect", [
    (">a\nACGTAC\nGGT\n", b"ACGTACGGT"),              # multi-line record
    (">a\nAAAAAAA\n>b\nCCCCCCC\n", b"CCCCCCC"),       # last record wins
    (">a\nAAAAAAA\n>b\nCC CCCC\nGGGGGGG\n", None),    # space invalidates the open record
    (">a\nAAAAAAA\n\n", None),                       # empty line closes it: nothing open at EOF
    (">a\r\nACGTACG\r\n", b"ACGTACG"),               # CRLF line ends
    ("ACGTACGT\n", None),                            # no header
    (">a\nACG\n", None),                              # shorter than one 6-mer
])
def test_fasta_rules(built_lib, tmp_path, text, expect):
    import dtwax_gb300 as d
    p = tmp_path / "x.fa"
    p.write_text(text)
    if expect is None:
        with pytest.raises(d.DtwxError):
            d.load_fasta(str(p))
    else:
        assert d.load_fasta(str(p)) == expect


def test_kmer_model_errors(built_lib, tmp_path):
    import dtwax_gb300 as d
    p = tmp_path / "m.txt"
    p.write_text("AAAAAA 80.0 1.0\n")
    with pytest.raises(d.DtwxError):
        d.load_kmer_model(str(p))      # 4095 k-mers missing
    p.write_text("AAAAXA 80.0 1.0\n")
    with pytest.raises(d.DtwxError):
        d.load_kmer_model(str(p))


def test_threshold_tuner_on_reference_logs(score_logs):
    from dtwax_gb300 import threshold
    th, acc = threshold.best_threshold(score_logs["target"], score_logs["other"])
    assert th == pytest.approx(float(score_logs["ref_threshold"]), rel=1e-12)
    assert acc == pytest.approx(float(score_logs["ref_accuracy"]), rel=1e-12)


def test_parse_log_reads_the_side_file():
    from dtwax_gb300 import threshold
    side = "0\tr0\t12.5\t100\t+\ttarget\n1\tr1\t300.25\t7\t-\tnon-target\n2\tr2\tinf\t-1\t+\tskipped\n"
    np.testing.assert_array_equal(threshold.parse_log(side), [12.5, 300.25])
    log = "Read_ID\tQUERY_LEN\tREF_LEN\tfwd\trev\n0\tr0\t2048\t100\t5.5\t4.25\n"
    np.testing.assert_array_equal(threshold.parse_log(log), [4.25])


def test_threshold_command_line(score_logs, tmp_path):
    """`python -m dtwax_gb300.threshold <target_log> <other_log>` prints what
    calc_classification_threshold.py prints for the same logs."""
    import subprocess
    import sys

    def write(path, scores):
        with open(path, "w") as f:
            f.write("Read_ID\tQUERY_LEN\tREF_LEN\tsDTW score: fwd-strand\tsDTW score: rev-strand\n")
            for i, v in enumerate(scores):
                f.write(f"{i}\tr{i}\t2048\t48128\t{float(v)!r}\t{float(v) + 1.0!r}\n")

    write(tmp_path / "t.log", score_logs["target"])
    write(tmp_path / "o.log", score_logs["other"])
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-m", "dtwax_gb300.threshold", str(tmp_path / "t.log"),
                          str(tmp_path / "o.log")], capture_output=True, text=True, check=True, cwd=root).stdout
    lines = out.splitlines()
    assert lines[0] == str(len(score_logs["target"])) and lines[1] == str(len(score_logs["other"]))
    th = float(lines[2].split("threshold: ")[1].split(",")[0])
    acc = float(lines[2].split("accuracy: ")[1])
    assert th == pytest.approx(float(score_logs["ref_threshold"]), rel=1e-12)
    assert acc == pytest.approx(float(score_logs["ref_accuracy"]), rel=1e-12)


def test_parse_log_roundtrip(built_lib):
    import dtwax_gb300 as d
    from dtwax_gb300 import threshold
    res = np.zeros(3, d.RESULT_DTYPE)
    res["score_fwd"] = [171.125, 120.5625, 300.0]
    res["score_rev"] = [292.5, 283.75, 250.25]
    res["n_samples"] = 2048
    text = d.format_log(res, ["r0", "r1", "r2"], 48128)
    lines = text.splitlines()
    assert lines[0].split("\t")[0] == "Read_ID"
    assert all(len(l.split()) == 6 for l in lines[1:])  # plot_realtime.py:39 needs 6 tokens
    np.testing.assert_allclose(threshold.parse_log(text), [171.125, 120.562, 250.25], rtol=1e-5)


def test_synthetic_generator_is_seeded():
    from dtwax_gb300 import synth
    a = synth.make_workload("C1", n_reads=8)
    b = synth.make_workload("C1", n_reads=8)
    np.testing.assert_array_equal(a.reads.raw, b.reads.raw)
    assert a.genome == b.genome and len(a.genome) == 48502
    assert a.ref_len == 48497
    assert a.reads.target.sum() == 4
    lens = np.diff(a.reads.offsets)
    assert (lens == 2000).all()
    # dwell model: mean samples per k-mer close to 9
    assert 7.5 < 2000 / a.reads.kmers.mean() < 10.5


def test_shard_assignment():
    from dtwax_gb300.shard import shard_range
    n = 2049
    parts = [shard_range(n, r, 4) for r in range(4)]
    assert parts[0][0] == 0 and parts[-1][1] == n
    assert all(parts[i][1] == parts[i + 1][0] for i in range(3))
    assert max(b - a for a, b in parts) - min(b - a for a, b in parts) <= 1


def test_f1_threshold_matches_find_threshold_py():
    """The F1 sweep against the output lines of the reference's
    src/test/find_threshold.py on the reference's FP16 logs (fixture made by
    tests/golden/make_golden.py)."""
    from dtwax_gb300 import threshold
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "find_threshold.npz"))
    r = threshold.f1_threshold(np.minimum(g["target_fwd"], g["target_rev"]),
                               np.minimum(g["other_fwd"], g["other_rev"]))
    got = [r["min"], r["max"], r["mean_target"], r["mean_other"], r["target_kept"], r["other_discarded"], r["f1"]]
    np.testing.assert_allclose(got, g["mode32"], rtol=1e-12)
    assert r["min"] < r["threshold"] < r["max"]


@pytest.mark.parametrize("bits", ["32", "16"])
def test_f1_command_line(tmp_path, bits):
    """`python -m dtwax_gb300.threshold f1 <32|16> <target> <other>` prints
    find_threshold.py's three lines (FP32 score files, or .fwd/.rev pairs)."""
    import subprocess
    import sys
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "find_threshold.npz"))

    def write(path, values):
        path.write_text("".join(f"{float(v)!r}\n" for v in values))

    if bits == "32":
        write(tmp_path / "t", np.minimum(g["target_fwd"], g["target_rev"]))
        write(tmp_path / "o", np.minimum(g["other_fwd"], g["other_rev"]))
    else:
        for name, key in (("t", "target"), ("o", "other")):
            write(tmp_path / f"{name}.fwd", g[f"{key}_fwd"])
            write(tmp_path / f"{name}.rev", g[f"{key}_rev"])
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-m", "dtwax_gb300.threshold", "f1", bits, str(tmp_path / "t"),
                          str(tmp_path / "o")], capture_output=True, text=True, check=True, cwd=root).stdout
    vals = [float(x) for line in out.splitlines()[:3] for x in line.split()]
    np.testing.assert_allclose(vals, g[f"mode{bits}"], rtol=1e-12)
