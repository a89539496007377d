"""Parity of the CUDA path with the FP64 oracle, through the C ABI.

Tolerances (the precision targets): FP32 scores within 1e-5 relative
of the FP64 oracle with the same end column; FP16 (half2 cells with the
per-strip running-minimum offset) within 1e-2 relative.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, write_kat_files
from gpu_util import make_classifier, oracle_classify, reads_of_lengths, small_genome
from dtwax_gb300 import synth

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5
FP16_RTOL = 1e-2
MIXED_RTOL = 1e-3  # FP16 differences, FP32 path cost


@pytest.fixture(scope="module")
def lib(built_lib):
    return built_lib


@pytest.fixture(scope="module")
def genome_pair():
    return small_genome(20_000, 11), small_genome(20_000, 12)


def check_fp32(res, ora, rtol=FP32_RTOL, ends=True):
    sf, ef, sr, er = ora
    np.testing.assert_allclose(res["score_fwd"], sf, rtol=rtol)
    np.testing.assert_allclose(res["score_rev"], sr, rtol=rtol)
    if ends:
        ok = res["n_samples"] > 0
        # end columns must match except where the oracle itself has a near tie
        mism = ok & ((res["strand"] == 0) & (res["end_pos"] != ef) | (res["strand"] == 1) & (res["end_pos"] != er))
        assert mism.sum() == 0, np.nonzero(mism)


def test_reference_builder_matches_oracle(lib, oracle):
    g = small_genome(30_011, 3)
    tab = synth.level_table()
    with make_classifier(g, tab, precision=1) as clf:
        fwd, rev = clf.reference()
    of, orv = oracle.build_levels(g, tab.astype(np.float64))
    assert fwd.size == len(g) - 5
    np.testing.assert_allclose(fwd, of, rtol=0, atol=2e-6)
    np.testing.assert_allclose(rev, orv, rtol=0, atol=2e-6)


def test_reference_builder_nonacgt_and_cap(lib, oracle):
    g = bytearray(small_genome(5_000, 4))
    g[100:103] = b"NNN"
    g[2000] = ord("a")
    g = bytes(g)
    tab = synth.level_table()
    with make_classifier(g, tab, precision=1, max_ref_len=3000) as clf:
        fwd, rev = clf.reference()
    of, orv = oracle.build_levels(g, tab.astype(np.float64), cap=3000)
    assert fwd.size == 3000
    np.testing.assert_allclose(fwd, of, atol=2e-6)
    np.testing.assert_allclose(rev, orv, atol=2e-6)


@pytest.mark.parametrize("precision,rtol", [(1, FP32_RTOL), (0, FP16_RTOL), (2, MIXED_RTOL)])
def test_kat_lambda_on_gpu(lib, kat, tmp_path, precision, rtol):
    """scripts/log on the GPU: the 4096 golden query samples against the
    lambda fwd||rev reference cut to 48,128 k-mers per strand."""
    import torch
    import dtwax_gb300 as d
    fasta, model = write_kat_files(kat, str(tmp_path))
    with d.Classifier(fasta=fasta, kmer_model=model, precision=precision, strand_mode=d.STRANDS_CONCAT,
                      max_ref_len=48128) as clf:
        q = torch.tensor(kat["query"].astype(np.float32), device="cuda")
        out = torch.zeros(32, dtype=torch.uint8, device="cuda")
        clf.distances(q.data_ptr(), np.array([0, q.numel()]), out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        res = np.frombuffer(out.cpu().numpy().tobytes(), d.RESULT_DTYPE)
    assert res["score"][0] == pytest.approx(float(kat["min_score"]), rel=rtol)
    if precision == 1:
        assert res["end_pos"][0] == 33305 and res["strand"][0] == 0


@pytest.mark.parametrize("precision", [1, 0, 2])
def test_classify_matches_oracle(lib, oracle, genome_pair, precision):
    g, o = genome_pair
    tab = synth.level_table()
    lengths = [2000, 1, 2, 31, 32, 33, 63, 64, 65, 100, 500, 1023, 1024, 1025, 1500, 2000, 2047, 2049, 3000, 777]
    reads = reads_of_lengths(g, o, tab, lengths)
    with make_classifier(g, tab, precision=precision) as clf:
        res = clf.classify(raw=reads.raw, offsets=reads.offsets)
        ora = oracle_classify(oracle, clf, reads.raw, reads.offsets)
    assert (res["n_samples"] == np.array(lengths)).all()
    if precision == 1:
        check_fp32(res, ora)
    else:
        sf, ef, sr, er = ora
        rtol = FP16_RTOL if precision == 0 else MIXED_RTOL
        np.testing.assert_allclose(res["score_fwd"], sf, rtol=rtol, atol=1e-2)
        np.testing.assert_allclose(res["score_rev"], sr, rtol=rtol, atol=1e-2)
        # targets (even indices, >= 500 samples) must end where the oracle ends
        for i, n in enumerate(lengths):
            if i % 2 == 0 and n >= 500:
                best_end = ef[i] if sf[i] <= sr[i] else er[i]
                assert abs(int(res["end_pos"][i]) - int(best_end)) <= 1


@pytest.mark.parametrize("cells,warps", [(16, 4), (32, 4), (32, 8), (16, 1)])
def test_ref_del_matches_oracle(lib, oracle, genome_pair, cells, warps):
    """The REF_DEL recurrence (left predecessor, DTW.cu:23-29) in FP32 cells
    against the FP64 oracle, on reads of window-edge lengths."""
    import dtwax_gb300 as d
    g, o = genome_pair
    tab = synth.level_table()
    lengths = [2000, 1, 2, 31, 32, 33, 1023, 1024, 1025, 2047, 2049, 3000, 500, 777]
    reads = reads_of_lengths(g, o, tab, lengths)
    with make_classifier(g, tab, precision=d.FP32, recurrence=d.REF_DEL, cells_per_thread=cells,
                         warps_per_cta=warps) as clf:
        res = clf.classify(raw=reads.raw, offsets=reads.offsets)
        t = clf.tuning()
        fwd, rev = clf.reference()
    assert t["cells_per_thread"] == cells and t["work_items"] == 2 * len(lengths)  # one chunk per read strand
    qs, offs = [], [0]
    for r in range(reads.n):
        z = oracle.zscore(reads.read(r).astype(np.float64), 1e-4).astype(np.float32).astype(np.float64)
        qs.append(z)
        offs.append(offs[-1] + z.size)
    ora = oracle.sdtw_batch(fwd.astype(np.float64), rev.astype(np.float64), np.concatenate(qs),
                            np.array(offs, np.int64), ref_del=True)
    check_fp32(res, ora)
    # the left term matters on these reads: NO_REF_DEL scores differ
    plain = oracle.sdtw_batch(fwd.astype(np.float64), rev.astype(np.float64), np.concatenate(qs),
                              np.array(offs, np.int64))
    assert (plain[0] > ora[0]).any()


def test_ref_del_fp16_matches_oracle(lib, oracle, genome_pair):
    """REF_DEL on FP16 pairs with the running-minimum frames: within the FP16
    tolerance of the FP64 REF_DEL oracle, end columns of target reads within 2."""
    import dtwax_gb300 as d
    g, o = genome_pair
    tab = synth.level_table()
    lengths = [2000, 1, 31, 32, 33, 1023, 1024, 1025, 2047, 2049, 3000, 500, 777, 64]
    reads = reads_of_lengths(g, o, tab, lengths)
    with make_classifier(g, tab, precision=d.FP16, recurrence=d.REF_DEL) as clf:
        res = clf.classify(raw=reads.raw, offsets=reads.offsets)
        assert clf.tuning()["work_items"] == len(lengths)  # one item per read (both strands)
    with make_classifier(g, tab, precision=d.FP32) as clf32:
        fwd, rev = clf32.reference()
    qs, offs = [], [0]
    for r in range(reads.n):
        z = oracle.zscore(reads.read(r).astype(np.float64), 1e-4).astype(np.float32).astype(np.float64)
        qs.append(z)
        offs.append(offs[-1] + z.size)
    sf, ef, sr, er = oracle.sdtw_batch(fwd.astype(np.float64), rev.astype(np.float64), np.concatenate(qs),
                                       np.array(offs, np.int64), ref_del=True)
    np.testing.assert_allclose(res["score_fwd"], sf, rtol=FP16_RTOL, atol=1e-2)
    np.testing.assert_allclose(res["score_rev"], sr, rtol=FP16_RTOL, atol=1e-2)
    for i, n in enumerate(lengths):
        if i % 2 == 0 and n >= 500:
            best_end = ef[i] if sf[i] <= sr[i] else er[i]
            assert abs(int(res["end_pos"][i]) - int(best_end)) <= 2


def test_ref_del_fp16_cta_shape_keeps_bits(lib, genome_pair):
    """A REF_DEL warp sweeps its read alone, in the same order, whatever CTA it
    sits in, so every CTA shape gives the same bits.  By default the reads are
    spread evenly over the SMs: ceil(reads / SMs) warps per CTA (at most 16),
    one CTA per SM."""
    import torch
    import dtwax_gb300 as d
    g, o = genome_pair
    tab = synth.level_table()
    lengths = [2000, 1, 33, 1025, 2049, 3000, 500, 777] * 3
    reads = reads_of_lengths(g, o, tab, lengths)
    outs, shapes = [], []
    for warps in (0, 1, 8, 16):
        with make_classifier(g, tab, precision=d.FP16, recurrence=d.REF_DEL, warps_per_cta=warps) as clf:
            outs.append(clf.classify(raw=reads.raw, offsets=reads.offsets))
            shapes.append(clf.tuning())
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    n = len(lengths)
    want = min(16, -(-n // sms))
    assert shapes[0]["warps_per_cta"] == want and shapes[0]["ctas"] == -(-n // want)
    assert [s["warps_per_cta"] for s in shapes[1:]] == [1, 8, 16]
    for res in outs[1:]:
        for k in ("score_fwd", "score_rev", "end_pos", "strand"):
            np.testing.assert_array_equal(res[k], outs[0][k])


def test_ref_del_rejects_other_cells(lib, genome_pair):
    import dtwax_gb300 as d
    g, _ = genome_pair
    with pytest.raises(d.DtwxError):
        make_classifier(g, synth.level_table(), precision=d.MIXED, recurrence=d.REF_DEL)


@pytest.mark.parametrize("cells,strips,warps", [(16, 1, 8), (32, 3, 2), (48, 2, 4), (32, 50, 1)])
def test_fp32_chunking_is_exact(lib, genome_pair, cells, strips, warps):
    """Chunks recompute a halo, so any chunk size gives the same FP32 bits."""
    g, o = genome_pair
    tab = synth.level_table()
    reads = reads_of_lengths(g, o, tab, [1500, 2000, 700, 2500, 90])
    with make_classifier(g, tab, precision=1) as clf:
        base = clf.classify(raw=reads.raw, offsets=reads.offsets)
    with make_classifier(g, tab, precision=1, cells_per_thread=cells, chunk_strips=strips,
                         warps_per_cta=warps) as clf:
        res = clf.classify(raw=reads.raw, offsets=reads.offsets)
        t = clf.tuning()
    strips_per_read = -(-(len(g) - 5) // (32 * cells))
    assert t["cells_per_thread"] == cells and t["chunk_strips"] == min(strips, strips_per_read)
    np.testing.assert_array_equal(res["score_fwd"], base["score_fwd"])
    np.testing.assert_array_equal(res["score_rev"], base["score_rev"])
    np.testing.assert_array_equal(res["end_pos"], base["end_pos"])


@pytest.mark.parametrize("cells,strips,warps", [(32, 1, 8), (48, 3, 2), (64, 2, 4), (32, 50, 1)])
def test_mixed_chunking_is_exact(lib, genome_pair, cells, strips, warps):
    """MIXED keeps FP32 cells with no rescale: any chunk size gives the same bits."""
    import dtwax_gb300 as d
    g, o = genome_pair
    tab = synth.level_table()
    reads = reads_of_lengths(g, o, tab, [1500, 2000, 700, 2500, 90])
    with make_classifier(g, tab, precision=d.MIXED) as clf:
        base = clf.classify(raw=reads.raw, offsets=reads.offsets)
    with make_classifier(g, tab, precision=d.MIXED, cells_per_thread=cells, chunk_strips=strips,
                         warps_per_cta=warps) as clf:
        res = clf.classify(raw=reads.raw, offsets=reads.offsets)
        t = clf.tuning()
    assert t["cells_per_thread"] == cells
    np.testing.assert_array_equal(res["score_fwd"], base["score_fwd"])
    np.testing.assert_array_equal(res["score_rev"], base["score_rev"])
    np.testing.assert_array_equal(res["end_pos"], base["end_pos"])


@pytest.mark.parametrize("cells,strips", [(32, 1), (48, 2), (32, 7), (48, 13)])
def test_fp16_chunking_within_tolerance(lib, oracle, genome_pair, cells, strips):
    """Narrow chunks run the kernel instance with 16-cell halo strips (the
    3,100-sample read's halo reaches column 0 for the first chunks); one chunk
    per read (13 strips of 1,536 columns) has no halo."""
    g, o = genome_pair
    tab = synth.level_table()
    reads = reads_of_lengths(g, o, tab, [1500, 2000, 2500, 3100])
    with make_classifier(g, tab, precision=0, cells_per_thread=cells, chunk_strips=strips) as clf:
        res = clf.classify(raw=reads.raw, offsets=reads.offsets)
        t = clf.tuning()
        sf, ef, sr, er = oracle_classify(oracle, clf, reads.raw, reads.offsets)
    strips_per_read = -(-(len(g) - 5) // (32 * cells))
    assert t["narrow_halo"] == (1 if strips < strips_per_read else 0)
    np.testing.assert_allclose(res["score_fwd"], sf, rtol=FP16_RTOL)
    np.testing.assert_allclose(res["score_rev"], sr, rtol=FP16_RTOL)
    for i in (0, 2):  # target reads: end column within 2 of the oracle's
        best_end = ef[i] if sf[i] <= sr[i] else er[i]
        assert abs(int(res["end_pos"][i]) - int(best_end)) <= 2


@pytest.mark.parametrize("precision", [1, 0])
def test_long_and_short_reads_in_one_batch(lib, oracle, genome_pair, precision):
    """Reads far longer than the reference window (40,000 and 12,345 samples)
    next to tiny ones: the seam buffers are sized by the longest read, halo
    strips of short reads stop early, and every read matches the oracle."""
    g, o = genome_pair
    tab = synth.level_table()
    lengths = [40_000, 3, 12_345, 1, 700]
    reads = reads_of_lengths(g, o, tab, lengths)
    with make_classifier(g, tab, precision=precision) as clf:
        res = clf.classify(raw=reads.raw, offsets=reads.offsets)
        ora = oracle_classify(oracle, clf, reads.raw, reads.offsets)
    assert (res["n_samples"] == np.array(lengths)).all()
    if precision == 1:
        check_fp32(res, ora)
    else:
        sf, ef, sr, er = ora
        np.testing.assert_allclose(res["score_fwd"], sf, rtol=FP16_RTOL, atol=1e-2)
        np.testing.assert_allclose(res["score_rev"], sr, rtol=FP16_RTOL, atol=1e-2)


def test_edge_cases(lib, oracle):
    import dtwax_gb300 as d
    tab = synth.level_table()
    tiny = small_genome(50, 9)  # 45 columns: less than one strip
    with make_classifier(tiny, tab, precision=1) as clf:
        assert clf.classify(raw=np.zeros(0, np.float32), offsets=np.zeros(1, np.int64)).size == 0
        raw = np.random.default_rng(0).normal(90, 10, 300).astype(np.float32)
        offs = np.array([0, 0, 1, 300])  # empty read, 1-sample read, 299-sample read
        res = clf.classify(raw=raw, offsets=offs)
        assert res["call"][0] == -1 and res["n_samples"][0] == 0 and np.isinf(res["score"][0])
        sf, ef, sr, er = oracle_classify(oracle, clf, raw, offs)
        np.testing.assert_allclose(res["score_fwd"][1:], sf[1:], rtol=FP32_RTOL, atol=1e-6)
        np.testing.assert_allclose(res["score_rev"][1:], sr[1:], rtol=FP32_RTOL, atol=1e-6)
        with pytest.raises(d.DtwxError):
            clf.classify(raw=raw, offsets=np.array([0, 200, 100]))  # decreasing offsets
    # reference window semantics: adapter skip + fixed query length, short reads skipped
    g = small_genome(8_000, 2)
    with make_classifier(g, tab, precision=1, adapter_skip=100, query_len=500, require_full=1) as clf:
        raw = np.random.default_rng(1).normal(90, 10, 1200).astype(np.float32)
        offs = np.array([0, 599, 1200])  # 599 < 600 -> skipped; 601 -> window [100, 600)
        res = clf.classify(raw=raw, offsets=offs)
        assert res["call"][0] == -1 and res["n_samples"][1] == 500
        sf, ef, sr, er = oracle_classify(oracle, clf, raw[599:], np.array([0, 601]), query_len=500, skip=100)
        assert res["score_fwd"][1] == pytest.approx(sf[0], rel=FP32_RTOL)


def test_int16_adc_scaling(lib, genome_pair):
    """pA = (raw + offset) * range / digitisation before the z-score."""
    g, o = genome_pair
    tab = synth.level_table()
    reads = reads_of_lengths(g, o, tab, [2000, 1500])
    off, rng_, dig = np.float32(12.0), np.float32(1400.0), np.float32(8192.0)
    adc = np.round(reads.raw / (rng_ / dig) - off).astype(np.int16)
    pa = ((adc.astype(np.float32) + off) * (rng_ / dig)).astype(np.float32)
    with make_classifier(g, tab, precision=1) as clf:
        a = clf.classify_i16(raw=adc, offsets=reads.offsets, offset=[off] * 2, range_=[rng_] * 2,
                             digitisation=[dig] * 2)
        b = clf.classify(raw=pa, offsets=reads.offsets)
    np.testing.assert_allclose(a["score"], b["score"], rtol=1e-6)
    np.testing.assert_array_equal(a["end_pos"], b["end_pos"])


def test_device_entry_points_match_host(lib, genome_pair):
    import torch
    import dtwax_gb300 as d
    g, o = genome_pair
    tab = synth.level_table()
    reads = reads_of_lengths(g, o, tab, [2000, 1000, 3000])
    with make_classifier(g, tab, precision=0) as clf:
        host = clf.classify(raw=reads.raw, offsets=reads.offsets)
        draw = torch.tensor(reads.raw, device="cuda")
        dout = torch.zeros(32 * reads.n, dtype=torch.uint8, device="cuda")
        s = torch.cuda.current_stream().cuda_stream
        clf.classify_device(draw.data_ptr(), reads.offsets, dout.data_ptr(), s)
        torch.cuda.synchronize()
        dev = np.frombuffer(dout.cpu().numpy().tobytes(), d.RESULT_DTYPE)
        assert clf.last_launch_count >= 3
    np.testing.assert_array_equal(dev["score"], host["score"])
    np.testing.assert_array_equal(dev["end_pos"], host["end_pos"])


def test_plain_fp32_matches_batched(lib, genome_pair):
    g, o = genome_pair
    tab = synth.level_table()
    reads = reads_of_lengths(g, o, tab, [2000, 1000, 1999, 40])
    with make_classifier(g, tab, precision=1) as clf:
        a = clf.classify(raw=reads.raw, offsets=reads.offsets)
        b = clf.classify_plain_fp32(raw=reads.raw, offsets=reads.offsets)
        assert clf.last_launch_count >= reads.n + 2
    np.testing.assert_array_equal(a["score_fwd"], b["score_fwd"])
    np.testing.assert_array_equal(a["end_pos"], b["end_pos"])


def test_targets_found_at_true_position(lib):
    """Size-independent property at a benchmark shape (C1 genome): target reads
    end within a few k-mers of where the simulator stopped, on the right strand,
    and score below every non-target read."""
    w = synth.make_workload("C1", n_reads=64)
    with make_classifier(w.genome, w.table, precision=0) as clf:
        res = clf.classify(raw=w.reads.raw, offsets=w.reads.offsets)
    t = w.reads.target == 1
    true_end = w.reads.start + w.reads.kmers - 1
    assert (res["strand"][t] == w.reads.strand[t]).all()
    assert (np.abs(res["end_pos"][t] - true_end[t]) <= 3).mean() >= 0.95
    assert res["score"][t].max() < res["score"][~t].min()


def test_c1_full_parity_all_precisions(lib, oracle):
    """All 512 reads of the C1 workload against the FP64 oracle, in FP32,
    FP16 and MIXED."""
    import dtwax_gb300 as d
    w = synth.make_workload("C1")
    with make_classifier(w.genome, w.table, precision=1) as clf:
        r32 = clf.classify(raw=w.reads.raw, offsets=w.reads.offsets)
        ora = oracle_classify(oracle, clf, w.reads.raw, w.reads.offsets)
    with make_classifier(w.genome, w.table, precision=0) as clf:
        r16 = clf.classify(raw=w.reads.raw, offsets=w.reads.offsets)
    with make_classifier(w.genome, w.table, precision=d.MIXED) as clf:
        rmx = clf.classify(raw=w.reads.raw, offsets=w.reads.offsets)
    sf, ef, sr, er = ora
    np.testing.assert_allclose(r32["score_fwd"], sf, rtol=FP32_RTOL)
    np.testing.assert_allclose(r32["score_rev"], sr, rtol=FP32_RTOL)
    best = np.minimum(sf, sr)
    np.testing.assert_allclose(r16["score"], best, rtol=FP16_RTOL)
    np.testing.assert_allclose(rmx["score_fwd"], sf, rtol=MIXED_RTOL)
    np.testing.assert_allclose(rmx["score_rev"], sr, rtol=MIXED_RTOL)
    score, end, strand = oracle.combine(sf, ef, sr, er)
    assert (r32["end_pos"] == end).mean() >= 0.999
    t = w.reads.target == 1
    assert ((np.abs(rmx["end_pos"] - end) <= 2) & (rmx["strand"] == strand))[t].mean() >= 0.999
    # classification agreement at the oracle-tuned threshold
    from dtwax_gb300 import threshold
    th, acc = threshold.best_threshold(best[t], best[~t])
    for r in (r16, rmx):
        agree = (threshold.call(r["score"], th) == threshold.call(best, th)).mean()
        assert agree >= 0.999


def test_cli_drop_in(lib, kat, tmp_path):
    """`dtwx_main <folder> <kmer_model> <ref.fasta>` prints the reference's
    6-column log for a folder of reads."""
    import dtwax_gb300 as d
    fasta, model = write_kat_files(kat, str(tmp_path))
    folder = tmp_path / "reads"
    folder.mkdir()
    rng = np.random.default_rng(5)
    raws = []
    for i in range(4):
        x = (rng.normal(0, 1, 4100) * 20 + 500).astype(np.int16)
        np.save(folder / f"read_{i:02d}.npy", x)
        raws.append(x)
    np.save(folder / "short.npy", np.zeros(3000, np.int16))  # < 1952 + 2048: skipped
    side = tmp_path / "side.tsv"
    out = subprocess.run([d.CLI_PATH, str(folder), model, fasta, "--side", str(side)], capture_output=True,
                         text=True, check=True).stdout.splitlines()
    assert out[0].startswith("Read_ID")
    rows = [l.split("\t") for l in out[1:]]
    assert len(rows) == 4 and all(len(r) == 6 for r in rows)
    assert [r[1] for r in rows] == [f"read_{i:02d}" for i in range(4)]
    assert all(r[2] == "2048" for r in rows)
    with d.Classifier(fasta=fasta, kmer_model=model, adapter_skip=1952, query_len=2048, require_full=1) as clf:
        res = clf.classify([x.astype(np.float32) for x in raws])
    np.testing.assert_allclose([float(r[4]) for r in rows], res["score_fwd"], rtol=1e-5)
    side_rows = [l.split("\t") for l in side.read_text().splitlines()]
    assert len(side_rows) == 5 and side_rows[-1][-1] == "skipped"
    # the build variants as flags: same log shape, scores of the same handle options
    for flags, kw, rtol in ((["--mixed"], dict(precision=d.MIXED), 1e-5),
                            (["--ref-del"], dict(recurrence=d.REF_DEL), 1e-5),
                            (["--fp32", "--ref-del"], dict(precision=d.FP32, recurrence=d.REF_DEL), 1e-5)):
        out = subprocess.run([d.CLI_PATH, str(folder), model, fasta] + flags, capture_output=True, text=True,
                             check=True).stdout.splitlines()
        rows = [l.split("\t") for l in out[1:]]
        assert len(rows) == 4 and all(len(r) == 6 for r in rows)
        with d.Classifier(fasta=fasta, kmer_model=model, adapter_skip=1952, query_len=2048, require_full=1,
                          **kw) as clf:
            res = clf.classify([x.astype(np.float32) for x in raws])
        np.testing.assert_allclose([float(r[4]) for r in rows], res["score_fwd"], rtol=rtol)


def _fifo_write_session(fifo, payload, proc, timeout=120):
    """One writer session as the reference's Read Until scripts do it: open the
    pipe, write, close (ont_readuntil.py:49-50).  The open is retried without
    blocking until the reader has (re)opened its end."""
    import os
    import time
    fd = None
    t0 = time.time()
    while fd is None and time.time() - t0 < timeout and proc.poll() is None:
        try:
            fd = os.open(fifo, os.O_WRONLY | os.O_NONBLOCK)
        except OSError:
            time.sleep(0.05)
    assert fd is not None, proc.stderr.read() if proc.poll() is not None else "reader never opened the pipe"
    os.set_blocking(fd, True)
    os.write(fd, payload)
    os.close(fd)


def test_cli_read_until_fifo(lib, kat, tmp_path):
    """`dtwx_main --fifo <kmer_model> <ref.fasta> <pipe>`: the reference's Read
    Until binary protocol (ru_main.cu, generate_load_squiggle.hpp:303-343).
    Batches of 10 reads x 2,048 uint8 samples arrive on a named pipe, and one
    6-token line per read comes back with the scores of dtwx_classify_batch.
    The writers open, write and close the pipe per session, as
    ont_readuntil.py does (16,000 bytes per open): the first batch is split
    across two sessions, and the reader keeps filling it across the reopen."""
    import os
    import dtwax_gb300 as d
    fasta, model = write_kat_files(kat, str(tmp_path))
    fifo = str(tmp_path / "pipe")
    os.mkfifo(fifo)
    rng = np.random.default_rng(9)
    data = rng.integers(0, 256, size=2 * 10 * 2048, dtype=np.uint8).tobytes()
    proc = subprocess.Popen([d.CLI_PATH, "--fifo", model, fasta, fifo, "--batches", "2"], stdout=subprocess.PIPE,
                            stderr=subprocess.PIPE, text=True)
    try:
        _fifo_write_session(fifo, data[:16000], proc)   # part of batch 1, then the writer closes
        _fifo_write_session(fifo, data[16000:], proc)   # the rest of batch 1 and batch 2
        out, err = proc.communicate(timeout=120)
    finally:
        if proc.poll() is None:
            proc.kill()
    assert proc.returncode == 0, err
    rows = [l.split("\t") for l in out.splitlines()]
    assert len(rows) == 20 and all(len(r) == 6 for r in rows)
    assert [r[0] for r in rows] == [str(j) for j in range(10)] * 2
    with d.Classifier(fasta=fasta, kmer_model=model) as clf:
        x = np.frombuffer(data, np.uint8).astype(np.float32)
        res = clf.classify(raw=x, offsets=np.arange(21, dtype=np.int64) * 2048)
        assert all(r[3] == str(clf.ref_len) for r in rows)
    np.testing.assert_allclose([float(r[4]) for r in rows], res["score_fwd"], rtol=1e-5)
    np.testing.assert_allclose([float(r[5]) for r in rows], res["score_rev"], rtol=1e-5)


def test_cli_read_until_fifo_runs_until_signalled(lib, kat, tmp_path):
    """Without --batches the FIFO reader runs like the reference's (while
    (true), ru_main.cu:172): writers may come and go; SIGTERM ends it with
    status 0 after the batches it has printed."""
    import os
    import signal
    import time
    import dtwax_gb300 as d
    fasta, model = write_kat_files(kat, str(tmp_path))
    fifo = str(tmp_path / "pipe")
    os.mkfifo(fifo)
    data = np.random.default_rng(10).integers(0, 256, size=10 * 2048, dtype=np.uint8).tobytes()
    proc = subprocess.Popen([d.CLI_PATH, "--fifo", model, fasta, fifo], stdout=subprocess.PIPE,
                            stderr=subprocess.PIPE, text=True)
    try:
        _fifo_write_session(fifo, data, proc)
        lines = []
        t0 = time.time()
        while len(lines) < 10 and time.time() - t0 < 120 and proc.poll() is None:
            line = proc.stdout.readline()
            if line:
                lines.append(line)
        assert len(lines) == 10
        time.sleep(0.2)  # the reader is back in open(), waiting for the next writer
        assert proc.poll() is None
        proc.send_signal(signal.SIGTERM)
        out, err = proc.communicate(timeout=60)
    finally:
        if proc.poll() is None:
            proc.kill()
    assert proc.returncode == 0, err
    assert out == ""


def test_autotune_picks_a_compiled_shape_and_keeps_results(lib, genome_pair):
    g, o = genome_pair
    tab = synth.level_table()
    reads = reads_of_lengths(g, o, tab, [2000] * 6)
    with make_classifier(g, tab, precision=1) as clf:
        before = clf.classify(raw=reads.raw, offsets=reads.offsets)
        ms = clf.autotune(6, 2000)
        after = clf.classify(raw=reads.raw, offsets=reads.offsets)
        t = clf.tuning()
    assert ms > 0
    assert t["cells_per_thread"] in (16, 32, 48) and t["warps_per_cta"] in (4, 8) and t["ctas_per_sm"] >= 1
    np.testing.assert_array_equal(after["score"], before["score"])  # FP32: shape never changes the bits


def test_cuda_graph_replay_matches_direct_launches(lib, genome_pair):
    """A repeated device batch runs directly once, is captured the second
    time and replayed afterwards; every call returns the same results."""
    import torch
    import dtwax_gb300 as d
    g, o = genome_pair
    tab = synth.level_table()
    reads = reads_of_lengths(g, o, tab, [2000, 1200, 4000, 33, 1])
    with make_classifier(g, tab, precision=0, use_graphs=1) as clf:
        host = clf.classify(raw=reads.raw, offsets=reads.offsets)
        stream = torch.cuda.Stream()
        draw = torch.tensor(reads.raw, device="cuda")
        dout = torch.zeros(32 * reads.n, dtype=torch.uint8, device="cuda")
        got = []
        for _ in range(4):
            dout.zero_()
            torch.cuda.synchronize()
            clf.classify_device(draw.data_ptr(), reads.offsets, dout.data_ptr(), stream.cuda_stream)
            stream.synchronize()
            got.append(np.frombuffer(dout.cpu().numpy().tobytes(), d.RESULT_DTYPE).copy())
            assert clf.last_sweep_ms() > 0
        assert clf.tuning()["graph_replays"] == 2
    for r in got:
        np.testing.assert_array_equal(r["score"], host["score"])
        np.testing.assert_array_equal(r["end_pos"], host["end_pos"])


def test_full_size_properties_c3_genome(lib):
    """Size-independent properties on the 5 Mb genome of the uneven-read
    workload (where the FP64 oracle is too slow for every read): FP32 results
    do not depend on the order of the reads in a batch, on how the batch is
    split, on the launch shape, or on graph replay."""
    import torch
    import dtwax_gb300 as d
    w = synth.make_workload("C3", n_reads=48)
    raw, offs = w.reads.raw, w.reads.offsets
    lens = np.diff(offs)
    with make_classifier(w.genome, w.table, precision=d.FP32) as clf:
        base = clf.classify(raw=raw, offsets=offs)
        perm = np.random.default_rng(1).permutation(w.reads.n)
        praw = np.concatenate([w.reads.read(i) for i in perm])
        poffs = np.concatenate([[0], np.cumsum(lens[perm])]).astype(np.int64)
        permuted = clf.classify(raw=praw, offsets=poffs)
        half = w.reads.n // 2
        first = clf.classify(raw=raw[: offs[half]], offsets=offs[: half + 1])
        second = clf.classify(raw=raw[offs[half]:], offsets=offs[half:] - offs[half])
    np.testing.assert_array_equal(permuted["score"], base["score"][perm])
    np.testing.assert_array_equal(permuted["end_pos"], base["end_pos"][perm])
    np.testing.assert_array_equal(np.concatenate([first["score"], second["score"]]), base["score"])
    with make_classifier(w.genome, w.table, precision=d.FP32, cells_per_thread=16, warps_per_cta=8,
                         use_graphs=1) as clf:
        d_raw = torch.tensor(raw, device="cuda")
        out = torch.zeros(32 * w.reads.n, dtype=torch.uint8, device="cuda")
        s = torch.cuda.Stream()
        got = []
        for _ in range(3):  # direct, captured, replayed
            clf.classify_device(d_raw.data_ptr(), offs, out.data_ptr(), s.cuda_stream)
            s.synchronize()
            got.append(np.frombuffer(out.cpu().numpy().tobytes(), d.RESULT_DTYPE).copy())
    for g in got:
        np.testing.assert_array_equal(g["score"], base["score"])
        np.testing.assert_array_equal(g["end_pos"], base["end_pos"])
