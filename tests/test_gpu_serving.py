"""Read Until serving: per-read DP row state kept on the GPU between chunks.

The oracle for a read served in chunks c1, c2, ... is the FP64 sDTW of
z(c1) || z(c2) || ... where each chunk is z-scored with its own statistics
(the serving normaliser), resumed from the previous chunk's last row; the
decision after chunk k is the best (score, end, strand) over the last row of
chunk k.  FP32 within 1e-5 relative with the same end column; FP16 within 1e-2.
"""
import numpy as np
import pytest

from gpu_util import make_classifier, small_genome
from dtwax_gb300 import synth

pytestmark = pytest.mark.gpu


def oracle_decisions(oracle, fwd, rev, chunks, ref_del=False):
    """Best hit after each chunk, resumed from the saved rows."""
    out = []
    rf = rr = None
    run = oracle.sdtw_ref_del if ref_del else oracle.sdtw
    for c in chunks:
        z = oracle.zscore(c.astype(np.float64), 1e-4).astype(np.float32).astype(np.float64)
        sf, ef, rf = run(fwd, z, init_row=rf, want_row=True)
        sr, er, rr = run(rev, z, init_row=rr, want_row=True)
        score, end, strand = oracle.combine([sf], [ef], [sr], [er])
        out.append((float(score[0]), int(end[0]), int(strand[0])))
    return out


def serve_reads(clf, reads_chunks, chunks_per_decision=3, max_in_flight=0, budget=0.0, interleave=True):
    """Submit chunks (round-robin across reads when interleave) and drain.
    Returns {read_number: [decision dicts in order]}."""
    clf.serve_start(max_in_flight=max_in_flight, state_budget_bytes=budget,
                    chunks_per_decision=chunks_per_decision)
    rounds = max(len(c) for c in reads_chunks.values())
    keys = list(reads_chunks)
    if interleave:
        for k in range(rounds):
            for rn in keys:
                ch = reads_chunks[rn]
                if k < len(ch):
                    clf.submit_chunk(rn % 512, rn, ch[k], is_last=(k == len(ch) - 1))
            clf.serve_step()
    else:
        for rn in keys:
            ch = reads_chunks[rn]
            for k, c in enumerate(ch):
                clf.submit_chunk(rn % 512, rn, c, is_last=(k == len(ch) - 1))
    clf.serve_drain()
    got = {}
    for d in clf.poll_decisions(100000):
        got.setdefault(d["read_number"], []).append(d)
    return got


def split(x, size):
    return [x[i:i + size] for i in range(0, x.size, size)]


@pytest.fixture(scope="module")
def setup(built_lib, oracle):
    g, o = small_genome(40_000, 31), small_genome(40_000, 32)
    tab = synth.level_table()
    reads = synth.simulate_reads(g, o, tab, [4800, 4000, 4800, 3300, 1600, 4800], [1, 0, 0, 1, 0, 0], seed=9)
    return g, o, tab, reads


@pytest.mark.parametrize("precision,rtol", [(1, 1e-5), (0, 1e-2), (2, 1e-3)])
def test_resume_matches_oracle(setup, oracle, precision, rtol):
    g, o, tab, reads = setup
    with make_classifier(g, tab, precision=precision, threshold=-1.0) as clf:  # never early: see every chunk
        fwd, rev = clf.reference()
        chunks = {i: split(reads.read(i), 1600) for i in range(reads.n)}
        got = serve_reads(clf, chunks, chunks_per_decision=3)
    for i in range(reads.n):
        want = oracle_decisions(oracle, fwd.astype(np.float64), rev.astype(np.float64), chunks[i][:3])
        ds = got[i]
        assert [d["chunks"] for d in ds] == list(range(1, len(want) + 1))
        assert ds[-1]["decided"] == 1
        for d, (s, e, st) in zip(ds, want):
            assert d["score"] == pytest.approx(s, rel=rtol)
            if precision == 1:
                assert (d["end_pos"], d["strand"]) == (e, st)


def test_resume_fp16_state_matches_oracle(setup, oracle):
    """FP16 row state (half2 cells + a frame offset per 512 columns) resumed
    chunk by chunk; a batch shape that differs between chunks (autotuned
    buckets) re-bases the saved frames."""
    import dtwax_gb300 as d
    g, o, tab, reads = setup
    for cells in (32, 48):
        with make_classifier(g, tab, precision=d.FP16, state_precision=d.STATE_FP16, threshold=-1.0,
                             cells_per_thread=cells) as clf:
            fwd, rev = clf.reference()
            chunks = {i: split(reads.read(i), 1600) for i in range(reads.n)}
            got = serve_reads(clf, chunks, chunks_per_decision=3)
        for i in range(reads.n):
            want = oracle_decisions(oracle, fwd.astype(np.float64), rev.astype(np.float64), chunks[i][:3])
            for dd, (s, e, st) in zip(got[i], want):
                assert dd["score"] == pytest.approx(s, rel=1e-2)


@pytest.mark.parametrize("state", ["fp32", "fp16"])
def test_resume_narrow_halo_matches_oracle(setup, oracle, state):
    """Chunks of 3 strips run the kernel instance with 16-cell halo strips,
    for both row-state layouts: resumed decisions stay within the FP16
    tolerance of the FP64 oracle."""
    import dtwax_gb300 as d
    g, o, tab, reads = setup
    sp = d.STATE_FP16 if state == "fp16" else d.STATE_FP32
    with make_classifier(g, tab, precision=d.FP16, state_precision=sp, threshold=-1.0, cells_per_thread=48,
                         chunk_strips=3) as clf:
        fwd, rev = clf.reference()
        chunks = {i: split(reads.read(i), 1600) for i in range(reads.n)}
        got = serve_reads(clf, chunks, chunks_per_decision=3)
        t = clf.tuning()
    assert t["narrow_halo"] == 1 and t["chunk_strips"] == 3
    for i in range(reads.n):
        want = oracle_decisions(oracle, fwd.astype(np.float64), rev.astype(np.float64), chunks[i][:3])
        for dd, (sc, e, st) in zip(got[i], want):
            assert dd["score"] == pytest.approx(sc, rel=1e-2)


def test_int16_chunks_match_float_chunks(setup):
    """Raw int16 ADC chunks with their scaling give the decisions of the same
    chunks converted to pA on the host."""
    import dtwax_gb300 as d
    g, o, tab, reads = setup
    x = reads.read(0)
    offset, rng_, digi = 12.0, 1400.0, 8192.0
    raw = np.round(x * digi / rng_ - offset).astype(np.int16)
    pa = ((raw.astype(np.float32) + offset) * (rng_ / digi)).astype(np.float32)
    out = []
    for use_i16 in (False, True):
        with make_classifier(g, tab, precision=d.FP32, threshold=-1.0) as clf:
            clf.serve_start(chunks_per_decision=3)
            for k, lo in enumerate(range(0, 4800, 1600)):
                last = lo + 1600 >= 4800
                if use_i16:
                    clf.submit_chunk_i16(1, 7, raw[lo:lo + 1600], offset, rng_, digi, is_last=last)
                else:
                    clf.submit_chunk(1, 7, pa[lo:lo + 1600], is_last=last)
                clf.serve_step()
            clf.serve_drain()
            out.append([(dd["score"], dd["end_pos"]) for dd in clf.poll_decisions(100)])
    assert out[0] == out[1] and len(out[0]) == 3


def test_fp16_state_halves_the_row_bytes(setup):
    import dtwax_gb300 as d
    g, o, tab, reads = setup
    budget = 64 * 8 * (40_000 + 6144.0)  # 64 reads of FP32 rows
    with make_classifier(g, tab, precision=d.FP16) as clf:
        clf.serve_start(state_budget_bytes=budget)
        n32 = clf.stats()["max_in_flight"]
    with make_classifier(g, tab, precision=d.FP16, state_precision=d.STATE_FP16) as clf:
        clf.serve_start(state_budget_bytes=budget)
        n16 = clf.stats()["max_in_flight"]
    assert n16 >= 2 * n32 - 2 and n32 >= 60
    with pytest.raises(d.DtwxError):
        make_classifier(g, tab, precision=d.FP32, state_precision=d.STATE_FP16)


@pytest.mark.parametrize("precision,rtol", [(1, 1e-5), (0, 1e-2)])
def test_resume_ref_del_matches_oracle(setup, oracle, precision, rtol):
    """The REF_DEL recurrence resumed chunk by chunk from the saved rows."""
    import dtwax_gb300 as d
    g, o, tab, reads = setup
    with make_classifier(g, tab, precision=precision, recurrence=d.REF_DEL, threshold=-1.0) as clf:
        fwd, rev = clf.reference()
        chunks = {i: split(reads.read(i), 1600) for i in range(reads.n)}
        got = serve_reads(clf, chunks, chunks_per_decision=3)
    for i in range(reads.n):
        want = oracle_decisions(oracle, fwd.astype(np.float64), rev.astype(np.float64), chunks[i][:3], ref_del=True)
        for dd, (s, e, st) in zip(got[i], want):
            assert dd["score"] == pytest.approx(s, rel=rtol)
            if precision == 1:
                assert (dd["end_pos"], dd["strand"]) == (e, st)


@pytest.mark.parametrize("precision", [1, 0, 2])
def test_same_result_alone_and_in_the_mix(setup, precision):
    """Continuous batching must not change a read's result: read 0 served alone
    equals read 0 served while 5 other reads share its batches."""
    g, o, tab, reads = setup
    chunks = {i: split(reads.read(i), 1600) for i in range(reads.n)}
    with make_classifier(g, tab, precision=precision, threshold=-1.0) as clf:
        alone = serve_reads(clf, {0: chunks[0]})[0]
    with make_classifier(g, tab, precision=precision, threshold=-1.0) as clf:
        mixed = serve_reads(clf, chunks)[0]
    assert len(alone) == len(mixed) == 3
    for a, b in zip(alone, mixed):
        if precision in (1, 2):  # FP32 cells: the same bits for any batch
            assert a["score"] == b["score"] and a["end_pos"] == b["end_pos"]
        else:
            assert a["score"] == pytest.approx(b["score"], rel=1e-2)


def test_admission_and_deferral(setup):
    """Two row-state slots for six reads: four wait, all are decided, the
    results equal unlimited admission."""
    g, o, tab, reads = setup
    chunks = {i: split(reads.read(i), 1600) for i in range(reads.n)}
    with make_classifier(g, tab, precision=1, threshold=-1.0) as clf:
        free = serve_reads(clf, chunks)
    with make_classifier(g, tab, precision=1, threshold=-1.0) as clf:
        tight = serve_reads(clf, chunks, max_in_flight=2)
        st = clf.stats()
    assert st["max_in_flight"] == 2 and st["reads_deferred"] == 4
    assert st["reads_decided"] == reads.n and st["queue_depth"] == 0 and st["in_flight"] == 0
    for i in range(reads.n):
        assert [d["score"] for d in tight[i]] == [d["score"] for d in free[i]]
    assert st["p99_latency_ms"] >= st["p50_latency_ms"] > 0


def test_target_decided_early_and_later_chunks_ignored(setup):
    g, o, tab, reads = setup
    chunks = {0: split(reads.read(0), 1600)}  # read 0 is a target
    with make_classifier(g, tab, precision=0, threshold=1e9) as clf:  # everything is a target
        got = serve_reads(clf, chunks)
        st = clf.stats()
    assert len(got[0]) == 1 and got[0][0]["decided"] == 1 and got[0][0]["call"] == 1
    assert st["chunks_processed"] == 1


def test_state_budget_admits_by_bytes(setup):
    import dtwax_gb300 as d
    g, o, tab, reads = setup
    with make_classifier(g, tab, precision=1) as clf:
        with pytest.raises(d.DtwxError):
            clf.serve_start(state_budget_bytes=10.0)  # not one read's row
    with make_classifier(g, tab, precision=1) as clf:
        # one read's row: 8 bytes per column, columns padded by less than 6144
        clf.serve_start(state_budget_bytes=3 * 8 * (clf.ref_len + 6144.0))
        st = clf.stats()
        assert st["max_in_flight"] == 3 and st["state_bytes"] >= 3 * 8 * clf.ref_len


def test_read_until_loop_real_time(built_lib):
    """A short real-time run of the simulated sequencer through the serving API:
    reads are decided, calls are right, latencies are recorded."""
    from dtwax_gb300 import readuntil
    g, o = small_genome(200_000, 41), small_genome(200_000, 42)
    tab = synth.level_table()
    cfg = readuntil.ServeConfig(channels=64, duration_s=2.0, warmup_s=0.5, pool_reads=128)
    pool = readuntil.make_pool(g, o, tab, cfg)
    with make_classifier(g, tab, precision=0) as clf:
        accept, reject = readuntil.calibrate(clf, pool, cfg, n=128)
        rec = readuntil.run(clf, pool, cfg, accept, reject)
    assert rec["reads_per_s"] > 20
    assert rec["call_accuracy"] >= 0.95
    assert 0 < rec["p50_latency_ms"] <= rec["p99_latency_ms"] < 1000
