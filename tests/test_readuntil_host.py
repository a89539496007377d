"""CPU tests of the Read Until loop (dtwax_gb300/readuntil.py) against a fake
serving library: chunk flow, decisions, latency bookkeeping and the
simulated sequencer's channel handling."""
import numpy as np

from dtwax_gb300 import readuntil, synth


class FakeServer:
    """Decides every read on its first chunk: target iff the pool says so.
    Decisions come back on the next serve_step, one batch per step."""

    def __init__(self, truth):
        self.truth = truth
        self.pending = []
        self.out = []
        self.steps = 0
        self.submitted = 0

    def autotune(self, k, n):
        return 0.0

    def serve_start(self, **kw):
        self.kw = kw

    def submit_chunk(self, ch, rn, x, is_last=False, arrival_ms=-1.0):
        assert x.size > 0
        self.submitted += 1
        self.pending.append((ch, rn, arrival_ms))

    def serve_step(self):
        from dtwax_gb300 import now_ms
        self.steps += 1
        t = now_ms()
        for ch, rn, arr in self.pending:
            self.out.append({"channel": ch, "read_number": rn, "decided": 1, "call": self.truth(rn),
                             "latency_ms": t - arr, "queue_ms": 0.0})
        self.pending = []

    def poll_decisions(self, cap):
        out, self.out = self.out[:cap], self.out[cap:]
        return out

    def stats(self):
        return {"mean_batch_reads": 1.0, "batches": self.steps, "mean_batch_ms": 0.0, "max_batch_ms": 0.0,
                "chunks_processed": self.submitted,
                "reads_deferred": 0, "max_in_flight": 0, "queue_depth": 0, "state_bytes": 0.0}


def test_loop_with_fake_library():
    cfg = readuntil.ServeConfig(channels=16, chunk=200, duration_s=0.6, warmup_s=0.2, pool_reads=32,
                                read_rate=20.0)
    g, o = synth.random_genome(6000, 1), synth.random_genome(6000, 2)
    pool = readuntil.make_pool(g, o, synth.level_table(), cfg)
    seq = readuntil.SimulatedSequencer(pool, cfg)
    srv = FakeServer(lambda rn: seq.truth.get(rn, 0))  # answers with the sequencer's ground truth
    rec = readuntil.run(srv, pool, cfg, accept=0.1, reject=0.2, sequencer=seq)
    assert rec["reads_per_s"] > 0 and rec["call_accuracy"] == 1.0
    assert rec["p50_latency_ms"] is not None and rec["p99_latency_ms"] >= rec["p50_latency_ms"] >= 0
    assert rec["accept_per_sample"] == 0.1 and rec["reject_per_sample"] == 0.2
    assert srv.kw["chunks_per_decision"] == cfg.chunks_per_read


def test_sequencer_drops_chunks_of_decided_reads():
    cfg = readuntil.ServeConfig(channels=4, chunk=50, pool_reads=8, read_rate=1000.0, chunks_per_read=3)
    g, o = synth.random_genome(3000, 1), synth.random_genome(3000, 2)
    pool = readuntil.make_pool(g, o, synth.level_table(), cfg)
    seq = readuntil.SimulatedSequencer(pool, cfg)
    first = seq.due(0.1)  # every channel has started a read and sent its first chunk
    assert sorted(c for _, c, _, _, _ in first) == [0, 1, 2, 3]
    ch, rn = first[0][1], first[0][2]
    seq.decided(ch, rn, 0.1)
    later = seq.due(10.0)
    # the decided read sends nothing more; its channel starts new reads
    assert all(not (c == ch and r == rn) for _, c, r, _, _ in later)
    assert any(c == ch and r > rn for _, c, r, _, _ in later)
    # reads that were not decided deliver their remaining chunks in order
    others = [(c, r) for _, c, r, _, _ in first if c != ch]
    for c, r in others:
        ks = [x for x in later if x[1] == c and x[2] == r]
        assert len(ks) == cfg.chunks_per_read - 1 and ks[-1][4]
    assert np.isfinite([t for t, _, _, _, _ in later]).all()
