"""CPU tests of the Read Until loop (dtwax_gb300/readuntil.py) against a fake
serving library: chunk flow, decisions, latency bookkeeping, the simulated
sequencer's channel handling, and a fake live Read Until client whose
unblock / stop actions the decisions drive."""
import numpy as np
import pytest

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


class FakeRead:
    def __init__(self, number, data):
        self.number = number
        self.id = f"read-{number}"
        self.raw_data = data.tobytes()


class FakeClient:
    """The read_until ReadUntilClient surface the loop uses: chunks arrive in
    rounds (every read's first chunk, then every read's second, ...), one
    round per get_read_chunks call; actions are recorded."""

    def __init__(self, rounds, dtype):
        self.rounds = rounds
        self.signal_dtype = dtype
        self.unblocked, self.stopped = [], []

    @property
    def is_running(self):
        return bool(self.rounds)

    def get_read_chunks(self, batch_size=1, last=True):
        return self.rounds.pop(0)[:batch_size] if self.rounds else []

    def unblock_read(self, read_channel, read_number, duration=0.1):
        self.unblocked.append((read_channel, read_number))

    def stop_receiving_read(self, read_channel, read_number):
        self.stopped.append((read_channel, read_number))


class RecordingServer(FakeServer):
    def __init__(self, truth):
        super().__init__(truth)
        self.samples = {}

    def submit_chunk(self, ch, rn, x, is_last=False, arrival_ms=-1.0):
        self.samples.setdefault(rn, []).append(np.array(x, copy=True))
        super().submit_chunk(ch, rn, x, is_last, arrival_ms)


def test_live_client_decisions_drive_unblock():
    """Reads 1-6 on channels 1-6, three chunks each; the library decides each
    read on its first chunk.  Non-targets (odd read numbers) are ejected,
    every decided read stops receiving data, and later chunks of decided reads
    never reach the library."""
    rng = np.random.default_rng(0)
    chunks = {rn: [rng.normal(90, 10, 400).astype(np.float32) for _ in range(3)] for rn in range(1, 7)}
    rounds = [[(rn, FakeRead(rn, chunks[rn][k])) for rn in range(1, 7)] for k in range(3)]
    client = FakeClient(rounds, np.float32)
    src = readuntil.ReadUntilClientSource(client, batch_size=16, max_chunks=3)
    srv = RecordingServer(lambda rn: rn % 2 == 0)
    cfg = readuntil.ServeConfig(channels=6, chunk=400, duration_s=0.3, warmup_s=0.0)
    rec = readuntil.run(srv, None, cfg, accept=0.1, reject=0.2, sequencer=src)
    assert sorted(client.unblocked) == [(rn, rn) for rn in (1, 3, 5)]
    assert sorted(client.stopped) == [(rn, rn) for rn in range(1, 7)]
    assert src.reads_started() == 6 and rec["reads_started"] == 6
    for rn in range(1, 7):
        assert len(srv.samples[rn]) == 1  # decided on its first chunk
        np.testing.assert_array_equal(srv.samples[rn][0], chunks[rn][0])
    assert np.isnan(rec["call_accuracy"])  # live reads carry no ground truth


def test_live_client_int16_signal_is_calibrated():
    raw = (np.arange(400) % 50 - 10).astype(np.int16)
    client = FakeClient([[(3, FakeRead(9, raw))]], np.int16)
    src = readuntil.ReadUntilClientSource(client, max_chunks=1, calibration=lambda ch: (12.0, 1400.0, 8192.0))
    (t, ch, rn, x, last), = src.due(0.0)
    assert (ch, rn, last) == (3, 9, True)
    np.testing.assert_allclose(x, (raw.astype(np.float32) + 12.0) * np.float32(1400.0 / 8192.0), rtol=1e-6)
    src_nocal = readuntil.ReadUntilClientSource(FakeClient([[(3, FakeRead(9, raw))]], np.int16))
    with pytest.raises(ValueError):
        src_nocal.due(0.0)
