"""Read Until loop over the ctypes serving API, with a simulated sequencer.

Replaces the reference's FIFO protocol (src/ReadUntil/ont_readuntil.py:29-59
feeding src/ru_main.cu:172-326, and the fake sequencer
src/ReadUntil/simulate_minion.py): chunks go straight into the library, each
read's last DP row stays on the GPU between its chunks, and a decision
(target / eject) comes back per read.

`SimulatedSequencer` produces, in real time, `channels` channels; a channel
carries one read at a time, a new read starts after an exponential gap (mean
1 / read_rate s), and an active read delivers one chunk of `chunk` samples every
`period_s` seconds until the library decides it (or its last chunk is sent).
Reads come from a pool of seeded synthetic squiggles (targets from the target
genome, others from a second genome).  Latency is measured from the scheduled
arrival of a read's last needed chunk to its decision.

`ReadUntilClientSource` takes the chunks from a live Read Until client instead
(the read_until package's ReadUntilClient), and its decisions drive the
client: non-target reads are ejected with unblock_read, and no more data is
requested for any decided read.
"""
from __future__ import annotations

import gc
import heapq
import time
from dataclasses import dataclass

import numpy as np

from . import synth


@dataclass
class ServeConfig:
    channels: int = 512
    chunk: int = 1600
    period_s: float = 0.4
    read_rate: float = 1.0          # read starts per second per channel
    chunks_per_read: int = 3        # chunks available per read (and max before deciding)
    duration_s: float = 10.0        # measured window
    warmup_s: float = 2.0
    target_fraction: float = 0.5
    pool_reads: int = 1024
    seed: int = 7


def make_pool(genome: bytes, other: bytes, table, cfg: ServeConfig, held_out: bool = False, n: int = 0):
    """Reads the simulated sequencer serves.  held_out=True draws a separate
    set from the same generator with other seeds (for calibrating the accept /
    reject rates on reads that are never served)."""
    n = n or cfg.pool_reads
    seed = cfg.seed + (1000 if held_out else 0)
    rng = np.random.default_rng(seed)
    mask = (rng.random(n) < cfg.target_fraction).astype(np.int8)
    reads = synth.simulate_reads(genome, other, table, [cfg.chunk * cfg.chunks_per_read] * n, mask,
                                 seed=seed + 1)
    return reads


def calibrate(clf, reads, cfg: ServeConfig, n: int = 256):
    """Per-sample accept / reject rates from the first chunk of n reads,
    classified offline: accept below the lowest non-target rate, reject above
    the highest target rate (so one chunk decides every read the data
    separates, and ambiguous reads get more chunks).  Pass reads that are not
    served (make_pool(..., held_out=True)) for a held-out call accuracy."""
    n = min(n, reads.n)
    first = [reads.read(i)[: cfg.chunk] for i in range(n)]
    res = clf.classify(first)
    per = res["score"] / cfg.chunk
    t = reads.target[:n] == 1
    if t.any() and (~t).any():
        accept = float(min(per[~t].min(), np.quantile(per[t], 0.99)))
        reject = float(max(per[t].max(), np.quantile(per[~t], 0.01)))
    else:
        accept, reject = float(np.median(per)), 0.0
    return accept, reject


class SimulatedSequencer:
    def __init__(self, reads, cfg: ServeConfig):
        self.reads = reads
        self.cfg = cfg
        self.rng = np.random.default_rng(cfg.seed + 2)
        self.events = []            # (time_s, channel, generation)
        self.gen = [0] * cfg.channels  # events of older generations are stale
        self.active = {}            # channel -> [read_number, pool index, next chunk k]
        self.next_read = 1
        self.truth = {}             # read_number -> target flag
        t0 = 0.0
        for ch in range(cfg.channels):
            heapq.heappush(self.events, (t0 + self.rng.exponential(1.0 / cfg.read_rate), ch, 0))

    def due(self, now_s: float):
        """Chunks whose arrival time has come: (arrival_s, channel, read_number, samples, is_last)."""
        out = []
        cfg = self.cfg
        while self.events and self.events[0][0] <= now_s:
            t, ch, g = heapq.heappop(self.events)
            if g != self.gen[ch]:
                continue
            st = self.active.get(ch)
            if st is None:  # a new read starts on this channel
                idx = int(self.rng.integers(0, self.reads.n))
                st = [self.next_read, idx, 0]
                self.truth[self.next_read] = int(self.reads.target[idx])
                self.next_read += 1
                self.active[ch] = st
            rn, idx, k = st
            x = self.reads.read(idx)[k * cfg.chunk:(k + 1) * cfg.chunk]
            last = k + 1 >= cfg.chunks_per_read
            out.append((t, ch, rn, x, last))
            st[2] += 1
            if not last:
                heapq.heappush(self.events, (t + cfg.period_s, ch, g))
            else:
                self.active.pop(ch)
                heapq.heappush(self.events, (t + cfg.period_s + self.rng.exponential(1.0 / cfg.read_rate), ch, g))
        return out

    def reads_started(self) -> int:
        return self.next_read - 1

    def decided(self, ch: int, rn: int, now_s: float, call: int = -1):
        """The library decided read rn: the sequencer stops sending its chunks
        (ejected, or no more chunks needed) and the channel starts a new read
        after an exponential gap."""
        st = self.active.get(ch)
        if st is not None and st[0] == rn:
            self.active.pop(ch)
            self.gen[ch] += 1  # the channel's pending chunk event is dropped
            heapq.heappush(self.events, (now_s + self.rng.exponential(1.0 / self.cfg.read_rate), ch, self.gen[ch]))


class ReadUntilClientSource:
    """Chunks from a live Read Until client, in place of the reference's FIFO
    bridge (src/ReadUntil/ont_readuntil.py:29-59, which pipes raw chunks to
    src/ru_main.cu and ejects every read it sees).

    `client` follows the read_until package's ReadUntilClient
    (read_until/base.py:344-378): `is_running`, `get_read_chunks(batch_size,
    last)` yielding (channel, read) with `read.number` and `read.raw_data`,
    `signal_dtype`, `unblock_read(channel, read_number, duration)` and
    `stop_receiving_read(channel, read_number)`.  Calibrated (float) signal is
    used as it comes; integer ADC signal needs `calibration(channel) ->
    (offset, range, digitisation)` and is scaled to pA as
    (raw + offset) * range / digitisation.

    The library's decision drives the client:
    * a target keeps sequencing and gets stop_receiving_read;
    * a non-target (early or final) gets unblock_read, then
      stop_receiving_read.
    Chunks of a decided read that were already queued are dropped.  A read's
    `max_chunks`-th chunk is marked last, so the library decides it there."""

    def __init__(self, client, batch_size: int = 512, max_chunks: int = 3, unblock_duration: float = 0.1,
                 calibration=None):
        self.client = client
        self.batch_size = batch_size
        self.max_chunks = max_chunks
        self.unblock_duration = unblock_duration
        self.calibration = calibration
        self.seen = {}        # (channel, read_number) -> chunks submitted
        self.done = set()     # decided (channel, read_number)
        self.truth = {}       # unknown for live reads
        self.started = 0
        self.actions = {"unblock": 0, "stop": 0}

    def reads_started(self) -> int:
        return self.started

    def _samples(self, channel, read) -> np.ndarray:
        dt = np.dtype(self.client.signal_dtype)
        x = np.frombuffer(read.raw_data, dt)
        if dt.kind in "iu":
            if self.calibration is None:
                raise ValueError("integer signal needs calibration(channel) -> (offset, range, digitisation)")
            off, rng_, digi = self.calibration(channel)
            return ((x.astype(np.float32) + np.float32(off)) * np.float32(rng_ / digi)).astype(np.float32)
        return x.astype(np.float32, copy=False)

    def due(self, now_s: float):
        out = []
        if not self.client.is_running:
            return out
        for channel, read in self.client.get_read_chunks(batch_size=self.batch_size, last=True):
            key = (channel, read.number)
            if key in self.done:
                continue
            k = self.seen.get(key, 0)
            if k >= self.max_chunks:
                continue
            if k == 0:
                self.started += 1
            self.seen[key] = k + 1
            x = self._samples(channel, read)
            if x.size:
                out.append((now_s, channel, read.number, x, k + 1 >= self.max_chunks))
        return out

    def decided(self, ch: int, rn: int, now_s: float, call: int = -1):
        key = (ch, rn)
        if key in self.done:
            return
        self.done.add(key)
        self.seen.pop(key, None)
        if call != 1:
            self.client.unblock_read(ch, rn, duration=self.unblock_duration)
            self.actions["unblock"] += 1
        self.client.stop_receiving_read(ch, rn)
        self.actions["stop"] += 1


def run(clf, reads, cfg: ServeConfig, accept: float, reject: float, state_budget_bytes: float = 0.0,
        max_in_flight: int = 0, drain: bool = False, sequencer: "SimulatedSequencer | None" = None) -> dict:
    """Real-time serving loop for warmup + duration seconds.  Returns the
    measured-window statistics.  Work still queued at the end is dropped
    unless `drain` (an overloaded configuration can hold minutes of it).
    `sequencer` defaults to a SimulatedSequencer over `reads`."""
    from . import now_ms

    # serving batches hold a few chunk-steps each: tune the launch shape for them
    for k in (1, 2, 4):
        clf.autotune(k, cfg.chunk)
    clf.serve_start(max_in_flight=max_in_flight, state_budget_bytes=state_budget_bytes,
                    chunks_per_decision=cfg.chunks_per_read, accept_per_sample=accept, reject_per_sample=reject)
    seq = sequencer if sequencer is not None else SimulatedSequencer(reads, cfg)
    # no garbage-collector pauses inside the real-time loop
    gc_was_on = gc.isenabled()
    gc.disable()
    try:
        rec = _loop(clf, seq, cfg, drain)
    finally:
        if gc_was_on:
            gc.enable()
    rec["accept_per_sample"], rec["reject_per_sample"] = accept, reject
    return rec


def _loop(clf, seq, cfg: ServeConfig, drain: bool) -> dict:
    from . import now_ms

    t_base = now_ms()
    lat, queue, calls, truth = [], [], [], []
    decided_in_window = 0
    chunks_in_window = 0
    end_s = cfg.warmup_s + cfg.duration_s
    st0 = None
    while True:
        now_s = (now_ms() - t_base) / 1e3
        if now_s >= end_s:
            break
        if st0 is None and now_s >= cfg.warmup_s:
            st0 = clf.stats()
        for (t, ch, rn, x, last) in seq.due(now_s):
            clf.submit_chunk(ch, rn, x, is_last=last, arrival_ms=t_base + t * 1e3)
            if t >= cfg.warmup_s:
                chunks_in_window += 1
        clf.serve_step()
        for d in clf.poll_decisions(8192):
            if d["decided"]:
                seq.decided(d["channel"], d["read_number"], now_s, d["call"])
                if now_s >= cfg.warmup_s:
                    decided_in_window += 1
                    lat.append(d["latency_ms"])
                    queue.append(d["queue_ms"])
                    calls.append(d["call"])
                    truth.append(seq.truth.get(d["read_number"], -1))
        time.sleep(0.00005)
    st = clf.stats()
    if drain:
        clf.serve_drain()
    lat = np.asarray(lat)
    queue = np.asarray(queue)
    calls = np.asarray(calls)
    truth = np.asarray(truth)
    known = truth >= 0  # reads of a live client have no ground truth
    acc = float((calls[known] == truth[known]).mean()) if known.any() else float("nan")
    return {
        "channels": cfg.channels, "chunk_samples": cfg.chunk, "duration_s": cfg.duration_s,
        "reads_per_s": decided_in_window / cfg.duration_s,
        "chunks_per_s": chunks_in_window / cfg.duration_s,
        # chunk-steps the GPU aligned per second in the window (offered load is chunks_per_s)
        "chunks_processed_per_s": (st["chunks_processed"] - (st0 or st)["chunks_processed"]) / cfg.duration_s,
        "p50_latency_ms": float(np.percentile(lat, 50)) if lat.size else None,
        "p99_latency_ms": float(np.percentile(lat, 99)) if lat.size else None,
        "max_latency_ms": float(lat.max()) if lat.size else None,
        # latency = queue (arrival -> batch launch) + batch on the device + harvest
        "p50_queue_ms": float(np.percentile(queue, 50)) if queue.size else None,
        "p99_queue_ms": float(np.percentile(queue, 99)) if queue.size else None,
        "p99_after_launch_ms": float(np.percentile(lat - queue, 99)) if lat.size else None,
        "call_accuracy": acc,
        "mean_batch_reads": st["mean_batch_reads"], "batches": st["batches"],
        "mean_batch_ms": st["mean_batch_ms"], "max_batch_ms": st["max_batch_ms"],
        "reads_deferred": st["reads_deferred"], "max_in_flight": st["max_in_flight"],
        "reads_started": seq.reads_started(),
        "deferred_fraction": st["reads_deferred"] / max(seq.reads_started(), 1),
        "queue_depth_end": st["queue_depth"],
        "state_bytes": st["state_bytes"],
    }
