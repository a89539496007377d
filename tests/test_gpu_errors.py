"""Device-side error status on every entry point, and a bounded wait that runs out.

Every TMA wait of the sweep is bounded: after a number of polls the warp gives
up, sets a device error flag and leaves with no copy in flight.  The library's
test hook (dtwx_debug_stall_next) withholds one work item's first
reference-strip copy, so that item's wait can only run out; nothing faults or
hangs.  Checked here through the C ABI:

* the host entry point (dtwx_classify_batch) returns DTWX_E_TIMEOUT;
* the device entry points (dtwx_classify_device, dtwx_distances) mark every
  result of the call with DTWX_CALL_DEVICE_ERROR and dtwx_sync returns
  DTWX_E_TIMEOUT, once;
* the next call on the same handle returns the same results as before the
  stall (the reference's own error convention is print-and-exit,
  src/include/hpc_helpers.hpp:103-113, so there is nothing to resume there).
"""
import time

import numpy as np
import pytest

from gpu_util import make_classifier, reads_of_lengths, small_genome
from dtwax_gb300 import synth

pytestmark = pytest.mark.gpu

E_TIMEOUT = -6
SPIN = 4096  # polls before the stalled wait gives up


@pytest.fixture(scope="module")
def case(built_lib):
    genome = small_genome(60_000, 31)
    other = small_genome(60_000, 32)
    table = synth.level_table()
    reads = reads_of_lengths(genome, other, table, [1500, 900, 2000, 1200, 64, 1700], seed=9)
    return genome, table, reads


def _same(a, b):
    np.testing.assert_array_equal(a["score"], b["score"])
    np.testing.assert_array_equal(a["end_pos"], b["end_pos"])
    np.testing.assert_array_equal(a["strand"], b["strand"])
    np.testing.assert_array_equal(a["call"], b["call"])


def test_host_entry_reports_timeout_and_recovers(case):
    import dtwax_gb300 as d
    genome, table, reads = case
    with make_classifier(genome, table, precision=d.FP16) as clf:
        want = clf.classify(raw=reads.raw, offsets=reads.offsets)
        assert (want["call"] >= 0).all()
        clf.debug_stall_next(0, SPIN)
        t = time.perf_counter()
        with pytest.raises(d.DtwxError) as ei:
            clf.classify(raw=reads.raw, offsets=reads.offsets)
        stalled_ms = (time.perf_counter() - t) * 1e3
        assert ei.value.code == E_TIMEOUT
        print(f"\nstalled call with a {SPIN}-poll limit: {stalled_ms:.1f} ms")
        _same(clf.classify(raw=reads.raw, offsets=reads.offsets), want)


@pytest.mark.parametrize("entry", ["classify_device", "distances"])
def test_device_entries_mark_results_and_sync_reports(case, entry):
    import torch
    import dtwax_gb300 as d
    genome, table, reads = case
    n = reads.n
    with make_classifier(genome, table, precision=d.FP16) as clf:
        if entry == "classify_device":
            src = torch.tensor(reads.raw, device="cuda")
            offsets = reads.offsets
        else:
            z = [((x - x.mean()) / np.sqrt(x.var() + 1e-4)).astype(np.float32)
                 for x in (reads.read(i).astype(np.float64) for i in range(n))]
            src = torch.tensor(np.concatenate(z), device="cuda")
            offsets = reads.offsets
        call = getattr(clf, entry)
        stream = torch.cuda.Stream()

        def run():
            out = torch.zeros(32 * n, dtype=torch.uint8, device="cuda")
            call(src.data_ptr(), offsets, out.data_ptr(), stream.cuda_stream)
            stream.synchronize()
            return np.frombuffer(out.cpu().numpy().tobytes(), d.RESULT_DTYPE).copy()

        want = run()
        clf.sync()
        assert (want["call"] >= 0).all()

        clf.debug_stall_next(0, SPIN)
        bad = run()
        assert (bad["call"] == d.CALL_DEVICE_ERROR).all()
        assert (bad["strand"] == 1).all()  # the timeout bit
        assert np.isnan(bad["score"]).all()
        with pytest.raises(d.DtwxError) as ei:
            clf.sync()
        assert ei.value.code == E_TIMEOUT
        clf.sync()  # reported once

        again = run()
        clf.sync()
        _same(again, want)


def test_offsets_before_the_buffer_are_refused(case):
    """A negative first offset would start a read before the caller's buffer:
    every handle entry point refuses it with DTWX_E_ARG before any device
    work, and the handle keeps working."""
    import torch
    import dtwax_gb300 as d
    genome, table, reads = case
    bad = reads.offsets - 5
    with make_classifier(genome, table, precision=d.FP16) as clf:
        want = clf.classify(raw=reads.raw, offsets=reads.offsets)
        d_raw = torch.tensor(reads.raw, dtype=torch.float32, device="cuda")
        d_q = torch.zeros(reads.raw.size, dtype=torch.float32, device="cuda")
        d_out = torch.zeros(32 * reads.n, dtype=torch.uint8, device="cuda")
        calls = {"classify": lambda: clf.classify(raw=reads.raw, offsets=bad),
                 "classify_device": lambda: clf.classify_device(d_raw.data_ptr(), bad, d_out.data_ptr()),
                 "distances": lambda: clf.distances(d_q.data_ptr(), bad, d_out.data_ptr()),
                 "normalize": lambda: clf.normalize(d_raw.data_ptr(), bad, d_q.data_ptr())}
        for name, call in calls.items():
            with pytest.raises(d.DtwxError) as ei:
                call()
            assert ei.value.code == -1, name
            assert "start at 0" in str(ei.value), name
        torch.cuda.synchronize()
        _same(clf.classify(raw=reads.raw, offsets=reads.offsets), want)
