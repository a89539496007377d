"""dtwx_distances_static, the entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc: processes sharing the GPU with
a basecaller whose memory pool already holds the device, and real-time Read
Until loops that cannot take the device-wide synchronisation an allocation or
free may cause.  Its scratch is one static device array inside the library.

Checked here through the C ABI: two calls in a row return what the regular
device entry point (dtwx_distances, handle-owned scratch) returns for the same
reads, within the FP32 tolerance of the other GPU tests, and what the FP64
oracle gives for the same z-scored reads and reference (1e-5 relative, exact
end columns); no result carries the device-error mark; requests beyond the
array's limits are refused with DTWX_E_CAPACITY, and misaligned buffers with
DTWX_E_ARG.  This file is collected last so that a failure here does not hide
any other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5


def _pairs(fwd, rev):
    m = fwd.size
    cols = -(-m // 512) * 512  # the sweep reads whole 512-column strips
    pairs = np.zeros((cols, 2), np.float32)
    pairs[:m, 0] = fwd
    pairs[:m, 1] = rev
    return pairs


def test_static_scratch_matches_regular_entry(built_lib, oracle):
    import torch
    import dtwax_gb300 as d
    from dtwax_gb300 import synth

    lib = d.load_library()
    genome = synth.random_genome(30_000, 21)
    other = synth.random_genome(30_000, 22)
    table = synth.level_table()
    lengths = [2000, 1500, 2048, 700, 1, 33]
    reads = synth.simulate_reads(genome, other, table, lengths, [1, 0, 1, 0, 1, 0], seed=8)
    # z-scored reads on the host, plus one empty read at the end
    zs = [((x - x.mean()) / np.sqrt(x.var() + 1e-4)).astype(np.float32)
          for x in (reads.read(i).astype(np.float64) for i in range(reads.n))]
    zs.append(np.zeros(0, np.float32))
    offsets = np.concatenate([[0], np.cumsum([z.size for z in zs])]).astype(np.int64)
    n = offsets.size - 1

    with d.Classifier(sequence=genome, level_table=table, precision=d.FP32) as clf:
        fwd, rev = clf.reference()
        stream = torch.cuda.Stream()
        d_q = torch.tensor(np.concatenate(zs), device="cuda")
        d_ref = torch.tensor(_pairs(fwd, rev), device="cuda")
        outs = [torch.zeros(32 * n, dtype=torch.uint8, device="cuda") for _ in range(3)]
        clf.distances(d_q.data_ptr(), offsets, outs[0].data_ptr(), stream.cuda_stream)
        for k in (1, 2):  # two calls in a row on the shared static scratch
            rc = lib.dtwx_distances_static(ctypes.c_void_p(d_ref.data_ptr()), fwd.size,
                                           ctypes.c_void_p(d_q.data_ptr()),
                                           offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n,
                                           ctypes.c_float(clf.cfg.threshold), ctypes.c_void_p(outs[k].data_ptr()),
                                           ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0, lib.dtwx_last_error(None)
        stream.synchronize()
        res = [np.frombuffer(o.cpu().numpy().tobytes(), d.RESULT_DTYPE) for o in outs]

    want = res[0]
    assert want["call"][-1] == -1  # the empty read
    # the FP64 oracle on the very inputs the GPU saw (FP32 reference, FP32 reads)
    sf, ef, sr, er = oracle.sdtw_batch(fwd.astype(np.float64), rev.astype(np.float64),
                                       np.concatenate(zs).astype(np.float64), offsets)
    live = want["n_samples"] > 0
    for got in res[1:]:
        assert (got["call"] != d.CALL_DEVICE_ERROR).all()
        np.testing.assert_allclose(got["score_fwd"][live], sf[live], rtol=FP32_RTOL)
        np.testing.assert_allclose(got["score_rev"][live], sr[live], rtol=FP32_RTOL)
        score, end, strand = oracle.combine(sf, ef, sr, er)
        np.testing.assert_array_equal(got["end_pos"][live], end[live])
        np.testing.assert_array_equal(got["strand"][live], strand[live])
    for got in res[1:]:
        np.testing.assert_allclose(got["score_fwd"], want["score_fwd"], rtol=FP32_RTOL)
        np.testing.assert_allclose(got["score_rev"], want["score_rev"], rtol=FP32_RTOL)
        np.testing.assert_array_equal(got["end_pos"], want["end_pos"])
        np.testing.assert_array_equal(got["strand"], want["strand"])
        np.testing.assert_array_equal(got["call"], want["call"])
        np.testing.assert_array_equal(got["n_samples"], want["n_samples"])


def test_static_scratch_refuses_oversized_requests(built_lib):
    import torch
    import dtwax_gb300 as d

    lib = d.load_library()
    d_ref = torch.zeros(1024, 2, dtype=torch.float32, device="cuda")
    d_q = torch.zeros(8192, dtype=torch.float32, device="cuda")
    d_out = torch.zeros(32 * 4097, dtype=torch.uint8, device="cuda")
    i64p = ctypes.POINTER(ctypes.c_int64)

    too_many = np.arange(4098, dtype=np.int64)  # 4097 reads of one sample
    rc = lib.dtwx_distances_static(ctypes.c_void_p(d_ref.data_ptr()), 1000, ctypes.c_void_p(d_q.data_ptr()),
                                   too_many.ctypes.data_as(i64p), 4097, ctypes.c_float(1.0),
                                   ctypes.c_void_p(d_out.data_ptr()), None)
    assert rc == -7  # DTWX_E_CAPACITY
    assert b"4096" in lib.dtwx_last_error(None)

    too_long = np.array([0, 2049], np.int64)
    rc = lib.dtwx_distances_static(ctypes.c_void_p(d_ref.data_ptr()), 1000, ctypes.c_void_p(d_q.data_ptr()),
                                   too_long.ctypes.data_as(i64p), 1, ctypes.c_float(1.0),
                                   ctypes.c_void_p(d_out.data_ptr()), None)
    assert rc == -7
    assert b"2048" in lib.dtwx_last_error(None)

    one = np.array([0, 100], np.int64)
    rc = lib.dtwx_distances_static(ctypes.c_void_p(d_ref.data_ptr() + 8), 1000, ctypes.c_void_p(d_q.data_ptr()),
                                   one.ctypes.data_as(i64p), 1, ctypes.c_float(1.0),
                                   ctypes.c_void_p(d_out.data_ptr()), None)
    assert rc == -1  # DTWX_E_ARG: the reference pairs are read in 16-byte loads
    assert b"16-byte" in lib.dtwx_last_error(None)

    before = np.array([-5, 100], np.int64)  # would start the read before d_query
    rc = lib.dtwx_distances_static(ctypes.c_void_p(d_ref.data_ptr()), 1000, ctypes.c_void_p(d_q.data_ptr()),
                                   before.ctypes.data_as(i64p), 1, ctypes.c_float(1.0),
                                   ctypes.c_void_p(d_out.data_ptr()), None)
    assert rc == -1 and b"start at 0" in lib.dtwx_last_error(None)
    torch.cuda.synchronize()
