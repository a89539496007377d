"""The library's window + z-score kernel against cuDNN, the arithmetic the
reference's normaliser actually runs.

normalizer::normalize (src/include/normalizer.cu:71-113) z-scores reads x
length samples with cudnnBatchNormalizationForwardTraining (SPATIAL mode over
a (1, reads, length, 1) tensor, scale 1, bias 0, epsilon 1e-4).  The library
restates that from cuDNN's documented formula in its own kernel
(dtwx_normalize, FP64 statistics).  Here both run on the same device buffers:
oracle/cudnn_bn.cpp makes the reference's cuDNN call, and the outputs must
agree to FP32 precision (1e-5) on the reference's own shapes: 10 reads of the
2,048-sample window after the 1,952-sample adapter (main.cu / ru_main.cu
batches, raw 8-bit FIFO samples and int16-range ADC values), and 2,048 reads
of 2,000 pA samples of the precision-study generator.
"""
import numpy as np
import pytest

from dtwax_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def cudnn(built_lib):
    from oracle import cudnn_bn
    if not cudnn_bn.available():
        pytest.skip(f"cuDNN unavailable here: {cudnn_bn.why_unavailable()}")
    return cudnn_bn


def _cudnn_windows(cudnn, windows: np.ndarray) -> np.ndarray:
    import torch
    reads, length = windows.shape
    d_x = torch.tensor(np.ascontiguousarray(windows, np.float32), device="cuda")
    scale = torch.ones(reads, dtype=torch.float32, device="cuda")
    bias = torch.zeros(reads, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    cudnn.normalize(d_x.data_ptr(), reads, length, scale.data_ptr(), bias.data_ptr(), 1e-4)
    torch.cuda.synchronize()
    return d_x.cpu().numpy().reshape(reads, length)


def _ours(raw: np.ndarray, offsets: np.ndarray, **cfg) -> tuple:
    import torch
    import dtwax_gb300 as d
    genome = synth.random_genome(5_000, 3)
    with d.Classifier(sequence=genome, level_table=synth.level_table(), **cfg) as clf:
        d_raw = torch.tensor(raw.astype(np.float32), device="cuda")
        d_q = torch.zeros(max(raw.size, 1), dtype=torch.float32, device="cuda")
        out = clf.normalize(d_raw.data_ptr(), offsets, d_q.data_ptr())
        torch.cuda.synchronize()
        return d_q.cpu().numpy(), out


@pytest.mark.parametrize("kind", ["fifo_u8", "adc_i16"])
def test_reference_window_matches_cudnn(cudnn, kind):
    """10 reads x 5,000 samples; window [1952, 4000) as ADAPTER_LEN / QUERY_LEN
    of the reference (generate_load_squiggle.hpp:412-430)."""
    rng = np.random.default_rng(41 if kind == "fifo_u8" else 42)
    if kind == "fifo_u8":
        raw = rng.integers(0, 256, size=(10, 5000)).astype(np.float32)
    else:
        raw = (rng.normal(500.0, 60.0, size=(10, 5000)) + rng.integers(-20, 20, size=(10, 1))).round()
        raw = raw.astype(np.float32)
    offsets = np.arange(11, dtype=np.int64) * 5000
    ours, out_off = _ours(raw.reshape(-1), offsets, adapter_skip=1952, query_len=2048, require_full=1)
    assert (np.diff(out_off) == 2048).all()
    want = _cudnn_windows(cudnn, raw[:, 1952:4000])
    np.testing.assert_allclose(ours[: 10 * 2048].reshape(10, 2048), want, rtol=TOL, atol=TOL)


def test_precision_study_reads_match_cudnn(cudnn, capsys):
    w = synth.make_workload("C2")
    raw, offsets = w.reads.raw, w.reads.offsets
    ours, out_off = _ours(raw, offsets)
    n, length = w.reads.n, 2000
    want = _cudnn_windows(cudnn, raw.reshape(n, length))
    err = np.abs(ours.reshape(n, length) - want)
    with capsys.disabled():
        print(f"\nnormalize_kernel vs cuDNN {cudnn.version()} batch norm, {n} reads x {length}: "
              f"max abs diff {err.max():.2e}")
    np.testing.assert_allclose(ours.reshape(n, length), want, rtol=TOL, atol=TOL)
