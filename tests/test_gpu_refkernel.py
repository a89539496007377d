"""The reference's own sDTW kernel beside this library's, on the same inputs.

FullDTW::DTW (src/include/DTW.cu:151-572 of the reference) is compiled from
the reference's sources into oracle/_ref/*.cubin and launched through the
driver API (oracle/ref_kernel.py).  These tests need those cubins: they are
built wherever the reference's sources are present and travel with the
repository.

1. The FP64 model of the reference kernel's evaluation order
   (oracle.sdtw_refkernel: 832-column tiles, 1,024-row query chunks and the
   kernel's three departures from the recurrence) reproduces the kernel: the
   FP32 build within 1e-5, the FP16 build within its accumulation error.
   Crafted reads whose alignment crosses a tile edge at the rows where a
   departure acts show that each departure is real on the GPU: dropping any
   one of them from the model misses the kernel by more than 10 %.
2. On identical inputs (a genome of whole tiles, 2,048-sample reads, the same
   z-scored levels) this library's FP16 calls agree with the reference
   kernel's FP16 calls and with the FP64 oracle at the FP64-tuned threshold on
   >= 99.9 % of reads (the target the precision study also holds).
   The reference kernel reports no end column, so end columns are compared
   with the FP64 oracle only.
Run with -s for the tables.
"""
import numpy as np
import pytest

from dtwax_gb300 import synth, threshold
from gpu_util import make_classifier

pytestmark = pytest.mark.gpu

RK = pytest.importorskip("oracle.ref_kernel")
TILE = 832
QLEN = 2048
NOISE = 0.2          # crafted reads: the strand's levels plus N(0, 0.2) per sample
CRAFTED = (640, 666, 694, 1472)   # alignment start column; see test 1


def need(name):
    if not RK.available(name):
        pytest.skip(f"{RK.cubin_path(name)} is not built (the reference's sources were absent at build time)")


def zscore_reads(oracle, reads):
    return np.stack([oracle.zscore(reads.read(i).astype(np.float64), 1e-4) for i in range(reads.n)]
                    ).astype(np.float32)


@pytest.fixture(scope="module")
def small(built_lib, oracle):
    """5-tile genome (4,165 bases -> 4,160 columns per strand), 16 simulated
    reads of 2,048 samples and the crafted reads."""
    g = synth.random_genome(5 * TILE + 5, 1)
    o = synth.random_genome(5 * TILE + 5, 2)
    table = synth.level_table()
    with make_classifier(g, table, precision=1) as clf:
        fwd, rev = clf.reference()
    assert fwd.size == 5 * TILE
    reads = synth.simulate_reads(g, o, table, [QLEN] * 16, (np.arange(16) % 2 == 0).astype(np.int8), seed=5)
    z = zscore_reads(oracle, reads)
    rng = np.random.default_rng(3)
    crafted = np.stack([fwd[s:s + QLEN] + NOISE * rng.standard_normal(QLEN) for s in CRAFTED]).astype(np.float32)
    # FP32 concatenated strands: one more read across the forward/reverse junction
    cat = np.concatenate([fwd, rev])
    junction = (cat[fwd.size - 1000: fwd.size - 1000 + QLEN] + NOISE * rng.standard_normal(QLEN)).astype(np.float32)
    return fwd, rev, z, crafted, junction


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-12)


def test_refkernel_fp32_matches_model(small, oracle):
    need("fp32_8320")
    fwd, rev, z, crafted, junction = small
    cat = np.concatenate([fwd, rev]).astype(np.float64)
    q = np.concatenate([z, crafted, junction[None]])
    with RK.RefKernel("fp32_8320") as k:
        d_ref = k.reference(fwd, rev)
        got = k.run(d_ref, q)
        got10 = k.run(d_ref, q, reads_per_launch=RK.BLOCK_NUM)
    np.testing.assert_array_equal(got, got10)  # main.cu's 10-read launches give the same bits
    model = oracle.sdtw_refkernel_batch(cat, q.astype(np.float64), oracle.REFK_ALL)
    exact = oracle.sdtw_refkernel_batch(cat, q.astype(np.float64), 0)
    e = rel(got, model)
    print(f"\nFP32 reference kernel vs FP64 model: max rel {e.max():.2e}; vs exact recurrence: "
          f"max rel {rel(got, exact).max():.2e}")
    assert e.max() <= 1e-5
    nz = len(z)
    # each departure is needed to explain the kernel on some crafted read
    for bit in (oracle.REFK_CHUNK_SEAM_DIAG, oracle.REFK_CHUNK_LANE1_DIAG, oracle.REFK_SEAM_SHIFT):
        without = oracle.sdtw_refkernel_batch(cat, crafted.astype(np.float64), oracle.REFK_ALL ^ bit)
        assert (rel(got[nz:nz + len(crafted)], without) > 0.1).any(), bit


def test_refkernel_fp32_at_the_1mb_geometry(built_lib, oracle):
    """The FP32 geometry the benchmark's reference arm times one read per
    launch (a 1 Mb genome, fwd and rev concatenated, 2,404 tiles) computes the
    kernel's recurrence there too: a target and a non-target read, each in its
    own launch, against the FP64 model within 1e-5."""
    need("fp32_2000128")
    g = synth.random_genome(1_000_000, 1)
    o = synth.random_genome(1_000_000, 2)
    table = synth.level_table()
    with make_classifier(g, table, precision=1) as clf:
        fwd, rev = clf.reference()
    reads = synth.simulate_reads(g, o, table, [QLEN] * 2, np.array([1, 0], np.int8), seed=5)
    z = zscore_reads(oracle, reads)
    with RK.RefKernel("fp32_2000128") as k:
        got = k.run(k.reference(fwd, rev), z, reads_per_launch=1)
        half = k.ref_len // 2
    cat = np.full(2 * half, np.inf)
    cat[: fwd.size] = fwd
    cat[half: half + rev.size] = rev
    model = oracle.sdtw_refkernel_batch(cat, z.astype(np.float64), oracle.REFK_ALL)
    print(f"\nFP32 reference kernel, 1 Mb geometry: scores {got}, max rel vs model {rel(got, model).max():.2e}")
    assert rel(got, model).max() <= 1e-5
    assert got[0] < got[1]  # the target read scores lower


def test_refkernel_fp16_matches_model(small, oracle):
    need("fp16_4160")
    fwd, rev, z, crafted, _ = small
    q = np.concatenate([z, crafted])
    with RK.RefKernel("fp16_4160") as k:
        d_ref = k.reference(fwd, rev)
        gf, gr = k.run(d_ref, q)
        gf10, gr10 = k.run(d_ref, q, reads_per_launch=RK.BLOCK_NUM)
    np.testing.assert_array_equal(gf, gf10)
    np.testing.assert_array_equal(gr, gr10)
    # the kernel stores the levels as half: model them the same way
    f16 = fwd.astype(np.float16).astype(np.float64)
    r16 = rev.astype(np.float16).astype(np.float64)
    q16 = q.astype(np.float16).astype(np.float64)
    mf = oracle.sdtw_refkernel_batch(f16, q16, oracle.REFK_ALL)
    mr = oracle.sdtw_refkernel_batch(r16, q16, oracle.REFK_ALL)
    ef, er = rel(gf, mf), rel(gr, mr)
    print(f"\nFP16 reference kernel vs FP64 model (half inputs): fwd max rel {ef.max():.2e} "
          f"(mean signed {np.mean((gf - mf) / mf):+.2e}), rev max rel {er.max():.2e}")
    assert max(ef.max(), er.max()) <= 0.08
    nz = len(z)
    for bit in (oracle.REFK_CHUNK_SEAM_DIAG, oracle.REFK_CHUNK_LANE1_DIAG, oracle.REFK_SEAM_SHIFT):
        without = oracle.sdtw_refkernel_batch(f16, q16[nz:], oracle.REFK_ALL ^ bit)
        assert (rel(gf[nz:], without) > 0.1).any(), bit


def test_concat_mode_matches_refkernel_fp32(small, oracle, built_lib):
    """This library's FP32 concatenated-strand mode (the reference's FP32
    layout, load_reference.hpp:36-37) against the reference's FP32 kernel on
    reads whose best alignment avoids the departures."""
    need("fp32_8320")
    import dtwax_gb300 as d
    fwd, rev, z, _, _ = small
    g = synth.random_genome(5 * TILE + 5, 1)
    o = synth.random_genome(5 * TILE + 5, 2)
    table = synth.level_table()
    reads = synth.simulate_reads(g, o, table, [QLEN] * 16, (np.arange(16) % 2 == 0).astype(np.int8), seed=5)
    with make_classifier(g, table, precision=d.FP32, strand_mode=d.STRANDS_CONCAT) as clf:
        ours = clf.classify(raw=reads.raw, offsets=reads.offsets)["score"]
    cat = np.concatenate([fwd, rev]).astype(np.float64)
    exact = oracle.sdtw_refkernel_batch(cat, z.astype(np.float64), 0)
    model = oracle.sdtw_refkernel_batch(cat, z.astype(np.float64), oracle.REFK_ALL)
    with RK.RefKernel("fp32_8320") as k:
        theirs = k.run(k.reference(fwd, rev), z)
    same = model == exact
    print(f"\nconcat FP32: {same.sum()} of {same.size} reads unaffected by the departures; "
          f"ours vs reference kernel max rel {rel(ours[same], theirs[same]).max():.2e}")
    assert rel(ours, exact).max() <= 1e-5
    assert rel(ours[same], theirs[same]).max() <= 2e-5


def test_refkernel_ref_del_matches_model(small, oracle):
    """The reference kernel built without -DNO_REF_DEL (left predecessor,
    DTW.cu:23-29) against the same FP64 model with the REF_DEL switch: FP32
    within 1e-5, FP16 within its accumulation error; without the switch the
    model misses the kernel."""
    need("fp32_8320_rd")
    need("fp16_4160_rd")
    fwd, rev, z, crafted, junction = small
    cat = np.concatenate([fwd, rev]).astype(np.float64)
    q = np.concatenate([z, crafted, junction[None]])
    with RK.RefKernel("fp32_8320_rd") as k:
        got = k.run(k.reference(fwd, rev), q)
    model = oracle.sdtw_refkernel_batch(cat, q.astype(np.float64), oracle.REFK_ALL | oracle.REFK_REF_DEL)
    no_left = oracle.sdtw_refkernel_batch(cat, q.astype(np.float64), oracle.REFK_ALL)
    e = rel(got, model)
    print(f"\nREF_DEL FP32 reference kernel vs FP64 model: max rel {e.max():.2e}; "
          f"vs the model without the left term: max rel {rel(got, no_left).max():.2e}")
    assert e.max() <= 1e-5
    assert (rel(got, no_left) > 1e-3).any()
    q16s = np.concatenate([z, crafted])
    with RK.RefKernel("fp16_4160_rd") as k:
        gf, gr = k.run(k.reference(fwd, rev), q16s)
    f16 = fwd.astype(np.float16).astype(np.float64)
    r16 = rev.astype(np.float16).astype(np.float64)
    q16 = q16s.astype(np.float16).astype(np.float64)
    mf = oracle.sdtw_refkernel_batch(f16, q16, oracle.REFK_ALL | oracle.REFK_REF_DEL)
    mr = oracle.sdtw_refkernel_batch(r16, q16, oracle.REFK_ALL | oracle.REFK_REF_DEL)
    e16 = max(rel(gf, mf).max(), rel(gr, mr).max())
    print(f"REF_DEL FP16 reference kernel vs FP64 model (half inputs): max rel {e16:.2e}")
    assert e16 <= 0.08


def test_ref_del_concat_matches_refkernel_fp32(small, oracle, built_lib):
    """This library's REF_DEL FP32 cells on the concatenated strands against
    the reference's REF_DEL FP32 kernel, on reads the departures leave alone."""
    need("fp32_8320_rd")
    import dtwax_gb300 as d
    fwd, rev, z, _, _ = small
    g = synth.random_genome(5 * TILE + 5, 1)
    o = synth.random_genome(5 * TILE + 5, 2)
    table = synth.level_table()
    reads = synth.simulate_reads(g, o, table, [QLEN] * 16, (np.arange(16) % 2 == 0).astype(np.int8), seed=5)
    with make_classifier(g, table, precision=d.FP32, strand_mode=d.STRANDS_CONCAT, recurrence=d.REF_DEL) as clf:
        ours = clf.classify(raw=reads.raw, offsets=reads.offsets)["score"]
    cat = np.concatenate([fwd, rev]).astype(np.float64)
    exact = oracle.sdtw_refkernel_batch(cat, z.astype(np.float64), oracle.REFK_REF_DEL)
    model = oracle.sdtw_refkernel_batch(cat, z.astype(np.float64), oracle.REFK_ALL | oracle.REFK_REF_DEL)
    with RK.RefKernel("fp32_8320_rd") as k:
        theirs = k.run(k.reference(fwd, rev), z)
    same = model == exact
    print(f"\nREF_DEL concat FP32: {same.sum()} of {same.size} reads unaffected by the departures; "
          f"ours vs reference kernel max rel {rel(ours[same], theirs[same]).max():.2e}")
    assert rel(ours, exact).max() <= 1e-5
    assert same.sum() >= 8
    assert rel(ours[same], theirs[same]).max() <= 2e-5


@pytest.fixture(scope="module")
def c1_tiles(built_lib, oracle):
    """C1 shape on whole tiles: a 47,429-base genome (47,424 = 57 x 832
    columns per strand, the columns the shipped FP16 geometry scores),
    512 reads x 2,048 samples (256 target, 256 from a second genome)."""
    import dtwax_gb300 as d
    g = synth.random_genome(57 * TILE + 5, synth.GENOME_SEED)
    o = synth.random_genome(57 * TILE + 5, synth.OTHER_SEED)
    table = synth.level_table()
    n = 512
    mask = np.zeros(n, np.int8)
    mask[: n // 2] = 1
    np.random.default_rng(synth.READ_SEED).shuffle(mask)
    reads = synth.simulate_reads(g, o, table, [QLEN] * n, mask, seed=synth.READ_SEED)
    with make_classifier(g, table, precision=d.FP16) as clf:
        ours = clf.classify(raw=reads.raw, offsets=reads.offsets)
        fwd, rev = clf.reference()
    z = zscore_reads(oracle, reads)
    offs = np.arange(n + 1, dtype=np.int64) * QLEN
    sf, ef, sr, er = oracle.sdtw_batch(fwd.astype(np.float64), rev.astype(np.float64),
                                       z.reshape(-1).astype(np.float64), offs)
    with RK.RefKernel("fp16_48128") as k:
        tf, tr = k.run(k.reference(fwd, rev), z)
    f16 = fwd.astype(np.float16).astype(np.float64)
    r16 = rev.astype(np.float16).astype(np.float64)
    q16 = z.astype(np.float16).astype(np.float64)
    mf = oracle.sdtw_refkernel_batch(f16, q16, oracle.REFK_ALL)
    mr = oracle.sdtw_refkernel_batch(r16, q16, oracle.REFK_ALL)
    xf = oracle.sdtw_refkernel_batch(f16, q16, 0)
    xr = oracle.sdtw_refkernel_batch(r16, q16, 0)
    return reads, ours, (sf, ef, sr, er), (tf, tr), (mf, mr), (xf, xr)


def test_c1_calls_agree_with_reference_kernel(c1_tiles, oracle):
    need("fp16_48128")
    reads, ours, (sf, ef, sr, er), (tf, tr), (mf, mr), (xf, xr) = c1_tiles
    score64, end64, strand64 = oracle.combine(sf, ef, sr, er)
    theirs = np.minimum(tf, tr)
    model = np.minimum(mf, mr)
    t = reads.target == 1
    th, acc = threshold.best_threshold(score64[t], score64[~t], plateau="center")
    c64 = threshold.call(score64, th)
    c_ours = threshold.call(ours["score"], th)
    c_theirs = threshold.call(theirs, th)
    th16, acc16 = threshold.best_threshold(theirs[t], theirs[~t])
    rows = {
        "ours FP16 vs FP64": rel(ours["score"], score64),
        "reference FP16 vs FP64": rel(theirs, score64),
        "reference FP16 vs its FP64 model": rel(theirs, model),
    }
    print(f"\nC1 on whole tiles: 512 reads x 2,048 samples vs 2 x 47,424 columns; FP64-tuned threshold "
          f"{th:.3f} ({acc:.2f} %), reference-FP16-tuned {th16:.3f} ({acc16:.2f} %)")
    for k, e in rows.items():
        print(f"  {k:34s} max rel {e.max():.2e}  median rel {np.median(e):.2e}")
    changed = model != np.minimum(xf, xr)
    print(f"  departures change the FP64 score of {changed.sum()} of {changed.size} reads "
          f"(max {rel(model, np.minimum(xf, xr)).max():.2e} relative)")
    exact_end = (ours["end_pos"] == end64) & (ours["strand"] == strand64)
    near_end = (np.abs(ours["end_pos"] - end64) <= 2) & (ours["strand"] == strand64)
    print(f"  ours FP16 end column vs FP64: exact {exact_end.mean():.4f} (targets {exact_end[t].mean():.4f}), "
          f"within 2 columns {near_end.mean():.4f} (targets {near_end[t].mean():.4f})")
    print(f"  call agreement: ours/FP64 {np.mean(c_ours == c64):.4f}, reference/FP64 "
          f"{np.mean(c_theirs == c64):.4f}, ours/reference {np.mean(c_ours == c_theirs):.4f}")
    assert rows["ours FP16 vs FP64"].max() <= 1e-2
    assert rows["reference FP16 vs its FP64 model"].max() <= 0.08
    assert np.mean(c_ours == c64) >= 0.999
    assert np.mean(c_ours == c_theirs) >= 0.999
    # FP16 end columns: within 2 columns of FP64 on the reads that align
    # (targets); the last row holds near ties (adjacent columns within the
    # FP16 error) that rounding may order differently.  FP32 ends are exact
    # (test_gpu_sdtw.py).
    assert near_end[t].mean() >= 0.999


def test_c1_ref_del_calls_agree_with_reference_kernel(oracle, built_lib):
    """The REF_DEL builds side by side on the C1 shape on whole tiles: this
    library's FP16 REF_DEL cells, the reference's FP16 REF_DEL kernel and the
    FP64 REF_DEL oracle call the same reads at the FP64-tuned threshold."""
    need("fp16_48128_rd")
    import dtwax_gb300 as d
    g = synth.random_genome(57 * TILE + 5, synth.GENOME_SEED)
    o = synth.random_genome(57 * TILE + 5, synth.OTHER_SEED)
    table = synth.level_table()
    n = 256
    mask = (np.arange(n) % 2 == 0).astype(np.int8)
    reads = synth.simulate_reads(g, o, table, [QLEN] * n, mask, seed=synth.READ_SEED + 1)
    with make_classifier(g, table, precision=d.FP16, recurrence=d.REF_DEL) as clf:
        ours = clf.classify(raw=reads.raw, offsets=reads.offsets)
        fwd, rev = clf.reference()
    z = zscore_reads(oracle, reads)
    offs = np.arange(n + 1, dtype=np.int64) * QLEN
    sf, ef, sr, er = oracle.sdtw_batch(fwd.astype(np.float64), rev.astype(np.float64),
                                       z.reshape(-1).astype(np.float64), offs, ref_del=True)
    with RK.RefKernel("fp16_48128_rd") as k:
        tf, tr = k.run(k.reference(fwd, rev), z)
    score64 = np.minimum(sf, sr)
    theirs = np.minimum(tf, tr)
    t = reads.target == 1
    th, acc = threshold.best_threshold(score64[t], score64[~t], plateau="center")
    c64, c_ours, c_theirs = (threshold.call(x, th) for x in (score64, ours["score"], theirs))
    e_ours = rel(ours["score"], score64)
    e_theirs = rel(theirs, score64)
    print(f"\nC1 REF_DEL on whole tiles, 256 reads: ours FP16 vs FP64 max rel {e_ours.max():.2e}, reference "
          f"FP16 vs FP64 max rel {e_theirs.max():.2e}; calls ours/FP64 {np.mean(c_ours == c64):.4f}, "
          f"reference/FP64 {np.mean(c_theirs == c64):.4f}, ours/reference {np.mean(c_ours == c_theirs):.4f}")
    assert e_ours.max() <= 1e-2
    assert np.mean(c_ours == c64) >= 0.999 and np.mean(c_ours == c_theirs) >= 0.999
