"""CPU checks of the FP64 model of the reference kernel's evaluation order
(oracle.sdtw_refkernel) and of the host-side layout used to run the
reference's own kernel (oracle/ref_kernel.py)."""
import os

import numpy as np
import pytest

from dtwax_gb300 import synth

TILE = 832


@pytest.mark.parametrize("tiles", [2, 3, 5])
def test_tile_order_without_departures_is_the_recurrence(oracle, tiles):
    rng = np.random.default_rng(tiles)
    ref = rng.standard_normal(tiles * TILE)
    for n in (1024, 2048, 3072):
        q = rng.standard_normal(n)
        assert oracle.sdtw_refkernel(ref, q, 0) == oracle.sdtw(ref, q)[0]
        assert oracle.sdtw_refkernel(ref, q, oracle.REFK_REF_DEL) == oracle.sdtw_ref_del(ref, q)[0]


def test_ref_del_oracle_matches_numpy(oracle):
    """The C REF_DEL recurrence against the plain numpy loop, and the left
    term can only lower a score."""
    rng = np.random.default_rng(11)
    for m, n in ((40, 7), (300, 50), (1000, 120)):
        ref = rng.standard_normal(m)
        q = rng.standard_normal(n)
        s, j = oracle.sdtw_ref_del(ref, q)
        s_np, j_np, _ = oracle.np_sdtw(ref, q, ref_del=True)
        assert s == pytest.approx(s_np, rel=1e-12) and j == j_np
        assert s <= oracle.sdtw(ref, q)[0]
        init = rng.random(m) * 5
        s2, _, row = oracle.sdtw_ref_del(ref, q, init_row=init, want_row=True)
        s2_np, _, row_np = oracle.np_sdtw(ref, q, init_row=init, ref_del=True)
        np.testing.assert_allclose(row, row_np, rtol=1e-12)


def test_each_departure_acts_where_expected(oracle):
    """An alignment that enters tile 2 diagonally at row 1,024 (start 640) is
    cut by the chunk-seam diagonal; one that enters tile 2's column 26 there
    (start 666) by the lane-1 diagonal; one that crosses the tile edge at a
    row of 962..992 (start 694) by the seam shift."""
    g = synth.random_genome(5 * TILE + 5, 1)
    fwd, _ = oracle.build_levels(g, np.asarray(synth.level_table(), np.float64))
    rng = np.random.default_rng(3)
    cases = {640: oracle.REFK_CHUNK_SEAM_DIAG, 666: oracle.REFK_CHUNK_LANE1_DIAG, 694: oracle.REFK_SEAM_SHIFT}
    for s, bit in cases.items():
        q = fwd[s:s + 2048] + 0.2 * rng.standard_normal(2048)
        exact = oracle.sdtw(fwd, q)[0]
        assert oracle.sdtw_refkernel(fwd, q, 0) == exact
        assert oracle.sdtw_refkernel(fwd, q, bit) > 1.1 * exact
        for other in set(cases.values()) - {bit}:
            assert oracle.sdtw_refkernel(fwd, q, other) == exact


def test_departures_never_lower_a_score(oracle):
    g = synth.random_genome(4 * TILE + 5, 7)
    o = synth.random_genome(4 * TILE + 5, 8)
    table = synth.level_table()
    fwd, _ = oracle.build_levels(g, np.asarray(table, np.float64))
    reads = synth.simulate_reads(g, o, table, [2048] * 12, (np.arange(12) % 2).astype(np.int8), seed=9)
    q = np.stack([oracle.zscore(reads.read(i).astype(np.float64), 1e-4) for i in range(reads.n)])
    exact = oracle.sdtw_refkernel_batch(fwd, q, 0)
    model = oracle.sdtw_refkernel_batch(fwd, q, oracle.REFK_ALL)
    np.testing.assert_array_equal(exact, [oracle.sdtw(fwd, x)[0] for x in q])
    assert (model >= exact).all()


def test_bad_shapes_give_nan(oracle):
    assert np.isnan(oracle.sdtw_refkernel(np.zeros(TILE), np.zeros(1024), 0))       # one tile
    assert np.isnan(oracle.sdtw_refkernel(np.zeros(2 * TILE + 1), np.zeros(1024), 0))
    assert np.isnan(oracle.sdtw_refkernel(np.zeros(2 * TILE), np.zeros(1000), 0))


def test_tile_interleave_is_the_reference_host_layout():
    from oracle import ref_kernel as RK
    tiles = 3
    cols = np.arange(tiles * TILE + 100, dtype=np.uint32)
    h = RK.tile_interleave(cols, tiles)
    # main.cu:93-109: h[l*832 + i*32 + j] = tmp[l*832 + j*26 + i]
    for l in range(tiles):
        for i in range(26):
            for j in range(32):
                assert h[l * TILE + i * 32 + j] == cols[l * TILE + j * 26 + i]
    np.testing.assert_array_equal(h[tiles * TILE:], cols[tiles * TILE:])


def test_half2_words():
    from oracle import ref_kernel as RK
    w = RK._half2_bits(np.array([1.0, -2.0], np.float32), np.array([0.5, np.inf], np.float32))
    assert w[0] == (0x3C00 | (0x3800 << 16))
    assert w[1] == (0xC000 | (0x7C00 << 16))


def test_reference_kernel_cubins_build():
    """Where the reference's sources are present the harness compiles every
    geometry (device code only, no GPU needed)."""
    from oracle import ref_kernel as RK
    if not RK.sources_present():
        pytest.skip("reference sources not present")
    paths = RK.build()
    for p in paths:
        assert os.path.getsize(p) > 0
