"""CPU models of the REF_DEL kernels' anti-diagonal schedule
(dtwax_gb300/csrc/refdel.cu) against the FP64 REF_DEL oracle: the plain
schedule (FP32 cells) and the same schedule with the FP16-pair kernel's
per-lane frames, both evaluated in FP64.

The model replays the kernel's index arithmetic with a small warp (LANES
lanes of S cells): strips left to right, at step t lane l computes rows
2(t - l) and 2(t - l) + 1, takes its left inputs from lane l-1's last cells of
the previous step (lane 0 from the left strip's seam column, row i at
[i + 1]), takes the diagonal of the pair's first row from the step before,
and keeps its cells when it has no row.  Lane LANES-1 writes the seam column.
The schedule is exact, so the model must equal the plain recurrence (in FP64)
for every read length, including lengths shorter than the warp and odd ones,
and for resumed rows."""
import numpy as np
import pytest

INF = np.inf


def model_refdel(ref, q, lanes=4, S=3, init_row=None):
    m, n = ref.size, q.size
    W = lanes * S
    strips = -(-m // W)
    cols = strips * W
    r = np.full(cols, 0.0)
    r[:m] = ref
    row0 = np.zeros(cols) if init_row is None else np.concatenate([init_row, np.full(cols - m, 0.0)])
    seam_in = np.full(n + 1, INF)
    last_row = np.empty(cols)
    for s in range(strips):
        first = s == 0
        seam_out = np.full(n + 1, INF)
        D = [row0[s * W + l * S: s * W + (l + 1) * S].copy() for l in range(lanes)]
        seam_out[0] = D[lanes - 1][S - 1]
        pairs = (n + 1) // 2
        # values each lane exposes to its right neighbour after a step
        expo_a = [D[l][S - 1] for l in range(lanes)]
        expo_b = [D[l][S - 1] for l in range(lanes)]
        diag_next = [(INF if first else seam_in[0]) if l == 0 else D[l - 1][S - 1] for l in range(lanes)]
        for st in range(pairs + lanes - 1):
            ua = [expo_a[l - 1] if l > 0 else None for l in range(lanes)]
            ub = [expo_b[l - 1] if l > 0 else None for l in range(lanes)]
            for l in range(lanes):
                rr = 2 * (st - l)
                if l == 0:
                    left0 = INF if first or rr + 1 > n else seam_in[rr + 1]
                    left1 = INF if first or rr + 2 > n else seam_in[rr + 2]
                else:
                    left0, left1 = ua[l], ub[l]
                diag0 = diag_next[l]
                diag_next[l] = left1
                ok0, ok1 = 0 <= rr < n, 0 <= rr + 1 < n
                if not ok0:
                    expo_a[l] = INF
                    expo_b[l] = D[l][S - 1]
                    continue
                base = s * W + l * S
                diag1, a_left, b_left, d0 = left0, left0, left1, diag0
                for k in range(S):
                    up = D[l][k]
                    a = (r[base + k] - q[rr]) ** 2 + min(up, d0, a_left)
                    if ok1:
                        b = (r[base + k] - q[rr + 1]) ** 2 + min(a, diag1, b_left)
                        D[l][k] = b
                        b_left = b
                    else:
                        D[l][k] = a
                    d0, a_left, diag1 = up, a, a
                expo_a[l] = a_left
                expo_b[l] = D[l][S - 1]
                if l == lanes - 1:
                    seam_out[rr + 1] = a_left
                    if ok1:
                        seam_out[rr + 2] = D[l][S - 1]
        for l in range(lanes):
            last_row[s * W + l * S: s * W + (l + 1) * S] = D[l]
        seam_in = seam_out
    row = last_row[:m]
    j = int(np.argmin(row))
    return float(row[j]), j, row


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 9, 16, 31])
def test_schedule_matches_recurrence(oracle, n):
    rng = np.random.default_rng(n)
    ref = rng.standard_normal(29)  # 3 strips of 12 columns, the last one partial
    q = rng.standard_normal(n)
    score, end, row = model_refdel(ref, q)
    s_o, e_o, row_o = oracle.sdtw_ref_del(ref, q, want_row=True)
    np.testing.assert_allclose(row, row_o, rtol=1e-12)
    assert score == pytest.approx(s_o, rel=1e-12) and end == e_o


@pytest.mark.parametrize("n", [1, 6, 11])
def test_schedule_resumes_from_a_saved_row(oracle, n):
    rng = np.random.default_rng(100 + n)
    ref = rng.standard_normal(30)
    init = rng.random(30) * 4
    q = rng.standard_normal(n)
    _, _, row = model_refdel(ref, q, lanes=5, S=2, init_row=init)
    _, _, row_o = oracle.sdtw_ref_del(ref, q, init_row=init, want_row=True)
    np.testing.assert_allclose(row, row_o, rtol=1e-12)


def model_refdel_framed(ref, q, lanes=4, S=3, K=2, init_row=None):
    """The same schedule with the FP16 kernel's bookkeeping, in FP64: each lane
    keeps its cells relative to its own frame offset O[l] (its minimum at the
    last rescale, every K steps); a value crossing from lane l-1 is re-based
    by O[l-1] - O[l]; the held diagonal is re-based at a rescale; the seam
    column travels between strips as absolute values."""
    m, n = ref.size, q.size
    W = lanes * S
    strips = -(-m // W)
    cols = strips * W
    r = np.zeros(cols)
    r[:m] = ref
    row0 = np.zeros(cols) if init_row is None else np.concatenate([init_row, np.zeros(cols - m)])
    seam_in = np.full(n + 1, INF)   # absolute values
    last_row = np.empty(cols)
    for s in range(strips):
        first = s == 0
        seam_out = np.full(n + 1, INF)
        absD = [row0[s * W + l * S: s * W + (l + 1) * S].copy() for l in range(lanes)]
        O = [float(x.min()) for x in absD]
        D = [absD[l] - O[l] for l in range(lanes)]
        seam_out[0] = D[lanes - 1][S - 1] + O[lanes - 1]
        pairs = (n + 1) // 2
        expo = [(D[l][S - 1], D[l][S - 1], O[l]) for l in range(lanes)]  # (a, b, frame) after a step
        diag_next = [None] * lanes
        for l in range(lanes):
            if l == 0:
                diag_next[l] = INF if first else seam_in[0] - O[0]
            else:
                diag_next[l] = D[l - 1][S - 1] + O[l - 1] - O[l]
        for st in range(pairs + lanes - 1):
            recv = [expo[l - 1] if l > 0 else None for l in range(lanes)]
            for l in range(lanes):
                rr = 2 * (st - l)
                if l == 0:
                    left0 = INF if first or rr + 1 > n else seam_in[rr + 1] - O[0]
                    left1 = INF if first or rr + 2 > n else seam_in[rr + 2] - O[0]
                else:
                    ua, ub, of = recv[l]
                    left0, left1 = ua + (of - O[l]), ub + (of - O[l])
                diag0 = diag_next[l]
                diag_next[l] = left1
                ok0, ok1 = 0 <= rr < n, 0 <= rr + 1 < n
                a_left = left0
                if ok0:
                    base = s * W + l * S
                    diag1, b_left, d0 = left0, left1, diag0
                    for k in range(S):
                        up = D[l][k]
                        a = (r[base + k] - q[rr]) ** 2 + min(up, d0, a_left)
                        if ok1:
                            b = (r[base + k] - q[rr + 1]) ** 2 + min(a, diag1, b_left)
                            D[l][k] = b
                            b_left = b
                        else:
                            D[l][k] = a
                        d0, a_left, diag1 = up, a, a
                    if l == lanes - 1:
                        seam_out[rr + 1] = a_left + O[l]
                        if ok1:
                            seam_out[rr + 2] = D[l][S - 1] + O[l]
                if st % K == K - 1:  # rescale: every lane, its own minimum
                    mn = float(D[l].min())
                    if np.isfinite(mn):
                        D[l] -= mn
                        O[l] += mn
                        a_left -= mn
                        diag_next[l] -= mn
                expo[l] = (a_left, D[l][S - 1], O[l])
        for l in range(lanes):
            last_row[s * W + l * S: s * W + (l + 1) * S] = D[l] + O[l]
        seam_in = seam_out
    return last_row[:m]


@pytest.mark.parametrize("n,K", [(1, 1), (5, 1), (8, 2), (13, 3), (31, 2)])
def test_framed_schedule_matches_recurrence(oracle, n, K):
    rng = np.random.default_rng(7 * n + K)
    ref = rng.standard_normal(29)
    q = rng.standard_normal(n)
    row = model_refdel_framed(ref, q, K=K)
    _, _, row_o = oracle.sdtw_ref_del(ref, q, want_row=True)
    np.testing.assert_allclose(row, row_o, rtol=1e-9, atol=1e-9)
    init = rng.random(29) * 4 + 10
    row = model_refdel_framed(ref, q, K=K, lanes=5, S=2, init_row=init)
    _, _, row_o = oracle.sdtw_ref_del(ref, q, init_row=init, want_row=True)
    np.testing.assert_allclose(row, row_o, rtol=1e-9, atol=1e-9)
