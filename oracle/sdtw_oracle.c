/*
 * FP64 CPU oracle for the subsequence-DTW (sDTW) read-classification path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA library
 * in dtwax_gb300/ is compared against.  Only tests/, __graft_entry__.smoke()
 * and the CPU-baseline leg of bench.py may load it; the product path never
 * links, loads or falls back to it.
 *
 * It restates, in plain C with OpenMP, the algorithm of the reference
 * (harisankarsadasivan/DTWax):
 *   - scripts/sdtw.py:205-225 `sdtw_default` (FP64 sDTW, free start/end) and
 *     src/include/DTW.cu:37-39 (`COST_FUNCTION` under -DNO_REF_DEL: only the
 *     vertical and diagonal predecessors);
 *   - scripts/sdtw.py:86-99 `discrete_normalize` (population z-score) and
 *     src/include/normalizer.cu:397-399 (batch-norm z-score, eps 1e-4);
 *   - scripts/sdtw.py:101-116 `ref_signal` and
 *     src/include/load_reference.hpp:33-108 `load_ref_coeffs` (6-mer levels
 *     of the forward strand and of the reverse complement, z-scored).
 *
 * Pinned against the reference's golden trace scripts/log (every logged DP
 * cell of a 4096-sample read against the 96,256-sample lambda reference, and
 * the final minimum 286.8895631) by tests/test_oracle_golden.py.
 *
 * Build (no GPU needed):
 *   gcc -O3 -fopenmp -ffp-contract=off -shared -fPIC sdtw_oracle.c -o liboracle.so
 * -ffp-contract=off keeps `d*d + m` as two rounded operations, as the
 * reference's Python/numba code computes it.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KMER 6

/* 2-bit base code in the lexicographic order of the k-mer model file
 * (src/ref/dna_kmer_model.txt lists AAAAAA, AAAAAC, AAAAAG, ...).
 * Returns -1 for anything that is not A/C/G/T (lower case is accepted). */
static int base_code(char c) {
  switch (c) {
  case 'A': case 'a': return 0;
  case 'C': case 'c': return 1;
  case 'G': case 'g': return 2;
  case 'T': case 't': return 3;
  default: return -1;
  }
}

/* Complement as in load_reference.hpp:111-128 (A<->T, C<->G, others kept). */
static char complement(char c) {
  switch (c) {
  case 'A': return 'T'; case 'C': return 'G';
  case 'G': return 'C'; case 'T': return 'A';
  case 'a': return 't'; case 'c': return 'g';
  case 'g': return 'c'; case 't': return 'a';
  default: return c;
  }
}

/* 6-mer code of s[0..6); -1 when a base is not ACGT. */
static int kmer_code(const char *s) {
  int code = 0;
  for (int k = 0; k < KMER; ++k) {
    int b = base_code(s[k]);
    if (b < 0) return -1;
    code = (code << 2) | b;
  }
  return code;
}

/* Population z-score, two-pass FP64: y = (x - mean) / sqrt(var + eps).
 * eps = 0 reproduces sdtw.py:97-99; eps = 1e-4 reproduces the batch-norm
 * normaliser of normalizer.cu:397-399 (biased variance, scale 1, bias 0).
 * Values flagged invalid (isnan) are excluded from the statistics and
 * mapped to 0. */
int64_t oracle_zscore(const double *x, int64_t n, double eps, double *y) {
  double sum = 0.0;
  int64_t cnt = 0;
  for (int64_t i = 0; i < n; ++i)
    if (!isnan(x[i])) { sum += x[i]; ++cnt; }
  if (cnt == 0) {
    for (int64_t i = 0; i < n; ++i) y[i] = 0.0;
    return 0;
  }
  const double mean = sum / (double)cnt;
  double ss = 0.0;
  for (int64_t i = 0; i < n; ++i)
    if (!isnan(x[i])) { double d = x[i] - mean; ss += d * d; }
  const double sd = sqrt(ss / (double)cnt + eps);
  for (int64_t i = 0; i < n; ++i)
    y[i] = isnan(x[i]) ? 0.0 : (x[i] - mean) / sd;
  return cnt;
}

/* Expected-level squiggle of both strands (sdtw.py:101-116 and
 * load_reference.hpp:33-108).  table[4096] holds the k-mer means indexed by
 * the 2-bit code.  For k-mer position j in [0, L-5):
 *   fwd[j] = table[code(seq[j..j+6))]
 *   rev[j] = table[code(rc[j..j+6))],  rc = reverse complement of seq.
 * Each strand is truncated to `cap` positions when cap > 0 (sdtw.py:116
 * truncates to R//2; the GPU reference caps at REF_LEN) and then z-scored
 * with eps 0.  K-mers holding a non-ACGT base get level 0 after z-scoring
 * and are left out of the statistics.  Returns the positions per strand. */
int64_t oracle_build_levels(const char *seq, int64_t L, const double *table,
                            int64_t cap, double *fwd, double *rev) {
  if (L < KMER) return 0;
  int64_t m = L - KMER + 1;
  if (cap > 0 && cap < m) m = cap;
  char *rc = (char *)malloc((size_t)L);
  if (!rc) return -1;
  for (int64_t i = 0; i < L; ++i) rc[i] = complement(seq[L - 1 - i]);
  double *tmp = (double *)malloc(sizeof(double) * (size_t)m);
  if (!tmp) { free(rc); return -1; }
  for (int strand = 0; strand < 2; ++strand) {
    const char *s = strand == 0 ? seq : rc;
    for (int64_t j = 0; j < m; ++j) {
      int c = kmer_code(s + j);
      tmp[j] = c < 0 ? NAN : table[c];
    }
    oracle_zscore(tmp, m, 0.0, strand == 0 ? fwd : rev);
  }
  free(tmp);
  free(rc);
  return m;
}

/* Single-sequence sDTW in FP64 (sdtw.py:205-225, NO_REF_DEL recurrence):
 *   D[0][j] = (r_j - q_0)^2                       (free start)
 *   D[i][0] = D[i-1][0] + (r_0 - q_i)^2
 *   D[i][j] = (r_j - q_i)^2 + min(D[i-1][j], D[i-1][j-1])
 * Free start is the same as starting from a "row -1" of zeros; a non-NULL
 * init_row (length m) replaces those zeros, which resumes a read whose
 * earlier samples were already aligned (the row state of the serving path).
 * Returns min_j D[n-1][j]; *argmin gets the smallest j reaching it.
 * final_row (nullable, length m) receives D[n-1][*].
 * trace_cols/trace_out (nullable) record D[i][trace_cols[t]] for every row
 * into trace_out[i*n_trace + t], the layout of the golden log. */
static double sdtw_rows(const double *ref, int64_t m, const double *q, int64_t n,
                        const double *init_row, double *final_row, int64_t *argmin,
                        const int64_t *trace_cols, int n_trace, double *trace_out, int ref_del);

double oracle_sdtw(const double *ref, int64_t m, const double *q, int64_t n,
                   const double *init_row, double *final_row, int64_t *argmin,
                   const int64_t *trace_cols, int n_trace, double *trace_out) {
  return sdtw_rows(ref, m, q, n, init_row, final_row, argmin, trace_cols, n_trace, trace_out, 0);
}

/* The REF_DEL recurrence of the reference's kernel built without -DNO_REF_DEL
 * (src/include/DTW.cu:23-29): a third predecessor, the cell to the left in the
 * same row, D[i][j] = d^2 + min(D[i][j-1], D[i-1][j], D[i-1][j-1]).  Row 0 is
 * the cost alone (the free start's zero row above wins every minimum). */
double oracle_sdtw_ref_del(const double *ref, int64_t m, const double *q, int64_t n,
                           const double *init_row, double *final_row, int64_t *argmin) {
  return sdtw_rows(ref, m, q, n, init_row, final_row, argmin, NULL, 0, NULL, 1);
}

static double sdtw_rows(const double *ref, int64_t m, const double *q, int64_t n,
                        const double *init_row, double *final_row, int64_t *argmin,
                        const int64_t *trace_cols, int n_trace, double *trace_out, int ref_del) {
  if (m <= 0 || n <= 0) {
    if (argmin) *argmin = -1;
    return INFINITY;
  }
  double *prev = (double *)malloc(sizeof(double) * (size_t)m);
  double *cur = (double *)malloc(sizeof(double) * (size_t)m);
  if (!prev || !cur) {
    free(prev); free(cur);
    if (argmin) *argmin = -1;
    return NAN;
  }
  if (init_row)
    memcpy(prev, init_row, sizeof(double) * (size_t)m);
  else
    memset(prev, 0, sizeof(double) * (size_t)m);
  for (int64_t i = 0; i < n; ++i) {
    const double qi = q[i];
    double d0 = ref[0] - qi;
    cur[0] = d0 * d0 + prev[0];
    for (int64_t j = 1; j < m; ++j) {
      double d = ref[j] - qi;
      double a = prev[j], b = prev[j - 1];
      double mn = a < b ? a : b;
      if (ref_del && cur[j - 1] < mn) mn = cur[j - 1];
      cur[j] = d * d + mn;
    }
    if (trace_out)
      for (int t = 0; t < n_trace; ++t) trace_out[i * n_trace + t] = cur[trace_cols[t]];
    double *sw = prev; prev = cur; cur = sw;
  }
  double best = prev[0];
  int64_t bj = 0;
  for (int64_t j = 1; j < m; ++j)
    if (prev[j] < best) { best = prev[j]; bj = j; }
  if (argmin) *argmin = bj;
  if (final_row) memcpy(final_row, prev, sizeof(double) * (size_t)m);
  free(prev);
  free(cur);
  return best;
}

/* Batch of reads against both strands, OpenMP over (read, strand) tasks.
 * queries holds the normalised reads back to back; read r is
 * queries[offsets[r] .. offsets[r+1]).  Outputs per read and strand:
 * min score and smallest end column.  n_threads <= 0 uses all cores. */
void oracle_sdtw_batch_rec(const double *fwd, const double *rev, int64_t m,
                           const double *queries, const int64_t *offsets, int n_reads,
                           double *score_fwd, int64_t *end_fwd, double *score_rev,
                           int64_t *end_rev, int n_threads, int ref_del);

void oracle_sdtw_batch(const double *fwd, const double *rev, int64_t m,
                       const double *queries, const int64_t *offsets, int n_reads,
                       double *score_fwd, int64_t *end_fwd, double *score_rev,
                       int64_t *end_rev, int n_threads) {
  oracle_sdtw_batch_rec(fwd, rev, m, queries, offsets, n_reads, score_fwd, end_fwd, score_rev, end_rev,
                        n_threads, 0);
}

/* oracle_sdtw_batch with the recurrence chosen: ref_del 0 (NO_REF_DEL) or 1. */
void oracle_sdtw_batch_rec(const double *fwd, const double *rev, int64_t m,
                           const double *queries, const int64_t *offsets, int n_reads,
                           double *score_fwd, int64_t *end_fwd, double *score_rev,
                           int64_t *end_rev, int n_threads, int ref_del) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  const int64_t tasks = 2 * (int64_t)n_reads;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t t = 0; t < tasks; ++t) {
    const int r = (int)(t >> 1);
    const int strand = (int)(t & 1);
    const double *q = queries + offsets[r];
    const int64_t n = offsets[r + 1] - offsets[r];
    int64_t am = -1;
    double s = sdtw_rows(strand == 0 ? fwd : rev, m, q, n, NULL, NULL, &am, NULL, 0, NULL, ref_del);
    if (strand == 0) { score_fwd[r] = s; end_fwd[r] = am; }
    else { score_rev[r] = s; end_rev[r] = am; }
  }
}

/* The reference GPU kernel's evaluation order, restated in FP64, with its
 * departures from the recurrence as switches (src/include/DTW.cu:151-572 at
 * its shipped shape: 832-column tiles of 32 lanes x 26 cells, the query in
 * 1,024-row chunks, one warp per read).
 *
 * The kernel sweeps chunk by chunk and, inside a chunk, tile by tile; a tile
 * gets the column to its left from the previous tile through a 1,024-entry
 * seam buffer (DTW.cu:155, :237-262, :369-389) and a chunk gets the row above
 * it from the previous chunk's last row (DTW.cu:205-209, :325-331, :447-455).
 * With quirks == 0 this order gives exactly the values of oracle_sdtw.
 * Switches (OR them):
 *   REFK_CHUNK_SEAM_DIAG (1): first row of a chunk after the first, first
 *     column of a tile after the first: diagonal = +inf (the tile starts with
 *     penalty_diag = inf, DTW.cu:313-315, :441-443);
 *   REFK_CHUNK_LANE1_DIAG (2): same row, column 26 of every tile (lane 1's
 *     first cell): diagonal = +inf (lane 1's first update reads the
 *     penalty_left value set before the wave loop, DTW.cu:178-179, :216-227);
 *   REFK_SEAM_SHIFT (4): seam rows 961..991 written by a middle tile hold the
 *     value of the row 31 below (the write index wave - 63 at DTW.cu:387
 *     against wave - 32 in the first tile, DTW.cu:267), seen by the next tile.
 * REFK_REF_DEL (8) is not a departure but the recurrence of the kernel built
 * without -DNO_REF_DEL (DTW.cu:23-29): the cell to the left in the same row is
 * a third predecessor; a tile's first column takes it from the seam buffer
 * (penalty_left = penalty_last_col[wave], DTW.cu:384, :516), so the seam shift
 * reaches it too.
 * m must be a multiple of 832 with at least two tiles (the kernel's own
 * geometry, its last partial tile is never scored) and n a multiple of 1024.
 * Returns min_j D[n-1][j] (the kernel reports no column), or NaN on a bad
 * shape. */
#define REFK_TILE 832
#define REFK_CHUNK 1024
#define REFK_LANE_CELLS 26
#define REFK_CHUNK_SEAM_DIAG 1
#define REFK_CHUNK_LANE1_DIAG 2
#define REFK_SEAM_SHIFT 4
#define REFK_REF_DEL 8

double oracle_sdtw_refkernel(const double *ref, int64_t m, const double *q, int64_t n, int quirks) {
  if (m < 2 * REFK_TILE || m % REFK_TILE != 0 || n <= 0 || n % REFK_CHUNK != 0) return NAN;
  const int64_t tiles = m / REFK_TILE;
  double *last_in = (double *)calloc((size_t)m, sizeof(double));
  double *last_out = (double *)malloc(sizeof(double) * (size_t)m);
  double *seam_prev = (double *)malloc(sizeof(double) * REFK_CHUNK);
  double *seam_cur = (double *)malloc(sizeof(double) * REFK_CHUNK);
  double *ra = (double *)malloc(sizeof(double) * REFK_TILE);
  double *rb = (double *)malloc(sizeof(double) * REFK_TILE);
  double best = NAN;
  if (!last_in || !last_out || !seam_prev || !seam_cur || !ra || !rb) goto done;
  for (int64_t c = 0; c < n / REFK_CHUNK; ++c) {
    for (int64_t k = 0; k < tiles; ++k) {
      const int64_t c0 = k * REFK_TILE;
      const double *up = last_in + c0;
      double *cur = ra, *spare = rb;
      for (int64_t r = 0; r < REFK_CHUNK; ++r) {
        const double qi = q[c * REFK_CHUNK + r];
        for (int64_t j = 0; j < REFK_TILE; ++j) {
          const double d = ref[c0 + j] - qi;
          const double cost = d * d;
          if (c == 0 && r == 0) {  /* free start */
            cur[j] = cost;
            continue;
          }
          const double top = up[j];
          double diag;
          if (j > 0)
            diag = up[j - 1];
          else if (k == 0)
            diag = INFINITY;
          else if (r == 0)
            diag = (quirks & REFK_CHUNK_SEAM_DIAG) ? INFINITY : last_in[c0 - 1];
          else
            diag = seam_prev[r - 1];
          if (r == 0 && j == REFK_LANE_CELLS && (quirks & REFK_CHUNK_LANE1_DIAG)) diag = INFINITY;
          double mn = top < diag ? top : diag;
          if (quirks & REFK_REF_DEL) {
            const double left = j > 0 ? cur[j - 1] : (k == 0 ? INFINITY : seam_prev[r]);
            if (left < mn) mn = left;
          }
          cur[j] = cost + mn;
        }
        seam_cur[r] = cur[REFK_TILE - 1];
        if (r == REFK_CHUNK - 1) memcpy(last_out + c0, cur, sizeof(double) * REFK_TILE);
        up = cur;
        double *sw = cur; cur = spare; spare = sw;
      }
      if ((quirks & REFK_SEAM_SHIFT) && k >= 1 && k <= tiles - 2)
        for (int x = 961; x <= 991; ++x) seam_cur[x] = seam_cur[x + 31];
      double *sw = seam_prev; seam_prev = seam_cur; seam_cur = sw;
    }
    double *sw = last_in; last_in = last_out; last_out = sw;
  }
  best = last_in[0];
  for (int64_t j = 1; j < m; ++j)
    if (last_in[j] < best) best = last_in[j];
done:
  free(last_in); free(last_out); free(seam_prev); free(seam_cur); free(ra); free(rb);
  return best;
}

/* oracle_sdtw_refkernel over reads of qlen samples stored back to back,
 * OpenMP over reads. */
void oracle_sdtw_refkernel_batch(const double *ref, int64_t m, const double *queries, int64_t qlen,
                                 int n_reads, int quirks, double *score, int n_threads) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int r = 0; r < n_reads; ++r)
    score[r] = oracle_sdtw_refkernel(ref, m, queries + (int64_t)r * qlen, qlen, quirks);
}

/* Threads OpenMP will use (reported as the CPU baseline's core count). */
int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
