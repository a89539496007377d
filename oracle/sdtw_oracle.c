/*
 * FP64 CPU oracle for the subsequence-DTW (sDTW) read-classification path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA library
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
double oracle_sdtw(const double *ref, int64_t m, const double *q, int64_t n,
                   const double *init_row, double *final_row, int64_t *argmin,
                   const int64_t *trace_cols, int n_trace, double *trace_out) {
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
      cur[j] = d * d + (a < b ? a : b);
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
void oracle_sdtw_batch(const double *fwd, const double *rev, int64_t m,
                       const double *queries, const int64_t *offsets, int n_reads,
                       double *score_fwd, int64_t *end_fwd, double *score_rev,
                       int64_t *end_rev, int n_threads) {
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
    double s = oracle_sdtw(strand == 0 ? fwd : rev, m, q, n, NULL, NULL, &am, NULL, 0, NULL);
    if (strand == 0) { score_fwd[r] = s; end_fwd[r] = am; }
    else { score_rev[r] = s; end_rev[r] = am; }
  }
}

/* Threads OpenMP will use (reported as the CPU baseline's core count). */
int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
