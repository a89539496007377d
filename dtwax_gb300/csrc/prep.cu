// Kernels around the sDTW sweep: the reference-squiggle builder, the per-read
// window + z-score normaliser, the reset of the result keys and the finalize
// step that turns per-strand (score, end column) keys into read results.
#include "dtwx_internal.h"

namespace dtwx {

// Layout of the public dtwx_result (include/dtwx.h); the host checks sizeof.
struct ResultRec {
  float score;
  float score_fwd;
  float score_rev;
  int32_t strand;
  int64_t end_pos;
  int32_t call;
  int32_t n_samples;
};
static_assert(sizeof(ResultRec) == 32, "dtwx_result layout");

constexpr int kBlock = 256;

__device__ __forceinline__ int base2(unsigned char c) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return -1;
  }
}

// Block-wide sum of doubles (deterministic order for a fixed block size).
__device__ double block_sum(double v, double *sh) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
    sh[32] = r;
  }
  __syncthreads();
  r = sh[32];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------- reference builder
// Follows src/include/load_reference.hpp:33-128 (6-mer levels of the forward
// strand and of the reverse complement, z-scored per strand) and
// scripts/sdtw.py:101-116.  Statistics are two-pass FP64 over the valid
// k-mers; k-mers with a non-ACGT base become 0 and are left out.
//
// work layout (doubles): lev[2*m] (fwd then rev; NaN = invalid),
// partial[2 * 3 * nblk] (sum, count, sumsq per block and strand), stats[4].

__global__ void kmer_levels_kernel(const unsigned char *seq, int64_t L, const double *table,
                                   int64_t m, double *lev, double *partial, int nblk) {
  __shared__ double sh[33];
  double s0 = 0, c0 = 0, s1 = 0, c1 = 0;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    int cf = 0, cr = 0;
    bool okf = true, okr = true;
#pragma unroll
    for (int k = 0; k < kKmer; ++k) {
      const int bf = base2(seq[j + k]);
      // reverse complement: rc[t] = comp(seq[L-1-t]); comp of code c is 3-c
      const int br = base2(seq[L - 1 - j - k]);
      okf &= bf >= 0;
      okr &= br >= 0;
      cf = (cf << 2) | (bf & 3);
      cr = (cr << 2) | ((3 - br) & 3);
    }
    const double vf = okf ? table[cf] : __longlong_as_double(0x7ff8000000000000ll);
    const double vr = okr ? table[cr] : __longlong_as_double(0x7ff8000000000000ll);
    lev[j] = vf;
    lev[m + j] = vr;
    if (okf) { s0 += vf; c0 += 1; }
    if (okr) { s1 += vr; c1 += 1; }
  }
  s0 = block_sum(s0, sh);
  c0 = block_sum(c0, sh);
  s1 = block_sum(s1, sh);
  c1 = block_sum(c1, sh);
  if (threadIdx.x == 0) {
    partial[0 * nblk + blockIdx.x] = s0;
    partial[1 * nblk + blockIdx.x] = c0;
    partial[3 * nblk + blockIdx.x] = s1;
    partial[4 * nblk + blockIdx.x] = c1;
  }
}

// stats[strand*2 + 0] = mean; second pass reads it.
__global__ void reduce_mean_kernel(const double *partial, int nblk, double *stats) {
  __shared__ double sh[33];
  for (int strand = 0; strand < 2; ++strand) {
    double s = 0, c = 0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
      s += partial[(3 * strand + 0) * nblk + i];
      c += partial[(3 * strand + 1) * nblk + i];
    }
    s = block_sum(s, sh);
    c = block_sum(c, sh);
    if (threadIdx.x == 0) {
      stats[strand * 2 + 0] = c > 0 ? s / c : 0.0;
      stats[strand * 2 + 1] = c;
    }
  }
}

__global__ void sumsq_kernel(const double *lev, int64_t m, const double *stats, double *partial,
                             int nblk) {
  __shared__ double sh[33];
  const double mf = stats[0], mr = stats[2];
  double q0 = 0, q1 = 0;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    const double vf = lev[j], vr = lev[m + j];
    if (!isnan(vf)) q0 += (vf - mf) * (vf - mf);
    if (!isnan(vr)) q1 += (vr - mr) * (vr - mr);
  }
  q0 = block_sum(q0, sh);
  q1 = block_sum(q1, sh);
  if (threadIdx.x == 0) {
    partial[2 * nblk + blockIdx.x] = q0;
    partial[5 * nblk + blockIdx.x] = q1;
  }
}

__global__ void reduce_sd_kernel(const double *partial, int nblk, double *stats) {
  __shared__ double sh[33];
  for (int strand = 0; strand < 2; ++strand) {
    double q = 0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) q += partial[(3 * strand + 2) * nblk + i];
    q = block_sum(q, sh);
    if (threadIdx.x == 0) {
      const double c = stats[strand * 2 + 1];
      stats[4 + strand] = c > 0 ? sqrt(q / c) : 1.0;
    }
  }
}

// Writes the z-scored levels: FP16 pairs (fwd[j], rev[j]) and FP32 planes.
// PAIRED: column j < m holds k-mer j of each strand.  CONCAT: one sequence
// fwd||rev of 2m columns, stored in both strand slots (the FP32 sweep then
// aligns only plane 0).
__global__ void zscore_pairs_kernel(const double *lev, int64_t m, int64_t m_pad, int concat,
                                    const double *stats, __half2 *ref16, float *ref32, __half *ref16p,
                                    float *fwd32, float *rev32) {
  const double mf = stats[0], mr = stats[2];
  const double sf = stats[4] > 0 ? stats[4] : 1.0, sr = stats[5] > 0 ? stats[5] : 1.0;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m_pad;
       j += (int64_t)gridDim.x * blockDim.x) {
    float a = 0.f, b = 0.f;
    if (!concat) {
      if (j < m) {
        const double vf = lev[j], vr = lev[m + j];
        a = isnan(vf) ? 0.f : (float)((vf - mf) / sf);
        b = isnan(vr) ? 0.f : (float)((vr - mr) / sr);
        fwd32[j] = a;
        rev32[j] = b;
      }
    } else if (j < 2 * m) {
      const bool rv = j >= m;
      const double v = lev[j];
      a = isnan(v) ? 0.f : (float)((v - (rv ? mr : mf)) / (rv ? sr : sf));
      b = a;
      if (rv) rev32[j - m] = a; else fwd32[j] = a;
    }
    ref32[j] = a;          // fwd plane
    ref32[m_pad + j] = b;  // rev plane
    ref16[j] = __floats2half2_rn(a, b);
    ref16p[j] = __float2half_rn(a);          // FP16 planes (MIXED precision)
    ref16p[m_pad + j] = __float2half_rn(b);
  }
}

size_t build_reference_work_bytes(int64_t m) {
  const int nblk = 1024;
  return sizeof(double) * (size_t)(2 * m + 6 * nblk + 8);
}

cudaError_t launch_build_reference(const char *d_seq, int64_t L, const double *d_table, int64_t m,
                                   int64_t m_pad, int concat, double *d_work, __half2 *d_ref16,
                                   float *d_ref32, __half *d_ref16p, float *d_fwd32, float *d_rev32,
                                   cudaStream_t s) {
  const int nblk = 1024;
  double *lev = d_work;
  double *partial = d_work + 2 * m;
  double *stats = partial + 6 * nblk;
  const unsigned char *seq = reinterpret_cast<const unsigned char *>(d_seq);
  kmer_levels_kernel<<<nblk, kBlock, 0, s>>>(seq, L, d_table, m, lev, partial, nblk);
  reduce_mean_kernel<<<1, kBlock, 0, s>>>(partial, nblk, stats);
  sumsq_kernel<<<nblk, kBlock, 0, s>>>(lev, m, stats, partial, nblk);
  reduce_sd_kernel<<<1, kBlock, 0, s>>>(partial, nblk, stats);
  zscore_pairs_kernel<<<1024, kBlock, 0, s>>>(lev, m, m_pad, concat, stats, d_ref16, d_ref32, d_ref16p,
                                              d_fwd32, d_rev32);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- normaliser
// Per read: y = (x - mean) / sqrt(var + eps) over the window, population
// variance, statistics in FP64, two passes (src/include/normalizer.cu:370-413
// uses cuDNN batch norm in SPATIAL mode with eps 1e-4 for the same formula).
// int16 input is first scaled to pA: (raw + add) * mul.

template <typename T>
__global__ void __launch_bounds__(kBlock) normalize_kernel(const T *src, const int64_t *src_off,
                                                           const int64_t *dst_off, const int32_t *dst_len,
                                                           const float *scale_mul,
                                                           const float *scale_add, float eps,
                                                           float *dst) {
  __shared__ double sh[33];
  const int r = blockIdx.x;
  const int n = dst_len[r];
  if (n <= 0) return;
  const T *x = src + src_off[r];
  float *y = dst + dst_off[r];
  const float mul = scale_mul ? scale_mul[r] : 1.f;
  const float add = scale_add ? scale_add[r] : 0.f;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += (double)(((float)x[i] + add) * mul);
  const double mean = block_sum(s, sh) / (double)n;
  double q = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = (double)(((float)x[i] + add) * mul) - mean;
    q += d * d;
  }
  const double var = block_sum(q, sh) / (double)n;
  const double inv = 1.0 / sqrt(var + (double)eps);
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    y[i] = (float)(((double)(((float)x[i] + add) * mul) - mean) * inv);
}

cudaError_t launch_normalize(const void *src, int is_i16, const int64_t *src_off,
                             const int64_t *dst_off, const int32_t *dst_len, const float *scale_mul,
                             const float *scale_add, int n_reads, float eps, float *dst,
                             cudaStream_t s) {
  if (n_reads <= 0) return cudaSuccess;
  if (is_i16)
    normalize_kernel<int16_t><<<n_reads, kBlock, 0, s>>>(static_cast<const int16_t *>(src), src_off,
                                                         dst_off, dst_len, scale_mul, scale_add, eps,
                                                         dst);
  else
    normalize_kernel<float><<<n_reads, kBlock, 0, s>>>(static_cast<const float *>(src), src_off,
                                                       dst_off, dst_len, scale_mul, scale_add, eps,
                                                       dst);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- reset / finalize

__global__ void reset_kernel(unsigned long long *keys, int n_keys, int32_t *counter, int32_t *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_keys) keys[i] = ~0ull;
  if (i == 0 && counter) *counter = 0;
  if (i == 0 && err) *err = 0;
}

cudaError_t launch_reset(unsigned long long *keys, int n_keys, int32_t *counter, int32_t *err,
                         cudaStream_t s) {
  const int n = n_keys > 1 ? n_keys : 1;
  reset_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(keys, n_keys, counter, err);
  return cudaGetLastError();
}

// The min/argmin of the last DP row was reduced inside the sweep into one key
// per read and strand: (orderable score << 32) | end column, combined with
// atomicMin, so the smallest score wins and ties go to the smallest column.
// Here the two strands are combined (ties: forward strand) and the call is
// made: target when score < threshold (calc_classification_threshold.py:52).
__global__ void finalize_kernel(const unsigned long long *keys, const int32_t *n_samples,
                                int n_reads, int concat, int64_t m_fwd, float threshold,
                                const int32_t *err, ResultRec *out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_reads) return;
  ResultRec o;
  const int32_t ns = n_samples ? n_samples[r] : 1;
  o.n_samples = ns;
  const unsigned long long kf = keys[2 * r], kr = keys[2 * r + 1];
  const float inf = __int_as_float(0x7f800000);
  float sf = kf == ~0ull ? inf : ordered_to_float((uint32_t)(kf >> 32));
  float sr = kr == ~0ull ? inf : ordered_to_float((uint32_t)(kr >> 32));
  const int64_t ef = kf == ~0ull ? -1 : (int64_t)(uint32_t)(kf & 0xffffffffu);
  const int64_t er = kr == ~0ull ? -1 : (int64_t)(uint32_t)(kr & 0xffffffffu);
  if (!concat) {
    const bool rev = sr < sf || (sr == sf && er < ef);
    o.score_fwd = sf;
    o.score_rev = sr;
    o.score = rev ? sr : sf;
    o.strand = rev ? 1 : 0;
    o.end_pos = rev ? er : ef;
  } else {
    // one sequence fwd||rev: the column tells the strand
    o.score = sf;
    o.score_fwd = sf;
    o.score_rev = sf;
    o.strand = ef >= m_fwd ? 1 : 0;
    o.end_pos = ef >= m_fwd ? ef - m_fwd : ef;
  }
  o.call = ns <= 0 ? -1 : (o.score < threshold ? 1 : 0);
  if (ns <= 0) {
    o.score = o.score_fwd = o.score_rev = inf;
    o.end_pos = -1;
    o.strand = 0;
  }
  const int32_t e = err ? *err : 0;
  if (e != 0) {
    // a bounded wait gave up or a task was refused: the keys are incomplete
    o.score = o.score_fwd = o.score_rev = __int_as_float(0x7fc00000);
    o.end_pos = -1;
    o.strand = e;
    o.call = kCallDeviceError;
  }
  out[r] = o;
}

cudaError_t launch_finalize(const unsigned long long *keys, const int32_t *n_samples, int n_reads,
                            int concat, int64_t m_fwd, float threshold, const int32_t *err,
                            void *d_results, cudaStream_t s) {
  if (n_reads <= 0) return cudaSuccess;
  finalize_kernel<<<(n_reads + kBlock - 1) / kBlock, kBlock, 0, s>>>(
      keys, n_samples, n_reads, concat, m_fwd, threshold, err, static_cast<ResultRec *>(d_results));
  return cudaGetLastError();
}

}  // namespace dtwx
