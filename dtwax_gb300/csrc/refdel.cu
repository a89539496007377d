// The REF_DEL recurrence on FP32 cells and on FP16 pairs (src/include/DTW.cu:
// 23-29, the build without -DNO_REF_DEL; scripts/sdtw.py keeps no such
// variant):
//
//   D[i][j] = (r_j - q_i)^2 + min(D[i-1][j], D[i-1][j-1], D[i][j-1])
//
// with the free start of sDTW (row -1 is zero, or the saved row of a resumed
// read) and +inf left of column 0.
//
// The left predecessor chains the cells of one row, so a warp sweeps a strip
// of 32*S columns along anti-diagonals instead of row by row:
// * lane l owns S consecutive columns and, at step t, computes rows
//   2(t - l) and 2(t - l) + 1 of them from left to right, so the horizontal
//   chain stays inside the lane;
// * the left predecessors of its first column are lane l-1's last cells of
//   the same rows, which lane l-1 computed at step t-1 (two shuffles per
//   step), and the diagonal one of the first row is the value received one
//   step earlier;
// * lane 0 takes both from the seam column of the strip to the left, and lane
//   31 writes the seam column for the strip to its right.
// Each step a lane computes two consecutive rows, interleaved (two dependency
// chains).  A cell costs one subtraction, two minima and one FMA.  A strip
// takes ceil(n / 2) + 31 steps; in the first and last 31 some lanes have no
// rows and keep their cells, so after the last step every lane holds row
// n - 1.
//
// A horizontal run can cross any column, so a task is one work item (per
// strand for FP32 cells) that sweeps every strip (the host launches it with
// one chunk).  The FP16-pair kernel further down adds per-lane
// running-minimum frames.
#include "dtwx_internal.h"
#include "warp_ops.cuh"

namespace dtwx {

// One step of one lane: its S cells of two consecutive rows r and r + 1,
// left to right, interleaved.  Row r + 1's cell k needs row r's cells k and
// k - 1 and its own cell k - 1, so the two rows are two dependency chains one
// cell apart, which doubles the instruction-level parallelism of the lane.
// D holds row r - 1 on entry and the last valid row on exit.  diag0 is the
// left neighbour's cell on row r - 1, left0 / left1 on rows r / r + 1;
// left0 returns this lane's last cell of row r.  RAMP: rows that do not exist
// (ok0 / ok1 false) leave the cells as they were.
template <int S, bool RAMP>
__device__ __forceinline__ void refdel_step2(float (&D)[S], const float (&R)[S], float q0, float q1, float diag0,
                                             float &left0, float left1, bool ok0, bool ok1) {
  float diag1 = left0;
#pragma unroll
  for (int k = 0; k < S; ++k) {
    const float d0 = R[k] - q0;
    const float d1 = R[k] - q1;
    const float up = D[k];
    const float a = fmaf(d0, d0, fminf(fminf(up, diag0), left0));
    const float b = fmaf(d1, d1, fminf(fminf(a, diag1), left1));
    if constexpr (RAMP)
      D[k] = ok1 ? b : (ok0 ? a : up);
    else
      D[k] = b;
    diag0 = up;
    left0 = a;
    diag1 = a;
    left1 = b;
  }
}

// A step's chain of S dependent min/FMA pairs needs several warps per
// scheduler to hide: 16 cells per lane fit in 128 registers (16 warps per
// SM); 32 cells take about 142 (12 warps) rather than spill.
template <int S>
__global__ void __launch_bounds__(256, S <= 16 ? 2 : 1) sdtw_refdel_kernel(const SdtwParams p) {
  static_assert(S % 4 == 0, "row state moves in 16-byte groups");
  constexpr int W = kWarp * S;
  const int lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const uint32_t is0 = lane == 0 ? 1u : 0u;
  const float inf = __int_as_float(0x7f800000);
  const int64_t gwarp = (int64_t)blockIdx.x * nwarps + (threadIdx.x >> 5);
  char *seam_base = p.seam + gwarp * p.seam_stride;
  const int64_t seam_half = p.seam_stride / 2;
  const int nstr = p.strands > 0 ? p.strands : 2;
  const int per_task = p.n_chunks * nstr;
  const int64_t n_items = (int64_t)p.n_tasks * per_task;
  const int64_t strips = (p.m + W - 1) / W;

  for (;;) {
    const int item = __shfl_sync(FULL_MASK, ticket_if(p.counter, is0), 0);
    if (item >= n_items) break;
    const int tr = item / per_task;
    const int rem = item - tr * per_task;
    const int strand = rem / p.n_chunks;
    if (rem - strand * p.n_chunks != 0) continue;  // one chunk per task: chunk 0 sweeps every strip
    const int ti = p.order ? p.order[tr] : tr;
    const Task t = p.tasks[ti];
    const int n = t.n;
    if (n <= 0 || n > p.max_rows) {
      if (n > p.max_rows) atomicOr(p.err, kErrBadTask);  // every lane: same bit
      continue;
    }
    const float *q = p.query + t.q_off;
    const bool resume = (t.flags & kTaskResume) != 0 && p.state != nullptr;
    const bool save = (t.flags & kTaskSaveState) != 0 && p.state != nullptr;
    // planar reference and row state: strand s at s * m_pad
    const int64_t plane = (int64_t)strand * p.m_pad;
    const float *ref = static_cast<const float *>(p.ref_plain) + plane;

    float best = inf;
    int64_t bcol = -1;
    for (int64_t s = 0; s < strips; ++s) {
      const int64_t c0 = s * W + (int64_t)lane * S;
      const bool first = s == 0;
      // seam column of the left strip: row -1 at [0], row i at [i + 1]
      const float *seam_in = reinterpret_cast<const float *>(seam_base + ((s + 1) & 1) * seam_half);
      float *seam_out = reinterpret_cast<float *>(seam_base + (s & 1) * seam_half);

      float D[S], R[S];
      if (resume) {
        const float4 *f = reinterpret_cast<const float4 *>(p.state + t.state_off + plane + c0);
#pragma unroll
        for (int k = 0; k < S / 4; ++k) {
          const float4 u = f[k];
          D[4 * k] = u.x, D[4 * k + 1] = u.y, D[4 * k + 2] = u.z, D[4 * k + 3] = u.w;
        }
      } else {
#pragma unroll
        for (int k = 0; k < S; ++k) D[k] = 0.f;
      }
      {
        const float4 *g = reinterpret_cast<const float4 *>(ref + c0);
#pragma unroll
        for (int k = 0; k < S / 4; ++k) {
          const float4 u = __ldg(g + k);
          R[4 * k] = u.x, R[4 * k + 1] = u.y, R[4 * k + 2] = u.z, R[4 * k + 3] = u.w;
        }
      }
      if (lane == kWarp - 1) seam_out[0] = D[S - 1];

      // Lane l computes row pair t - l (rows 2(t - l) and 2(t - l) + 1) at
      // step t.  From lane l-1 it takes the last cells of the same two rows
      // (computed at step t - 1) and, as the diagonal of the pair's first row,
      // the last cell of the row before (received one step earlier).
      const int pairs = (n + 1) >> 1;
      const float up0 = __shfl_up_sync(FULL_MASK, D[S - 1], 1);  // every lane takes part in the shuffle
      float diag_next = lane == 0 ? (first ? inf : seam_in[0]) : up0;
      float q0n = q[0], q1n = n > 1 ? q[1] : 0.f;  // lane 0's first pair
      float s0n = first ? inf : seam_in[1], s1n = first || n < 2 ? inf : seam_in[2];
      float last_a = D[S - 1];  // this lane's last cell of the pair's first row (after each step)

      for (int st = 0; st < pairs + kWarp - 1; ++st) {
        const int pi = st - lane;  // this lane's pair
        const int r = 2 * pi;
        const float q0 = q0n, q1 = q1n, s0 = s0n, s1 = s1n;
        {
          // next step's pair, clamped (rows outside [0, n) compute nothing)
          int j = r + 2;
          j = j < 0 ? 0 : (j >= n ? n - 1 : j);
          q0n = q[j];
          q1n = q[j + 1 < n ? j + 1 : n - 1];
          if (!first) {
            const int rr = 2 * (st + 1);  // lane 0's next rows rr, rr + 1 at seam [rr + 1], [rr + 2]
            s0n = rr + 1 <= n ? seam_in[rr + 1] : inf;
            s1n = rr + 2 <= n ? seam_in[rr + 2] : inf;
          }
        }
        const float ua = __shfl_up_sync(FULL_MASK, last_a, 1);
        const float ub = __shfl_up_sync(FULL_MASK, D[S - 1], 1);
        float left0 = lane == 0 ? s0 : ua;
        const float left1 = lane == 0 ? s1 : ub;
        const float diag0 = diag_next;
        diag_next = left1;
        const bool ok0 = (unsigned)r < (unsigned)n, ok1 = (unsigned)(r + 1) < (unsigned)n;
        if (st >= kWarp - 1 && 2 * st + 1 < n) {
          refdel_step2<S, false>(D, R, q0, q1, diag0, left0, left1, true, true);
        } else {
          refdel_step2<S, true>(D, R, q0, q1, diag0, left0, left1, ok0, ok1);
        }
        last_a = left0;
        if (lane == kWarp - 1) {
          if (ok0) seam_out[r + 1] = left0;
          if (ok1) seam_out[r + 2] = D[S - 1];
        }
      }

      // every lane now holds row n - 1 of its columns
#pragma unroll
      for (int k = 0; k < S; ++k) {
        const int64_t col = c0 + k;
        if (col < p.m && D[k] < best) {
          best = D[k];
          bcol = col;
        }
      }
      if (save) {
        float4 *f = reinterpret_cast<float4 *>(p.state + t.state_off + plane + c0);
#pragma unroll
        for (int k = 0; k < S / 4; ++k) f[k] = make_float4(D[4 * k], D[4 * k + 1], D[4 * k + 2], D[4 * k + 3]);
      }
      __syncwarp();  // the next strip reads this strip's seam column
    }
    warp_argmin(best, bcol);
    red_min_if(&p.keys[2 * (int64_t)t.out_slot + strand], make_key(best, bcol), is0 & (bcol >= 0 ? 1u : 0u));
  }
}

// ---------------------------------------------------------------- FP16 pairs
// The same sweep on __half2 cells (fwd strand in .x, rev in .y; one work item
// covers both).  FP16 keeps the path cost in range with running-minimum
// frames, here one per lane: lane l holds its cells relative to a float2
// offset O_l, its own minimum at the last rescale (every kRefDelPairsRescale
// steps, i.e. 32 rows, all lanes at the same step).  A value crossing from
// lane l-1 is re-based by O_{l-1} - O_l in FP32 and rounded to FP16 at the
// magnitude of the result.  With horizontal moves allowed, neighbouring
// frames differ by at most the cost of a horizontal run, so the re-based
// values stay in range.  Lane 0 re-bases the left strip's seam column, which
// travels as absolute FP32 pairs.

constexpr int kRefDelPairsRescale = 16;  // steps (2 rows each) between rescales

template <int S, bool RAMP>
__device__ __forceinline__ void refdel_step2_pairs(__half2 (&D)[S], const __half2 (&R)[S], __half2 q0, __half2 q1,
                                                   __half2 diag0, __half2 &left0, __half2 left1, bool ok0,
                                                   bool ok1) {
  __half2 diag1 = left0;
#pragma unroll
  for (int k = 0; k < S; ++k) {
    const __half2 d0 = __hsub2(R[k], q0);
    const __half2 d1 = __hsub2(R[k], q1);
    const __half2 up = D[k];
    const __half2 a = __hfma2(d0, d0, __hmin2(__hmin2(up, diag0), left0));
    const __half2 b = __hfma2(d1, d1, __hmin2(__hmin2(a, diag1), left1));
    if constexpr (RAMP)
      D[k] = ok1 ? b : (ok0 ? a : up);
    else
      D[k] = b;
    diag0 = up;
    left0 = a;
    diag1 = a;
    left1 = b;
  }
}

__device__ __forceinline__ __half2 rebase(float2 v, float2 dl) {
  return __floats2half2_rn(v.x + dl.x, v.y + dl.y);
}

// 128 registers: the kernel would take 165 (12 warps per SM); capped, a few
// values spill outside the cell loop and 16 warps per SM hide more of the
// cell chain's fixed latencies (measured on a 2,048-read batch: +6 % with
// 4-warp CTAs, +10 % with 8-warp CTAs).  With no launch bounds it takes up
// to 16-warp CTAs, one per SM: the default spreads a batch that way.
template <int S>
__global__ void __maxnreg__(128) sdtw_refdel_pairs_kernel(const SdtwParams p) {
  static_assert(S % 4 == 0, "row state moves in 16-byte groups");
  constexpr int W = kWarp * S;
  const int lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const uint32_t is0 = lane == 0 ? 1u : 0u;
  const float inf = __int_as_float(0x7f800000);
  const __half2 hinf = __half2half2(__ushort_as_half((unsigned short)0x7c00u));
  const int64_t gwarp = (int64_t)blockIdx.x * nwarps + (threadIdx.x >> 5);
  char *seam_base = p.seam + gwarp * p.seam_stride;
  const int64_t seam_half = p.seam_stride / 2;
  const int per_task = p.n_chunks;
  const int64_t n_items = (int64_t)p.n_tasks * per_task;
  const int64_t strips = (p.m + W - 1) / W;

  for (;;) {
    const int item = __shfl_sync(FULL_MASK, ticket_if(p.counter, is0), 0);
    if (item >= n_items) break;
    const int tr = item / per_task;
    if (item - tr * per_task != 0) continue;  // one chunk per task: chunk 0 sweeps every strip
    const int ti = p.order ? p.order[tr] : tr;
    const Task t = p.tasks[ti];
    const int n = t.n;
    if (n <= 0 || n > p.max_rows) {
      if (n > p.max_rows) atomicOr(p.err, kErrBadTask);  // every lane: same bit
      continue;
    }
    const float *q = p.query + t.q_off;
    const bool resume = (t.flags & kTaskResume) != 0 && p.state != nullptr;
    const bool save = (t.flags & kTaskSaveState) != 0 && p.state != nullptr;
    const __half2 *ref = static_cast<const __half2 *>(p.ref_plain);

    float bestx = inf, besty = inf;
    int64_t colx = -1, coly = -1;
    for (int64_t s = 0; s < strips; ++s) {
      const int64_t c0 = s * W + (int64_t)lane * S;
      const bool first = s == 0;
      // seam column of the left strip, absolute FP32 pairs: row -1 at [0], row i at [i + 1]
      const float2 *seam_in = reinterpret_cast<const float2 *>(seam_base + ((s + 1) & 1) * seam_half);
      float2 *seam_out = reinterpret_cast<float2 *>(seam_base + (s & 1) * seam_half);

      __half2 D[S], R[S];
      float2 O = make_float2(0.f, 0.f);  // this lane's frame
      if (resume) {
        // FP32 row state (fwd plane, rev plane at m_pad): the frame is the lane's minimum
        const float4 *f0 = reinterpret_cast<const float4 *>(p.state + t.state_off + c0);
        const float4 *f1 = reinterpret_cast<const float4 *>(p.state + t.state_off + p.m_pad + c0);
        float mx = inf, my = inf;
#pragma unroll
        for (int k = 0; k < S / 4; ++k) {
          const float4 u = f0[k], v = f1[k];
          mx = fminf(mx, fminf(fminf(u.x, u.y), fminf(u.z, u.w)));
          my = fminf(my, fminf(fminf(v.x, v.y), fminf(v.z, v.w)));
        }
        O = make_float2(isinf(mx) ? 0.f : mx, isinf(my) ? 0.f : my);
#pragma unroll
        for (int k = 0; k < S / 4; ++k) {
          const float4 u = f0[k], v = f1[k];
          D[4 * k] = __floats2half2_rn(u.x - O.x, v.x - O.y);
          D[4 * k + 1] = __floats2half2_rn(u.y - O.x, v.y - O.y);
          D[4 * k + 2] = __floats2half2_rn(u.z - O.x, v.z - O.y);
          D[4 * k + 3] = __floats2half2_rn(u.w - O.x, v.w - O.y);
        }
      } else {
#pragma unroll
        for (int k = 0; k < S; ++k) D[k] = __float2half2_rn(0.f);
      }
      {
        const uint4 *g = reinterpret_cast<const uint4 *>(ref + c0);
#pragma unroll
        for (int k = 0; k < S / 4; ++k) {
          const uint4 u = __ldg(g + k);
          memcpy(&R[4 * k], &u.x, 4);
          memcpy(&R[4 * k + 1], &u.y, 4);
          memcpy(&R[4 * k + 2], &u.z, 4);
          memcpy(&R[4 * k + 3], &u.w, 4);
        }
      }
      if (lane == kWarp - 1) {
        const float2 v = __half22float2(D[S - 1]);
        seam_out[0] = make_float2(v.x + O.x, v.y + O.y);
      }

      // dl re-bases a value arriving on this lane's left into its frame: from
      // lane l-1 (that lane's frame minus this one) or, on lane 0, from the
      // absolute seam column (minus this frame)
      float2 dl;
      {
        const float ox = __shfl_up_sync(FULL_MASK, O.x, 1), oy = __shfl_up_sync(FULL_MASK, O.y, 1);
        dl = lane == 0 ? make_float2(-O.x, -O.y) : make_float2(ox - O.x, oy - O.y);
      }
      const __half2 up0 = __shfl_up_sync(FULL_MASK, D[S - 1], 1);  // every lane takes part in the shuffle
      __half2 diag_next = lane == 0 ? (first ? hinf : rebase(seam_in[0], dl)) : rebase(__half22float2(up0), dl);
      const int pairs = (n + 1) >> 1;
      float q0n = q[0], q1n = n > 1 ? q[1] : 0.f;  // lane 0's first pair
      const float2 finf = make_float2(inf, inf);
      float2 s0n = first ? finf : seam_in[1], s1n = first || n < 2 ? finf : seam_in[2];
      __half2 last_a = D[S - 1];

      for (int st = 0; st < pairs + kWarp - 1; ++st) {
        const int r = 2 * (st - lane);  // this lane's rows r, r + 1
        const __half2 q0 = __float2half2_rn(q0n), q1 = __float2half2_rn(q1n);
        const float2 s0 = s0n, s1 = s1n;
        {
          int j = r + 2;  // next step's rows, clamped (rows outside [0, n) compute nothing)
          j = j < 0 ? 0 : (j >= n ? n - 1 : j);
          q0n = q[j];
          q1n = q[j + 1 < n ? j + 1 : n - 1];
          if (!first) {
            const int rr = 2 * (st + 1);
            s0n = rr + 1 <= n ? seam_in[rr + 1] : finf;
            s1n = rr + 2 <= n ? seam_in[rr + 2] : finf;
          }
        }
        const __half2 ua = __shfl_up_sync(FULL_MASK, last_a, 1);
        const __half2 ub = __shfl_up_sync(FULL_MASK, D[S - 1], 1);
        __half2 left0 = rebase(lane == 0 ? s0 : __half22float2(ua), dl);
        const __half2 left1 = rebase(lane == 0 ? s1 : __half22float2(ub), dl);
        const __half2 diag0 = diag_next;
        diag_next = left1;
        const bool ok0 = (unsigned)r < (unsigned)n, ok1 = (unsigned)(r + 1) < (unsigned)n;
        if (st >= kWarp - 1 && 2 * st + 1 < n) {
          refdel_step2_pairs<S, false>(D, R, q0, q1, diag0, left0, left1, true, true);
        } else {
          refdel_step2_pairs<S, true>(D, R, q0, q1, diag0, left0, left1, ok0, ok1);
        }
        last_a = left0;
        if (lane == kWarp - 1) {
          if (ok0) {
            const float2 v = __half22float2(left0);
            seam_out[r + 1] = make_float2(v.x + O.x, v.y + O.y);
          }
          if (ok1) {
            const float2 v = __half22float2(D[S - 1]);
            seam_out[r + 2] = make_float2(v.x + O.x, v.y + O.y);
          }
        }
        if (st % kRefDelPairsRescale == kRefDelPairsRescale - 1) {
          // rescale (every lane at the same step): subtract this lane's minimum
          __half2 mn = D[0];
#pragma unroll
          for (int k = 1; k < S; ++k) mn = __hmin2(mn, D[k]);
          float2 mf = __half22float2(mn);
          mf.x = isinf(mf.x) ? 0.f : mf.x;  // all-infinite cells stay as they are
          mf.y = isinf(mf.y) ? 0.f : mf.y;
          mn = __floats2half2_rn(mf.x, mf.y);  // exact: the components are FP16 values
#pragma unroll
          for (int k = 0; k < S; ++k) D[k] = __hsub2(D[k], mn);
          last_a = __hsub2(last_a, mn);
          diag_next = __hsub2(diag_next, mn);
          O.x += mf.x;
          O.y += mf.y;
          const float ox = __shfl_up_sync(FULL_MASK, O.x, 1), oy = __shfl_up_sync(FULL_MASK, O.y, 1);
          dl = lane == 0 ? make_float2(-O.x, -O.y) : make_float2(ox - O.x, oy - O.y);
        }
      }

      // every lane now holds row n - 1 of its columns (relative to O)
#pragma unroll
      for (int k = 0; k < S; ++k) {
        const float2 v = __half22float2(D[k]);
        const float vx = v.x + O.x, vy = v.y + O.y;
        const int64_t col = c0 + k;
        if (col < p.m) {
          if (vx < bestx) {
            bestx = vx;
            colx = col;
          }
          if (vy < besty) {
            besty = vy;
            coly = col;
          }
        }
      }
      if (save) {
        float4 *f0 = reinterpret_cast<float4 *>(p.state + t.state_off + c0);
        float4 *f1 = reinterpret_cast<float4 *>(p.state + t.state_off + p.m_pad + c0);
#pragma unroll
        for (int k = 0; k < S / 4; ++k) {
          const float2 v0 = __half22float2(D[4 * k]), v1 = __half22float2(D[4 * k + 1]);
          const float2 v2 = __half22float2(D[4 * k + 2]), v3 = __half22float2(D[4 * k + 3]);
          f0[k] = make_float4(v0.x + O.x, v1.x + O.x, v2.x + O.x, v3.x + O.x);
          f1[k] = make_float4(v0.y + O.y, v1.y + O.y, v2.y + O.y, v3.y + O.y);
        }
      }
      __syncwarp();  // the next strip reads this strip's seam column
    }
    warp_argmin(bestx, colx);
    warp_argmin(besty, coly);
    const int64_t base = 2 * (int64_t)t.out_slot;
    red_min_if(&p.keys[base], make_key(bestx, colx), is0 & (colx >= 0 ? 1u : 0u));
    red_min_if(&p.keys[base + 1], make_key(besty, coly), is0 & (coly >= 0 ? 1u : 0u));
  }
}

namespace {

template <int S>
cudaError_t launch_refdel_inst(int warps, int grid, const SdtwParams &p, cudaStream_t s) {
  sdtw_refdel_kernel<S><<<grid, warps * kWarp, 0, s>>>(p);
  return cudaGetLastError();
}

template <int S>
cudaError_t launch_refdel_pairs_inst(int warps, int grid, const SdtwParams &p, cudaStream_t s) {
  sdtw_refdel_pairs_kernel<S><<<grid, warps * kWarp, 0, s>>>(p);
  return cudaGetLastError();
}

template <int S>
int occ_refdel_pairs_inst(int warps) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sdtw_refdel_pairs_kernel<S>, warps * kWarp, 0) !=
      cudaSuccess)
    return 0;
  return n;
}

template <int S>
int occ_refdel_inst(int warps) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sdtw_refdel_kernel<S>, warps * kWarp, 0) != cudaSuccess)
    return 0;
  return n;
}

}  // namespace

cudaError_t launch_refdel_fp32(int cells_per_thread, int warps_per_cta, int grid, const SdtwParams &p,
                               cudaStream_t s) {
  if (cells_per_thread == 16) return launch_refdel_inst<16>(warps_per_cta, grid, p, s);
  if (cells_per_thread == 32) return launch_refdel_inst<32>(warps_per_cta, grid, p, s);
  return cudaErrorInvalidValue;
}

int refdel_fp32_ctas_per_sm(int cells_per_thread, int warps_per_cta) {
  if (cells_per_thread == 16) return occ_refdel_inst<16>(warps_per_cta);
  if (cells_per_thread == 32) return occ_refdel_inst<32>(warps_per_cta);
  return 0;
}

cudaError_t launch_refdel_pairs(int cells_per_thread, int warps_per_cta, int grid, const SdtwParams &p,
                                cudaStream_t s) {
  if (cells_per_thread == 32) return launch_refdel_pairs_inst<32>(warps_per_cta, grid, p, s);
  return cudaErrorInvalidValue;
}

int refdel_pairs_ctas_per_sm(int cells_per_thread, int warps_per_cta) {
  if (cells_per_thread == 32) return occ_refdel_pairs_inst<32>(warps_per_cta);
  return 0;
}

}  // namespace dtwx
