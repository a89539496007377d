// Internal definitions shared by the CUDA kernels and the host side of libdtwx.
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace dtwx {

constexpr int kWarp = 32;
constexpr int kKmer = 6;
constexpr int kTableSize = 4096;
// Rows between two running-minimum rescales of the FP16 cells.
constexpr int kRescaleRows = 32;

// Narrow halo strips.  A column chunk starting at a > 0 recomputes a halo on
// its left; the columns that still reach column a shrink by one per row, so
// narrower halo strips stop sooner: 16-cell strips cut the halo of a
// 1,600-row chunk from about 1.04 to 0.69 strips of 1,536 columns.  FP16-pair
// kernels come in a second instance with such strips, launched when chunks
// are narrow (at most kNarrowHaloMaxStrips strips, i.e. small batches) and
// the halo is a large part of an item; wide-chunk batches keep the
// full-width-halo instance, whose register allocation the halo loop would
// otherwise change.
constexpr int kNarrowHaloCells = 16;
constexpr int kNarrowHaloMaxStrips = 32;
// Bounded device-side waits: polls of mbarrier.try_wait before a wait gives up
// and flags an error.  A poll that finds the phase incomplete suspends the
// warp for a few microseconds (measured on GB300: 4,096 polls in about 15 ms),
// so 2^18 polls bound a wait at about one second; a strip copy lands in
// microseconds.  The count does not advance while the context is switched out.
constexpr uint32_t kSpinLimit = 1u << 18;

// Task flags.
constexpr int32_t kTaskResume = 1;    // start from the saved row state instead of free start
constexpr int32_t kTaskSaveState = 2; // write the final DP row to the row state

// One unit of DP work: a read (offline) or one chunk of a read (serving).
// Rows are query samples query[q_off .. q_off + n); every output column of the
// reference is covered by the work items (task, chunk) of the task.
struct Task {
  int64_t q_off;     // offset of the first sample in the query buffer
  int32_t n;         // rows (samples) in this task
  int32_t flags;     // kTaskResume | kTaskSaveState
  int64_t state_off; // offset, in columns, of this read's row state
  int32_t out_slot;  // result slot: keys[2*out_slot + strand]
  int32_t pad;
};
static_assert(sizeof(Task) == 32, "Task layout");

// Device error flags (bit mask in *err).
constexpr int32_t kErrTmaTimeout = 1;
constexpr int32_t kErrBadTask = 2;
// dtwx_result.call of every read of a call whose kernels set a device error
// flag (DTWX_CALL_DEVICE_ERROR of include/dtwx.h).
constexpr int32_t kCallDeviceError = -2;

struct SdtwParams {
  const float *query;          // z-scored samples, FP32
  const Task *tasks;           // n_tasks
  const int32_t *order;        // processing order of tasks (longest first); NULL = identity
  unsigned long long *keys;    // 2 per out slot: (orderable score << 32) | end column
  float *state;                // row-state pool (absolute FP32 values, per read a fwd and a rev
                               // plane of m_pad floats; or the FP16 layout of state_fp16), NULL if unused
  char *seam;                  // per-warp scratch (seam columns + epoch offsets)
  int32_t *counter;            // work-queue ticket counter (zeroed before launch)
  int32_t *err;                // device error flags
  const void *ref_plain;       // reference in global memory (used when TMA is off)
  int64_t m;                   // valid columns per strand
  int64_t m_pad;               // padded columns (multiple of the strip width)
  int64_t seam_stride;         // bytes of scratch per warp
  int32_t n_tasks;
  int32_t n_chunks;            // chunks per task
  int32_t chunk_strips;        // strips per chunk
  int32_t max_rows;            // capacity of the seam buffers (rows)
  int32_t n_items;             // informational: the kernel derives the queue length itself
  int32_t use_tma;
  int32_t ref_layout;          // FP32: 0 = interleaved (fwd, rev) float pairs, 1 = planar (rev plane at m_pad);
                               // MIXED is always planar FP16
  int32_t strands;             // FP32/MIXED strands per task: 2 (paired), 1 (concatenated sequence); 0 = 2
  int32_t ref_del;             // 1: REF_DEL recurrence (left predecessor); needs one chunk per task
  int32_t state_fp16;          // FP16 cells: row state as half2 cells (m_pad) then one float2
                               // frame offset per 512-column group (m_pad / 512)
  int32_t narrow_halo;         // FP16 pairs: launch the instance with kNarrowHaloCells-wide halo strips
  uint32_t spin_limit;         // polls before a bounded wait gives up; 0 = kSpinLimit
  int32_t stall_item;          // test hook: 1 + the queue ticket whose first reference-strip copy
                               // is not issued, so that its warp's bounded wait runs out; 0 = none
};

// Per-warp scratch layout, in bytes, for cells of `pair_bytes` bytes.
// Each half (one per strip parity) holds the seam column, (max_rows + 1)
// cells plus 32 of slack (whole-warp stores past the last row land there),
// then from a 16-byte aligned position the FP32 offsets of the epochs,
// (max_rows / kRescaleRows + 2) float2 plus 32 of slack.
constexpr __host__ __device__ int64_t seam_offsets_pos(int pair_bytes, int max_rows) {
  return ((int64_t)(max_rows + 1 + 32) * pair_bytes + 15) & ~(int64_t)15;
}
constexpr __host__ __device__ int64_t seam_bytes_per_warp(int pair_bytes, int max_rows) {
  // ping-pong between consecutive strips
  return 2 * ((seam_offsets_pos(pair_bytes, max_rows) + (int64_t)(max_rows / kRescaleRows + 2 + 32) * 8 + 255) &
              ~(int64_t)255);
}

// Orderable 32-bit image of a float: unsigned order == float order.
__host__ __device__ inline uint32_t float_to_ordered(float f) {
  uint32_t u;
#ifdef __CUDA_ARCH__
  u = __float_as_uint(f);
#else
  memcpy(&u, &f, 4);
#endif
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float ordered_to_float(uint32_t o) {
  uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  float f;
#ifdef __CUDA_ARCH__
  f = __uint_as_float(u);
#else
  memcpy(&f, &u, 4);
#endif
  return f;
}

// ---------------------------------------------------------------- launchers
// (defined in the .cu files; all return cudaError_t of the launch)

// sDTW over all (task, chunk) items.  precision: 0 FP16, 1 FP32, 2 MIXED;
// p.ref_del selects the REF_DEL kernels (the anti-diagonal sweeps of
// refdel.cu for FP32 cells and FP16 pairs).  cells_per_thread must be one
// of the compiled instances.
cudaError_t launch_sdtw(int precision, int cells_per_thread, int warps_per_cta, int grid,
                        const SdtwParams &p, const CUtensorMap *tmap, cudaStream_t s);
// Dynamic shared memory the sDTW kernel needs per CTA.
size_t sdtw_smem_bytes(int precision, int cells_per_thread, int warps_per_cta);
// Resident CTAs per SM for the given shape (occupancy API), 0 on error.
int sdtw_ctas_per_sm(int precision, int cells_per_thread, int warps_per_cta, bool ref_del = false);
bool sdtw_instance_exists(int precision, int cells_per_thread, bool ref_del = false);
// The REF_DEL kernels of refdel.cu, one chunk per task: FP32 cells (16 or 32
// cells per lane) and FP16 pairs (32).
cudaError_t launch_refdel_fp32(int cells_per_thread, int warps_per_cta, int grid, const SdtwParams &p,
                               cudaStream_t s);
int refdel_fp32_ctas_per_sm(int cells_per_thread, int warps_per_cta);
cudaError_t launch_refdel_pairs(int cells_per_thread, int warps_per_cta, int grid, const SdtwParams &p,
                                cudaStream_t s);
int refdel_pairs_ctas_per_sm(int cells_per_thread, int warps_per_cta);
int sdtw_pair_bytes(int precision, bool ref_del = false);  // bytes per seam entry (per row)
int sdtw_ref_bytes(int precision);   // reference bytes per column of a strip

// Reference builder: genome bytes -> z-scored levels as FP16 (fwd, rev) pairs,
// as FP32 planes (fwd plane, then rev plane at m_pad) and as FP16 planes.
cudaError_t launch_build_reference(const char *d_seq, int64_t L, const double *d_table,
                                   int64_t m, int64_t m_pad, int concat, double *d_work,
                                   __half2 *d_ref16, float *d_ref32, __half *d_ref16p, float *d_fwd32,
                                   float *d_rev32, cudaStream_t s);
size_t build_reference_work_bytes(int64_t m);

// Window + z-score of raw reads into the query buffer.
// src: raw samples (float or int16 when is_i16); for read r the window starts at
// src_off[r] and has dst_len[r] samples written to dst + dst_off[r].
cudaError_t launch_normalize(const void *src, int is_i16, const int64_t *src_off,
                             const int64_t *dst_off, const int32_t *dst_len,
                             const float *scale_mul, const float *scale_add, int n_reads,
                             float eps, float *dst, cudaStream_t s);

// Keys -> dtwx_result records.  When the device error word `err` (may be
// NULL) is non-zero, every record of the call is marked call =
// DTWX_CALL_DEVICE_ERROR with the error bits in `strand` and NaN scores: the
// sweep did not finish, so no score of the call can be trusted.
cudaError_t launch_finalize(const unsigned long long *keys, const int32_t *n_samples,
                            int n_reads, int concat, int64_t m_fwd, float threshold,
                            const int32_t *err, void *d_results, cudaStream_t s);

// Reset keys to the empty value, the work counter and the device error word
// (either may be NULL) to zero.
cudaError_t launch_reset(unsigned long long *keys, int n_keys, int32_t *counter, int32_t *err,
                         cudaStream_t s);

// Record the message dtwx_last_error(NULL) reports (calls made without a handle).
void set_create_error(const char *msg);

// Issue-rate probe.
cudaError_t launch_peak_probe(int precision, int grid, int block, int iters,
                              float *sink, cudaStream_t s);

}  // namespace dtwx
