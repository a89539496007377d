// dtwx_distances_static: the FP32 sDTW sweep for callers that must not allocate
// device memory.
//
// Who needs it: a process that shares the GPU with a basecaller whose memory
// pool has already reserved the device (a foreign cudaMalloc may fail there, or
// squeeze the basecaller out of memory), and real-time Read Until loops that
// cannot afford cudaMalloc/cudaFree, which may synchronise the whole device and
// stall every decision behind them.  Such callers bring the reference squiggle,
// the z-scored reads and the result buffer in memory they already own; the
// scratch the sweep needs (task table, work counter, per-warp seam columns,
// per-read result keys) lives in the fixed array below, which the library
// reserves once when it is loaded onto a GPU and keeps until the process exits.
#include <mutex>

#include "dtwx.h"
#include "dtwx_internal.h"

namespace dtwx {
namespace {

// Limits of the static scratch.
constexpr int kStMaxReads = 4096;   // reads per call
constexpr int kStMaxRows = 2048;    // samples per read (QUERY_LEN of the reference)
constexpr int kStCells = 16;        // FP32 instance: 16 column pairs per lane (512-column strips)
constexpr int kStWarps = 4;         // warps per CTA
constexpr int kStCtas = 64;         // CTAs: 256 warps share the queue
constexpr int kStPairBytes = 8;     // float2 (fwd, rev)

constexpr int64_t align256(int64_t x) { return (x + 255) & ~(int64_t)255; }
// seam scratch of one warp: the kernel's own layout (seam_bytes_per_warp, with
// its slack for whole-warp stores past the last row) for the widest seam entry
// the FP32 sweep could use, so that a change of the cell size or the slack
// cannot let a warp write past the array
constexpr int64_t kStSeamPerWarp = seam_bytes_per_warp(kStPairBytes, kStMaxRows);
static_assert(kStPairBytes >= 4, "FP32 seam cells are 4 bytes");
static_assert(kStSeamPerWarp % 256 == 0, "per-warp seam scratch keeps 256-byte alignment");

constexpr int64_t kStFlagsOff = 0;                                                // counter, error flags
constexpr int64_t kStKeysOff = 256;                                               // 2 x u64 per read
constexpr int64_t kStTasksOff = align256(kStKeysOff + 16 * (int64_t)kStMaxReads);  // Task per read
constexpr int64_t kStNsampOff = align256(kStTasksOff + 32 * (int64_t)kStMaxReads); // int32 per read
constexpr int64_t kStSeamOff = align256(kStNsampOff + 4 * (int64_t)kStMaxReads);
constexpr int64_t kStBytes = kStSeamOff + kStSeamPerWarp * kStWarps * kStCtas;     // about 9 MiB
static_assert(kStSeamOff + seam_bytes_per_warp(4, kStMaxRows) * kStWarps * kStCtas <= kStBytes,
              "every warp's seam columns fit in the static scratch");

// The scratch itself.  Host code must never pass this name to a kernel: on the
// host it is only a stand-in symbol, not a device address.  The device address
// comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_static_scratch[kStBytes];

constexpr int kStMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kStMaxDevices] = {};

// Device address of g_static_scratch on the current device (looked up once).
cudaError_t scratch_address(int dev, unsigned char **out) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = p;
  }
  *out = static_cast<unsigned char *>(g_addr[dev]);
  return cudaSuccess;
}

int st_fail(int code, const char *msg) {
  set_create_error(msg);
  return code;
}

}  // namespace
}  // namespace dtwx

using namespace dtwx;

extern "C" int dtwx_distances_static(const void *d_ref_pairs, int64_t ref_len, const float *d_query,
                                     const int64_t *offsets, int32_t n_reads, float threshold,
                                     dtwx_result *d_out, void *stream) {
  if (n_reads < 0 || ref_len <= 0 || !offsets || (n_reads > 0 && (!d_ref_pairs || !d_query || !d_out)))
    return st_fail(DTWX_E_ARG, "dtwx_distances_static: bad arguments");
  if (n_reads > 0 && offsets[0] < 0)
    return st_fail(DTWX_E_ARG, "dtwx_distances_static: offsets must start at 0 or later");
  if ((reinterpret_cast<uintptr_t>(d_ref_pairs) & 15) != 0)
    return st_fail(DTWX_E_ARG, "dtwx_distances_static: d_ref_pairs must be 16-byte aligned");
  if ((reinterpret_cast<uintptr_t>(d_out) & 7) != 0)
    return st_fail(DTWX_E_ARG, "dtwx_distances_static: d_out must be 8-byte aligned");
  if (n_reads > kStMaxReads)
    return st_fail(DTWX_E_CAPACITY, "dtwx_distances_static: more than 4096 reads in one call");
  if (ref_len >= ((int64_t)1 << 32)) return st_fail(DTWX_E_CAPACITY, "dtwx_distances_static: reference too long");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return st_fail(DTWX_E_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kStMaxDevices) return st_fail(DTWX_E_CAPACITY, "dtwx_distances_static: device ordinal");
  unsigned char *base = nullptr;
  e = scratch_address(dev, &base);
  if (e != cudaSuccess) return st_fail(DTWX_E_CUDA, cudaGetErrorString(e));
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  // Host-side task table in a fixed host array (no allocation either).
  static thread_local Task h_tasks[kStMaxReads];
  static thread_local int32_t h_nsamp[kStMaxReads];
  int32_t n_tasks = 0;
  for (int r = 0; r < n_reads; ++r) {
    const int64_t n = offsets[r + 1] - offsets[r];
    if (n < 0) return st_fail(DTWX_E_ARG, "dtwx_distances_static: offsets must be non-decreasing");
    if (n > kStMaxRows)
      return st_fail(DTWX_E_CAPACITY, "dtwx_distances_static: a read is longer than 2048 samples");
    h_nsamp[r] = (int32_t)n;
    if (n == 0) continue;
    Task &t = h_tasks[n_tasks++];
    t.q_off = offsets[r];
    t.n = (int32_t)n;
    t.flags = 0;
    t.state_off = 0;
    t.out_slot = r;
    t.pad = 0;
  }
  if (n_reads == 0) return DTWX_OK;

  int32_t *flags = reinterpret_cast<int32_t *>(base + kStFlagsOff);
  unsigned long long *keys = reinterpret_cast<unsigned long long *>(base + kStKeysOff);
  Task *d_tasks = reinterpret_cast<Task *>(base + kStTasksOff);
  int32_t *d_nsamp = reinterpret_cast<int32_t *>(base + kStNsampOff);
  // Every call reuses the same bytes: zero the counter and error flags, reset
  // the keys, then overwrite the task table.  Seam columns are always written
  // before they are read, so they need no clearing.
  if ((e = cudaMemsetAsync(flags, 0, 64, st)) != cudaSuccess) return st_fail(DTWX_E_CUDA, cudaGetErrorString(e));
  if (n_tasks &&
      (e = cudaMemcpyAsync(d_tasks, h_tasks, sizeof(Task) * n_tasks, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return st_fail(DTWX_E_CUDA, cudaGetErrorString(e));
  if ((e = cudaMemcpyAsync(d_nsamp, h_nsamp, sizeof(int32_t) * n_reads, cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return st_fail(DTWX_E_CUDA, cudaGetErrorString(e));
  if ((e = launch_reset(keys, 2 * n_reads, flags, flags + 4, st)) != cudaSuccess)
    return st_fail(DTWX_E_CUDA, cudaGetErrorString(e));
  if (n_tasks) {
    SdtwParams p{};
    p.query = d_query;
    p.tasks = d_tasks;
    p.order = nullptr;
    p.keys = keys;
    p.state = nullptr;
    p.seam = reinterpret_cast<char *>(base + kStSeamOff);
    p.counter = flags;
    p.err = flags + 4;
    p.ref_plain = d_ref_pairs;
    p.m = ref_len;
    p.m_pad = ref_len;
    p.seam_stride = kStSeamPerWarp;
    p.n_tasks = n_tasks;
    const int64_t W = (int64_t)kWarp * kStCells;
    const int64_t strips = (ref_len + W - 1) / W;
    // one chunk of G strips per item: about 4 items per warp for the whole batch
    int64_t g = (strips * n_tasks + 4LL * kStWarps * kStCtas - 1) / (4LL * kStWarps * kStCtas);
    if (g < 1) g = 1;
    if (g > strips) g = strips;
    p.chunk_strips = (int32_t)g;
    p.n_chunks = (int32_t)((strips + g - 1) / g);
    p.max_rows = kStMaxRows;
    p.n_items = (int32_t)((int64_t)n_tasks * p.n_chunks);
    p.use_tma = 0;
    if ((e = launch_sdtw(1, kStCells, kStWarps, kStCtas, p, nullptr, st)) != cudaSuccess)
      return st_fail(DTWX_E_CUDA, cudaGetErrorString(e));
  }
  if ((e = launch_finalize(keys, d_nsamp, n_reads, 0, ref_len, threshold, flags + 4, d_out, st)) != cudaSuccess)
    return st_fail(DTWX_E_CUDA, cudaGetErrorString(e));
  return DTWX_OK;
}
