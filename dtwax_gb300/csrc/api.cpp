// libdtwx host side: the C ABI of include/dtwx.h.
//
// One handle = one target genome on one GPU.  The handle owns the z-scored
// reference squiggle (FP16 and FP32 pair layouts), a TMA tensor map per kernel
// instance, the batch scratch (query buffer, task table, seam columns, result
// keys) and, once serving is started, the pool of per-read DP row states.
#include "dtwx.h"

#include <cudaTypedefs.h>
#include <time.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <deque>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "dtwx_internal.h"
#include "host_util.h"

using namespace dtwx;

static_assert(sizeof(dtwx_result) == 32, "dtwx_result must match the finalize kernel's record");
static_assert(offsetof(dtwx_result, end_pos) == 16, "dtwx_result layout");
static_assert(sizeof(dtwx_config) == 96, "dtwx_config layout (mirrored by the Python binding)");

namespace {

thread_local std::string g_create_err;

constexpr int64_t kPadCols = 6144;  // a multiple of every compiled strip width (512, 1024, 1536, 2048 columns)
constexpr int kServeSlots = 4;      // most serving batches in flight at once, each on its own stream

struct Shape {
  int S = 0;      // cells (column pairs) per lane
  int G = 0;      // strips per chunk
  int warps = 0;  // warps per CTA
  int grid = 0;   // CTAs
  int64_t items = 0;  // work items (while tuning: the candidate's chunk factor per mille)
  bool nh = false;  // narrow halo strips (FP16 pairs, narrow chunks)
};

// Buffers of one batch that may be in flight on its own stream.
struct BatchCtx {
  cudaStream_t stream = nullptr;
  cudaEvent_t meta_free = nullptr;  // pinned meta blob may be rewritten
  cudaEvent_t done = nullptr;
  cudaEvent_t sweep_beg = nullptr, sweep_end = nullptr;  // bracket the last sweep launch
  bool sweep_timed = false;
  DevBuf raw, query, meta, keys, results, seam, flags;
  HostBuf h_raw, h_meta, h_results, h_flags;
  int64_t seam_bytes = 0;
  bool meta_pending = false;
};

struct ServeRead {
  int32_t channel = 0;
  uint64_t read_number = 0;
  int slot = -1;
  int chunks_done = 0;
  int samples_done = 0;
  bool in_batch = false;
  bool queued = false;
  bool last_seen = false;
  std::deque<std::vector<float>> pending;
  std::deque<double> arrivals;
  std::deque<int> is_last;
};

struct ServeTask {
  std::pair<int32_t, uint64_t> key;
  int n;
  double arrival;
  int last;
  double launched = 0;  // host time the batch holding this chunk was launched
};

}  // namespace

struct dtwx_handle {
  dtwx_config cfg{};
  int device = 0;
  int sms = 0;
  int64_t m = 0;       // k-mer positions per strand
  int64_t m_cols = 0;  // DP columns (m, or 2m for the concatenated mode)
  int64_t m_pad = 0;
  DevBuf ref16, ref32, ref16p, fwd32, rev32;  // FP16 pairs, FP32 planes, FP16 planes (MIXED)
  CUtensorMap tmap[3][3]{};  // [precision][instance index]
  bool tmap_ok[3][3]{};
  Shape fixed[3];            // user-fixed parts of the shape (0 = choose)
  // autotuned shapes by (precision, log2 tasks, log2 rows): S, warps and a
  // factor on the analytic chunk width
  struct Tuned {
    int S, warps;
    double g_scale;
  };
  std::map<std::tuple<int, int, int>, Tuned> tuned;
  Shape override_shape;      // set while the autotuner times a candidate
  // CUDA graph of the most recent repeated device batch
  uint64_t graph_key = 0, graph_pending = 0;
  cudaGraphExec_t graph_exec = nullptr;
  int32_t graph_launches = 0;
  int64_t graph_replays = 0;
  bool capturing = false;
  BatchCtx ctx[1 + kServeSlots];  // [0] offline calls, [1..] the serving batches
  std::string err;
  int32_t last_launches = 0;
  Shape last_shape[3];
  // a device-pointer call (dtwx_distances / dtwx_classify_device) was enqueued
  // since the last dtwx_sync; ctx[0].done marks its end on the caller's stream
  bool device_call_pending = false;
  // one-shot test hook of dtwx_debug_stall_next for the next sweep launch
  int32_t stall_item = 0;
  uint32_t stall_spin = 0;
  // serving
  bool serving = false;
  int32_t chunks_per_decision = 3;
  int32_t max_in_flight = 0;
  DevBuf state;  // max_in_flight * m_pad float2
  std::vector<int> free_slots;
  std::map<std::pair<int32_t, uint64_t>, ServeRead> reads;
  std::map<std::pair<int32_t, uint64_t>, double> finished;  // decided reads -> decision time
  std::deque<std::pair<int32_t, uint64_t>> admit_queue;
  std::vector<dtwx_decision> decisions;
  std::vector<double> latencies, queue_times;  // decided reads
  std::vector<ServeTask> inflight[kServeSlots];  // tasks of the serving batch in ctx[1 + s]
  bool running[kServeSlots] = {};
  float accept_per_sample = 0.f, reject_per_sample = 0.f;
  int64_t chunks_submitted = 0, chunks_processed = 0, reads_decided = 0, reads_deferred = 0;
  int32_t batches = 0;
  double batch_reads_sum = 0;
  double batch_ms_sum = 0, batch_ms_max = 0;  // device time of the serving sweeps
};

namespace {

int fail(dtwx_handle *h, int code, const std::string &msg) {
  if (h)
    h->err = msg;
  else
    g_create_err = msg;
  return code;
}

// Ends a stream capture that an error left open, so the caller's stream stays usable.
struct CaptureGuard {
  dtwx_handle *h;
  cudaStream_t st;
  ~CaptureGuard();
};

#define CK(h, call)                                                                         \
  do {                                                                                      \
    cudaError_t _e = (call);                                                                \
    if (_e != cudaSuccess)                                                                  \
      return fail((h), _e == cudaErrorMemoryAllocation ? DTWX_E_NOMEM : DTWX_E_CUDA,        \
                  std::string(#call) + ": " + cudaGetErrorString(_e));                      \
  } while (0)

// compiled sweep instances (cells per lane) by precision
constexpr int kInstS[3][3] = {{32, 48, 0}, {16, 32, 48}, {32, 48, 64}};
int inst_count(int precision) { return precision == 0 ? 2 : 3; }
int inst_index(int precision, int S) {
  for (int i = 0; i < inst_count(precision); ++i)
    if (kInstS[precision][i] == S) return i;
  return 0;
}
int inst_S(int precision, int idx) { return kInstS[precision][idx]; }

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// The reference viewed as rows of 128 bytes (32 x u32); one box = one strip
// (32 lanes x S columns of ref_bytes each), loaded with 128-byte swizzling so
// that each lane's 16-byte reads of its own slice are free of bank conflicts.
// `bytes` = size of the buffer (m_pad FP16 pairs, two planes of m_pad floats,
// or two planes of m_pad halves).
bool make_tmap(CUtensorMap *map, void *base, int64_t bytes, int S, int ref_bytes) {
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t rows = (cuuint64_t)(bytes / 128);
  cuuint64_t dims[2] = {32, rows};
  cuuint64_t strides[1] = {128};
  cuuint32_t box[2] = {32, (cuuint32_t)(32 * S * ref_bytes / 128)};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Analytic launch-shape model: with dynamic work stealing of equal-sized items
// the sweep takes about ceil(items / warps) item times; an item of G strips
// costs G strips plus the recomputed halo.  Halo strips (WH columns wide) stop
// at the last row that still reaches the chunk, so the halo is about the
// triangle n^2/2 rounded up to WH-wide steps: (n + WH) / (2 W) strips of W
// columns, plus about 10 % for the per-row overhead of a narrow strip.
int choose_chunk_strips(int64_t strips_per_read, int64_t n_tasks, double mean_rows, int W, int WH,
                        int64_t total_warps) {
  if (strips_per_read <= 1) return 1;
  const double halo = (mean_rows + WH) / (2.0 * W) * (WH < W ? 1.1 : 1.0);
  double best_t = 1e300;
  int best_g = (int)strips_per_read;
  for (int64_t g = 1; g <= strips_per_read; ++g) {
    const int64_t chunks = (strips_per_read + g - 1) / g;
    if (g > 1 && chunks == (strips_per_read + (g - 1) - 1) / (g - 1)) continue;
    const int64_t items = n_tasks * chunks;
    const double waves = std::ceil((double)items / (double)total_warps);
    const double cost = (double)g + (chunks > 1 ? halo * (double)(chunks - 1) / chunks : 0.0);
    const double t = waves * cost;
    if (t < best_t * 0.999) {
      best_t = t;
      best_g = (int)g;
    }
  }
  return best_g;
}

// Serving row state kept as FP16 cells plus frame offsets (FP16 handles only).
bool state_fp16(const dtwx_handle *h) {
  return h->cfg.state_precision == DTWX_STATE_FP16 && h->cfg.precision == DTWX_FP16;
}

// Floats of row state per read slot: FP32 fwd and rev planes, or half2 cells
// (one float each) then a float2 offset per 512-column group.
int64_t state_slot_floats(const dtwx_handle *h) {
  return state_fp16(h) ? h->m_pad + 2 * (h->m_pad / 512) : 2 * h->m_pad;
}

// Reference buffer a sweep of this precision reads when TMA is off.
const void *ref_for(const dtwx_handle *h, int precision) {
  return precision == 0 ? h->ref16.p : (precision == 2 ? h->ref16p.p : h->ref32.p);
}

int log2_bucket(double x) { return x < 1.0 ? 0 : (int)std::floor(std::log2(x)); }

// Largest CTA each sweep kernel launches with: the FP16-pair REF_DEL kernel is
// capped at 128 registers, so 16 warps fill an SM's register file; the others
// are compiled for at most 256 threads.
int max_warps_per_cta(int precision, bool rd) { return rd && precision == 0 ? 16 : 8; }

// Default warps per CTA of a REF_DEL sweep.  A REF_DEL work item is a whole
// read (strand), so the batch alone sets the parallelism; the items are spread
// evenly over the SMs, one CTA per SM.  Measured on the FP16-pair kernel with
// 2,000-sample reads against 1 Mb: a warp takes 370 ms per read alone or 4 to
// an SM, 487 ms 8 to an SM and 794 ms 16 to an SM, and 16 warps in one CTA
// beat two 8-warp CTAs on the same SM (2,048 reads: 793 against 846 ms;
// 4,096: 1,416 against 1,637 ms).  FP32 keeps 4-warp CTAs for large batches.
int refdel_spread_warps(int precision, int64_t items, int sms) {
  const int64_t per_sm = (std::max<int64_t>(items, 1) + sms - 1) / sms;
  const int cap = precision == 0 ? max_warps_per_cta(precision, true) : 4;
  return (int)std::min<int64_t>(per_sm, cap);
}

// Rows a warp's seam buffers are sized for: the longest read rounded up to
// 1,024 (at least 1,024), or -1 when the buffer offsets would leave int range.
int seam_rows_capacity(int64_t max_rows) {
  const int64_t cap = std::max<int64_t>(1024, (max_rows + 1023) / 1024 * 1024);
  return cap + 64 > INT32_MAX / 8 ? -1 : (int)cap;
}

// Launch shape of a sweep: user-fixed fields win, then an autotuned entry for
// this (precision, batch size, read length) bucket, then the defaults; the
// chunk width comes from the analytic model (times the tuned factor).
Shape pick_shape(dtwx_handle *h, int precision, int64_t n_tasks, double mean_rows) {
  Shape s;
  const Shape &f = h->fixed[precision];
  const Shape &o = h->override_shape;
  double g_scale = 1.0;
  auto t = h->tuned.find(std::make_tuple(precision, log2_bucket((double)n_tasks), log2_bucket(mean_rows)));
  const bool use_t = t != h->tuned.end();
  // defaults measured on the 1 Mb / 2,048-read batch: 48 cells per lane (64 for
  // MIXED, whose reference takes half the registers) in 4-warp CTAs; the REF_DEL
  // kernels default to 32 cells per lane (FP32 cells also have a 16-cell instance)
  const bool rd = h->cfg.recurrence == DTWX_REF_DEL;
  const int def_S = rd ? 32 : (precision == 2 ? 64 : 48);
  s.S = o.S ? o.S : (f.S ? f.S : (use_t ? t->second.S : def_S));
  const int strands = precision == 0 ? 1 : (h->cfg.strand_mode == DTWX_STRANDS_CONCAT ? 1 : 2);
  // warps per CTA: while tuning the candidate's (0 = the default below), else
  // user-fixed, then autotuned, then the default
  s.warps = o.S ? o.warps : (f.warps ? f.warps : (use_t ? t->second.warps : 0));
  if (s.warps <= 0) s.warps = rd ? refdel_spread_warps(precision, n_tasks * strands, h->sms) : 4;
  s.warps = std::min(s.warps, max_warps_per_cta(precision, rd));
  if (use_t && !f.G) g_scale = t->second.g_scale;
  if (o.S) g_scale = o.items > 0 ? o.items / 1000.0 : 1.0;  // candidate factor (per mille) while tuning
  int occ = sdtw_ctas_per_sm(precision, s.S, s.warps, rd);
  if (occ <= 0) occ = 1;
  const int W = kWarp * s.S;
  const int64_t strips = (h->m_cols + W - 1) / W;
  const int64_t total_warps = (int64_t)h->sms * occ * s.warps;
  if (rd) {
    s.G = (int)strips;  // REF_DEL: one chunk per task (a horizontal run crosses any chunk edge)
  } else if (f.G && !o.S) {
    s.G = f.G;
  } else {
    // FP16 pairs: narrow chunks get the narrow-halo instance, so price their halo that way
    const int64_t nt = std::max<int64_t>(n_tasks, 1) * strands;
    int g0 = choose_chunk_strips(strips, nt, mean_rows, W, precision == 0 ? kWarp * kNarrowHaloCells : W,
                                 total_warps);
    if (precision == 0 && g0 > kNarrowHaloMaxStrips) g0 = choose_chunk_strips(strips, nt, mean_rows, W, W, total_warps);
    s.G = std::max(1, (int)std::lround(g0 * g_scale));
  }
  if (s.G > strips) s.G = (int)strips;
  const int64_t chunks = (strips + s.G - 1) / s.G;
  s.nh = precision == 0 && !rd && chunks > 1 && s.G <= kNarrowHaloMaxStrips && s.S % kNarrowHaloCells == 0;
  const int64_t items = n_tasks * chunks * strands;
  // FP16 pairs, default shape, a batch of several waves: the SM's warps in one
  // CTA instead of occ 4-warp CTAs (the same warps per SM, so the same chunks
  // and bits).  Measured on the 2,048-read / 1 Mb batch at 48 cells per lane:
  // 487 against 501 ms; equal on the 8,192-read / 5 Mb one.  Single-wave
  // batches (serving) keep 4-warp CTAs, which leave room for the next batch.
  if (!rd && precision == 0 && !o.S && !f.warps && !use_t && items >= 2 * total_warps && occ > 1) {
    const int full = occ * s.warps;
    if (sdtw_ctas_per_sm(precision, s.S, full, false) == 1) {
      s.warps = full;
      occ = 1;
    }
  }
  s.items = items;
  const int64_t want = (items + s.warps - 1) / s.warps;
  s.grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)h->sms * occ, want));
  return s;
}

char *align16(char *p) { return reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15)); }

// Enqueue reset + sweep + finalize for `tasks` on ctx's stream (or `stream`).
// d_query: device samples; d_nsamp: device per-slot sample counts; d_out:
// n_slots result records.  The task/order arrays travel inside the meta blob
// that the caller already placed at meta offsets off_tasks / off_order.
int enqueue_sweep(dtwx_handle *h, BatchCtx &c, int precision, cudaStream_t st, const float *d_query,
                  const Task *d_tasks, const int32_t *d_order, int64_t n_tasks, int max_rows,
                  double mean_rows, int n_slots, const int32_t *d_nsamp, void *d_out,
                  float *state, bool finalize, int &launches) {
  Shape sh = pick_shape(h, precision, n_tasks, mean_rows);
  // the work counter hands out 32-bit tickets, each warp one past the last item
  if (sh.items + (int64_t)sh.grid * sh.warps >= INT32_MAX)
    return fail(h, DTWX_E_CAPACITY, "batch has more work items than one sweep can number");
  h->last_shape[precision] = sh;
  const int pb = sdtw_pair_bytes(precision, h->cfg.recurrence == DTWX_REF_DEL);
  const int rows_cap = seam_rows_capacity(max_rows);
  if (rows_cap < 0) return fail(h, DTWX_E_CAPACITY, "read longer than a seam buffer can index");
  const int64_t per_warp = seam_bytes_per_warp(pb, rows_cap);
  const int64_t need = per_warp * (int64_t)sh.grid * sh.warps;
  const int strands = h->cfg.strand_mode == DTWX_STRANDS_CONCAT ? 1 : 2;
  CK(h, c.seam.ensure((size_t)need));
  CK(h, c.keys.ensure(sizeof(unsigned long long) * 2 * (size_t)std::max(n_slots, 1)));
  if (!c.flags.p) {
    // counter and error flags start at zero; errors stay set until the host reads them
    CK(h, c.flags.ensure(64));
    CK(h, cudaMemsetAsync(c.flags.p, 0, 64, st));
  }
  int32_t *counter = c.flags.as<int32_t>();
  int32_t *err = counter + 4;
  CK(h, launch_reset(c.keys.as<unsigned long long>(), 2 * n_slots, counter, err, st));
  ++launches;
  if (n_tasks > 0) {
    SdtwParams p{};
    p.query = d_query;
    p.tasks = d_tasks;
    p.order = d_order;
    p.keys = c.keys.as<unsigned long long>();
    p.state = state;
    p.seam = c.seam.as<char>();
    p.counter = counter;
    p.err = err;
    p.ref_plain = ref_for(h, precision);
    p.m = h->m_cols;
    p.m_pad = h->m_pad;
    p.seam_stride = per_warp;
    p.n_tasks = (int32_t)n_tasks;
    const int W = kWarp * sh.S;
    const int64_t strips = (h->m_cols + W - 1) / W;
    p.n_chunks = (int32_t)((strips + sh.G - 1) / sh.G);
    p.chunk_strips = sh.G;
    p.max_rows = rows_cap;
    p.n_items = (int32_t)(n_tasks * p.n_chunks * (precision != 0 ? strands : 1));
    p.ref_layout = 1;
    p.strands = strands;
    p.ref_del = h->cfg.recurrence == DTWX_REF_DEL ? 1 : 0;
    p.state_fp16 = state_fp16(h) ? 1 : 0;
    p.narrow_halo = sh.nh ? 1 : 0;
    p.stall_item = h->stall_item;
    p.spin_limit = h->stall_spin;
    h->stall_item = 0;
    h->stall_spin = 0;
    const int ii = inst_index(precision, sh.S);
    p.use_tma = h->tmap_ok[precision][ii] ? 1 : 0;
    // inside a stream capture the timing events become event-record nodes
    const unsigned ev_flags = h->capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    CK(h, cudaEventRecordWithFlags(c.sweep_beg, st, ev_flags));
    CK(h, launch_sdtw(precision, sh.S, sh.warps, sh.grid, p, p.use_tma ? &h->tmap[precision][ii] : nullptr,
                      st));
    CK(h, cudaEventRecordWithFlags(c.sweep_end, st, ev_flags));
    c.sweep_timed = true;
    ++launches;
  }
  if (finalize) {
    CK(h, launch_finalize(c.keys.as<unsigned long long>(), d_nsamp, n_slots,
                          h->cfg.strand_mode == DTWX_STRANDS_CONCAT, h->m, h->cfg.threshold, err, d_out, st));
    ++launches;
  }
  return DTWX_OK;
}

int check_device_flags(dtwx_handle *h, BatchCtx &c) {
  int32_t f[8] = {0};
  if (!c.flags.p) return DTWX_OK;
  CK(h, cudaMemcpy(f, c.flags.p, sizeof(f), cudaMemcpyDeviceToHost));
  if (f[4]) CK(h, cudaMemset(c.flags.as<int32_t>() + 4, 0, sizeof(int32_t)));  // reported once
  if (f[4] & kErrTmaTimeout) return fail(h, DTWX_E_TIMEOUT, "device: TMA wait gave up");
  if (f[4] & kErrBadTask) return fail(h, DTWX_E_CAPACITY, "device: task longer than the seam buffers");
  return DTWX_OK;
}

// Read windows (adapter skip + query_len) of a batch.
struct Windows {
  std::vector<int64_t> src_off, dst_off;
  std::vector<int32_t> len;
  int64_t total = 0;
  int max_len = 0;
};

Windows make_windows(const dtwx_config &cfg, const int64_t *offsets, int n_reads) {
  Windows w;
  w.src_off.resize(n_reads);
  w.dst_off.resize(n_reads);
  w.len.resize(n_reads);
  for (int r = 0; r < n_reads; ++r) {
    const int64_t L = offsets[r + 1] - offsets[r];
    const int64_t skip = cfg.adapter_skip > 0 ? cfg.adapter_skip : 0;
    int64_t n = cfg.query_len > 0 ? cfg.query_len : L - skip;
    if (L - skip < n) n = cfg.require_full ? 0 : L - skip;
    if (n < 0) n = 0;
    w.src_off[r] = offsets[r] + skip;
    w.dst_off[r] = w.total;
    w.len[r] = (int32_t)n;
    w.total += n;
    w.max_len = std::max<int>(w.max_len, (int)n);
  }
  return w;
}

// Meta blob: tasks | order | nsamp | src_off | dst_off | scale_mul | scale_add.
struct MetaLayout {
  size_t tasks, order, nsamp, src_off, dst_off, smul, sadd, total;
};
MetaLayout meta_layout(int64_t n_tasks, int n_reads) {
  MetaLayout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o += (bytes + 15) & ~size_t(15);
    return at;
  };
  L.tasks = take(sizeof(Task) * (size_t)std::max<int64_t>(n_tasks, 1));
  L.order = take(sizeof(int32_t) * (size_t)std::max<int64_t>(n_tasks, 1));
  L.nsamp = take(sizeof(int32_t) * (size_t)std::max(n_reads, 1));
  L.src_off = take(sizeof(int64_t) * (size_t)std::max(n_reads, 1));
  L.dst_off = take(sizeof(int64_t) * (size_t)std::max(n_reads, 1));
  L.smul = take(sizeof(float) * (size_t)std::max(n_reads, 1));
  L.sadd = take(sizeof(float) * (size_t)std::max(n_reads, 1));
  L.total = o;
  return L;
}

// Order tasks longest first (LPT) so that the tail of the dynamic queue holds
// the short reads.
void lpt_order(const std::vector<Task> &tasks, int32_t *order) {
  std::vector<int32_t> idx(tasks.size());
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return tasks[a].n > tasks[b].n; });
  std::copy(idx.begin(), idx.end(), order);
}

int wait_meta(dtwx_handle *h, BatchCtx &c) {
  if (c.meta_pending) {
    CK(h, cudaEventSynchronize(c.meta_free));
    c.meta_pending = false;
  }
  return DTWX_OK;
}

// Shared body of the classify entry points.  raw_host != NULL: samples are on
// the host (copied window by window into pinned memory); otherwise raw_dev.
int classify_common(dtwx_handle *h, const void *raw_host, const void *raw_dev, int is_i16,
                    const int64_t *offsets, int n_reads, const float *sc_off, const float *sc_range,
                    const float *sc_digi, dtwx_result *out_host, dtwx_result *out_dev, cudaStream_t st,
                    bool use_given_stream, int precision, bool one_launch_per_read) {
  if (!h) return fail(nullptr, DTWX_E_ARG, "null handle");
  if (n_reads < 0 || (n_reads > 0 && !offsets)) return fail(h, DTWX_E_ARG, "bad read batch");
  if (n_reads > 0 && offsets[0] < 0) return fail(h, DTWX_E_ARG, "offsets must start at 0 or later");
  for (int r = 0; r < n_reads; ++r)
    if (offsets[r + 1] < offsets[r]) return fail(h, DTWX_E_ARG, "offsets must be non-decreasing");
  CK(h, cudaSetDevice(h->device));
  BatchCtx &c = h->ctx[0];
  if (!use_given_stream) st = c.stream;
  int launches = 0;
  const Windows w = make_windows(h->cfg, offsets, n_reads);
  const size_t es = is_i16 ? 2 : 4;
  std::vector<Task> tasks;
  tasks.reserve(n_reads);
  double sum_rows = 0;
  for (int r = 0; r < n_reads; ++r) {
    if (w.len[r] <= 0) continue;
    Task t{};
    t.q_off = w.dst_off[r];
    t.n = w.len[r];
    t.flags = 0;
    t.state_off = 0;
    t.out_slot = r;
    tasks.push_back(t);
    sum_rows += w.len[r];
  }
  const int64_t n_tasks = (int64_t)tasks.size();
  const double mean_rows = n_tasks ? sum_rows / n_tasks : 0.0;
  const MetaLayout L = meta_layout(n_tasks, n_reads);
  if (int rc = wait_meta(h, c)) return rc;
  CK(h, c.h_meta.ensure(L.total));
  CK(h, c.meta.ensure(L.total));
  char *hm = c.h_meta.as<char>();
  if (n_tasks) memcpy(hm + L.tasks, tasks.data(), sizeof(Task) * tasks.size());
  lpt_order(tasks, reinterpret_cast<int32_t *>(hm + L.order));
  int32_t *nsamp = reinterpret_cast<int32_t *>(hm + L.nsamp);
  int64_t *src_off = reinterpret_cast<int64_t *>(hm + L.src_off);
  int64_t *dst_off = reinterpret_cast<int64_t *>(hm + L.dst_off);
  float *smul = reinterpret_cast<float *>(hm + L.smul);
  float *sadd = reinterpret_cast<float *>(hm + L.sadd);
  for (int r = 0; r < n_reads; ++r) {
    nsamp[r] = w.len[r];
    dst_off[r] = w.dst_off[r];
    src_off[r] = raw_host ? w.dst_off[r] : w.src_off[r];
    smul[r] = 1.f;
    sadd[r] = 0.f;
    if (is_i16 && sc_range && sc_digi) smul[r] = sc_digi[r] != 0.f ? sc_range[r] / sc_digi[r] : 1.f;
    if (is_i16 && sc_off) sadd[r] = sc_off[r];
  }
  // ---- CUDA graph of a repeated device batch
  CaptureGuard capture_guard{h, st};
  const bool graphable = h->cfg.use_graphs && raw_dev && out_dev && !raw_host && !one_launch_per_read;
  uint64_t key = 0;
  if (graphable) {
    uint64_t hsh = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
      for (int i = 0; i < 8; ++i) {
        hsh ^= (v >> (8 * i)) & 0xff;
        hsh *= 1099511628211ull;
      }
    };
    mix(reinterpret_cast<uintptr_t>(raw_dev));
    mix(reinterpret_cast<uintptr_t>(out_dev));
    mix(reinterpret_cast<uintptr_t>(st));
    mix((uint64_t)n_reads);
    mix((uint64_t)precision);
    for (int r = 0; r <= n_reads; ++r) mix((uint64_t)offsets[r]);
    key = hsh | 1;
    if (key == h->graph_key && h->graph_exec) {
      // the pinned metadata blob was refilled above; the graph's copy reads it at replay
      CK(h, cudaGraphLaunch(h->graph_exec, st));
      CK(h, cudaEventRecord(c.meta_free, st));
      c.meta_pending = true;
      h->last_launches = h->graph_launches;
      ++h->graph_replays;
      return DTWX_OK;
    }
    if (key == h->graph_pending) {
      CK(h, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      h->capturing = true;
    } else {
      h->graph_pending = key;
    }
  }
  const void *src_dev = raw_dev;
  if (raw_host) {
    CK(h, c.h_raw.ensure(std::max<size_t>(es * (size_t)w.total, 16)));
    CK(h, c.raw.ensure(std::max<size_t>(es * (size_t)w.total, 16)));
    char *dst = c.h_raw.as<char>();
    const char *src = static_cast<const char *>(raw_host);
    for (int r = 0; r < n_reads; ++r)
      if (w.len[r] > 0) memcpy(dst + es * w.dst_off[r], src + es * w.src_off[r], es * (size_t)w.len[r]);
    if (w.total) CK(h, cudaMemcpyAsync(c.raw.p, c.h_raw.p, es * (size_t)w.total, cudaMemcpyHostToDevice, st));
    src_dev = c.raw.p;
  }
  CK(h, cudaMemcpyAsync(c.meta.p, c.h_meta.p, L.total, cudaMemcpyHostToDevice, st));
  if (!h->capturing) {
    CK(h, cudaEventRecord(c.meta_free, st));
    c.meta_pending = true;
  }
  const char *dm = c.meta.as<char>();
  CK(h, c.query.ensure(sizeof(float) * (size_t)std::max<int64_t>(w.total, 4)));
  CK(h, c.results.ensure(sizeof(dtwx_result) * (size_t)std::max(n_reads, 1)));
  if (w.total) {
    CK(h, launch_normalize(src_dev, is_i16, reinterpret_cast<const int64_t *>(dm + L.src_off),
                           reinterpret_cast<const int64_t *>(dm + L.dst_off),
                           reinterpret_cast<const int32_t *>(dm + L.nsamp),
                           is_i16 ? reinterpret_cast<const float *>(dm + L.smul) : nullptr,
                           is_i16 ? reinterpret_cast<const float *>(dm + L.sadd) : nullptr, n_reads,
                           h->cfg.norm_eps, c.query.as<float>(), st));
    ++launches;
  }
  void *d_out = out_dev ? static_cast<void *>(out_dev) : c.results.p;
  const Task *d_tasks = reinterpret_cast<const Task *>(dm + L.tasks);
  const int32_t *d_order = reinterpret_cast<const int32_t *>(dm + L.order);
  if (!one_launch_per_read) {
    if (int rc = enqueue_sweep(h, c, precision, st, c.query.as<float>(), d_tasks, d_order, n_tasks,
                               w.max_len, mean_rows, n_reads, reinterpret_cast<const int32_t *>(dm + L.nsamp),
                               d_out, nullptr, true, launches))
      return rc;
  } else {
    // one sweep launch per read; keys are reset once and finalized once
    if (int rc = enqueue_sweep(h, c, precision, st, c.query.as<float>(), d_tasks, d_order, 0, w.max_len,
                               mean_rows, n_reads, reinterpret_cast<const int32_t *>(dm + L.nsamp), d_out,
                               nullptr, false, launches))
      return rc;
    const int pb = sdtw_pair_bytes(precision, h->cfg.recurrence == DTWX_REF_DEL);
    const int rows_cap = seam_rows_capacity(w.max_len);
    if (rows_cap < 0) return fail(h, DTWX_E_CAPACITY, "read longer than a seam buffer can index");
    const int64_t per_warp = seam_bytes_per_warp(pb, rows_cap);
    int64_t seam_need = 0;
    for (int64_t t = 0; t < n_tasks; ++t) {
      const Shape sh = pick_shape(h, precision, 1, tasks[t].n);
      seam_need = std::max<int64_t>(seam_need, per_warp * (int64_t)sh.grid * sh.warps);
    }
    CK(h, c.seam.ensure((size_t)std::max<int64_t>(seam_need, 256)));
    for (int64_t t = 0; t < n_tasks; ++t) {
      // the keys were reset once above; each read gets its own sweep launch
      const Shape sh = pick_shape(h, precision, 1, tasks[t].n);
      int32_t *counter = c.flags.as<int32_t>();
      CK(h, cudaMemsetAsync(counter, 0, sizeof(int32_t), st));
      SdtwParams p{};
      p.query = c.query.as<float>();
      p.tasks = d_tasks + t;
      p.order = nullptr;
      p.keys = c.keys.as<unsigned long long>();
      p.seam = c.seam.as<char>();
      p.counter = counter;
      p.err = counter + 4;
      p.ref_plain = ref_for(h, precision);
      p.m = h->m_cols;
      p.m_pad = h->m_pad;
      p.seam_stride = per_warp;
      p.n_tasks = 1;
      const int W = kWarp * sh.S;
      const int64_t strips = (h->m_cols + W - 1) / W;
      p.n_chunks = (int32_t)((strips + sh.G - 1) / sh.G);
      p.chunk_strips = sh.G;
      p.max_rows = rows_cap;
      p.strands = h->cfg.strand_mode == DTWX_STRANDS_CONCAT ? 1 : 2;
      p.ref_del = h->cfg.recurrence == DTWX_REF_DEL ? 1 : 0;
      p.n_items = p.n_chunks * (precision != 0 ? p.strands : 1);
      p.ref_layout = 1;
      p.narrow_halo = sh.nh ? 1 : 0;
      const int ii = inst_index(precision, sh.S);
      p.use_tma = h->tmap_ok[precision][ii] ? 1 : 0;
      CK(h, launch_sdtw(precision, sh.S, sh.warps, sh.grid, p, p.use_tma ? &h->tmap[precision][ii] : nullptr,
                        st));
      ++launches;
    }
    CK(h, launch_finalize(c.keys.as<unsigned long long>(), reinterpret_cast<const int32_t *>(dm + L.nsamp),
                          n_reads, h->cfg.strand_mode == DTWX_STRANDS_CONCAT, h->m, h->cfg.threshold,
                          c.flags.as<int32_t>() + 4, d_out, st));
    ++launches;
  }
  h->last_launches = launches;
  if (h->capturing) {
    h->capturing = false;
    cudaGraph_t graph = nullptr;
    CK(h, cudaStreamEndCapture(st, &graph));
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(h, ie);
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    h->graph_exec = exec;
    h->graph_key = key;
    h->graph_launches = launches;
    CK(h, cudaGraphLaunch(exec, st));
    CK(h, cudaEventRecord(c.meta_free, st));
    c.meta_pending = true;
  }
  if (out_host) {
    if (n_reads)
      CK(h, cudaMemcpyAsync(out_host, d_out, sizeof(dtwx_result) * (size_t)n_reads, cudaMemcpyDeviceToHost, st));
    CK(h, cudaStreamSynchronize(st));
    c.meta_pending = false;
    if (int rc = check_device_flags(h, c)) return rc;
  } else {
    // device results: the error word is read by dtwx_sync (and marked in the results)
    CK(h, cudaEventRecord(c.done, st));
    h->device_call_pending = true;
  }
  return DTWX_OK;
}

double now_ms() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

int create_common(const dtwx_config *cfg_in, const std::vector<double> &table, const std::string &seq,
                  dtwx_handle **out) {
  if (!out) return fail(nullptr, DTWX_E_ARG, "out is NULL");
  *out = nullptr;
  dtwx_config cfg;
  dtwx_config_default(&cfg);
  if (cfg_in) {
    if (cfg_in->abi_version != DTWX_ABI_VERSION) return fail(nullptr, DTWX_E_ARG, "dtwx_config ABI mismatch");
    cfg = *cfg_in;
  }
  if (cfg.precision != DTWX_FP16 && cfg.precision != DTWX_FP32 && cfg.precision != DTWX_MIXED)
    return fail(nullptr, DTWX_E_ARG, "bad precision");
  if (cfg.strand_mode != DTWX_STRANDS_PAIRED && cfg.strand_mode != DTWX_STRANDS_CONCAT)
    return fail(nullptr, DTWX_E_ARG, "bad strand_mode");
  if (cfg.recurrence != DTWX_NO_REF_DEL && cfg.recurrence != DTWX_REF_DEL)
    return fail(nullptr, DTWX_E_ARG, "bad recurrence");
  if (cfg.state_precision != DTWX_STATE_FP32 && cfg.state_precision != DTWX_STATE_FP16)
    return fail(nullptr, DTWX_E_ARG, "bad state_precision");
  if (cfg.state_precision == DTWX_STATE_FP16 && cfg.precision != DTWX_FP16)
    return fail(nullptr, DTWX_E_ARG, "FP16 row state needs DTWX_FP16 cells");
  if (cfg.recurrence == DTWX_REF_DEL && cfg.precision == DTWX_MIXED)
    return fail(nullptr, DTWX_E_ARG, "the REF_DEL recurrence is built for FP16 and FP32 cells");
  if (cfg.recurrence == DTWX_REF_DEL && cfg.state_precision == DTWX_STATE_FP16)
    return fail(nullptr, DTWX_E_ARG, "REF_DEL keeps an FP32 row state");
  if (cfg.cells_per_thread &&
      !sdtw_instance_exists(cfg.precision, cfg.cells_per_thread, cfg.recurrence == DTWX_REF_DEL))
    return fail(nullptr, DTWX_E_ARG, "cells_per_thread has no compiled kernel for this precision");
  if (cfg.warps_per_cta < 0 || cfg.warps_per_cta > max_warps_per_cta(cfg.precision, cfg.recurrence == DTWX_REF_DEL))
    return fail(nullptr, DTWX_E_ARG, "warps_per_cta must be 1..8 (1..16 for FP16 REF_DEL cells)");
  if (cfg.chunk_strips < 0) return fail(nullptr, DTWX_E_ARG, "chunk_strips must be >= 0");
  const int64_t L = (int64_t)seq.size();
  if (L < kKmer) return fail(nullptr, DTWX_E_FORMAT, "reference shorter than one 6-mer");
  int64_t m = L - kKmer + 1;
  if (cfg.max_ref_len > 0 && cfg.max_ref_len < m) m = cfg.max_ref_len;
  const int64_t m_cols = cfg.strand_mode == DTWX_STRANDS_CONCAT ? 2 * m : m;
  if (m_cols >= ((int64_t)1 << 32)) return fail(nullptr, DTWX_E_CAPACITY, "reference too long");

  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(nullptr, DTWX_E_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (cfg.device < 0 || cfg.device >= ndev) return fail(nullptr, DTWX_E_ARG, "device ordinal out of range");
  e = cudaSetDevice(cfg.device);
  if (e != cudaSuccess) return fail(nullptr, DTWX_E_CUDA, cudaGetErrorString(e));

  dtwx_handle *h = new dtwx_handle();
  h->cfg = cfg;
  h->device = cfg.device;
  cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device);
  h->m = m;
  h->m_cols = m_cols;
  h->m_pad = (m_cols + kPadCols - 1) / kPadCols * kPadCols;
  for (int p = 0; p < 3; ++p) {
    h->fixed[p].S = (p == cfg.precision && cfg.cells_per_thread) ? cfg.cells_per_thread : 0;
    h->fixed[p].G = cfg.chunk_strips;
    h->fixed[p].warps = cfg.warps_per_cta;
  }
  auto bad = [&](cudaError_t err, const char *what) {
    g_create_err = std::string(what) + ": " + cudaGetErrorString(err);
    dtwx_destroy(h);
    return err == cudaErrorMemoryAllocation ? DTWX_E_NOMEM : DTWX_E_CUDA;
  };
  for (auto &c : h->ctx) {
    if ((e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking)) != cudaSuccess) return bad(e, "stream");
    if ((e = cudaEventCreateWithFlags(&c.meta_free, cudaEventDisableTiming)) != cudaSuccess) return bad(e, "event");
    if ((e = cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming)) != cudaSuccess) return bad(e, "event");
    if ((e = cudaEventCreate(&c.sweep_beg)) != cudaSuccess) return bad(e, "event");
    if ((e = cudaEventCreate(&c.sweep_end)) != cudaSuccess) return bad(e, "event");
  }
  cudaStream_t st = h->ctx[0].stream;
  if ((e = h->ref16.ensure(sizeof(__half2) * h->m_pad)) != cudaSuccess) return bad(e, "alloc ref16");
  if ((e = h->ref32.ensure(2 * sizeof(float) * h->m_pad)) != cudaSuccess) return bad(e, "alloc ref32");
  if ((e = h->ref16p.ensure(2 * sizeof(__half) * h->m_pad)) != cudaSuccess) return bad(e, "alloc ref16p");
  if ((e = h->fwd32.ensure(sizeof(float) * m)) != cudaSuccess) return bad(e, "alloc fwd32");
  if ((e = h->rev32.ensure(sizeof(float) * m)) != cudaSuccess) return bad(e, "alloc rev32");
  DevBuf d_seq, d_table, d_work;
  if ((e = d_seq.ensure(L)) != cudaSuccess) return bad(e, "alloc seq");
  if ((e = d_table.ensure(sizeof(double) * kTableSize)) != cudaSuccess) return bad(e, "alloc table");
  if ((e = d_work.ensure(build_reference_work_bytes(m))) != cudaSuccess) return bad(e, "alloc work");
  cudaMemcpyAsync(d_seq.p, seq.data(), L, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_table.p, table.data(), sizeof(double) * kTableSize, cudaMemcpyHostToDevice, st);
  e = launch_build_reference(d_seq.as<char>(), L, d_table.as<double>(), m, h->m_pad,
                             cfg.strand_mode == DTWX_STRANDS_CONCAT, d_work.as<double>(), h->ref16.as<__half2>(),
                             h->ref32.as<float>(), h->ref16p.as<__half>(), h->fwd32.as<float>(),
                             h->rev32.as<float>(), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  d_seq.release();
  d_table.release();
  d_work.release();
  if (e != cudaSuccess) return bad(e, "reference build");
  for (int p = 0; p < 3; ++p) {
    const int64_t bytes = p == 0 ? 4 * h->m_pad : (p == 1 ? 8 * h->m_pad : 4 * h->m_pad);
    for (int i = 0; i < inst_count(p); ++i)
      h->tmap_ok[p][i] = make_tmap(&h->tmap[p][i], const_cast<void *>(ref_for(h, p)), bytes, inst_S(p, i),
                                   sdtw_ref_bytes(p));
  }
  *out = h;
  return DTWX_OK;
}

}  // namespace

void dtwx::set_create_error(const char *msg) { g_create_err = msg ? msg : ""; }

CaptureGuard::~CaptureGuard() {
  if (h && h->capturing) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(st, &g);
    if (g) cudaGraphDestroy(g);
    h->capturing = false;
    h->graph_pending = 0;
  }
}

// =================================================================== C ABI

extern "C" {

int dtwx_config_default(dtwx_config *cfg) {
  if (!cfg) return DTWX_E_ARG;
  memset(cfg, 0, sizeof(*cfg));
  cfg->abi_version = DTWX_ABI_VERSION;
  cfg->precision = DTWX_FP16;
  cfg->strand_mode = DTWX_STRANDS_PAIRED;
  cfg->device = 0;
  cfg->max_ref_len = 0;
  cfg->adapter_skip = 0;
  cfg->query_len = 0;
  cfg->require_full = 0;
  cfg->norm_eps = 1e-4f;
  cfg->threshold = 194.0f;
  return DTWX_OK;
}

int dtwx_create(const dtwx_config *cfg, const char *kmer_model_path, const float *level_table,
                const char *fasta_path, dtwx_handle **out) {
  if (!fasta_path) return fail(nullptr, DTWX_E_ARG, "fasta_path is NULL");
  if ((kmer_model_path == nullptr) == (level_table == nullptr))
    return fail(nullptr, DTWX_E_ARG, "give exactly one of kmer_model_path and level_table");
  std::vector<double> table;
  std::string err;
  if (kmer_model_path) {
    std::string text;
    if (!read_file(kmer_model_path, text)) return fail(nullptr, DTWX_E_IO, std::string("cannot read ") + kmer_model_path);
    if (!parse_kmer_model(text, table, err)) return fail(nullptr, DTWX_E_FORMAT, err);
  } else {
    table.assign(level_table, level_table + kTableSize);
  }
  std::string text, seq, name;
  if (!read_file(fasta_path, text)) return fail(nullptr, DTWX_E_IO, std::string("cannot read ") + fasta_path);
  if (!parse_fasta(text, seq, name, err)) return fail(nullptr, DTWX_E_FORMAT, err);
  return create_common(cfg, table, seq, out);
}

int dtwx_load_fasta(const char *fasta_path, char *seq_out, int64_t cap, int64_t *len_out) {
  if (!fasta_path || !len_out || cap < 0) return fail(nullptr, DTWX_E_ARG, "bad arguments");
  std::string text, seq, name, err;
  if (!read_file(fasta_path, text)) return fail(nullptr, DTWX_E_IO, std::string("cannot read ") + fasta_path);
  if (!parse_fasta(text, seq, name, err)) return fail(nullptr, DTWX_E_FORMAT, err);
  *len_out = (int64_t)seq.size();
  if (seq_out) memcpy(seq_out, seq.data(), (size_t)std::min<int64_t>(cap, (int64_t)seq.size()));
  return DTWX_OK;
}

int dtwx_load_kmer_model(const char *path, float *table_out) {
  if (!path || !table_out) return fail(nullptr, DTWX_E_ARG, "bad arguments");
  std::string text, err;
  std::vector<double> table;
  if (!read_file(path, text)) return fail(nullptr, DTWX_E_IO, std::string("cannot read ") + path);
  if (!parse_kmer_model(text, table, err)) return fail(nullptr, DTWX_E_FORMAT, err);
  for (int i = 0; i < kTableSize; ++i) table_out[i] = (float)table[i];
  return DTWX_OK;
}

int dtwx_create_from_sequence(const dtwx_config *cfg, const float *level_table, const char *seq,
                              int64_t seq_len, dtwx_handle **out) {
  if (!level_table || !seq || seq_len < 0) return fail(nullptr, DTWX_E_ARG, "bad arguments");
  std::vector<double> table(level_table, level_table + kTableSize);
  return create_common(cfg, table, std::string(seq, seq + seq_len), out);
}

int dtwx_destroy(dtwx_handle *h) {
  if (!h) return DTWX_OK;
  cudaSetDevice(h->device);
  for (auto &c : h->ctx) {
    if (c.stream) cudaStreamSynchronize(c.stream);
    c.raw.release();
    c.query.release();
    c.meta.release();
    c.keys.release();
    c.results.release();
    c.seam.release();
    c.flags.release();
    c.h_raw.release();
    c.h_meta.release();
    c.h_results.release();
    c.h_flags.release();
    if (c.meta_free) cudaEventDestroy(c.meta_free);
    if (c.sweep_beg) cudaEventDestroy(c.sweep_beg);
    if (c.sweep_end) cudaEventDestroy(c.sweep_end);
    if (c.done) cudaEventDestroy(c.done);
    if (c.stream) cudaStreamDestroy(c.stream);
  }
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  h->ref16.release();
  h->ref32.release();
  h->fwd32.release();
  h->rev32.release();
  h->state.release();
  delete h;
  return DTWX_OK;
}

const char *dtwx_last_error(const dtwx_handle *h) {
  if (!h) return g_create_err.c_str();
  return h->err.c_str();
}

int64_t dtwx_ref_len(const dtwx_handle *h) { return h ? h->m : -1; }

int dtwx_get_reference(dtwx_handle *h, float *fwd, float *rev) {
  if (!h || !fwd || !rev) return DTWX_E_ARG;
  CK(h, cudaSetDevice(h->device));
  CK(h, cudaMemcpy(fwd, h->fwd32.p, sizeof(float) * h->m, cudaMemcpyDeviceToHost));
  CK(h, cudaMemcpy(rev, h->rev32.p, sizeof(float) * h->m, cudaMemcpyDeviceToHost));
  return DTWX_OK;
}

int dtwx_classify_batch(dtwx_handle *h, const float *raw, const int64_t *offsets, int32_t n_reads,
                        dtwx_result *out) {
  if (!h) return DTWX_E_ARG;
  if (n_reads > 0 && (!raw || !out)) return fail(h, DTWX_E_ARG, "raw/out is NULL");
  return classify_common(h, raw, nullptr, 0, offsets, n_reads, nullptr, nullptr, nullptr, out, nullptr, nullptr,
                         false, h->cfg.precision, false);
}

int dtwx_classify_batch_i16(dtwx_handle *h, const int16_t *raw, const int64_t *offsets, int32_t n_reads,
                            const float *offset, const float *range, const float *digitisation,
                            dtwx_result *out) {
  if (!h) return DTWX_E_ARG;
  if (n_reads > 0 && (!raw || !out)) return fail(h, DTWX_E_ARG, "raw/out is NULL");
  return classify_common(h, raw, nullptr, 1, offsets, n_reads, offset, range, digitisation, out, nullptr,
                         nullptr, false, h->cfg.precision, false);
}

int dtwx_classify_device(dtwx_handle *h, const float *d_raw, const int64_t *offsets, int32_t n_reads,
                         dtwx_result *d_out, void *stream) {
  if (!h) return DTWX_E_ARG;
  if (n_reads > 0 && (!d_raw || !d_out)) return fail(h, DTWX_E_ARG, "d_raw/d_out is NULL");
  return classify_common(h, nullptr, d_raw, 0, offsets, n_reads, nullptr, nullptr, nullptr, nullptr, d_out,
                         static_cast<cudaStream_t>(stream), true, h->cfg.precision, false);
}

int dtwx_classify_plain_fp32(dtwx_handle *h, const float *raw, const int64_t *offsets, int32_t n_reads,
                             dtwx_result *out) {
  if (!h) return DTWX_E_ARG;
  if (n_reads > 0 && (!raw || !out)) return fail(h, DTWX_E_ARG, "raw/out is NULL");
  return classify_common(h, raw, nullptr, 0, offsets, n_reads, nullptr, nullptr, nullptr, out, nullptr, nullptr,
                         false, DTWX_FP32, true);
}

int dtwx_distances(dtwx_handle *h, const float *d_query, const int64_t *offsets, int32_t n_reads,
                   dtwx_result *d_out, void *stream) {
  if (!h) return DTWX_E_ARG;
  if (n_reads < 0 || (n_reads > 0 && (!d_query || !offsets || !d_out)))
    return fail(h, DTWX_E_ARG, "bad arguments");
  if (n_reads > 0 && offsets[0] < 0) return fail(h, DTWX_E_ARG, "offsets must start at 0 or later");
  CK(h, cudaSetDevice(h->device));
  BatchCtx &c = h->ctx[0];
  cudaStream_t st = static_cast<cudaStream_t>(stream);  // 0 = the legacy default stream
  std::vector<Task> tasks;
  int max_len = 0;
  double sum = 0;
  for (int r = 0; r < n_reads; ++r) {
    const int64_t n = offsets[r + 1] - offsets[r];
    if (n < 0) return fail(h, DTWX_E_ARG, "offsets must be non-decreasing");
    if (n == 0) continue;
    if (n > INT32_MAX) return fail(h, DTWX_E_CAPACITY, "read too long");
    Task t{};
    t.q_off = offsets[r];
    t.n = (int32_t)n;
    t.out_slot = r;
    tasks.push_back(t);
    max_len = std::max<int>(max_len, (int)n);
    sum += n;
  }
  const int64_t n_tasks = (int64_t)tasks.size();
  const MetaLayout L = meta_layout(n_tasks, n_reads);
  if (int rc = wait_meta(h, c)) return rc;
  CK(h, c.h_meta.ensure(L.total));
  CK(h, c.meta.ensure(L.total));
  char *hm = c.h_meta.as<char>();
  if (n_tasks) memcpy(hm + L.tasks, tasks.data(), sizeof(Task) * tasks.size());
  lpt_order(tasks, reinterpret_cast<int32_t *>(hm + L.order));
  int32_t *nsamp = reinterpret_cast<int32_t *>(hm + L.nsamp);
  for (int r = 0; r < n_reads; ++r) nsamp[r] = (int32_t)(offsets[r + 1] - offsets[r]);
  CK(h, cudaMemcpyAsync(c.meta.p, c.h_meta.p, L.total, cudaMemcpyHostToDevice, st));
  CK(h, cudaEventRecord(c.meta_free, st));
  c.meta_pending = true;
  const char *dm = c.meta.as<char>();
  int launches = 0;
  int rc = enqueue_sweep(h, c, h->cfg.precision, st, d_query, reinterpret_cast<const Task *>(dm + L.tasks),
                         reinterpret_cast<const int32_t *>(dm + L.order), n_tasks, max_len,
                         n_tasks ? sum / n_tasks : 0.0, n_reads, reinterpret_cast<const int32_t *>(dm + L.nsamp),
                         d_out, nullptr, true, launches);
  h->last_launches = launches;
  if (rc) return rc;
  CK(h, cudaEventRecord(c.done, st));
  h->device_call_pending = true;
  return DTWX_OK;
}

int dtwx_normalize(dtwx_handle *h, const float *d_raw, const int64_t *offsets, int32_t n_reads, float *d_query,
                   int64_t *out_offsets, void *stream) {
  if (!h) return DTWX_E_ARG;
  if (n_reads < 0 || (n_reads > 0 && (!d_raw || !offsets || !d_query)))
    return fail(h, DTWX_E_ARG, "bad arguments");
  if (n_reads > 0 && offsets[0] < 0) return fail(h, DTWX_E_ARG, "offsets must start at 0 or later");
  for (int r = 0; r < n_reads; ++r)
    if (offsets[r + 1] < offsets[r]) return fail(h, DTWX_E_ARG, "offsets must be non-decreasing");
  CK(h, cudaSetDevice(h->device));
  BatchCtx &c = h->ctx[0];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Windows w = make_windows(h->cfg, offsets, n_reads);
  if (out_offsets) {
    for (int r = 0; r < n_reads; ++r) out_offsets[r] = w.dst_off[r];
    out_offsets[n_reads] = w.total;
  }
  if (n_reads == 0 || w.total == 0) return DTWX_OK;
  const MetaLayout L = meta_layout(0, n_reads);
  if (int rc = wait_meta(h, c)) return rc;
  CK(h, c.h_meta.ensure(L.total));
  CK(h, c.meta.ensure(L.total));
  char *hm = c.h_meta.as<char>();
  int32_t *len = reinterpret_cast<int32_t *>(hm + L.nsamp);
  int64_t *src_off = reinterpret_cast<int64_t *>(hm + L.src_off);
  int64_t *dst_off = reinterpret_cast<int64_t *>(hm + L.dst_off);
  for (int r = 0; r < n_reads; ++r) {
    len[r] = w.len[r];
    src_off[r] = w.src_off[r];
    dst_off[r] = w.dst_off[r];
  }
  CK(h, cudaMemcpyAsync(c.meta.p, c.h_meta.p, L.total, cudaMemcpyHostToDevice, st));
  CK(h, cudaEventRecord(c.meta_free, st));
  c.meta_pending = true;
  const char *dm = c.meta.as<char>();
  CK(h, launch_normalize(d_raw, 0, reinterpret_cast<const int64_t *>(dm + L.src_off),
                         reinterpret_cast<const int64_t *>(dm + L.dst_off),
                         reinterpret_cast<const int32_t *>(dm + L.nsamp), nullptr, nullptr, n_reads, h->cfg.norm_eps,
                         d_query, st));
  h->last_launches = 1;
  return DTWX_OK;
}

int dtwx_sync(dtwx_handle *h) {
  if (!h) return DTWX_E_ARG;
  CK(h, cudaSetDevice(h->device));
  BatchCtx &c = h->ctx[0];
  if (!h->device_call_pending) return DTWX_OK;
  CK(h, cudaEventSynchronize(c.done));
  h->device_call_pending = false;
  return check_device_flags(h, c);
}

int dtwx_debug_stall_next(dtwx_handle *h, int32_t item, uint32_t spin_limit) {
  if (!h) return DTWX_E_ARG;
  if (item < 0) return fail(h, DTWX_E_ARG, "item must be >= 0");
  h->stall_item = item + 1;
  h->stall_spin = spin_limit;
  return DTWX_OK;
}

int dtwx_autotune(dtwx_handle *h, int32_t n_reads_req, int32_t read_len, float *best_ms) {
  if (!h || n_reads_req <= 0 || read_len <= 0) return DTWX_E_ARG;
  CK(h, cudaSetDevice(h->device));
  const int prec = h->cfg.precision;
  // candidates are timed on the requested batch, cut to about 1.2e13 cells
  // (under a second per candidate) and to 2,048 reads; the winner is kept for
  // the requested batch size (its chunk width is a factor on the analytic
  // model, which rescales with the batch)
  const double per_read = 2.0 * (double)read_len * (double)h->m;
  const int32_t by_cells = (int32_t)std::max(16.0, std::min(2048.0, 1.2e13 / std::max(per_read, 1.0)));
  const int32_t n_reads = std::min<int32_t>(n_reads_req, by_cells);
  // synthetic z-scored reads of the requested shape (the sweep's cost does not
  // depend on the sample values)
  std::vector<float> q((size_t)n_reads * read_len);
  uint64_t x = 0x9e3779b97f4a7c15ull;
  for (auto &v : q) {
    x ^= x << 13, x ^= x >> 7, x ^= x << 17;
    v = (float)((double)(x >> 11) * (1.0 / 9007199254740992.0) * 3.4641016 - 1.7320508);  // mean 0, var 1
  }
  DevBuf dq, dout;
  CK(h, dq.ensure(sizeof(float) * q.size()));
  CK(h, dout.ensure(sizeof(dtwx_result) * (size_t)n_reads));
  CK(h, cudaMemcpy(dq.p, q.data(), sizeof(float) * q.size(), cudaMemcpyHostToDevice));
  std::vector<int64_t> offs((size_t)n_reads + 1);
  for (int r = 0; r <= n_reads; ++r) offs[r] = (int64_t)r * read_len;
  BatchCtx &c = h->ctx[0];
  cudaStream_t st = c.stream;
  struct Cand { int S, warps, permille; };
  std::vector<Cand> cands;
  const bool rd = h->cfg.recurrence == DTWX_REF_DEL;
  // warps 0: the default shape (for REF_DEL the batch spread evenly over the SMs)
  for (int si = 0; si < inst_count(prec); ++si)
    for (int w : {0, 4, 8})
      for (int pm : {500, 1000, 2000}) {
        if (!sdtw_instance_exists(prec, inst_S(prec, si), rd)) continue;
        if (rd && pm != 1000) continue;  // one chunk per task: no chunk width to tune
        if (w == 0 && !rd) continue;     // the default is 4 warps
        if (w && !sdtw_ctas_per_sm(prec, inst_S(prec, si), w, rd)) continue;
        cands.push_back({inst_S(prec, si), w, pm});
      }
  float best = 1e30f;
  Cand win{0, 0, 1000};
  int rc = DTWX_OK;
  // one untimed pass first: the first sweep of a handle pays one-time costs
  rc = dtwx_distances(h, dq.as<float>(), offs.data(), n_reads, dout.as<dtwx_result>(), st);
  for (const Cand &cd : cands) {
    if (rc != DTWX_OK) break;
    h->override_shape = Shape{};
    h->override_shape.S = cd.S;
    h->override_shape.warps = cd.warps;
    h->override_shape.items = cd.permille;
    float ms = 0.f;
    rc = dtwx_distances(h, dq.as<float>(), offs.data(), n_reads, dout.as<dtwx_result>(), st);
    if (rc == DTWX_OK) rc = dtwx_last_sweep_ms(h, &ms);
    if (rc != DTWX_OK) break;
    if (ms < best) {
      best = ms;
      win = cd;
    }
  }
  h->override_shape = Shape{};
  if (rc != DTWX_OK) return rc;
  CK(h, cudaStreamSynchronize(st));
  const dtwx_handle::Tuned tw{win.S, win.warps, win.permille / 1000.0};
  h->tuned[std::make_tuple(prec, log2_bucket(n_reads_req), log2_bucket(read_len))] = tw;
  h->tuned[std::make_tuple(prec, log2_bucket(n_reads), log2_bucket(read_len))] = tw;
  if (best_ms) *best_ms = best;
  return DTWX_OK;
}

int32_t dtwx_last_launch_count(const dtwx_handle *h) { return h ? h->last_launches : -1; }

int dtwx_last_sweep_ms(dtwx_handle *h, float *ms) {
  if (!h || !ms) return DTWX_E_ARG;
  BatchCtx &c = h->ctx[0];
  if (!c.sweep_timed) return fail(h, DTWX_E_STATE, "no sweep launched yet");
  CK(h, cudaEventSynchronize(c.sweep_end));
  CK(h, cudaEventElapsedTime(ms, c.sweep_beg, c.sweep_end));
  return DTWX_OK;
}

int dtwx_get_tuning(const dtwx_handle *h, int32_t *out, int32_t n) {
  if (!h || !out || n < 0) return DTWX_E_ARG;
  const Shape &s = h->last_shape[h->cfg.precision];
  const int32_t v[8] = {s.S, s.G, s.warps, s.grid, (int32_t)std::min<int64_t>(s.items, INT32_MAX),
                        s.S ? sdtw_ctas_per_sm(h->cfg.precision, s.S, s.warps,
                                               h->cfg.recurrence == DTWX_REF_DEL)
                            : 0,
                        (int32_t)h->graph_replays, s.nh ? 1 : 0};
  for (int i = 0; i < n && i < 8; ++i) out[i] = v[i];
  return DTWX_OK;
}

int dtwx_peak_probe(int32_t device, int32_t precision, float ms_target, double *cells_per_s) {
  if (!cells_per_s || precision < 0 || precision > 2) return DTWX_E_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return DTWX_E_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int block = 256, grid = sms * 8;
  float *sink = nullptr;
  if (cudaMalloc(&sink, sizeof(float) * block) != cudaSuccess) return DTWX_E_NOMEM;
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  int iters = 256;
  float ms = 0.f;
  int rc = DTWX_OK;
  for (int round = 0; round < 12; ++round) {
    cudaEventRecord(a, s);
    if (launch_peak_probe(precision, grid, block, iters, sink, s) != cudaSuccess) {
      rc = DTWX_E_CUDA;
      break;
    }
    cudaEventRecord(b, s);
    if (cudaEventSynchronize(b) != cudaSuccess) {
      rc = DTWX_E_CUDA;
      break;
    }
    cudaEventElapsedTime(&ms, a, b);
    if (ms >= ms_target * 0.5f) break;
    const double scale = ms > 0.01f ? ms_target / ms : 8.0;
    iters = (int)std::min<double>(iters * std::min(scale, 16.0) + 1, 1 << 30);
  }
  if (rc == DTWX_OK) {
    // timed run at the calibrated length (after the calibration warmed up)
    cudaEventRecord(a, s);
    launch_peak_probe(precision, grid, block, iters, sink, s);
    cudaEventRecord(b, s);
    if (cudaEventSynchronize(b) != cudaSuccess) rc = DTWX_E_CUDA;
    cudaEventElapsedTime(&ms, a, b);
    const double cells = (double)grid * block * (double)iters * 32.0 * (precision == 0 ? 2.0 : 1.0);
    *cells_per_s = cells / (ms * 1e-3);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamDestroy(s);
  cudaFree(sink);
  return rc;
}

double dtwx_now_ms(void) { return now_ms(); }

// ----------------------------------------------------------------- serving

int dtwx_serve_start(dtwx_handle *h, int32_t max_in_flight, double state_budget_bytes,
                     int32_t chunks_per_decision, float accept_per_sample, float reject_per_sample) {
  if (!h) return DTWX_E_ARG;
  if (h->serving) return fail(h, DTWX_E_STATE, "serving already started");
  if (chunks_per_decision <= 0) return fail(h, DTWX_E_ARG, "chunks_per_decision must be > 0");
  CK(h, cudaSetDevice(h->device));
  const double slot_bytes = (double)state_slot_floats(h) * sizeof(float);
  int64_t slots = max_in_flight > 0 ? max_in_flight : 0;
  if (slots == 0 && state_budget_bytes <= 0) {
    // neither given: the row-state pool may take half of the free device memory
    size_t free_b = 0, total_b = 0;
    CK(h, cudaMemGetInfo(&free_b, &total_b));
    state_budget_bytes = std::min(0.5 * (double)free_b, 4096.0 * slot_bytes);
  }
  if (state_budget_bytes > 0) {
    const int64_t by_budget = (int64_t)(state_budget_bytes / slot_bytes);
    slots = slots > 0 ? std::min(slots, by_budget) : by_budget;
  }
  if (slots <= 0) return fail(h, DTWX_E_CAPACITY, "row-state budget holds no read");
  CK(h, h->state.ensure((size_t)(slot_bytes * slots)));
  h->max_in_flight = (int32_t)slots;
  h->chunks_per_decision = chunks_per_decision;
  h->accept_per_sample = accept_per_sample;
  h->reject_per_sample = reject_per_sample;
  h->free_slots.clear();
  for (int64_t i = slots - 1; i >= 0; --i) h->free_slots.push_back((int)i);
  h->serving = true;
  return DTWX_OK;
}

int dtwx_submit_chunk_i16(dtwx_handle *h, int32_t channel, uint64_t read_number, const int16_t *samples,
                          int32_t n, int32_t is_last, double arrival_ms, float offset, float range,
                          float digitisation) {
  if (!h) return DTWX_E_ARG;
  if (n <= 0 || !samples) return fail(h, DTWX_E_ARG, "empty chunk");
  if (!(digitisation != 0.f)) return fail(h, DTWX_E_ARG, "digitisation must be non-zero");
  std::vector<float> pa((size_t)n);
  const float mul = range / digitisation;
  for (int32_t i = 0; i < n; ++i) pa[i] = ((float)samples[i] + offset) * mul;
  return dtwx_submit_chunk(h, channel, read_number, pa.data(), n, is_last, arrival_ms);
}

int dtwx_submit_chunk(dtwx_handle *h, int32_t channel, uint64_t read_number, const float *samples, int32_t n,
                      int32_t is_last, double arrival_ms) {
  if (!h) return DTWX_E_ARG;
  if (!h->serving) return fail(h, DTWX_E_STATE, "call dtwx_serve_start first");
  if (n <= 0 || !samples) return fail(h, DTWX_E_ARG, "empty chunk");
  const auto key = std::make_pair(channel, read_number);
  if (h->finished.count(key)) return DTWX_OK;  // already decided: later chunks are moot
  auto it = h->reads.find(key);
  if (it == h->reads.end()) {
    ServeRead r;
    r.channel = channel;
    r.read_number = read_number;
    it = h->reads.emplace(key, std::move(r)).first;
  }
  ServeRead &r = it->second;
  if (r.last_seen) return fail(h, DTWX_E_STATE, "chunk after the read's last chunk");
  r.pending.emplace_back(samples, samples + n);
  r.arrivals.push_back(arrival_ms >= 0 ? arrival_ms : now_ms());
  r.is_last.push_back(is_last ? 1 : 0);
  if (is_last) r.last_seen = true;
  ++h->chunks_submitted;
  if (r.slot < 0 && !r.queued) {
    if (!h->free_slots.empty() && h->admit_queue.empty()) {
      r.slot = h->free_slots.back();
      h->free_slots.pop_back();
    } else {
      r.queued = true;
      h->admit_queue.push_back(key);
      ++h->reads_deferred;
    }
  }
  return DTWX_OK;
}

namespace {

void release_read(dtwx_handle *h, std::map<std::pair<int32_t, uint64_t>, ServeRead>::iterator it) {
  if (it->second.slot >= 0) h->free_slots.push_back(it->second.slot);
  h->finished[it->first] = now_ms();
  // forget decisions older than a minute: a channel's read numbers only grow
  if (h->finished.size() > 65536) {
    const double cut = now_ms() - 60e3;
    for (auto f = h->finished.begin(); f != h->finished.end();)
      f = f->second < cut ? h->finished.erase(f) : std::next(f);
  }
  h->reads.erase(it);
  while (!h->free_slots.empty() && !h->admit_queue.empty()) {
    auto k = h->admit_queue.front();
    h->admit_queue.pop_front();
    auto jt = h->reads.find(k);
    if (jt == h->reads.end()) continue;
    jt->second.queued = false;
    jt->second.slot = h->free_slots.back();
    h->free_slots.pop_back();
  }
}

// Turn the results of serving batch `slot` into decisions.  After each chunk:
// target when the score (or the score per aligned sample, if an accept rate
// was given) is below the threshold; an early non-target when the score per
// sample is above the reject rate; otherwise a final non-target once
// chunks_per_decision chunks (or the read's last chunk) are aligned.
int harvest(dtwx_handle *h, int slot) {
  BatchCtx &c = h->ctx[1 + slot];
  CK(h, cudaEventSynchronize(c.done));
  const int32_t dev_err = c.h_flags.as<int32_t>()[4];
  if (dev_err) {
    CK(h, cudaMemset(c.flags.as<int32_t>() + 4, 0, sizeof(int32_t)));
    return fail(h, (dev_err & kErrTmaTimeout) ? DTWX_E_TIMEOUT : DTWX_E_CAPACITY, "device error flag in a serving batch");
  }
  if (c.sweep_timed) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c.sweep_beg, c.sweep_end) == cudaSuccess) {
      h->batch_ms_sum += ms;
      h->batch_ms_max = std::max<double>(h->batch_ms_max, ms);
    }
  }
  const dtwx_result *res = c.h_results.as<dtwx_result>();
  const double t = now_ms();
  std::vector<ServeTask> &inflight = h->inflight[slot];
  for (size_t i = 0; i < inflight.size(); ++i) {
    const ServeTask &st = inflight[i];
    auto it = h->reads.find(st.key);
    if (it == h->reads.end()) continue;
    ServeRead &r = it->second;
    r.in_batch = false;
    r.chunks_done += 1;
    r.samples_done += st.n;
    ++h->chunks_processed;
    dtwx_decision d{};
    d.channel = r.channel;
    d.read_number = r.read_number;
    d.score = res[i].score;
    d.strand = res[i].strand;
    d.end_pos = res[i].end_pos;
    d.chunks = r.chunks_done;
    d.samples = r.samples_done;
    d.latency_ms = t - st.arrival;
    d.queue_ms = st.launched - st.arrival;
    const double per = (double)res[i].score / std::max(r.samples_done, 1);
    const bool target = h->accept_per_sample > 0 ? per < h->accept_per_sample : res[i].score < h->cfg.threshold;
    const bool reject = h->reject_per_sample > 0 && per > h->reject_per_sample;
    d.call = target ? 1 : 0;
    d.decided = (target || reject || r.chunks_done >= h->chunks_per_decision || st.last) ? 1 : 0;
    h->decisions.push_back(d);
    if (d.decided) {
      h->latencies.push_back(d.latency_ms);
      h->queue_times.push_back(d.queue_ms);
      ++h->reads_decided;
      release_read(h, it);
    }
  }
  inflight.clear();
  h->running[slot] = false;
  return DTWX_OK;
}

// Harvest every serving batch that has finished; `wait` blocks for running ones.
int harvest_done(dtwx_handle *h, bool wait) {
  for (int s = 0; s < kServeSlots; ++s) {
    if (!h->running[s]) continue;
    if (!wait) {
      const cudaError_t q = cudaEventQuery(h->ctx[1 + s].done);
      if (q == cudaErrorNotReady) continue;
      if (q != cudaSuccess) return fail(h, DTWX_E_CUDA, cudaGetErrorString(q));
    }
    if (int rc = harvest(h, s)) return rc;
  }
  return DTWX_OK;
}

}  // namespace

int dtwx_serve_step(dtwx_handle *h) {
  if (!h) return DTWX_E_ARG;
  if (!h->serving) return fail(h, DTWX_E_STATE, "call dtwx_serve_start first");
  CK(h, cudaSetDevice(h->device));
  if (int rc = harvest_done(h, false)) return rc;
  // Continuous batching: up to kServeSlots batches are in flight, each on its
  // own stream with its own scratch; a new batch starts as soon as a slot is
  // free, so chunks that arrive while batches run reach the GPU without
  // waiting for them to end.  A read is in at most one batch at a time (its
  // row state).
  int slot = -1;
  const int slots = h->cfg.serve_batches > 0 ? std::min(h->cfg.serve_batches, kServeSlots) : 2;
  for (int s = 0; s < slots && slot < 0; ++s)
    if (!h->running[s]) slot = s;
  if (slot < 0) return 0;
  BatchCtx &c = h->ctx[1 + slot];
  // decided reads whose remaining chunks are moot are dropped at decision time;
  // gather one chunk per admitted read that has one waiting
  std::vector<ServeTask> batch;
  int64_t total = 0;
  int max_len = 0;
  for (auto &kv : h->reads) {
    ServeRead &r = kv.second;
    if (r.slot < 0 || r.in_batch || r.pending.empty()) continue;
    ServeTask t;
    t.key = kv.first;
    t.n = (int)r.pending.front().size();
    t.arrival = r.arrivals.front();
    t.last = r.is_last.front();
    batch.push_back(t);
    total += t.n;
    max_len = std::max(max_len, t.n);
  }
  if (batch.empty()) return 0;
  const int nb = (int)batch.size();
  std::vector<Task> tasks(nb);
  const MetaLayout L = meta_layout(nb, nb);
  CK(h, c.h_meta.ensure(L.total));
  CK(h, c.meta.ensure(L.total));
  CK(h, c.h_raw.ensure(sizeof(float) * (size_t)total));
  CK(h, c.raw.ensure(sizeof(float) * (size_t)total));
  CK(h, c.query.ensure(sizeof(float) * (size_t)total));
  CK(h, c.results.ensure(sizeof(dtwx_result) * nb));
  CK(h, c.h_results.ensure(sizeof(dtwx_result) * nb));
  char *hm = c.h_meta.as<char>();
  int32_t *nsamp = reinterpret_cast<int32_t *>(hm + L.nsamp);
  int64_t *src_off = reinterpret_cast<int64_t *>(hm + L.src_off);
  int64_t *dst_off = reinterpret_cast<int64_t *>(hm + L.dst_off);
  float *hraw = c.h_raw.as<float>();
  int64_t off = 0;
  for (int i = 0; i < nb; ++i) {
    ServeRead &r = h->reads[batch[i].key];
    std::vector<float> &chunk = r.pending.front();
    memcpy(hraw + off, chunk.data(), sizeof(float) * chunk.size());
    Task &t = tasks[i];
    t.q_off = off;
    t.n = batch[i].n;
    t.flags = kTaskSaveState | (r.chunks_done > 0 ? kTaskResume : 0);
    t.state_off = (int64_t)r.slot * state_slot_floats(h);
    t.out_slot = i;
    nsamp[i] = batch[i].n;
    src_off[i] = off;
    dst_off[i] = off;
    off += batch[i].n;
    r.pending.pop_front();
    r.arrivals.pop_front();
    r.is_last.pop_front();
    r.in_batch = true;
  }
  memcpy(hm + L.tasks, tasks.data(), sizeof(Task) * nb);
  lpt_order(tasks, reinterpret_cast<int32_t *>(hm + L.order));
  cudaStream_t st = c.stream;
  CK(h, cudaMemcpyAsync(c.raw.p, c.h_raw.p, sizeof(float) * total, cudaMemcpyHostToDevice, st));
  CK(h, cudaMemcpyAsync(c.meta.p, c.h_meta.p, L.total, cudaMemcpyHostToDevice, st));
  const char *dm = c.meta.as<char>();
  int launches = 0;
  CK(h, launch_normalize(c.raw.p, 0, reinterpret_cast<const int64_t *>(dm + L.src_off),
                         reinterpret_cast<const int64_t *>(dm + L.dst_off),
                         reinterpret_cast<const int32_t *>(dm + L.nsamp), nullptr, nullptr, nb, h->cfg.norm_eps,
                         c.query.as<float>(), st));
  ++launches;
  double mean = (double)total / nb;
  if (int rc = enqueue_sweep(h, c, h->cfg.precision, st, c.query.as<float>(), reinterpret_cast<const Task *>(dm + L.tasks),
                             reinterpret_cast<const int32_t *>(dm + L.order), nb, max_len, mean, nb,
                             reinterpret_cast<const int32_t *>(dm + L.nsamp), c.results.p, h->state.as<float>(), true,
                             launches))
    return rc;
  CK(h, cudaMemcpyAsync(c.h_results.p, c.results.p, sizeof(dtwx_result) * nb, cudaMemcpyDeviceToHost, st));
  CK(h, c.h_flags.ensure(64));
  CK(h, cudaMemcpyAsync(c.h_flags.p, c.flags.p, 64, cudaMemcpyDeviceToHost, st));  // read at harvest
  CK(h, cudaEventRecord(c.done, st));
  const double launched = now_ms();
  for (ServeTask &t : batch) t.launched = launched;
  h->inflight[slot] = batch;
  h->running[slot] = true;
  h->batches += 1;
  h->batch_reads_sum += nb;
  h->last_launches = launches;
  return nb;
}

int dtwx_poll_decisions(dtwx_handle *h, dtwx_decision *out, int32_t cap) {
  if (!h || (cap > 0 && !out)) return DTWX_E_ARG;
  if (int rc = harvest_done(h, false)) return rc;
  const int n = (int)std::min<size_t>((size_t)std::max(cap, 0), h->decisions.size());
  for (int i = 0; i < n; ++i) out[i] = h->decisions[i];
  h->decisions.erase(h->decisions.begin(), h->decisions.begin() + n);
  return n;
}

int dtwx_serve_drain(dtwx_handle *h) {
  if (!h) return DTWX_E_ARG;
  if (!h->serving) return fail(h, DTWX_E_STATE, "call dtwx_serve_start first");
  for (;;) {
    if (int rc = harvest_done(h, true)) return rc;
    const int rc = dtwx_serve_step(h);
    if (rc < 0) return rc;
    bool any = false;
    for (int s = 0; s < kServeSlots; ++s) any |= h->running[s];
    if (rc == 0 && !any) break;
  }
  return DTWX_OK;
}

int dtwx_stats_get(dtwx_handle *h, dtwx_stats *out) {
  if (!h || !out) return DTWX_E_ARG;
  memset(out, 0, sizeof(*out));
  out->chunks_submitted = h->chunks_submitted;
  out->chunks_processed = h->chunks_processed;
  out->reads_decided = h->reads_decided;
  out->reads_deferred = h->reads_deferred;
  int64_t q = 0;
  for (auto &kv : h->reads) q += (int64_t)kv.second.pending.size();
  out->queue_depth = (int32_t)q;
  out->in_flight = h->max_in_flight - (int32_t)h->free_slots.size();
  out->max_in_flight = h->max_in_flight;
  out->batches = h->batches;
  out->mean_batch_reads = h->batches ? h->batch_reads_sum / h->batches : 0.0;
  out->mean_batch_ms = h->batches ? h->batch_ms_sum / h->batches : 0.0;
  out->max_batch_ms = h->batch_ms_max;
  out->state_bytes = (double)h->state.cap;
  auto pct = [](std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * (double)(v.size() - 1);
    const size_t lo = (size_t)pos;
    const size_t hi = std::min(lo + 1, v.size() - 1);
    return v[lo] + (v[hi] - v[lo]) * (pos - (double)lo);
  };
  out->p50_latency_ms = pct(h->latencies, 0.50);
  out->p99_latency_ms = pct(h->latencies, 0.99);
  out->p50_queue_ms = pct(h->queue_times, 0.50);
  out->p99_queue_ms = pct(h->queue_times, 0.99);
  return DTWX_OK;
}

}  // extern "C"
