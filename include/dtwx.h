/*
 * dtwx.h -- C ABI of the GB300 subsequence-DTW (sDTW) nanopore read classifier.
 *
 * Drop-in for the sDTW call of DTWax (harisankarsadasivan/DTWax).  Each entry
 * point names the reference interface it replaces (paths are inside that
 * project).  Conventions:
 *   - every call returns DTWX_OK (0) or a negative DTWX_E* status; the text of
 *     the last failure is available from dtwx_last_error(handle) (the reference
 *     prints and calls exit(), src/include/hpc_helpers.hpp:103-113);
 *   - host pointers are borrowed for the duration of the call only; device
 *     state (reference squiggle, scratch, serving row state) is owned by the
 *     handle;
 *   - one handle is driven by one host thread at a time; separate handles are
 *     independent;
 *   - nothing here falls back to a CPU implementation: without a usable CUDA
 *     device dtwx_create fails with DTWX_E_CUDA.
 */
#ifndef DTWX_H
#define DTWX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DTWX_ABI_VERSION 2

/* status codes */
#define DTWX_OK 0
#define DTWX_E_ARG (-1)      /* invalid argument */
#define DTWX_E_IO (-2)       /* file could not be read */
#define DTWX_E_FORMAT (-3)   /* FASTA / k-mer model / input format error */
#define DTWX_E_CUDA (-4)     /* CUDA runtime or driver error */
#define DTWX_E_NOMEM (-5)    /* device or host allocation failed */
#define DTWX_E_TIMEOUT (-6)  /* a bounded device-side wait gave up */
#define DTWX_E_CAPACITY (-7) /* request exceeds a configured capacity */
#define DTWX_E_STATE (-8)    /* call not valid in the handle's current state */

/* arithmetic of the DP */
#define DTWX_FP16 0  /* half2 (fwd, rev) cells, per-strip running-min offset kept in FP32 */
#define DTWX_FP32 1  /* float cells, one strand per work item */
#define DTWX_MIXED 2 /* FP16 differences (half2: two columns of one strand), FP32 cells:
                        each cell is one f32 = f16*f16 + f32 FMA */

/* the recurrence */
#define DTWX_NO_REF_DEL 0 /* D = d^2 + min(up, diag): the reference's build (-DNO_REF_DEL, src/Makefile:8) */
#define DTWX_REF_DEL 1    /* D = d^2 + min(left, up, diag) (DTW.cu:23-29 without -DNO_REF_DEL);
                             FP16 or FP32 cells; a read is one work item (per strand in
                             FP32): a horizontal run can cross any column chunk */

/* serving row state (the last DP row of a read between its chunks) */
#define DTWX_STATE_FP32 0 /* absolute FP32 values: 8 bytes per column pair */
#define DTWX_STATE_FP16 1 /* DTWX_FP16 cells only: half2 cells relative to a float2 frame offset per
                             512 columns, about 4 bytes per column pair (twice the reads per budget) */

/* how the two strands are scored */
#define DTWX_STRANDS_PAIRED 0 /* fwd and rev aligned separately (DTW.cu half2 .x/.y) */
#define DTWX_STRANDS_CONCAT 1 /* one sequence fwd||rev (load_reference.hpp:36-37, sdtw.py:234) */

typedef struct dtwx_config {
  int32_t abi_version;     /* DTWX_ABI_VERSION */
  int32_t precision;       /* DTWX_FP16 (default), DTWX_FP32 or DTWX_MIXED */
  int32_t strand_mode;     /* DTWX_STRANDS_PAIRED (default) or DTWX_STRANDS_CONCAT */
  int32_t device;          /* CUDA device ordinal */
  int64_t max_ref_len;     /* cap on k-mer positions per strand, 0 = none
                              (REF_LEN of src/include/common.hpp:70-74) */
  int32_t adapter_skip;    /* samples dropped at the read start (ADAPTER_LEN, 1952 in
                              the reference; 0 for the synthetic squiggles) */
  int32_t query_len;       /* samples aligned per read after the skip (QUERY_LEN,
                              2048 in the reference); 0 = the rest of the read */
  int32_t require_full;    /* 1: reads shorter than adapter_skip + query_len are
                              skipped, as generate_load_squiggle.hpp:412-430 does */
  float norm_eps;          /* z-score epsilon (normalizer.cu:399 uses 1e-4) */
  float threshold;         /* call = target when score < threshold
                              (calc_classification_threshold.py:52) */
  int32_t max_batch_reads; /* capacity hint for one classify call, 0 = grow on demand */
  int32_t cells_per_thread;/* DP columns per lane; 0 = autotune */
  int32_t chunk_strips;    /* strips (32 lanes x cells_per_thread columns) per work item; 0 = autotune */
  int32_t warps_per_cta;   /* 1..8, 1..16 for FP16 REF_DEL cells; 0 = autotune, else 4, or for
                              REF_DEL the batch spread evenly over the SMs (one CTA per SM) */
  int32_t use_graphs;      /* 1: dtwx_classify_device replays a captured CUDA graph when a batch
                              repeats (same buffers, offsets and stream): the first such batch runs
                              directly, the second is captured, later ones are replays */
  int32_t serve_batches;   /* serving batches in flight at once (1..4), 0 = 2 */
  int32_t recurrence;      /* DTWX_NO_REF_DEL (default) or DTWX_REF_DEL */
  int32_t state_precision; /* DTWX_STATE_FP32 (default) or DTWX_STATE_FP16 */
  int32_t reserved[4];
} dtwx_config;

/* dtwx_result.call of every read of a call whose kernels reported a device
 * error (a bounded wait gave up, or a task exceeded the scratch it was given):
 * the sweep did not finish, the scores are NaN and `strand` holds the device
 * error bits (1: a wait gave up, 2: a task was refused).  Device-pointer calls
 * return before their kernels run, so this mark, and dtwx_sync, are how their
 * callers learn of such an error. */
#define DTWX_CALL_DEVICE_ERROR (-2)

/* Per-read outcome.  end_pos is the DP column (0-based k-mer position on the
 * chosen strand's own 5'->3' axis) where the best alignment ends; score is
 * min(score_fwd, score_rev) with ties going to the smaller end column, then to
 * the forward strand.  n_samples = 0 marks a read that was skipped; call =
 * DTWX_CALL_DEVICE_ERROR a read whose call hit a device error. */
typedef struct dtwx_result {
  float score;
  float score_fwd;
  float score_rev;
  int32_t strand; /* 0 forward, 1 reverse complement */
  int64_t end_pos;
  int32_t call;   /* 1 target, 0 non-target, -1 skipped, DTWX_CALL_DEVICE_ERROR */
  int32_t n_samples;
} dtwx_result;

typedef struct dtwx_handle dtwx_handle;

/* Fill *cfg with the defaults above.  No reference counterpart (the reference
 * uses compile-time macros, src/include/common.hpp:60-98). */
int dtwx_config_default(dtwx_config *cfg);

/* Build a classifier for one target genome.
 * Replaces load_reference::ref_loader + read_kmer_model + load_ref_coeffs
 * (src/include/load_reference.hpp:131-212) and the host tile re-layout of
 * src/main.cu:93-119.  Exactly one of kmer_model_path (text "KMER mean stdev"
 * per line) and level_table (4096 means by 2-bit code, A<C<G<T, first base most
 * significant) is non-NULL.  The squiggle of both strands is built and
 * z-scored on the GPU. */
int dtwx_create(const dtwx_config *cfg, const char *kmer_model_path,
                const float *level_table, const char *fasta_path,
                dtwx_handle **out);

/* Parse a FASTA file with the rules of load_reference::ref_loader
 * (src/include/load_reference.hpp:164-212): a '>' line or an empty line ends
 * the open record, a sequence line holding a space invalidates it, and only the
 * record still open at the end of the file is kept (so the last record wins).
 * Writes up to `cap` bases to seq_out (may be NULL to query the length) and the
 * full length to *len_out.  Host only; needs no GPU. */
int dtwx_load_fasta(const char *fasta_path, char *seq_out, int64_t cap, int64_t *len_out);

/* Parse a k-mer model text file ("KMER mean stdev" per line; read_kmer_model,
 * src/include/load_reference.hpp:131-161) into table_out[4096] by 2-bit code.
 * Host only; needs no GPU. */
int dtwx_load_kmer_model(const char *path, float *table_out);

/* Same, from an in-memory base sequence (no FASTA parsing). */
int dtwx_create_from_sequence(const dtwx_config *cfg, const float *level_table,
                              const char *seq, int64_t seq_len,
                              dtwx_handle **out);

int dtwx_destroy(dtwx_handle *h);

/* Text of the last failure on this handle (never NULL).  With h == NULL it
 * reports the last failure of dtwx_create*. */
const char *dtwx_last_error(const dtwx_handle *h);

/* k-mer positions per strand of the loaded reference. */
int64_t dtwx_ref_len(const dtwx_handle *h);

/* Copy the z-scored squiggle (FP32, one strand each) to host arrays of
 * dtwx_ref_len() floats.  For checking the reference builder. */
int dtwx_get_reference(dtwx_handle *h, float *fwd, float *rev);

/* Offsets (all entry points): n_reads + 1 host int64 values, non-decreasing
 * and starting at 0 or later; anything else returns DTWX_E_ARG before any
 * device work.
 *
 * Classify reads given as raw FP32 samples on the host: read r is
 * raw[offsets[r] .. offsets[r+1]).  Window, z-score (FP64 statistics),
 * sDTW of both strands and the min/argmin all run on the GPU; out[n_reads] is
 * written on return.  Replaces the batch loop of src/main.cu:217-271
 * (normalizer::normalize, src/include/normalizer.cu:370-413, then
 * FullDTW::distances per 10-read batch). */
int dtwx_classify_batch(dtwx_handle *h, const float *raw, const int64_t *offsets,
                        int32_t n_reads, dtwx_result *out);

/* Same for int16 ADC samples; pA = (raw + offset) * range / digitisation per
 * read (fast5/nanopolish_fast5_io.cpp:279-315).  scale arrays may be NULL
 * (raw used as is). */
int dtwx_classify_batch_i16(dtwx_handle *h, const int16_t *raw, const int64_t *offsets,
                            int32_t n_reads, const float *offset, const float *range,
                            const float *digitisation, dtwx_result *out);

/* Device-pointer entry, the in-process launcher of the reference:
 * FullDTW::distances(ref, query, dists, num_entries, thresh, stream,
 * device_last_row) (src/include/DTW.hpp:287-295).  d_query holds z-scored
 * FP32 samples on the device, read r = d_query[offsets[r] .. offsets[r+1])
 * (offsets on the HOST); d_out (device, n_reads entries) receives the results.
 * Work is enqueued on `stream` (a cudaStream_t; 0 is the legacy default
 * stream, as for the reference's launcher) and the call returns without
 * synchronising.  Scratch (work queue, seam columns, keys) is owned by the
 * handle, so calls on one handle must not overlap on different streams.
 * Device-side errors surface in the results (DTWX_CALL_DEVICE_ERROR) and
 * through dtwx_sync.  (The reference's launcher checks nothing.) */
int dtwx_distances(dtwx_handle *h, const float *d_query, const int64_t *offsets,
                   int32_t n_reads, dtwx_result *d_out, void *stream);

/* Device-resident variant of dtwx_classify_batch: raw FP32 samples already on
 * the device (d_raw, offsets on the host), results to d_out on `stream`.
 * Runs the window + z-score kernel, the sDTW kernel and the finalize kernel.
 * Device-side errors surface as for dtwx_distances. */
int dtwx_classify_device(dtwx_handle *h, const float *d_raw, const int64_t *offsets,
                         int32_t n_reads, dtwx_result *d_out, void *stream);

/* The window + z-score step alone, on device buffers: for read r the window
 * of the handle's config (adapter_skip, query_len, require_full) of
 * d_raw[offsets[r] .. offsets[r+1]) (FP32 samples on the device, offsets on
 * the host) is z-scored per read, (x - mean) / sqrt(biased variance +
 * norm_eps) with FP64 statistics, into d_query (device), windows back to back.
 * out_offsets (host, n_reads + 1 entries, may be NULL) receives where each
 * window starts in d_query and the total.  Asynchronous on `stream`.
 * Replaces normalizer::normalize (src/include/normalizer.cu:71-113), which
 * runs cudnnBatchNormalizationForwardTraining over reads x length samples in
 * place (per read mean and biased variance, epsilon 1e-4). */
int dtwx_normalize(dtwx_handle *h, const float *d_raw, const int64_t *offsets, int32_t n_reads,
                   float *d_query, int64_t *out_offsets, void *stream);

/* Wait for the kernels of the handle's most recent dtwx_distances or
 * dtwx_classify_device call and return their device-side status: DTWX_OK,
 * DTWX_E_TIMEOUT (a bounded wait gave up) or DTWX_E_CAPACITY (a task exceeded
 * its scratch).  The status is reported once; DTWX_OK when no such call is
 * outstanding.  The host-buffer entry points check the same status before
 * they return.  Replaces the CUDA error check after the reference's launches
 * (CUERR, src/include/hpc_helpers.hpp:103-113). */
int dtwx_sync(dtwx_handle *h);

/* Test hook for the bounded device waits.  The next sweep launch of this
 * handle does not issue the first reference-strip copy of work item `item`
 * (its queue ticket), so the warp that takes that item waits for data that
 * never comes; every wait of that launch gives up after `spin_limit` polls
 * (0 = the library's limit of 2^18 polls, about one second).  The warp then flags the error and
 * leaves with no copy in flight, the call's results carry
 * DTWX_CALL_DEVICE_ERROR and the status is DTWX_E_TIMEOUT.  One-shot: later
 * launches are unaffected.  Applies to TMA-staged sweeps (the NO_REF_DEL
 * kernels).  No reference counterpart (the reference has no bounded waits). */
int dtwx_debug_stall_next(dtwx_handle *h, int32_t item, uint32_t spin_limit);

/* FP32 sDTW of device-resident reads with no device allocation at all.
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * a process whose GPU memory is reserved by a basecaller's pool (a foreign
 * cudaMalloc can fail or crowd the basecaller out), or a real-time loop that
 * cannot absorb the device-wide synchronisation cudaMalloc/cudaFree may cause.
 * No handle is needed: the caller passes the z-scored reference as FP32 pairs
 * (fwd, rev) per k-mer column in device memory it owns -- ref_len columns,
 * readable up to the next multiple of 512 columns, 16-byte aligned (the sweep
 * reads it in 16-byte loads; DTWX_E_ARG otherwise) -- the z-scored reads
 * (d_query on the device, offsets on the host) and d_out (n_reads results on
 * the device, 8-byte aligned).  Scratch (task table, work counter, seam columns, result keys)
 * is one static device array of about 9 MiB that every GPU loading the library
 * keeps until the process exits.  Limits: at most 4096 reads per call and 2048
 * samples per read; larger requests return DTWX_E_CAPACITY with a message in
 * dtwx_last_error(NULL).  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress).  All calls share the array, so calls that overlap on the GPU
 * (different streams, or several host threads) race and must be serialised by
 * the caller.  Asynchronous on `stream` (0 = legacy default stream).  A device
 * error of the call (a task the scratch cannot hold) marks every result with
 * DTWX_CALL_DEVICE_ERROR. */
int dtwx_distances_static(const void *d_ref_pairs, int64_t ref_len, const float *d_query,
                          const int64_t *offsets, int32_t n_reads, float threshold,
                          dtwx_result *d_out, void *stream);

/* One read per launch in FP32 (no persistent queue, no graph): the plain
 * comparator the batched path is measured against.  Host buffers. */
int dtwx_classify_plain_fp32(dtwx_handle *h, const float *raw, const int64_t *offsets,
                             int32_t n_reads, dtwx_result *out);

/* Kernel launches issued by the most recent classify/distances call. */
int32_t dtwx_last_launch_count(const dtwx_handle *h);

/* Device time of the most recent sDTW sweep kernel launch of a classify or
 * distances call (CUDA events recorded on its stream right before and after
 * the launch; waits for it to finish).  The reference prints the same kind of
 * figure with TIMERSTOP_CUDA (src/include/hpc_helpers.hpp:93-100). */
int dtwx_last_sweep_ms(dtwx_handle *h, float *ms);

/* Autotuner: time the sweep on a synthetic batch of n_reads reads of read_len
 * samples (cut to at most 2,048 reads and about 1.2e13 cells) for every
 * compiled cells-per-thread instance, 4 and 8 warps per CTA (and, for REF_DEL,
 * the batch spread evenly over the SMs), and half / once / twice the analytic
 * chunk width; the fastest shape is used from then on for
 * batches of n_reads reads of that length (log2 buckets of read count and
 * read length).  *best_ms gets its sweep time.  The reference fixes these at
 * compile time (SEGMENT_SIZE, BLOCK_NUM; src/include/common.hpp:64-79). */
int dtwx_autotune(dtwx_handle *h, int32_t n_reads, int32_t read_len, float *best_ms);

/* Launch shape of the handle's most recent batched sweep in its precision:
 * out[0..n) = cells per thread, strips per work item, warps per CTA, CTAs,
 * work items, resident CTAs per SM, CUDA-graph replays so far, 1 if the
 * narrow-halo kernel instance ran (as many as n asks for, up to 8). */
int dtwx_get_tuning(const dtwx_handle *h, int32_t *out, int32_t n);

/* Measured issue-rate ceiling of the cell update on this device: a kernel that
 * runs only the per-cell instruction mix (sub, min, fma) of the given
 * precision over register-resident cells for `ms_target` milliseconds.
 * Returns cells/s in *cells_per_s.  No reference counterpart (roofline). */
int dtwx_peak_probe(int32_t device, int32_t precision, float ms_target, double *cells_per_s);

/* ----------------------------------------------------------------- serving
 * Read Until: per-channel signal chunks arrive as the sequencer produces
 * them; each read's last DP row stays on the device between chunks and the
 * sDTW resumes from it.  Replaces the FIFO loop of src/ru_main.cu:172-326 and
 * the byte-pipe protocol of src/ReadUntil/ont_readuntil.py:29-59.  Reads are
 * admitted while the device row-state pool has room; the rest wait. */
typedef struct dtwx_decision {
  int32_t channel;
  int32_t decided;   /* 1 final (target or max chunks reached), 0 interim */
  uint64_t read_number;
  float score;
  int32_t strand;
  int32_t call;      /* 1 target, 0 non-target */
  int64_t end_pos;
  int32_t chunks;    /* chunks aligned so far */
  int32_t samples;   /* samples aligned so far */
  double latency_ms; /* last needed chunk arrival -> decision */
  double queue_ms;   /* that chunk's arrival -> launch of the batch that aligned it */
} dtwx_decision;

typedef struct dtwx_stats {
  int64_t chunks_submitted;
  int64_t chunks_processed;
  int64_t reads_decided;
  int64_t reads_deferred;    /* reads that waited for row-state memory */
  int32_t queue_depth;       /* chunks waiting now */
  int32_t in_flight;         /* reads holding row state */
  int32_t max_in_flight;     /* row-state slots */
  int32_t batches;           /* device batches launched */
  double p50_latency_ms;
  double p99_latency_ms;
  double mean_batch_reads;
  double state_bytes;        /* device bytes of the row-state pool */
  double mean_batch_ms;      /* device time of a serving batch's sweep, mean and max */
  double max_batch_ms;
  double p50_queue_ms;       /* decided reads: last chunk's arrival -> its batch launch */
  double p99_queue_ms;
} dtwx_stats;

/* Prepare the handle for serving.  max_in_flight = reads holding device row
 * state at once (0: as many as state_budget_bytes allows; both 0: the pool
 * takes half of the free device memory, at most 4096 reads); chunks_per_decision
 * = chunks after which a read is decided even if not a target (the reference
 * decides on one fixed window).  After each chunk a read is a target when its
 * score per aligned sample is below accept_per_sample (or, with
 * accept_per_sample = 0, when its score is below the config threshold), and an
 * early non-target when its score per sample is above reject_per_sample
 * (0 = never early). */
int dtwx_serve_start(dtwx_handle *h, int32_t max_in_flight, double state_budget_bytes,
                     int32_t chunks_per_decision, float accept_per_sample,
                     float reject_per_sample);

/* Queue one chunk (FP32 pA samples) of read `read_number` on `channel`.
 * arrival_ms is the caller's clock at arrival (for latency); < 0 = now. */
int dtwx_submit_chunk(dtwx_handle *h, int32_t channel, uint64_t read_number,
                      const float *samples, int32_t n, int32_t is_last, double arrival_ms);

/* Same for raw int16 ADC samples as the sequencer delivers them
 * (read_until/base.py:349 get_read_chunks, raw_data as int16):
 * pA = (raw + offset) * range / digitisation (fast5/nanopolish_fast5_io.cpp:279-315). */
int dtwx_submit_chunk_i16(dtwx_handle *h, int32_t channel, uint64_t read_number,
                          const int16_t *samples, int32_t n, int32_t is_last, double arrival_ms,
                          float offset, float range, float digitisation);

/* Harvest finished batches and launch the next continuous batch if a chunk
 * is ready and fewer than serve_batches batches are in flight (never blocks);
 * returns the chunks launched (>= 0) or a status. */
int dtwx_serve_step(dtwx_handle *h);

/* Collect decisions made so far (up to cap); returns the count. */
int dtwx_poll_decisions(dtwx_handle *h, dtwx_decision *out, int32_t cap);

/* Wait until every submitted chunk has been processed. */
int dtwx_serve_drain(dtwx_handle *h);

int dtwx_stats_get(dtwx_handle *h, dtwx_stats *out);

/* Host clock in ms used for latency bookkeeping (CLOCK_MONOTONIC). */
double dtwx_now_ms(void);

#ifdef __cplusplus
}
#endif
#endif /* DTWX_H */
