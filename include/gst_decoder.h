/*
 * gst_decoder.h -- C ABI of the GB300 GST decoder (GST stream -> DXT1 blocks).
 *
 * Drop-in replacement for the reference's decoder entry points,
 * codec/decoder.h:12-38 (namespace GenTC), with plain pointers, sizes and
 * status codes instead of std::unique_ptr<gpu::GPUContext>, std::vector and
 * OpenCL handles:
 *
 *   reference (codec/decoder.h)              this header
 *   ---------------------------------------  ----------------------------------
 *   gpu::GPUContext::InitializeOpenCL        gst_init / gst_destroy
 *     (gpu/gpu.h:35-60, gpu/gpu.cpp:394-529)
 *   InitializeDecoder             :15        gst_initialize_decoder
 *   DecompressDXT                 :16-17     gst_decompress_dxt
 *   LoadCompressedDXT             :19-21     gst_load_compressed_dxt
 *   LoadCompressedDXTs            :23-25     gst_load_compressed_dxts
 *   LoadRGB / LoadRGBs            :27-33     gst_load_rgb / gst_load_rgbs
 *   RequiredScratchMem            :35        gst_required_scratch
 *   PreallocateDecompressor       :36        gst_preallocate
 *   FreeDecompressor              :37        gst_free_decompressor
 *   GenTCHeader::LoadFrom (codec/codec_base.h:9-20)  gst_parse_header
 *
 * Device buffers replace cl_mem, a CUDA stream (passed as void*, a
 * cudaStream_t) replaces the cl_command_queue, and completion is stream order
 * (record an event on the stream) instead of a returned cl_event.  The
 * device-resident layout of the compressed data is the reference's
 * (codec/decoder.cpp:430-476, demo/photos_sf.cpp:753-791): a page of
 * 8*N u32 offsets padded to 512 bytes, then 4*N 512-byte frequency tables,
 * then every image's four sections back to back.  Unlike the reference,
 * a batch may mix image sizes.
 *
 * Every call returns a gst_status.  Malformed streams are rejected before any
 * launch where the host holds the bytes; on the device-resident path the
 * kernels check group offsets, table sums and palette indices themselves and
 * report GST_E_FORMAT through gst_sync_status.  There is no CPU fallback: if
 * the CUDA kernels cannot run, the calls fail with GST_E_CUDA.
 */
#ifndef GST_DECODER_H
#define GST_DECODER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gst_status {
  GST_OK = 0,
  GST_E_ARG = 1,     /* bad argument (null pointer, short buffer, bad count) */
  GST_E_FORMAT = 2,  /* malformed GST stream                                 */
  GST_E_OOM = 3,     /* device or pinned memory could not be allocated       */
  GST_E_CUDA = 4,    /* a CUDA call failed                                   */
  GST_E_TIMEOUT = 5  /* a bounded wait on the device gave up                 */
} gst_status;

/* codec/codec_base.h:9-20: seven little-endian u32 words at the stream start. */
typedef struct gst_header {
  uint32_t width;
  uint32_t height;
  uint32_t palette_bytes;
  uint32_t y_cmp_sz;
  uint32_t chroma_cmp_sz;
  uint32_t palette_sz;
  uint32_t indices_sz;
} gst_header;

typedef struct gst_ctx gst_ctx;

/* Creates a decoder context on CUDA device `device` (replaces
 * gpu::GPUContext::InitializeOpenCL, gpu/gpu.cpp:394-529). */
gst_status gst_init(int device, gst_ctx **ctx);
void gst_destroy(gst_ctx *ctx);

/* codec/decoder.cpp:558-591: loads the kernels and checks the device can run
 * them (sm_103 and the shared memory they use).  Optional, as in the reference. */
gst_status gst_initialize_decoder(gst_ctx *ctx);

/* codec/codec_base.cpp:18-25 plus validation of the whole stream: dimensions
 * (w, h multiples of 128, w*h a multiple of 131072), section sizes, the four
 * frequency tables (each sums to 2048) and every group's end offset. */
gst_status gst_parse_header(const uint8_t *gst, size_t len, gst_header *hdr);

/* codec/decoder.cpp:41-47: device scratch one image of this header needs. */
size_t gst_required_scratch(const gst_header *hdr);

/* codec/decoder.cpp:478-485: reserve scratch once for later calls, or free it.
 * Without it the context grows its scratch on demand. */
gst_status gst_preallocate(gst_ctx *ctx, size_t bytes);
gst_status gst_free_decompressor(gst_ctx *ctx);

/* codec/decoder.cpp:487-532: host stream in, host DXT1 out (w*h/2 bytes),
 * blocking. */
gst_status gst_decompress_dxt(gst_ctx *ctx, const uint8_t *gst, size_t len, uint8_t *dxt_out,
                              size_t out_cap);

/* codec/decoder.cpp:534-544: device-resident decode of one image or a batch.
 * d_cmp holds the reference's layout (see above); hdrs are the images'
 * headers in order; outputs are written back to back from d_out (w*h/2 bytes
 * per image).  Enqueued on `stream` (a cudaStream_t; NULL = legacy default). */
gst_status gst_load_compressed_dxt(gst_ctx *ctx, const gst_header *hdr, const void *d_cmp,
                                   void *d_out, void *stream);
gst_status gst_load_compressed_dxts(gst_ctx *ctx, const gst_header *hdrs, int n, const void *d_cmp,
                                    void *d_out, void *stream);

/* LoadRGB / LoadRGBs (codec/decoder.h:27-33, codec/decoder.cpp:546-556): the
 * same decode, written as 8-bit RGB instead of DXT1 -- w*h*3 bytes per image,
 * raster order, 3 bytes per pixel, images back to back from d_out (4-byte
 * aligned).  The pixels are the reference's assemble_rgb
 * (codec/assemble.cl:83-129): endpoints widened from 5:6:5 by bit
 * replication, the four-colour palette (2a + b) / 3, (a + 2b) / 3 whatever
 * the endpoints' order, and 2-bit selectors low bits first. */
gst_status gst_load_rgb(gst_ctx *ctx, const gst_header *hdr, const void *d_cmp, void *d_out, void *stream);
gst_status gst_load_rgbs(gst_ctx *ctx, const gst_header *hdrs, int n, const void *d_cmp, void *d_out,
                         void *stream);

/* Pipelined host-to-host LoadCompressedDXTs (the streaming form of
 * demo/photos_sf.cpp:688-830, no counterpart API in the reference): h_cmp is
 * the reference's layout (as for gst_load_compressed_dxts) and h_out the
 * DXT1 output, both in pinned host memory (cudaMallocHost / cudaHostAlloc).
 * The n images are split into `chunks` (0 = up to 8) contiguous runs whose
 * block counts rise as 1, 2, 4, ... and fall again towards the end; each
 * run's tables and sections are copied in, decoded and copied out on three
 * internal streams, so that copies in, decodes and copies out of different
 * runs overlap (small first and last runs: the copies out, the slowest stage,
 * start early and little is left after the last decode).  Enqueued after the work already on
 * `stream`, and `stream` waits for the last copy out: h_out is complete once
 * `stream` reaches that point.  Calls on one context run one after another. */
gst_status gst_load_host_dxts(gst_ctx *ctx, const gst_header *hdrs, int n, const void *h_cmp, void *h_out,
                              int chunks, void *stream);

/* Resident batches (the serving and benchmark form of LoadCompressedDXTs):
 * gst_batch_create builds the batch's work plan once, uploads it and reserves
 * the batch's own scratch (gst_batch_device_bytes in total), so that
 * gst_batch_launch enqueues only kernels -- no host work, no copies -- and may
 * be captured in a CUDA graph; gst_batch_graph_launch captures it once per
 * (d_cmp, d_out) pair and replays the graph.  Batches are independent of each
 * other and of the context's own scratch, so different batches may run
 * concurrently on different streams; one batch must not run concurrently with
 * itself.  No counterpart in the reference, whose every call rebuilds its
 * sub-buffers and re-enqueues its kernels (codec/decoder.cpp:98-428). */
typedef struct gst_batch gst_batch;
gst_status gst_batch_create(gst_ctx *ctx, const gst_header *hdrs, int n, gst_batch **batch);
void gst_batch_destroy(gst_batch *batch);
size_t gst_batch_device_bytes(const gst_batch *batch);
/* rANS CTAs of the batch's next two-kernel launch (its plan's rANS items):
 * runs of up to 4 groups of one section, or -- where the batch's groups fill
 * the launch's one wave of CTAs with 3.5 groups an item or more -- exactly
 * that wave's capacity of near-equal items.  0 for a null batch. */
int gst_batch_rans_items(const gst_batch *batch);
gst_status gst_batch_launch(gst_batch *batch, const void *d_cmp, void *d_out, void *stream);
gst_status gst_batch_graph_launch(gst_batch *batch, const void *d_cmp, void *d_out, void *stream);

/* The batch from pinned host memory to pinned host memory: gst_load_host_dxts's
 * pipeline (copies in, decodes and copies out of `chunks` runs overlapped,
 * 0 = 3) with the batch's own device mirrors and per-run plans, built once per
 * chunk count, and the whole pipeline captured as one CUDA graph per (h_cmp,
 * h_out, chunks, tuning) and replayed: a call costs one graph launch of host
 * work, while every copy and decode runs each time.  A batch without a tuning
 * of its own decodes each run with the run's own size-dependent
 * configuration (see gst_get_class_tuning).  The batch's device launches and
 * its host launches must not run concurrently. */
gst_status gst_batch_host_launch(gst_batch *batch, const void *h_cmp, void *h_out, int chunks, void *stream);

/* Per-batch tuning of the launch (no counterpart in the reference).
 * gst_batch_autotune decodes the batch under each of a fixed set of
 * configurations -- two kernels at (CTAs per SM, staging depth), or the
 * persistent kernel at a staging depth -- one warm-up and `iterations` timed
 * launches each, on `stream`, blocking, and keeps the fastest for the batch's
 * later launches, writing it to *blocks_per_sm / *stage_words / *persistent
 * when those are non-null.  It writes the decoded output to d_out as a launch
 * does and must not be called while `stream` is being captured.
 * gst_batch_set_tuning sets the configuration directly (values as for the
 * "rans_blocks_per_sm", "rans_stage_words" and "persistent" options); (0, 0, 0)
 * returns the batch to the context's configuration.  Every configuration
 * decodes bit-identically; only the time differs. */
gst_status gst_batch_autotune(gst_batch *batch, const void *d_cmp, void *d_out, void *stream, int iterations,
                              int *blocks_per_sm, int *stage_words, int *persistent);
gst_status gst_batch_set_tuning(gst_batch *batch, int blocks_per_sm, int stage_words, int persistent);

/* Per-size-class tuning of the context's launches (no counterpart in the
 * reference).  A launch's size class is set by its DXT1 block count: class 0
 * up to 2^14 blocks (one 512x512 image), each next class four times larger,
 * class 6 above 2^24.  Per-image and batched context calls, the server's
 * launches, the pipelined host calls and batches without their own tuning
 * use their class's configuration where one is set, else the context's
 * ("rans_blocks_per_sm" / "rans_stage_words" / "persistent" options) once
 * any of those options was set.  With neither, a launch whose rANS items
 * (runs of 4 groups) fit one wave of 8 CTAs per SM with 4352-word stages
 * uses that configuration, else one that fits at 1528 words, else the
 * context's default (12, 1016, two kernels): a launch of a few images needs
 * no more CTAs per SM, and every re-stage it avoids is on its critical path.
 * gst_set_class_tuning sets a class (values as for gst_batch_set_tuning;
 * 0, 0 clears it); gst_autotune_class runs gst_batch_autotune on a
 * representative batch and sets the result for that batch's class, which it
 * returns in *size_class; gst_get_class_tuning reads a class's configuration
 * (the context's for a class without one).
 * The server keeps the two-kernel form for its launches (they run side by
 * side on its slots), with the class's CTAs per SM and staging depth. */
int gst_size_class(uint64_t blocks);
gst_status gst_get_class_tuning(gst_ctx *ctx, int size_class, int *blocks_per_sm, int *stage_words, int *persistent);
gst_status gst_set_class_tuning(gst_ctx *ctx, int size_class, int blocks_per_sm, int stage_words, int persistent);
gst_status gst_autotune_class(gst_ctx *ctx, const gst_header *hdrs, int n, const void *d_cmp, void *d_out,
                              void *stream, int iterations, int *size_class);

/* The per-size-class configurations as a JSON table on disk (no counterpart
 * in the reference), so that tuning outlives the process:
 *   {"format": "gst_gb300 class tuning", "version": 1, "device": "<GPU name>",
 *    "classes": [{"class": c, "max_blocks": m, "blocks_per_sm": b,
 *                 "stage_words": w, "persistent": p}, ...]}
 * gst_save_class_tuning writes the classes that are set (atomically: a
 * temporary file renamed into place); gst_load_class_tuning replaces the
 * context's class table with the file's after validating every entry
 * (GST_E_FORMAT for a malformed table, GST_E_ARG for a missing file or one
 * written on another kind of GPU; nothing changes on error).  With the
 * environment variable GST_TUNING_TABLE naming a file, gst_init loads it when
 * it exists and matches the device, and gst_autotune_class saves the table
 * there after each run. */
gst_status gst_save_class_tuning(gst_ctx *ctx, const char *path);
gst_status gst_load_class_tuning(gst_ctx *ctx, const char *path);

/* One-image device-resident decode that allocates nothing -- no counterpart in
 * the reference, which allocates its decoder scratch per call or through
 * PreallocateDecompressor.  For callers that must not allocate device memory
 * while they decode: a render or streaming thread that cannot absorb the
 * device-wide synchronisation cudaMalloc/cudaFree may cause, or an engine that
 * owns all device memory through its own pools.  It needs no gst_ctx (creating one
 * allocates).  Input and output are the caller's, as for
 * gst_load_compressed_dxt; the scratch is a 4 MiB array built into the library,
 * held by every GPU that loads the library until the process exits.
 *   - Limit: the image's scratch (256 + 8*B + palette_bytes + B/8 + B/1024
 *     bytes, B = width*height/16) must fit in 4 MiB -- about 2048x2048;
 *     larger images return GST_E_ARG and nothing is enqueued.
 *   - All calls share that array and leave their data in it: each call clears
 *     the words that must start at zero; calls whose GPU work overlaps (other
 *     streams without ordering, other host threads) race -- serialise them.
 *   - The first call on a device looks up the array's address on that device;
 *     make it before any stream capture there.
 *   - With device_status non-null the call waits for `stream` and stores the
 *     kernels' error bits there (0 when the stream was well formed).  With
 *     device_status null nothing reports a malformed payload: the call returns
 *     GST_OK once the work is enqueued and the output is then undefined. */
gst_status gst_load_compressed_dxt_static(const gst_header *hdr, const void *d_cmp, void *d_out, void *stream,
                                          uint32_t *device_status);

/* Size of the reference's device layout for these headers (offsets page,
 * frequency tables, sections), and a host-side packer that writes it from
 * n complete GST streams (gst[i] of len[i] bytes) into `dst`. */
size_t gst_batch_layout_bytes(const gst_header *hdrs, int n);
gst_status gst_pack_batch(const uint8_t *const *gst, const size_t *len, int n, uint8_t *dst,
                          size_t dst_cap);

/* rANS stage alone (ans/ans_decode.cl:97-143 with the table of
 * ans/build_table.cl), as the reference's ans::ocl::OpenCLDecoder::Decode
 * (ans/ans_ocl.h:26-72) exposes it: d_freqs holds 256 u16 normalised
 * frequencies (sum 2048), d_body a section body in the format of
 * codec/entropy.cpp:174-265 (n_groups u32 end offsets, then the groups, each
 * ending in streams_per_group u32 final states).  Writes n_groups *
 * streams_per_group * 256 symbols to d_out, stream-major within a group
 * (out[(g * streams + s) * 256 + i]).  d_out must be 16-byte aligned. */
gst_status gst_decode_rans_groups(gst_ctx *ctx, const void *d_freqs, const void *d_body, uint32_t body_bytes,
                                  uint32_t n_groups, uint32_t streams_per_group, void *d_out, void *stream);

/* Waits for `stream` and returns the device-side status of the last decode
 * enqueued through this context (GST_E_FORMAT if the kernels met a malformed
 * stream), then clears it. */
gst_status gst_sync_status(gst_ctx *ctx, void *stream);

/* Number of kernel launches the last decode call made (for instrumentation). */
int gst_last_launch_count(gst_ctx *ctx);

/* Instrumentation (no counterpart in the reference, whose queues are created
 * without profiling, gpu/gpu.cpp:483): with profiling on, each decode call
 * records CUDA events on its stream around every kernel it launches;
 * gst_kernel_times waits for the last call and writes the kernels' durations
 * in milliseconds (and their names, if `names` is non-null); it returns the
 * number written. */
gst_status gst_set_profiling(gst_ctx *ctx, int enable);
int gst_kernel_times(gst_ctx *ctx, float *ms, const char **names, int cap);

/* Tuning knobs of a context (no counterpart in the reference; its work-group
 * sizes are fixed, codec/decoder.cpp:166-417).  Known names:
 *   "rans_blocks_per_sm"  register budget of the rANS kernel in CTAs of 128
 *                         threads per SM: 1-9 (eight, 64 registers), 10-13
 *                         (twelve, default) or 14-16 (sixteen).  The
 *                         persistent kernel always runs 8 per SM.  Setting
 *                         this, "rans_stage_words" or "persistent" also
 *                         turns off the size-dependent choice for launches
 *                         of a few images (gst_get_class_tuning).
 *   "rans_stage_words"    16-bit renormalisation words each warp stages in
 *                         shared memory: a multiple of 8 in [520, 4352];
 *                         default 1016.  Deeper stages re-stage less often
 *                         but leave room for fewer CTAs per SM (16 CTAs at
 *                         520 words, 13 at 1016, 8 at 2040, 5 at 4352, which
 *                         holds any group whole: for launches of a few
 *                         groups, where the re-stages are on the critical
 *                         path).
 *   "persistent"          0 (default): a rANS kernel, then a tile kernel;
 *                         1: one persistent kernel whose CTAs take rANS
 *                         items, then tiles, from a work queue in the plan
 *                         (a tile waits, bounded, for its image's groups;
 *                         GST_E_TIMEOUT from gst_sync_status if it gave up).
 *                         gst_decode_rans_groups always uses the rANS kernel.
 *   "persistent_wait_us"  bound of a persistent tile's wait for its image and
 *                         of an encoder group's look-back wait for the sizes
 *                         before it, microseconds (0 = 2 s, at most
 *                         2,000,000).
 *   "auto_tuning"         1: back to the default configuration (12, 1016,
 *                         two kernels) with the size-dependent choice for
 *                         launches of a few images; other values GST_E_ARG.
 *   "balance_rans_items"  1 (default): where a launch's rANS groups fill its
 *                         one wave of CTAs (SMs x resident CTAs per SM of the
 *                         two-kernel form) with 3.5 groups an item or more,
 *                         the plan cuts them into exactly that many items of
 *                         near-equal size, so that every SM holds the same
 *                         work; 0: runs of 4 groups of one section always.
 *                         Resident batches re-cut their plan at their next
 *                         launch outside stream capture.
 *   "encode_hist_match"   encoder byte counts (gst_encode.h): 0 (default)
 *                         issues one shared-memory atomic per byte; 1 merges
 *                         the lanes of a warp holding the same byte first
 *                         (a match-any per byte: slower on measured sections).
 *   "inject_encode_stall" fault injection for tests, 0 (default) or 1: in
 *                         encoder calls (gst_encode.h) group 1 never publishes
 *                         its size, so the later groups' bounded look-back
 *                         waits run out (bound: "persistent_wait_us") and the
 *                         call reports GST_E_TIMEOUT through gst_sync_status.
 *   "inject_drop_rans"    fault injection for tests, 0 (default) or 1: the
 *                         context's persistent launches leave out their rANS
 *                         items, so every tile waits until its bound and the
 *                         call reports GST_E_TIMEOUT; the decode is void.
 * Invalid values and unknown names return GST_E_ARG.  They apply to the
 * context's calls and to resident batches without a tuning of their own;
 * such batches re-capture their graph after a change. */
gst_status gst_set_option(gst_ctx *ctx, const char *name, int value);

/* Serving: a continuous-batching decode server (no counterpart in the
 * reference, whose demos decode fixed pages of pre-packed streams,
 * demo/photos_sf.cpp:688-830).
 *   - gst_server_submit copies one whole GST stream (header, tables, sections)
 *     into pinned host staging and queues it; it returns at once.  The stream
 *     is validated first (as gst_parse_header).  GST_E_OOM: the staging is
 *     full (retry later) or the request could never fit the device budget.
 *     arrival_ns (server clock, gst_server_now_ns) stamps the request's
 *     arrival for latency; 0 = now.
 *   - A scheduler thread admits queued requests in arrival order while their
 *     compressed bytes plus DXT1 output fit in device_budget_bytes, and
 *     launches everything admitted as one batch whenever one of max_inflight
 *     launch slots is free; launches run on their own streams and overlap on
 *     the device, and requests that arrive meanwhile ride in the next launch.
 *   - gst_server_poll returns finished requests (waiting up to wait_us for
 *     the first); each result's DXT1 blocks stay resident on the device at
 *     d_dxt until gst_server_release, which returns its memory to the budget.
 *     gst_server_read copies one result to host memory (blocking).
 *   - gst_server_cancel withdraws a request that has not been launched yet
 *     (queued, or admitted and waiting for a slot): its staging and device
 *     memory return at once and it never appears in gst_server_poll.
 *     GST_E_ARG for an unknown id or a request already launched (that one
 *     completes normally and is released after polling).
 *   - gst_server_read_stats reports counts and submit-to-finish latency
 *     percentiles since the last reset (reset != 0 starts a new period).
 *   - gst_server_destroy waits for the launches in flight and drops requests
 *     not yet launched.
 * Each request's result is bit-identical to its plain single-image decode:
 * images of a launch share nothing but the launch. */
typedef struct gst_server gst_server;
typedef struct {
  size_t device_budget_bytes; /* compressed input + DXT1 output of admitted requests; 0 = 32 GiB */
  size_t host_staging_bytes;  /* pinned staging of submitted streams; 0 = 1 GiB */
  size_t slot_scratch_bytes;  /* decode scratch of one launch, allocated per slot at creation; a launch takes images while they fit; 0 = 256 MiB */
  int max_inflight;           /* launches in flight, each on its own stream; 0 = 4 */
  int max_batch_images;       /* images per launch; 0 = 256; 1 decodes every request alone */
} gst_server_config;
typedef struct {
  uint64_t id;
  gst_status status; /* GST_E_FORMAT if the kernels met a malformed stream in its launch */
  void *d_dxt;       /* device address of the DXT1 blocks, valid until gst_server_release */
  size_t dxt_bytes;
  uint32_t width, height;
  uint64_t arrival_ns, launch_ns, done_ns; /* server clock */
} gst_server_result;
typedef struct {
  uint64_t submitted, completed, rejected, launches, launched_images, pixels, queued;
  size_t device_bytes_in_use, device_bytes_peak;
  double seconds; /* length of the statistics period */
  double latency_mean_us, latency_p50_us, latency_p99_us, latency_max_us;
  uint64_t cancelled; /* requests withdrawn by gst_server_cancel */
} gst_server_stats;
gst_status gst_server_create(gst_ctx *ctx, const gst_server_config *cfg, gst_server **server);
void gst_server_destroy(gst_server *server);
uint64_t gst_server_now_ns(gst_server *server);
gst_status gst_server_submit(gst_server *server, const void *gst, size_t len, uint64_t arrival_ns, uint64_t *id);
gst_status gst_server_poll(gst_server *server, gst_server_result *out, int cap, int *n, int wait_us);
gst_status gst_server_read(gst_server *server, uint64_t id, void *dst, size_t cap);
gst_status gst_server_release(gst_server *server, uint64_t id);
gst_status gst_server_cancel(gst_server *server, uint64_t id);
gst_status gst_server_read_stats(gst_server *server, gst_server_stats *stats, int reset);

/* Open-loop load from a native thread, so that no stall of the caller delays
 * a submission: stream i (gst[i], len[i] bytes) is submitted at server time
 * arrival_ns[i] (gst_server_now_ns clock, nondecreasing) and stamped with
 * it, while the caller polls and releases results.  ids[i] receives the
 * request's id as soon as it is submitted, or 0 if it was refused (staging
 * full at its arrival, or never admissible); the caller may read ids while
 * the schedule runs (each entry is written once, 8-byte aligned) and keeps
 * the streams, len, arrival_ns and ids alive until gst_server_schedule_wait,
 * which joins the thread and returns the submitted and refused counts and the
 * worst lateness of a submission behind its arrival.  One schedule at a time
 * (GST_E_ARG otherwise; concurrent calls from several threads are safe);
 * gst_server_destroy stops a running one. */
gst_status gst_server_schedule(gst_server *server, int n, const void *const *gst, const size_t *len,
                               const uint64_t *arrival_ns, uint64_t *ids);
gst_status gst_server_schedule_wait(gst_server *server, int *submitted, int *rejected, uint64_t *late_max_ns);

/* Human-readable name of a status code. */
const char *gst_status_string(gst_status s);

#ifdef __cplusplus
}
#endif
#endif /* GST_DECODER_H */
