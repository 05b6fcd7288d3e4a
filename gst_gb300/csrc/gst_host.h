// gst_host.h -- host-side helpers shared by the C ABI (gst_api.cpp) and the
// serving loop (gst_server.cpp).  Internal to the library.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <mutex>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "gst_decoder.h"
#include "gst_encode_plan.h"
#include "gst_plan.h"

namespace gst {

// An NVTX range over the host-side enqueue of one stage (rANS, tile, copy in,
// copy out, a server launch), so that a timeline tool shows each stage
// against the kernels and copies it issued.  NVTX is header-only: without an
// attached tool a range costs a few nanoseconds.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// gst_encode.cu
// Enqueues the encoder kernels of one plan (histogram, normalisation, rANS
// encode, tables); normalize_only runs the normalisation alone on counts
// already in place.
cudaError_t launch_encode(const EncPlanView &v, int sm_count, cudaStream_t stream, bool normalize_only,
                          int *launches, cudaEvent_t *ev = nullptr, const char **names = nullptr,
                          bool hist_match = true);

// gst_prepare.cu
// Enqueues the endpoint stages (forward wavelet planes, run palette) of the
// images of a plan.
cudaError_t launch_reencode(const ReImage *d_imgs, const uint32_t *d_order, ReState *d_states, uint32_t n_images,
                            const uint32_t *chunks_desc, uint32_t max_blocks, uint32_t *d_status, cudaStream_t stream,
                            int *launches);
cudaError_t launch_prepare(const EncPrepImage *d_images, uint32_t n_images, uint32_t n_tiles,
                           const EncPrepChunk *d_chunks, uint32_t n_chunks, uint32_t *d_counts,
                           uint32_t *d_palette_bytes, cudaStream_t stream, cudaEvent_t *ev = nullptr,
                           const char **names = nullptr);

// gst_kernels.cu
// Enqueues the kernels of one plan; names (may be null) receives the name of
// each kernel launched, in order.
cudaError_t launch_decode(const uint8_t *d_cmp, uint8_t *d_scratch, uint8_t *d_out, GstPlanView plan,
                          cudaStream_t stream, int *launches, cudaEvent_t *ev, const GstTuning &tuning,
                          const char **names = nullptr);

// CTAs of the two-kernel form's rANS kernel that the device holds at once
// under `t` (SMs x resident CTAs per SM, from the occupancy calculator); 0 for
// the persistent form.
uint32_t rans_wave_capacity(const GstTuning &t);

namespace host {

size_t align_up(size_t x, size_t a);
gst_status cuda_status(cudaError_t e);
// Dimension and size rules a header must meet before anything is launched.
gst_status check_header(const gst_header &h);
uint64_t image_blocks(const gst_header &h);
uint64_t total_blocks(const gst_header *hdrs, int n);
uint64_t section_bytes(const gst_header &h);

// Scratch layout of one image: decoded symbols, chunk prefixes, group sums.
struct ScratchLayout {
  size_t sym, chunk, gsum, total;
};
ScratchLayout scratch_layout(const gst_header &h);

// Where everything of a plan for these headers goes.
struct PlanLayout {
  size_t off_images, off_rans, off_tiles, off_order, off_counters, off_image_err, off_sync, bytes;
  int n_images;
  uint32_t n_rans, n_tiles;
  size_t scratch_bytes;
  std::vector<ScratchLayout> lay;
  // rANS items of image i's section s at [4 i + s]; `balanced` when their
  // sizes were evened out to fill a launch's one-wave capacity exactly.
  std::vector<uint32_t> items;
  bool balanced = false;
};
// `capacity`: how many rANS CTAs of the intended launch are resident at once
// (rans_wave_capacity), or 0.  Where the work fills that one wave with items
// of 3.5 groups or more on average, the sections are cut into exactly
// `capacity` items of near-equal size instead of runs of 4 groups, so that
// every SM holds the same number of CTAs and of groups.
PlanLayout plan_layout(const gst_header *hdrs, int n, uint32_t capacity = 0);
// out_block_bytes: output bytes per block, 8 (DXT1) or 48 (RGB8).
void write_plan(const PlanLayout &L, const gst_header *hdrs, int n, uint8_t *ph, const uint64_t *freq_at,
                const uint64_t *body_at, const uint64_t *out_at, uint32_t out_block_bytes = 8);
GstPlanView plan_view(const PlanLayout &L, uint8_t *plan_d, uint32_t *status_d);

int ctx_device(const gst_ctx *ctx);
// The one-wave capacity plan_layout balances rANS items for under tuning `t`
// (rans_wave_capacity), or 0 where the context's "balance_rans_items" option
// is off.
uint32_t plan_capacity(const gst_ctx *ctx, const GstTuning &t);
GstTuning ctx_tuning(gst_ctx *ctx);
// The configuration of a launch of these images: their size class's entry
// where one is set, else the context's where its tuning options were set,
// else the deepest stages whose one wave holds the launch (few images) or
// the context's default.
GstTuning ctx_tuning_for(gst_ctx *ctx, const gst_header *hdrs, int n);
int size_class(uint64_t blocks);

// Context state of the encoder calls (gst_encode_api.cpp), created on first use.
struct EncodeState;
void destroy_encode_state(EncodeState *s);
std::mutex &ctx_mutex(gst_ctx *ctx);
EncodeState *&ctx_encode_state(gst_ctx *ctx);
uint32_t *ctx_status(gst_ctx *ctx);
uint64_t ctx_wait_limit_ns(gst_ctx *ctx);
// Instrumentation of the context's last call (gst_set_profiling / gst_kernel_times):
// null when profiling is off or `capturing`.
cudaEvent_t *ctx_timing_events(gst_ctx *ctx, bool capturing);
void ctx_set_timed(gst_ctx *ctx, int kernels, int launches);
const char **ctx_timed_names(gst_ctx *ctx);
bool ctx_enc_hist_match(gst_ctx *ctx);
bool ctx_inject_encode_stall(gst_ctx *ctx);
// Waits for `stream` and turns the device error bits into a status (clears them).
gst_status read_device_status(gst_ctx *ctx, cudaStream_t stream);

}  // namespace host
}  // namespace gst
