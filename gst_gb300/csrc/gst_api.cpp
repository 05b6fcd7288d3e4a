// gst_api.cpp -- C ABI of the GB300 GST decoder (include/gst_decoder.h).
//
// Host half of the decode path: header parsing and stream validation, the
// per-call work plan (gst_plan.h), scratch management and the launches.  It
// replaces codec/decoder.cpp:41-591 and the OpenCL context of gpu/gpu.cpp; the
// device work is in gst_kernels.cu.  No CPU fallback exists: every decode goes
// through the CUDA kernels or fails with GST_E_CUDA.
#include "gst_decoder.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gst_host.h"
#include "gst_plan.h"

constexpr int kMaxTimedKernels = 4;

using namespace gst;
using namespace gst::host;

namespace gst {
namespace host {

constexpr size_t kAlign = 256;
size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

uint32_t rd32(const uint8_t *p) {
  return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}

// Dimension and size rules a header must meet before anything is launched
// (README.md:67-71 of the reference; blocks < 2^28 keeps every offset in u32).
gst_status check_header(const gst_header &h) {
  if (h.width == 0 || h.height == 0 || h.width % 128 || h.height % 128) return GST_E_FORMAT;
  const uint64_t px = uint64_t(h.width) * h.height;
  if (px % (16u * 256u * 32u)) return GST_E_FORMAT;
  const uint64_t B = px / 16;
  if (B >= (1u << 28)) return GST_E_FORMAT;
  if (h.palette_bytes == 0 || h.palette_bytes % kSymsPerGroup) return GST_E_FORMAT;
  if (8 * B + h.palette_bytes >= (1ull << 32)) return GST_E_FORMAT;
  const uint32_t lens[4] = {h.y_cmp_sz, h.chroma_cmp_sz, h.palette_sz, h.indices_sz};
  const uint64_t syms[4] = {2 * B, 4 * B, h.palette_bytes, B};
  for (int i = 0; i < 4; ++i) {
    const uint64_t G = syms[i] / kSymsPerGroup;
    if (lens[i] % 4 || G * (4 + 4 * kStreamsPerGroup) > lens[i]) return GST_E_FORMAT;
  }
  return GST_OK;
}

uint64_t image_blocks(const gst_header &h) { return uint64_t(h.width / 4) * (h.height / 4); }
uint64_t section_bytes(const gst_header &h) {
  return uint64_t(h.y_cmp_sz) + h.chroma_cmp_sz + h.palette_sz + h.indices_sz;
}

ScratchLayout scratch_layout(const gst_header &h) {
  const uint64_t B = image_blocks(h);
  ScratchLayout s;
  s.sym = 0;
  s.chunk = align_up(8 * B + h.palette_bytes, kAlign);  // index section: 2 bytes per block
  s.gsum = s.chunk + align_up(B / 32 * 4, kAlign);
  s.total = s.gsum + align_up(2 * (B / kSymsPerGroup) * 4, kAlign);
  return s;
}

size_t offsets_page_bytes(int n) { return align_up(size_t(n) * 8 * 4, 512); }

// Each decode call uploads its plan from one of kPlanRing pinned host buffers
// into the matching device buffer, so the host can prepare up to kPlanRing
// calls ahead of the GPU before it waits.
constexpr int kPlanRing = 8;
struct PlanBuf {
  uint8_t *d = nullptr;  // device copy read by the kernels
  size_t d_cap = 0;
  uint8_t *h = nullptr;  // pinned host staging
  size_t h_cap = 0;
  cudaEvent_t copied = nullptr;  // the pinned staging may be rewritten once this fires
  cudaEvent_t done = nullptr;    // the device copy may be rewritten once this fires
  cudaStream_t stream = nullptr;
  bool used = false;
};

}  // namespace host
}  // namespace gst

struct gst_ctx {
  int device = 0;
  std::mutex mu;
  // Scratch for decoded symbols and index prefixes, shared by all calls;
  // calls on different streams are ordered through scratch_done.
  uint8_t *scratch = nullptr;
  size_t scratch_cap = 0;
  bool preallocated = false;
  cudaEvent_t scratch_done = nullptr;
  cudaStream_t scratch_stream = nullptr;
  bool scratch_used = false;
  PlanBuf plans[kPlanRing];
  int next_plan = 0;
  uint32_t *status_d = nullptr;  // device error bits of the calls since the last status read
  cudaStream_t own_stream = nullptr;
  // Staging for the host-buffer path (gst_decompress_dxt).
  uint8_t *cmp_d = nullptr;
  size_t cmp_cap = 0;
  uint8_t *out_d = nullptr;
  size_t out_cap = 0;
  uint8_t *cmp_h = nullptr;  // pinned
  size_t cmp_h_cap = 0;
  uint8_t *out_h = nullptr;  // pinned
  size_t out_h_cap = 0;
  int last_launches = 0;
  GstTuning tuning;  // rANS launch configuration of the context's calls and untuned batches
  // Per size class (gst_size_class of a launch's blocks), set by
  // gst_set_class_tuning / gst_autotune_class; unset classes use `tuning`.
  GstTuning class_tuning[kSizeClasses];
  bool class_set[kSizeClasses] = {};
  uint64_t wait_limit_ns = 0;  // persistent tile wait bound (0: the kernel's 2 s)
  bool inject_drop_rans = false;  // fault injection for tests: persistent launches without their rANS items
  // Instrumentation: events around each kernel of the last decode call.
  bool profiling = false;
  cudaEvent_t ev[kMaxTimedKernels + 1] = {};
  int timed_kernels = 0;
  const char *timed_names[kMaxTimedKernels] = {};
  // Pipelined host-to-host decode (gst_load_host_dxts): device mirrors of the
  // caller's pinned input and output, and its copy-in / decode / copy-out
  // streams with one event pair per chunk.
  uint8_t *hs_cmp_d = nullptr;
  size_t hs_cmp_cap = 0;
  uint8_t *hs_out_d = nullptr;
  size_t hs_out_cap = 0;
  cudaStream_t hs_in = nullptr, hs_comp = nullptr, hs_out = nullptr;
  cudaEvent_t hs_start = nullptr, hs_done = nullptr;
  cudaEvent_t hs_copied[kPlanRing] = {}, hs_decoded[kPlanRing] = {};
  bool hs_used = false;
  gst::host::EncodeState *enc = nullptr;  // encoder calls (gst_encode_api.cpp)
  bool enc_hist_match = false;            // encoder byte counts: merge equal lanes before the atomic
  bool balance_items = true;              // cut rANS items to fill one wave where that pays (plan_layout)
  bool tuning_explicit = false;           // the tuning options were set: untuned launches use ctx->tuning
  bool inject_encode_stall = false;       // fault injection for tests: group 1 never publishes its size
};

namespace gst {
namespace host {

// Size class of a launch of `blocks` DXT1 blocks: up to 2^14 (one 512x512
// image) is class 0, each next class four times larger, the last open-ended.
int size_class(uint64_t blocks) {
  int c = 0;
  for (uint64_t limit = uint64_t(1) << 14; blocks > limit && c < kSizeClasses - 1; limit <<= 2) ++c;
  return c;
}
// The configuration of such a launch (the caller holds ctx->mu or owns ctx).
GstTuning tuning_for_locked(const gst_ctx *ctx, uint64_t blocks) {
  const int c = size_class(blocks);
  return ctx->class_set[c] ? ctx->class_tuning[c] : ctx->tuning;
}

// The configuration of a launch of these images: their size class's entry
// where one is set, else the context's where its tuning options were set.
// Otherwise the deepest stages whose one wave of CTAs still holds the
// launch's rANS items: a launch of a few images needs no more CTAs per SM
// than that, and each re-stage it avoids lies on its critical path (64
// one-image calls of the batch: 2.35 ms at 8 CTAs/SM with 4352-word stages,
// 2.72 ms at 12 with 1016).  Larger launches keep the context's default.
GstTuning launch_tuning_locked(const gst_ctx *ctx, const gst_header *hdrs, int n) {
  const int c = size_class(total_blocks(hdrs, n));
  if (ctx->class_set[c]) return ctx->class_tuning[c];
  if (ctx->tuning_explicit) return ctx->tuning;
  uint64_t items = 0;  // runs of 4 groups
  for (int i = 0; i < n; ++i) {
    const uint64_t B = image_blocks(hdrs[i]);
    for (uint64_t G : {2 * B / kSymsPerGroup, 4 * B / kSymsPerGroup, uint64_t(hdrs[i].palette_bytes) / kSymsPerGroup,
                       B / kSymsPerGroup})
      items += (G + kGroupsPerRansCta - 1) / kGroupsPerRansCta;
  }
  static const GstTuning kFew[] = {{8, 4352, 0}, {8, 1528, 0}};
  for (const GstTuning &t : kFew) {
    const uint32_t cap = rans_wave_capacity(t);
    if (cap > 0 && items <= cap) return t;
  }
  return ctx->tuning;
}

gst_status cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return GST_OK;
  if (e == cudaErrorMemoryAllocation) return GST_E_OOM;
  return GST_E_CUDA;
}

gst_status grow_device(uint8_t **p, size_t *cap, size_t need) {
  if (*cap >= need) return GST_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const size_t sz = std::max(need, size_t(1) << 20);
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), sz);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_status(e);
  }
  *cap = sz;
  return GST_OK;
}

gst_status grow_pinned(uint8_t **p, size_t *cap, size_t need) {
  if (*cap >= need) return GST_OK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  const size_t sz = std::max(need, size_t(1) << 16);
  cudaError_t e = cudaMallocHost(reinterpret_cast<void **>(p), sz);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_status(e);
  }
  *cap = sz;
  return GST_OK;
}

bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) return false;
  return st != cudaStreamCaptureStatusNone;
}

// Takes the next plan buffer of the ring with room for `bytes`; on return
// its pinned staging may be written and the device copy may be overwritten by
// work enqueued on `stream`.
gst_status acquire_plan(gst_ctx *ctx, size_t bytes, cudaStream_t stream, bool cap, PlanBuf **out) {
  PlanBuf &pb = ctx->plans[ctx->next_plan];
  ctx->next_plan = (ctx->next_plan + 1) % kPlanRing;
  if (pb.used && !cap) {
    cudaEventSynchronize(pb.copied);
    if (pb.stream != stream) cudaStreamWaitEvent(stream, pb.done, 0);
  }
  if (pb.d_cap < bytes || pb.h_cap < bytes) {
    if (cap) return GST_E_ARG;  // buffers cannot be reallocated during stream capture
    if (pb.used) cudaEventSynchronize(pb.done);
    gst_status st = grow_device(&pb.d, &pb.d_cap, bytes);
    if (st != GST_OK) return st;
    st = grow_pinned(&pb.h, &pb.h_cap, bytes);
    if (st != GST_OK) return st;
  }
  *out = &pb;
  return GST_OK;
}

// Makes ctx->scratch at least `bytes` and orders its use on `stream` after
// the previous call that used it.
gst_status acquire_scratch(gst_ctx *ctx, size_t bytes, cudaStream_t stream, bool cap) {
  if (ctx->scratch_used && !cap && ctx->scratch_stream != stream) cudaStreamWaitEvent(stream, ctx->scratch_done, 0);
  if (ctx->scratch_cap >= bytes) return GST_OK;
  if (ctx->preallocated) return GST_E_OOM;
  if (cap) return GST_E_ARG;
  if (ctx->scratch_used) cudaEventSynchronize(ctx->scratch_done);
  return grow_device(&ctx->scratch, &ctx->scratch_cap, bytes);
}

// Uploads the plan staged in pb->h (plan_bytes) and launches the kernels on
// `view`, whose pointers lie in pb->d.
gst_status upload_and_launch(gst_ctx *ctx, PlanBuf *pb, size_t plan_bytes, const GstPlanView &view,
                             const uint8_t *d_cmp, uint8_t *d_scratch, uint8_t *d_out, cudaStream_t stream,
                             bool cap, const GstTuning &tuning) {
  cudaError_t e = cudaMemcpyAsync(pb->d, pb->h, plan_bytes, cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return cuda_status(e);
  if (!cap) cudaEventRecord(pb->copied, stream);
  cudaEvent_t *ev = (ctx->profiling && !cap) ? ctx->ev : nullptr;
  GstPlanView v = view;
  v.wait_limit_ns = ctx->wait_limit_ns;
  if (ctx->inject_drop_rans && tuning.persistent && v.sync) v.n_rans = 0;
  e = launch_decode(d_cmp, d_scratch, d_out, v, stream, &ctx->last_launches, ev, tuning, ctx->timed_names);
  ctx->timed_kernels = ev ? ctx->last_launches : 0;
  if (e != cudaSuccess) return cuda_status(e);
  if (!cap) {
    cudaEventRecord(pb->done, stream);
    pb->stream = stream;
    pb->used = true;
  }
  return GST_OK;
}

uint64_t total_blocks(const gst_header *hdrs, int n) {
  uint64_t b = 0;
  for (int i = 0; i < n; ++i) b += image_blocks(hdrs[i]);
  return b;
}

PlanLayout plan_layout(const gst_header *hdrs, int n, uint32_t capacity) {
  PlanLayout L;
  L.lay.resize(n);
  L.scratch_bytes = 0;
  L.n_rans = L.n_tiles = 0;
  L.items.assign(4 * size_t(n), 0);
  std::vector<uint32_t> groups(4 * size_t(n));
  uint64_t total_groups = 0, min_items = 0;
  for (int i = 0; i < n; ++i) {
    L.lay[i] = scratch_layout(hdrs[i]);
    L.scratch_bytes += L.lay[i].total;
    const uint64_t B = image_blocks(hdrs[i]);
    const uint64_t g[4] = {2 * B / kSymsPerGroup, 4 * B / kSymsPerGroup, hdrs[i].palette_bytes / kSymsPerGroup,
                           B / kSymsPerGroup};
    for (int s = 0; s < 4; ++s) {
      groups[4 * size_t(i) + s] = uint32_t(g[s]);
      L.items[4 * size_t(i) + s] = uint32_t((g[s] + kGroupsPerRansCta - 1) / kGroupsPerRansCta);
      total_groups += g[s];
      min_items += L.items[4 * size_t(i) + s];
    }
    L.n_tiles += uint32_t(B / 1024);
  }
  // Runs of 4 groups leave the last SMs of a one-wave launch with a CTA more
  // than the others (1083 CTAs of a 8192x8192 texture on 8 x 152 places:
  // 19 SMs hold 8 CTAs, the rest 7, and those 19 end the kernel several
  // microseconds late).  Where the work fills the wave with items of 3.5
  // groups or more, cut the sections into exactly `capacity` items instead:
  // one more item at a time to the section whose items are largest on
  // average.  (Smaller items cost more than the balance gains: the 64-image
  // batch at 3.2 groups an item measured slower.)
  if (capacity > 0 && min_items < capacity && 2 * total_groups >= 7 * uint64_t(capacity)) {
    // Max-heap of sections by average item size: section a ranks below b
    // when G_a / k_a < G_b / k_b.
    auto below = [&](size_t a, size_t b) {
      return uint64_t(groups[a]) * L.items[b] < uint64_t(groups[b]) * L.items[a];
    };
    std::vector<size_t> heap;
    for (size_t k = 0; k < groups.size(); ++k)
      if (groups[k] > L.items[k]) heap.push_back(k);
    std::make_heap(heap.begin(), heap.end(), below);
    for (uint64_t extra = capacity - min_items; extra > 0 && !heap.empty(); --extra) {
      std::pop_heap(heap.begin(), heap.end(), below);
      const size_t k = heap.back();
      ++L.items[k];
      if (groups[k] > L.items[k]) std::push_heap(heap.begin(), heap.end(), below);
      else heap.pop_back();
    }
    L.balanced = true;
  }
  for (uint32_t k : L.items) L.n_rans += k;
  L.off_images = align_up(sizeof(GstPlanHead), 128);
  L.off_rans = L.off_images + sizeof(GstImageDesc) * n;
  L.off_tiles = align_up(L.off_rans + sizeof(GstRansItem) * L.n_rans, 16);
  L.off_order = align_up(L.off_tiles + sizeof(GstTileItem) * L.n_tiles, 16);
  L.off_counters = align_up(L.off_order + 4 * size_t(L.n_rans), 16);
  L.off_image_err = L.off_counters + 4 * size_t(n);
  L.off_sync = align_up(L.off_image_err + 4 * size_t(n), 16);
  L.bytes = align_up(L.off_sync + 16 + 4 * size_t(n), 16);
  L.n_images = n;
  return L;
}

// Writes the plan (L.bytes) for n images whose compressed data sit in the
// reference's layout: codec/decoder.cpp:132-149 and demo/photos_sf.cpp:753-791
// (offsets page, then 4n frequency tables, then each image's four sections),
// and whose DXT1 blocks go back to back.  With freq_at / body_at, image i's
// four frequency tables and first section are instead at those device
// addresses, and with out_at its blocks go to device address out_at[i]; the
// kernels then get null compressed and output bases.
void write_plan(const PlanLayout &L, const gst_header *hdrs, int n, uint8_t *ph, const uint64_t *freq_at,
                const uint64_t *body_at, const uint64_t *out_at, uint32_t out_block_bytes) {
  memset(ph, 0, L.bytes);
  GstPlanHead *head = reinterpret_cast<GstPlanHead *>(ph);
  head->n_images = uint32_t(n);
  head->n_rans = L.n_rans;
  head->n_tiles = L.n_tiles;
  GstImageDesc *imgs = reinterpret_cast<GstImageDesc *>(ph + L.off_images);
  GstRansItem *rans = reinterpret_cast<GstRansItem *>(ph + L.off_rans);
  GstTileItem *tiles = reinterpret_cast<GstTileItem *>(ph + L.off_tiles);
  const size_t page = offsets_page_bytes(n);
  uint64_t body = page + size_t(n) * 4 * kFreqTableBytes;
  uint64_t scratch_off = 0, out_off = 0;
  uint32_t ri = 0, ti = 0;
  struct SectionItems {
    uint64_t cost;  // compressed bytes per group (x16)
    uint32_t first, count;
  };
  std::vector<SectionItems> by_section;
  by_section.reserve(4 * size_t(n));
  for (int i = 0; i < n; ++i) {
    const gst_header &h = hdrs[i];
    GstImageDesc &d = imgs[i];
    const uint32_t B = uint32_t(image_blocks(h));
    d.freq_off = freq_at ? freq_at[i] : page + size_t(i) * 4 * kFreqTableBytes;
    d.body_off = body_at ? body_at[i] : body;
    d.sym_off = scratch_off + L.lay[i].sym;
    d.chunk_off = scratch_off + L.lay[i].chunk;
    d.gsum_off = scratch_off + L.lay[i].gsum;
    d.out_off = out_at ? out_at[i] : out_off;
    const uint32_t lens[4] = {h.y_cmp_sz, h.chroma_cmp_sz, h.palette_sz, h.indices_sz};
    const uint32_t syms[4] = {2 * B, 4 * B, h.palette_bytes, B};
    uint32_t in = 0, o = 0;
    for (int s = 0; s < 4; ++s) {
      d.sec_in[s] = in;
      d.sec_len[s] = lens[s];
      d.sec_groups[s] = syms[s] / kSymsPerGroup;
      d.sec_out[s] = o;
      in += lens[s];
      o += syms[s];
      by_section.push_back({uint64_t(lens[s]) * 16 / std::max<uint32_t>(1u, d.sec_groups[s]), ri, 0});
      // L.items[4 i + s] items of near-equal size (runs of 4 groups and a
      // shorter last one when the layout is not balanced).
      const uint32_t G = d.sec_groups[s], k = L.items[4 * size_t(i) + s];
      for (uint32_t j = 0, g = 0; j < k; ++j) {
        const uint32_t m = L.balanced ? G / k + (j < G % k ? 1u : 0u) : std::min(kGroupsPerRansCta, G - g);
        rans[ri++] = {uint32_t(i), uint32_t(s), g, uint16_t(m), uint16_t(kStreamsPerGroup)};
        g += m;
      }
      by_section.back().count = ri - by_section.back().first;
    }
    d.bx = h.width / 4;
    d.by = h.height / 4;
    d.palette_words = h.palette_bytes / 4;
    d.tiles_x = d.bx / kWaveletDim;
    for (uint32_t t = 0; t < B / 1024; ++t) tiles[ti++] = {uint32_t(i), t};
    body += section_bytes(h);
    scratch_off += L.lay[i].total;
    out_off += uint64_t(out_block_bytes) * B;
  }
  // The rANS kernel's launch order, longest first: items of sections with more
  // compressed bytes per group (more renormalisation words, more re-staging)
  // start first, so that the launch does not end on a few long items.  (The
  // persistent kernel keeps image order, so that images finish one after
  // another and their tiles can start early.)
  // The cost is a section's, so sorting the sections (stably) and emitting
  // each one's items in turn gives the items' stable order by cost.
  uint32_t *order = reinterpret_cast<uint32_t *>(ph + L.off_order);
  std::stable_sort(by_section.begin(), by_section.end(),
                   [](const SectionItems &a, const SectionItems &b) { return a.cost > b.cost; });
  uint32_t k = 0;
  for (const SectionItems &sec : by_section)
    for (uint32_t j = 0; j < sec.count; ++j) order[k++] = sec.first + j;
  // Balanced items: the larger first (by cost within a size), so that the
  // launch's rounds of CTAs over the SMs deal every SM the same mix.
  if (L.balanced)
    std::stable_sort(order, order + k, [&](uint32_t a, uint32_t b) { return rans[a].ngroups > rans[b].ngroups; });
}

GstPlanView plan_view(const PlanLayout &L, uint8_t *plan_d, uint32_t *status_d) {
  GstPlanView view = {};  // every field: wait_limit_ns 0 is the kernel's default bound
  view.err = status_d;
  view.images = reinterpret_cast<const GstImageDesc *>(plan_d + L.off_images);
  view.rans = reinterpret_cast<const GstRansItem *>(plan_d + L.off_rans);
  view.tiles = L.n_tiles ? reinterpret_cast<const GstTileItem *>(plan_d + L.off_tiles) : nullptr;
  view.counters = reinterpret_cast<uint32_t *>(plan_d + L.off_counters);
  view.image_err = reinterpret_cast<uint32_t *>(plan_d + L.off_image_err);
  view.rans_order = reinterpret_cast<const uint32_t *>(plan_d + L.off_order);
  view.sync = reinterpret_cast<uint32_t *>(plan_d + L.off_sync);
  view.n_images = uint32_t(L.n_images);
  view.rgb = 0;
  view.n_rans = L.n_rans;
  view.n_tiles = L.n_tiles;
  return view;
}

// Builds the plan for n images whose compressed data sit in the reference's
// layout at d_cmp, uploads it through the plan ring and launches.  hdrs have
// passed check_header.
gst_status decode_batch(gst_ctx *ctx, const gst_header *hdrs, int n, const uint8_t *d_cmp, uint8_t *d_out,
                        cudaStream_t stream, bool rgb = false) {
  const bool cap = capturing(stream);
  const GstTuning tuning = launch_tuning_locked(ctx, hdrs, n);
  const PlanLayout L = plan_layout(hdrs, n, plan_capacity(ctx, tuning));
  gst_status st = acquire_scratch(ctx, L.scratch_bytes, stream, cap);
  if (st != GST_OK) return st;
  PlanBuf *pb = nullptr;
  st = acquire_plan(ctx, L.bytes, stream, cap, &pb);
  if (st != GST_OK) return st;
  write_plan(L, hdrs, n, pb->h, nullptr, nullptr, nullptr, rgb ? 48 : 8);
  GstPlanView view = plan_view(L, pb->d, ctx->status_d);
  view.image_err = nullptr;  // the context reports per call
  view.rgb = rgb ? 1 : 0;
  st = upload_and_launch(ctx, pb, L.bytes, view, d_cmp, ctx->scratch, d_out, stream, cap, tuning);
  if (st != GST_OK) return st;
  if (!cap) {
    cudaEventRecord(ctx->scratch_done, stream);
    ctx->scratch_stream = stream;
    ctx->scratch_used = true;
  }
  return GST_OK;
}

// Chunk boundaries of a pipelined host-to-host decode: contiguous runs of
// images whose block counts rise as 1, 2, 4, ... and fall again towards the
// end (..., 4, 2, 1).  The copies out are the slowest stage (the decode runs
// ~2.4x faster than the device-to-host link), so a small first chunk starts
// them early, every later chunk is decoded while the copies out before it
// run, and a small last chunk leaves little to copy after the last decode.
std::vector<int> chunk_cuts(const gst_header *hdrs, int n, int chunks, uint64_t blocks) {
  std::vector<double> bound(chunks);  // cumulative fraction of the blocks at the end of chunk k
  double wsum = 0;
  auto weight = [&](int k) { return 1u << std::min(k, chunks - 1 - k); };
  for (int k = 0; k < chunks; ++k) wsum += double(weight(k));
  for (int k = 0, acc_w = 0; k < chunks; ++k) {
    acc_w += int(weight(k));
    bound[k] = double(acc_w) / wsum;
  }
  std::vector<int> cut(1, 0);
  uint64_t acc = 0;
  for (int i = 0; i < n; ++i) {
    acc += image_blocks(hdrs[i]);
    const int k = int(cut.size()) - 1;  // the chunk image i belongs to
    const int left_images = n - (i + 1), left_chunks = chunks - int(cut.size());
    if (left_chunks > 0 && left_images >= left_chunks &&
        (double(acc) >= bound[k] * double(blocks) || left_images == left_chunks))
      cut.push_back(i + 1);
  }
  cut.push_back(n);
  return cut;
}

gst_status read_device_status(gst_ctx *ctx, cudaStream_t stream) {
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_status(e);
  uint32_t bits = 0;
  e = cudaMemcpy(&bits, ctx->status_d, sizeof(bits), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  if (bits) {
    e = cudaMemset(ctx->status_d, 0, sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_status(e);
    return (bits & kErrTimeout) ? GST_E_TIMEOUT : GST_E_FORMAT;
  }
  return GST_OK;
}

}  // namespace host
}  // namespace gst

namespace gst {
namespace host {
int ctx_device(const gst_ctx *ctx) { return ctx->device; }
std::mutex &ctx_mutex(gst_ctx *ctx) { return ctx->mu; }
EncodeState *&ctx_encode_state(gst_ctx *ctx) { return ctx->enc; }
uint32_t *ctx_status(gst_ctx *ctx) { return ctx->status_d; }
uint64_t ctx_wait_limit_ns(gst_ctx *ctx) { return ctx->wait_limit_ns; }
cudaEvent_t *ctx_timing_events(gst_ctx *ctx, bool capturing) {
  return (ctx->profiling && !capturing) ? ctx->ev : nullptr;
}
void ctx_set_timed(gst_ctx *ctx, int kernels, int launches) {
  ctx->timed_kernels = kernels;
  ctx->last_launches = launches;
}
const char **ctx_timed_names(gst_ctx *ctx) { return ctx->timed_names; }
bool ctx_enc_hist_match(gst_ctx *ctx) { return ctx->enc_hist_match; }
uint32_t plan_capacity(const gst_ctx *ctx, const GstTuning &t) {
  return ctx->balance_items ? rans_wave_capacity(t) : 0;
}
bool ctx_inject_encode_stall(gst_ctx *ctx) { return ctx->inject_encode_stall; }
GstTuning ctx_tuning(gst_ctx *ctx) {
  std::lock_guard<std::mutex> lock(ctx->mu);
  return ctx->tuning;
}
GstTuning ctx_tuning_for(gst_ctx *ctx, const gst_header *hdrs, int n) {
  std::lock_guard<std::mutex> lock(ctx->mu);
  return launch_tuning_locked(ctx, hdrs, n);
}
}  // namespace host
}  // namespace gst

// A resident batch: its plan is uploaded once and it owns its scratch, so a
// launch enqueues kernels only (and can be captured in a CUDA graph).
struct gst_batch {
  gst_ctx *ctx = nullptr;
  PlanLayout layout;
  size_t compressed_bytes = 0;
  size_t out_bytes = 0;
  uint8_t *plan_d = nullptr;
  uint8_t *scratch = nullptr;
  bool tuned = false;  // tuning set by gst_batch_autotune / gst_batch_set_tuning
  GstTuning tuning;
  uint32_t plan_cap = 0;       // the one-wave capacity the plan's rANS items were cut for
  size_t plan_alloc = 0;       // bytes allocated at plan_d
  cudaGraphExec_t graph = nullptr;
  const void *graph_cmp = nullptr;
  void *graph_out = nullptr;
  GstTuning graph_tuning;
  std::vector<gst_header> hdrs;
  // Host-buffer launches (gst_batch_host_launch): device mirrors of the
  // caller's pinned input and output, per-chunk plans uploaded once, and the
  // captured pipeline per (input, output, chunks, tuning).
  uint8_t *hm_cmp = nullptr, *hm_out = nullptr;
  uint8_t *hm_plans = nullptr;
  int hm_chunks = 0;
  std::vector<int> hm_cut;
  std::vector<PlanLayout> hm_lay;
  std::vector<size_t> hm_plan_off;
  std::vector<GstTuning> hm_tun;  // each chunk's launch configuration (the plans are cut for it)
  std::vector<size_t> hm_scr_off;  // chunk c's scratch: b->scratch + hm_scr_off[c], disjoint per chunk
  cudaStream_t hm_stream[4] = {};  // copy in, decode (even chunks), copy out, decode (odd chunks)
  cudaGraphExec_t hm_graph = nullptr;
  const void *hm_graph_cmp = nullptr;
  void *hm_graph_out = nullptr;
  GstTuning hm_graph_tuning;
};

namespace {

GstTuning batch_tuning(const gst_batch *b) {
  return b->tuned ? b->tuning : launch_tuning_locked(b->ctx, b->hdrs.data(), int(b->hdrs.size()));
}

bool valid_tuning(int blocks_per_sm, int stage_words, int persistent = 0) {
  return blocks_per_sm >= 1 && blocks_per_sm <= 16 && stage_words >= int(kMinStageWords) &&
         stage_words <= int(kMaxStageWords) && (stage_words & 7) == 0 && (persistent == 0 || persistent == 1);
}

// Re-cuts the batch's rANS items for the one-wave capacity of tuning `t` when
// that differs from the one the plan was cut for (any cut decodes correctly;
// a balanced one is faster).  Waits for the device first, since earlier
// launches may still read the plan, and drops the captured graph (its rANS
// grid has the old item count).  The caller holds ctx->mu.
cudaError_t ensure_plan_locked(gst_batch *b, const GstTuning &t) {
  const uint32_t cap = plan_capacity(b->ctx, t);
  if (cap == b->plan_cap) return cudaSuccess;
  const int n = int(b->hdrs.size());
  PlanLayout L = plan_layout(b->hdrs.data(), n, cap);
  b->plan_cap = cap;
  if (L.balanced == b->layout.balanced && L.items == b->layout.items) return cudaSuccess;  // the same cut
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess && L.bytes > b->plan_alloc) {
    cudaFree(b->plan_d);
    b->plan_d = nullptr;
    b->plan_alloc = 0;
    e = cudaMalloc(reinterpret_cast<void **>(&b->plan_d), L.bytes);
    if (e == cudaSuccess) b->plan_alloc = L.bytes;
  }
  if (e != cudaSuccess) {
    b->plan_cap = ~0u;  // retried on the next launch
    return e;
  }
  std::vector<uint8_t> plan(L.bytes);
  write_plan(L, b->hdrs.data(), n, plan.data(), nullptr, nullptr, nullptr);
  e = cudaMemcpy(b->plan_d, plan.data(), L.bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    b->plan_cap = ~0u;
    return e;
  }
  b->layout = std::move(L);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  return cudaSuccess;
}

// Launches the batch's kernels under `t`; the caller holds ctx->mu.  Outside
// stream capture the plan is first re-cut for `t` where that pays.
cudaError_t batch_launch_locked(gst_batch *b, const void *d_cmp, void *d_out, cudaStream_t st, const GstTuning &t,
                                cudaEvent_t *ev) {
  gst_ctx *ctx = b->ctx;
  if (!capturing(st)) {
    const cudaError_t e = ensure_plan_locked(b, t);
    if (e != cudaSuccess) return e;
  }
  GstPlanView view = plan_view(b->layout, b->plan_d, ctx->status_d);
  view.wait_limit_ns = ctx->wait_limit_ns;
  return launch_decode(static_cast<const uint8_t *>(d_cmp), b->scratch, static_cast<uint8_t *>(d_out), view, st,
                       &ctx->last_launches, ev, t, ctx->timed_names);
}

}  // namespace

extern "C" {

const char *gst_status_string(gst_status s) {
  switch (s) {
    case GST_OK: return "ok";
    case GST_E_ARG: return "bad argument";
    case GST_E_FORMAT: return "malformed GST stream";
    case GST_E_OOM: return "out of memory";
    case GST_E_CUDA: return "CUDA error";
    case GST_E_TIMEOUT: return "device wait timed out";
  }
  return "unknown status";
}

gst_status gst_init(int device, gst_ctx **out) {
  if (!out) return GST_E_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return GST_E_CUDA;
  if (device < 0 || device >= count) return GST_E_ARG;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_status(e);
  gst_ctx *ctx = new gst_ctx();
  ctx->device = device;
  bool ok = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&ctx->scratch_done, cudaEventDisableTiming) == cudaSuccess &&
            cudaMalloc(reinterpret_cast<void **>(&ctx->status_d), sizeof(uint32_t)) == cudaSuccess &&
            cudaMemset(ctx->status_d, 0, sizeof(uint32_t)) == cudaSuccess;
  for (auto &pb : ctx->plans) {
    ok = ok && cudaEventCreateWithFlags(&pb.copied, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&pb.done, cudaEventDisableTiming) == cudaSuccess;
  }
  if (!ok) {
    gst_destroy(ctx);
    return GST_E_CUDA;
  }
  // A persisted per-size-class table, where one is named and matches this
  // device; a missing or foreign table leaves the built-in configuration.
  const char *table = std::getenv("GST_TUNING_TABLE");
  if (table && *table) gst_load_class_tuning(ctx, table);
  *out = ctx;
  return GST_OK;
}

void gst_destroy(gst_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  gst::host::destroy_encode_state(ctx->enc);
  cudaFree(ctx->scratch);
  cudaFree(ctx->status_d);
  for (auto &pb : ctx->plans) {
    cudaFree(pb.d);
    cudaFreeHost(pb.h);
    if (pb.copied) cudaEventDestroy(pb.copied);
    if (pb.done) cudaEventDestroy(pb.done);
  }
  cudaFree(ctx->cmp_d);
  cudaFree(ctx->out_d);
  cudaFreeHost(ctx->cmp_h);
  cudaFreeHost(ctx->out_h);
  if (ctx->scratch_done) cudaEventDestroy(ctx->scratch_done);
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  cudaFree(ctx->hs_cmp_d);
  cudaFree(ctx->hs_out_d);
  for (cudaStream_t s : {ctx->hs_in, ctx->hs_comp, ctx->hs_out})
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : {ctx->hs_start, ctx->hs_done})
    if (e) cudaEventDestroy(e);
  for (int k = 0; k < kPlanRing; ++k) {
    if (ctx->hs_copied[k]) cudaEventDestroy(ctx->hs_copied[k]);
    if (ctx->hs_decoded[k]) cudaEventDestroy(ctx->hs_decoded[k]);
  }
  delete ctx;
}

gst_status gst_initialize_decoder(gst_ctx *ctx) {
  if (!ctx) return GST_E_ARG;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, ctx->device);
  if (e != cudaSuccess) return cuda_status(e);
  if (prop.major * 10 + prop.minor < 100) return GST_E_CUDA;
  if (prop.sharedMemPerBlock < 48 * 1024) return GST_E_CUDA;
  return GST_OK;
}

gst_status gst_parse_header(const uint8_t *gst, size_t len, gst_header *hdr) {
  if (!gst || !hdr) return GST_E_ARG;
  if (len < 28 + 4 * kFreqTableBytes) return GST_E_FORMAT;
  uint32_t *w = reinterpret_cast<uint32_t *>(hdr);
  for (int i = 0; i < 7; ++i) w[i] = rd32(gst + 4 * i);
  gst_status st = check_header(*hdr);
  if (st != GST_OK) return st;
  if (28 + 4 * kFreqTableBytes + section_bytes(*hdr) > len) return GST_E_FORMAT;
  const uint8_t *freqs = gst + 28;
  const uint8_t *body = freqs + 4 * kFreqTableBytes;
  const uint64_t B = image_blocks(*hdr);
  const uint32_t lens[4] = {hdr->y_cmp_sz, hdr->chroma_cmp_sz, hdr->palette_sz, hdr->indices_sz};
  const uint64_t syms[4] = {2 * B, 4 * B, hdr->palette_bytes, B};
  for (int s = 0; s < 4; ++s) {
    uint32_t sum = 0;
    for (int k = 0; k < 256; ++k) sum += uint32_t(freqs[s * 512 + 2 * k]) | (uint32_t(freqs[s * 512 + 2 * k + 1]) << 8);
    if (sum != kTableSize) return GST_E_FORMAT;
    const uint32_t G = uint32_t(syms[s] / kSymsPerGroup);
    uint32_t prev = 4 * G;
    for (uint32_t g = 0; g < G; ++g) {
      const uint32_t e = rd32(body + 4 * g);
      if (e % 4 || e < prev + 4 * kStreamsPerGroup || e > lens[s]) return GST_E_FORMAT;
      prev = e;
    }
    body += lens[s];
  }
  return GST_OK;
}

size_t gst_required_scratch(const gst_header *hdr) {
  if (!hdr || check_header(*hdr) != GST_OK) return 0;
  return scratch_layout(*hdr).total;
}

gst_status gst_preallocate(gst_ctx *ctx, size_t bytes) {
  if (!ctx) return GST_E_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  if (ctx->scratch_used) cudaEventSynchronize(ctx->scratch_done);
  cudaFree(ctx->scratch);
  ctx->scratch = nullptr;
  ctx->scratch_cap = 0;
  const size_t sz = std::max<size_t>(bytes, 256);
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&ctx->scratch), sz);
  if (e != cudaSuccess) {
    ctx->scratch = nullptr;
    return cuda_status(e);
  }
  ctx->scratch_cap = sz;
  ctx->preallocated = true;
  return GST_OK;
}

gst_status gst_free_decompressor(gst_ctx *ctx) {
  if (!ctx) return GST_E_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  if (ctx->scratch_used) cudaEventSynchronize(ctx->scratch_done);
  cudaFree(ctx->scratch);
  ctx->scratch = nullptr;
  ctx->scratch_cap = 0;
  ctx->preallocated = false;
  return GST_OK;
}

size_t gst_batch_layout_bytes(const gst_header *hdrs, int n) {
  if (!hdrs || n <= 0) return 0;
  size_t total = offsets_page_bytes(n) + size_t(n) * 4 * kFreqTableBytes;
  for (int i = 0; i < n; ++i) total += section_bytes(hdrs[i]);
  return total;
}

gst_status gst_pack_batch(const uint8_t *const *gst, const size_t *len, int n, uint8_t *dst, size_t dst_cap) {
  if (!gst || !len || !dst || n <= 0) return GST_E_ARG;
  std::vector<gst_header> hdrs(n);
  for (int i = 0; i < n; ++i) {
    gst_status st = gst_parse_header(gst[i], len[i], &hdrs[i]);
    if (st != GST_OK) return st;
  }
  const size_t need = gst_batch_layout_bytes(hdrs.data(), n);
  if (dst_cap < need) return GST_E_ARG;
  memset(dst, 0, offsets_page_bytes(n));
  uint32_t *out_offsets = reinterpret_cast<uint32_t *>(dst);
  uint32_t *in_offsets = out_offsets + 4 * n;
  uint8_t *freqs = dst + offsets_page_bytes(n);
  uint8_t *body = freqs + size_t(n) * 4 * kFreqTableBytes;
  uint32_t in = 0, out = 0;
  for (int i = 0; i < n; ++i) {
    const gst_header &h = hdrs[i];
    const uint32_t B = uint32_t(image_blocks(h));
    const uint32_t lens[4] = {h.y_cmp_sz, h.chroma_cmp_sz, h.palette_sz, h.indices_sz};
    const uint32_t syms[4] = {2 * B, 4 * B, h.palette_bytes, B};
    for (int s = 0; s < 4; ++s) {
      out_offsets[4 * i + s] = out;
      in_offsets[4 * i + s] = in;
      out += syms[s];
      in += lens[s];
    }
    memcpy(freqs + size_t(i) * 4 * kFreqTableBytes, gst[i] + 28, 4 * kFreqTableBytes);
    const size_t sb = section_bytes(h);
    memcpy(body, gst[i] + 28 + 4 * kFreqTableBytes, sb);
    body += sb;
  }
  return GST_OK;
}

gst_status gst_load_compressed_dxts(gst_ctx *ctx, const gst_header *hdrs, int n, const void *d_cmp, void *d_out,
                                    void *stream) {
  if (!ctx || !hdrs || n <= 0 || !d_cmp || !d_out) return GST_E_ARG;
  if ((reinterpret_cast<uintptr_t>(d_cmp) & 15) || (reinterpret_cast<uintptr_t>(d_out) & 7)) return GST_E_ARG;
  for (int i = 0; i < n; ++i) {
    gst_status st = check_header(hdrs[i]);
    if (st != GST_OK) return st;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  return decode_batch(ctx, hdrs, n, static_cast<const uint8_t *>(d_cmp), static_cast<uint8_t *>(d_out),
                      static_cast<cudaStream_t>(stream));
}

gst_status gst_load_compressed_dxt(gst_ctx *ctx, const gst_header *hdr, const void *d_cmp, void *d_out,
                                   void *stream) {
  return gst_load_compressed_dxts(ctx, hdr, 1, d_cmp, d_out, stream);
}

gst_status gst_load_rgbs(gst_ctx *ctx, const gst_header *hdrs, int n, const void *d_cmp, void *d_out, void *stream) {
  if (!ctx || !hdrs || n <= 0 || !d_cmp || !d_out) return GST_E_ARG;
  if ((reinterpret_cast<uintptr_t>(d_cmp) & 15) || (reinterpret_cast<uintptr_t>(d_out) & 3)) return GST_E_ARG;
  for (int i = 0; i < n; ++i) {
    gst_status st = check_header(hdrs[i]);
    if (st != GST_OK) return st;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  return decode_batch(ctx, hdrs, n, static_cast<const uint8_t *>(d_cmp), static_cast<uint8_t *>(d_out),
                      static_cast<cudaStream_t>(stream), true);
}

gst_status gst_load_rgb(gst_ctx *ctx, const gst_header *hdr, const void *d_cmp, void *d_out, void *stream) {
  return gst_load_rgbs(ctx, hdr, 1, d_cmp, d_out, stream);
}

gst_status gst_load_host_dxts(gst_ctx *ctx, const gst_header *hdrs, int n, const void *h_cmp, void *h_out,
                              int chunks, void *stream) {
  if (!ctx || !hdrs || n <= 0 || !h_cmp || !h_out || chunks < 0) return GST_E_ARG;
  for (int i = 0; i < n; ++i) {
    gst_status st = check_header(hdrs[i]);
    if (st != GST_OK) return st;
  }
  if (chunks == 0) chunks = std::min(n, 8);
  chunks = std::min(std::min(chunks, n), kPlanRing);
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t caller = static_cast<cudaStream_t>(stream);
  if (capturing(caller)) return GST_E_ARG;  // host memory paths are not captured
  if (!ctx->hs_in) {
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->hs_in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->hs_comp, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->hs_out, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->hs_start, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->hs_done, cudaEventDisableTiming);
    for (int k = 0; k < kPlanRing && e == cudaSuccess; ++k) {
      e = cudaEventCreateWithFlags(&ctx->hs_copied[k], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->hs_decoded[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return cuda_status(e);
  }
  // Where each image's tables, sections and blocks are (the reference's
  // layout, codec/decoder.cpp:430-476), and the chunk boundaries.
  const size_t page = offsets_page_bytes(n);
  std::vector<uint64_t> body(n + 1), out(n + 1);
  body[0] = page + size_t(n) * 4 * kFreqTableBytes;
  out[0] = 0;
  uint64_t blocks = 0;
  for (int i = 0; i < n; ++i) {
    body[i + 1] = body[i] + section_bytes(hdrs[i]);
    out[i + 1] = out[i] + 8 * image_blocks(hdrs[i]);
    blocks += image_blocks(hdrs[i]);
  }
  const std::vector<int> cut = chunk_cuts(hdrs, n, chunks, blocks);
  const int nc = int(cut.size()) - 1;
  gst_status st = grow_device(&ctx->hs_cmp_d, &ctx->hs_cmp_cap, body[n]);
  if (st == GST_OK) st = grow_device(&ctx->hs_out_d, &ctx->hs_out_cap, out[n]);
  if (st != GST_OK) return st;
  size_t scratch = 0;
  std::vector<PlanLayout> lay(nc);
  for (int c = 0; c < nc; ++c) {
    const int m = cut[c + 1] - cut[c];
    const uint32_t cap = plan_capacity(ctx, launch_tuning_locked(ctx, hdrs + cut[c], m));
    lay[c] = plan_layout(hdrs + cut[c], m, cap);
    scratch = std::max(scratch, lay[c].scratch_bytes);
  }
  // A previous call's copies out of the mirrors must be done before this
  // call overwrites them.
  cudaEventRecord(ctx->hs_start, caller);
  cudaStreamWaitEvent(ctx->hs_in, ctx->hs_start, 0);
  if (ctx->hs_used) cudaStreamWaitEvent(ctx->hs_in, ctx->hs_done, 0);
  cudaStreamWaitEvent(ctx->hs_comp, ctx->hs_start, 0);
  cudaStreamWaitEvent(ctx->hs_out, ctx->hs_start, 0);
  st = acquire_scratch(ctx, scratch, ctx->hs_comp, false);
  if (st != GST_OK) return st;
  const uint8_t *hc = static_cast<const uint8_t *>(h_cmp);
  uint8_t *ho = static_cast<uint8_t *>(h_out);
  cudaError_t e = cudaSuccess;
  // The three passes are enqueued one after another (every copy in, then every
  // decode, then every copy out) so that copies sharing a copy engine queue in
  // the order they can run: a copy out never holds up a later copy in, and
  // each chunk's plan travels with its data instead of behind later chunks.
  // 1. Copy in each chunk's tables, sections (two contiguous ranges) and plan.
  PlanBuf *pbs[kPlanRing] = {};
  nvtxRangePushA("gst copy in");
  for (int c = 0; c < nc && e == cudaSuccess; ++c) {
    const int i0 = cut[c], i1 = cut[c + 1], m = i1 - i0;
    const size_t t0 = page + size_t(i0) * 4 * kFreqTableBytes, t1 = page + size_t(i1) * 4 * kFreqTableBytes;
    e = cudaMemcpyAsync(ctx->hs_cmp_d + t0, hc + t0, t1 - t0, cudaMemcpyHostToDevice, ctx->hs_in);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ctx->hs_cmp_d + body[i0], hc + body[i0], body[i1] - body[i0], cudaMemcpyHostToDevice,
                          ctx->hs_in);
    if (e != cudaSuccess) break;
    std::vector<uint64_t> fa(m), ba(m), oa(m);
    for (int k = 0; k < m; ++k) {
      fa[k] = reinterpret_cast<uint64_t>(ctx->hs_cmp_d + page + size_t(i0 + k) * 4 * kFreqTableBytes);
      ba[k] = reinterpret_cast<uint64_t>(ctx->hs_cmp_d + body[i0 + k]);
      oa[k] = reinterpret_cast<uint64_t>(ctx->hs_out_d + out[i0 + k]);
    }
    st = acquire_plan(ctx, lay[c].bytes, ctx->hs_in, false, &pbs[c]);
    if (st != GST_OK) {
      nvtxRangePop();
      return st;
    }
    write_plan(lay[c], hdrs + i0, m, pbs[c]->h, fa.data(), ba.data(), oa.data());
    e = cudaMemcpyAsync(pbs[c]->d, pbs[c]->h, lay[c].bytes, cudaMemcpyHostToDevice, ctx->hs_in);
    if (e == cudaSuccess) e = cudaEventRecord(pbs[c]->copied, ctx->hs_in);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->hs_copied[c], ctx->hs_in);
  }
  nvtxRangePop();
  // 2. Decode each chunk once it is in.
  nvtxRangePushA("gst decode");
  for (int c = 0; c < nc && e == cudaSuccess; ++c) {
    e = cudaStreamWaitEvent(ctx->hs_comp, ctx->hs_copied[c], 0);
    if (e != cudaSuccess) break;
    GstPlanView view = plan_view(lay[c], pbs[c]->d, ctx->status_d);
    view.image_err = nullptr;
    e = launch_decode(nullptr, ctx->scratch, nullptr, view, ctx->hs_comp, &ctx->last_launches, nullptr,
                      launch_tuning_locked(ctx, hdrs + cut[c], cut[c + 1] - cut[c]),
                      ctx->timed_names);
    if (e == cudaSuccess) e = cudaEventRecord(pbs[c]->done, ctx->hs_comp);
    pbs[c]->stream = ctx->hs_comp;
    pbs[c]->used = true;
    if (e == cudaSuccess) e = cudaEventRecord(ctx->hs_decoded[c], ctx->hs_comp);
  }
  nvtxRangePop();
  // 3. Copy each chunk's blocks out once decoded.
  nvtxRangePushA("gst copy out");
  for (int c = 0; c < nc && e == cudaSuccess; ++c) {
    const int i0 = cut[c], i1 = cut[c + 1];
    e = cudaStreamWaitEvent(ctx->hs_out, ctx->hs_decoded[c], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ho + out[i0], ctx->hs_out_d + out[i0], out[i1] - out[i0], cudaMemcpyDeviceToHost,
                          ctx->hs_out);
  }
  nvtxRangePop();
  if (e != cudaSuccess) return cuda_status(e);
  cudaEventRecord(ctx->scratch_done, ctx->hs_comp);
  ctx->scratch_stream = ctx->hs_comp;
  ctx->scratch_used = true;
  // hs_done: the last copy out, after every decode (the copy-out stream
  // waited for each chunk's decode in turn).
  e = cudaEventRecord(ctx->hs_done, ctx->hs_out);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(caller, ctx->hs_done, 0);
  ctx->hs_used = true;
  return cuda_status(e);
}

gst_status gst_decompress_dxt(gst_ctx *ctx, const uint8_t *gst, size_t len, uint8_t *dxt_out, size_t out_cap) {
  if (!ctx || !gst || !dxt_out) return GST_E_ARG;
  gst_header h;
  gst_status st = gst_parse_header(gst, len, &h);
  if (st != GST_OK) return st;
  const size_t out_bytes = size_t(image_blocks(h)) * 8;
  if (out_cap < out_bytes) return GST_E_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  // codec/decoder.cpp:430-476 (UploadData): the offsets page at byte 0, the
  // stream minus its 28-byte header from byte 512.
  const size_t body = 28 + 4 * kFreqTableBytes + section_bytes(h);
  const size_t cmp_bytes = 512 + body - 28;
  if ((st = grow_device(&ctx->cmp_d, &ctx->cmp_cap, cmp_bytes)) != GST_OK) return st;
  if ((st = grow_device(&ctx->out_d, &ctx->out_cap, out_bytes)) != GST_OK) return st;
  if ((st = grow_pinned(&ctx->cmp_h, &ctx->cmp_h_cap, cmp_bytes)) != GST_OK) return st;
  if ((st = grow_pinned(&ctx->out_h, &ctx->out_h_cap, out_bytes)) != GST_OK) return st;
  cudaStream_t s = ctx->own_stream;
  cudaStreamSynchronize(s);  // the pinned staging buffers may still feed the previous call
  memset(ctx->cmp_h, 0, 512);
  memcpy(ctx->cmp_h + 512, gst + 28, body - 28);
  cudaError_t e;
  {
    NvtxRange range("gst copy in");
    e = cudaMemcpyAsync(ctx->cmp_d, ctx->cmp_h, cmp_bytes, cudaMemcpyHostToDevice, s);
  }
  if (e != cudaSuccess) return cuda_status(e);
  st = decode_batch(ctx, &h, 1, ctx->cmp_d, ctx->out_d, s);
  if (st != GST_OK) return st;
  {
    NvtxRange range("gst copy out");
    e = cudaMemcpyAsync(ctx->out_h, ctx->out_d, out_bytes, cudaMemcpyDeviceToHost, s);
  }
  if (e != cudaSuccess) return cuda_status(e);
  st = read_device_status(ctx, s);
  memcpy(dxt_out, ctx->out_h, out_bytes);
  return st;
}

gst_status gst_decode_rans_groups(gst_ctx *ctx, const void *d_freqs, const void *d_body, uint32_t body_bytes,
                                  uint32_t n_groups, uint32_t streams_per_group, void *d_out, void *stream) {
  if (!ctx || !d_freqs || !d_body || !d_out || n_groups == 0) return GST_E_ARG;
  if (streams_per_group < 1 || streams_per_group > kStreamsPerGroup) return GST_E_ARG;
  if ((reinterpret_cast<uintptr_t>(d_freqs) & 1) || (reinterpret_cast<uintptr_t>(d_body) & 3) ||
      (reinterpret_cast<uintptr_t>(d_out) & 15))
    return GST_E_ARG;
  if (uint64_t(n_groups) * 4 > body_bytes) return GST_E_FORMAT;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool cap = capturing(st);
  const uint32_t n_rans = (n_groups + kGroupsPerRansCta - 1) / kGroupsPerRansCta;
  const size_t off_images = align_up(sizeof(GstPlanHead), 128);
  const size_t off_rans = off_images + sizeof(GstImageDesc);
  const size_t off_counters = align_up(off_rans + sizeof(GstRansItem) * n_rans, 16);
  const size_t plan_bytes = align_up(off_counters + 4, 16);
  PlanBuf *pb = nullptr;
  gst_status s2 = acquire_plan(ctx, plan_bytes, st, cap, &pb);
  if (s2 != GST_OK) return s2;
  uint8_t *ph = pb->h;
  memset(ph, 0, plan_bytes);
  GstPlanHead *head = reinterpret_cast<GstPlanHead *>(ph);
  head->n_images = 1;
  head->n_rans = n_rans;
  GstImageDesc *d = reinterpret_cast<GstImageDesc *>(ph + off_images);
  // Addresses are carried as offsets from a null base.
  d->freq_off = reinterpret_cast<uintptr_t>(d_freqs);
  d->body_off = reinterpret_cast<uintptr_t>(d_body);
  d->sym_off = reinterpret_cast<uintptr_t>(d_out);
  d->sec_len[0] = body_bytes;
  d->sec_groups[0] = n_groups;
  GstRansItem *rans = reinterpret_cast<GstRansItem *>(ph + off_rans);
  for (uint32_t g = 0, r = 0; g < n_groups; g += kGroupsPerRansCta, ++r)
    rans[r] = {0u, 0u, g, uint16_t(std::min(kGroupsPerRansCta, n_groups - g)), uint16_t(streams_per_group)};
  GstPlanView view = {};
  view.err = ctx->status_d;
  view.images = reinterpret_cast<const GstImageDesc *>(pb->d + off_images);
  view.rans = reinterpret_cast<const GstRansItem *>(pb->d + off_rans);
  view.counters = reinterpret_cast<uint32_t *>(pb->d + off_counters);
  view.n_images = 1;
  view.n_rans = n_rans;  // no sync words: always the rANS kernel alone
  return upload_and_launch(ctx, pb, plan_bytes, view, nullptr, nullptr, nullptr, st, cap, tuning_for_locked(ctx, 0));
}

gst_status gst_batch_create(gst_ctx *ctx, const gst_header *hdrs, int n, gst_batch **out) {
  if (!ctx || !hdrs || n <= 0 || !out) return GST_E_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    gst_status st = check_header(hdrs[i]);
    if (st != GST_OK) return st;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  gst_batch *b = new gst_batch();
  b->ctx = ctx;
  b->hdrs.assign(hdrs, hdrs + n);
  b->plan_cap = plan_capacity(ctx, launch_tuning_locked(ctx, hdrs, n));
  b->layout = plan_layout(hdrs, n, b->plan_cap);
  b->compressed_bytes = gst_batch_layout_bytes(hdrs, n);
  for (int i = 0; i < n; ++i) b->out_bytes += size_t(image_blocks(hdrs[i])) * 8;
  std::vector<uint8_t> plan(b->layout.bytes);
  write_plan(b->layout, hdrs, n, plan.data(), nullptr, nullptr, nullptr);
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&b->plan_d), b->layout.bytes);
  if (e == cudaSuccess) b->plan_alloc = b->layout.bytes;
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void **>(&b->scratch), std::max<size_t>(b->layout.scratch_bytes, 256));
  if (e == cudaSuccess) e = cudaMemcpy(b->plan_d, plan.data(), b->layout.bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    gst_batch_destroy(b);
    return cuda_status(e);
  }
  *out = b;
  return GST_OK;
}

void gst_batch_destroy(gst_batch *b) {
  if (!b) return;
  cudaSetDevice(b->ctx->device);
  cudaDeviceSynchronize();
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->hm_graph) cudaGraphExecDestroy(b->hm_graph);
  for (cudaStream_t s : b->hm_stream)
    if (s) cudaStreamDestroy(s);
  cudaFree(b->hm_cmp);
  cudaFree(b->hm_out);
  cudaFree(b->hm_plans);
  cudaFree(b->plan_d);
  cudaFree(b->scratch);
  delete b;
}

int gst_batch_rans_items(const gst_batch *b) { return b ? int(b->layout.n_rans) : 0; }

size_t gst_batch_device_bytes(const gst_batch *b) {
  return b ? b->layout.bytes + b->layout.scratch_bytes : 0;
}

gst_status gst_batch_launch(gst_batch *b, const void *d_cmp, void *d_out, void *stream) {
  if (!b || !d_cmp || !d_out) return GST_E_ARG;
  if ((reinterpret_cast<uintptr_t>(d_cmp) & 15) || (reinterpret_cast<uintptr_t>(d_out) & 7)) return GST_E_ARG;
  gst_ctx *ctx = b->ctx;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool cap = capturing(st);
  cudaEvent_t *ev = (ctx->profiling && !cap) ? ctx->ev : nullptr;
  cudaError_t e = batch_launch_locked(b, d_cmp, d_out, st, batch_tuning(b), ev);
  ctx->timed_kernels = ev ? ctx->last_launches : 0;
  return cuda_status(e);
}

gst_status gst_batch_graph_launch(gst_batch *b, const void *d_cmp, void *d_out, void *stream) {
  if (!b || !d_cmp || !d_out) return GST_E_ARG;
  gst_ctx *ctx = b->ctx;
  cudaSetDevice(ctx->device);
  GstTuning cur;
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    cur = batch_tuning(b);
    if (!capturing(static_cast<cudaStream_t>(stream))) {
      const cudaError_t e = ensure_plan_locked(b, cur);  // may drop the graph: captured again below
      if (e != cudaSuccess) return cuda_status(e);
    }
  }
  if (!b->graph || b->graph_cmp != d_cmp || b->graph_out != d_out || b->graph_tuning != cur) {
    // Capture the launch sequence once per (input, output) pair.
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e);
    {
      std::lock_guard<std::mutex> lock(ctx->mu);
      launch_decode(nullptr, nullptr, nullptr, GstPlanView{}, nullptr, &ctx->last_launches, nullptr,
                    GstTuning{});  // configure attributes
    }
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    gst_status st = GST_OK;
    if (e == cudaSuccess) st = gst_batch_launch(b, d_cmp, d_out, cs);
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return cuda_status(e != cudaSuccess ? e : e2);
    }
    if (st != GST_OK) {
      cudaGraphDestroy(g);
      return st;
    }
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_status(e);
    b->graph_cmp = d_cmp;
    b->graph_out = d_out;
    b->graph_tuning = cur;
  }
  return cuda_status(cudaGraphLaunch(b->graph, static_cast<cudaStream_t>(stream)));
}

gst_status gst_batch_host_launch(gst_batch *b, const void *h_cmp, void *h_out, int chunks, void *stream) {
  if (!b || !h_cmp || !h_out || chunks < 0) return GST_E_ARG;
  gst_ctx *ctx = b->ctx;
  const int n = int(b->hdrs.size());
  if (chunks == 0) chunks = std::min(n, 3);
  chunks = std::min(chunks, n);
  cudaSetDevice(ctx->device);
  cudaStream_t caller = static_cast<cudaStream_t>(stream);
  if (capturing(caller)) return GST_E_ARG;
  const gst_header *hdrs = b->hdrs.data();
  const size_t page = offsets_page_bytes(n);
  std::vector<uint64_t> body(n + 1), out(n + 1);
  body[0] = page + size_t(n) * 4 * kFreqTableBytes;
  out[0] = 0;
  uint64_t blocks = 0;
  for (int i = 0; i < n; ++i) {
    body[i + 1] = body[i] + section_bytes(hdrs[i]);
    out[i + 1] = out[i] + 8 * image_blocks(hdrs[i]);
    blocks += image_blocks(hdrs[i]);
  }
  cudaError_t e = cudaSuccess;
  if (!b->hm_cmp) {
    e = cudaMalloc(reinterpret_cast<void **>(&b->hm_cmp), body[n]);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void **>(&b->hm_out), out[n]);
    for (auto &s : b->hm_stream)
      if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e);
  }
  // Each chunk's configuration: the batch's own where it has one, else the
  // chunk's size-dependent one (a chunk is a launch of a few images).
  const std::vector<int> cut_now = chunk_cuts(hdrs, n, chunks, blocks);
  GstTuning tuning;
  std::vector<GstTuning> tun;
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    tuning = batch_tuning(b);
    tun.assign(cut_now.size() - 1, tuning);
    if (!b->tuned)
      for (size_t c = 0; c + 1 < cut_now.size(); ++c)
        tun[c] = launch_tuning_locked(ctx, hdrs + cut_now[c], cut_now[c + 1] - cut_now[c]);
  }
  if (b->hm_chunks != chunks || b->hm_tun != tun) {
    // Per-chunk plans with absolute addresses in the mirrors, uploaded once
    // per chunk count and chunk configurations.
    const std::vector<int> &cut = cut_now;
    const int nc = int(cut.size()) - 1;
    std::vector<PlanLayout> lay(nc);
    std::vector<size_t> off(nc + 1, 0);
    for (int c = 0; c < nc; ++c) {
      lay[c] = plan_layout(hdrs + cut[c], cut[c + 1] - cut[c], plan_capacity(ctx, tun[c]));
      off[c + 1] = align_up(off[c] + lay[c].bytes, 256);
    }
    if (b->hm_graph) cudaGraphExecDestroy(b->hm_graph);
    b->hm_graph = nullptr;
    cudaDeviceSynchronize();  // earlier launches may still read the old plans
    cudaFree(b->hm_plans);
    b->hm_plans = nullptr;
    b->hm_chunks = 0;
    e = cudaMalloc(reinterpret_cast<void **>(&b->hm_plans), std::max<size_t>(off[nc], 256));
    if (e != cudaSuccess) return cuda_status(e);
    std::vector<uint8_t> ph(off[nc]);
    for (int c = 0; c < nc; ++c) {
      const int i0 = cut[c], m = cut[c + 1] - i0;
      std::vector<uint64_t> fa(m), ba(m), oa(m);
      for (int k = 0; k < m; ++k) {
        fa[k] = reinterpret_cast<uint64_t>(b->hm_cmp + page + size_t(i0 + k) * 4 * kFreqTableBytes);
        ba[k] = reinterpret_cast<uint64_t>(b->hm_cmp + body[i0 + k]);
        oa[k] = reinterpret_cast<uint64_t>(b->hm_out + out[i0 + k]);
      }
      write_plan(lay[c], hdrs + i0, m, ph.data() + off[c], fa.data(), ba.data(), oa.data());
    }
    e = cudaMemcpy(b->hm_plans, ph.data(), off[nc], cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e);
    b->hm_cut = cut;
    b->hm_scr_off.assign(nc + 1, 0);
    for (int c = 0; c < nc; ++c) b->hm_scr_off[c + 1] = b->hm_scr_off[c] + lay[c].scratch_bytes;
    if (b->hm_scr_off[nc] > b->layout.scratch_bytes) return GST_E_ARG;  // cannot happen: same images
    b->hm_lay = std::move(lay);
    b->hm_plan_off = std::move(off);
    b->hm_chunks = chunks;
    b->hm_tun = tun;
  }
  if (!b->hm_graph || b->hm_graph_cmp != h_cmp || b->hm_graph_out != h_out || b->hm_graph_tuning != tuning) {
    // Capture the copies in, decodes and copies out of every chunk, enqueued
    // in three passes as gst_load_host_dxts does.  Consecutive chunks decode
    // on two streams, each into its own part of the batch's scratch: a decode
    // is bound by its rANS chains' latency more than by its size, so the next
    // chunk's decode starts as soon as its copy in lands instead of after the
    // previous decode, and the copies out (the slowest stage) wait less.
    {
      std::lock_guard<std::mutex> lock(ctx->mu);
      launch_decode(nullptr, nullptr, nullptr, GstPlanView{}, nullptr, &ctx->last_launches, nullptr,
                    GstTuning{});  // configure attributes
    }
    const int nc = int(b->hm_cut.size()) - 1;
    const uint8_t *hc = static_cast<const uint8_t *>(h_cmp);
    uint8_t *ho = static_cast<uint8_t *>(h_out);
    cudaStream_t cs = nullptr, si = b->hm_stream[0], so = b->hm_stream[2];
    const cudaStream_t sc[2] = {b->hm_stream[1], b->hm_stream[3]};
    std::vector<cudaEvent_t> evs(2 * nc + 5, nullptr);
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    for (auto &ev : evs)
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    cudaGraph_t g = nullptr;
    bool capturing_now = false;
    if (e == cudaSuccess) {
      e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      capturing_now = e == cudaSuccess;
    }
    cudaEvent_t fork = evs[2 * nc], end_i = evs[2 * nc + 1], end_c = evs[2 * nc + 2], end_o = evs[2 * nc + 3];
    cudaEvent_t end_c2 = evs[2 * nc + 4];
    if (e == cudaSuccess) e = cudaEventRecord(fork, cs);
    for (cudaStream_t s : {si, sc[0], sc[1], so})
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, fork, 0);
    nvtxRangePushA("gst copy in");
    for (int c = 0; c < nc && e == cudaSuccess; ++c) {
      const int i0 = b->hm_cut[c], i1 = b->hm_cut[c + 1];
      const size_t t0 = page + size_t(i0) * 4 * kFreqTableBytes, t1 = page + size_t(i1) * 4 * kFreqTableBytes;
      e = cudaMemcpyAsync(b->hm_cmp + t0, hc + t0, t1 - t0, cudaMemcpyHostToDevice, si);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->hm_cmp + body[i0], hc + body[i0], body[i1] - body[i0], cudaMemcpyHostToDevice, si);
      if (e == cudaSuccess) e = cudaEventRecord(evs[c], si);
    }
    nvtxRangePop();
    nvtxRangePushA("gst decode");
    for (int c = 0; c < nc && e == cudaSuccess; ++c) {
      const cudaStream_t s = sc[c & 1];
      e = cudaStreamWaitEvent(s, evs[c], 0);
      GstPlanView view = plan_view(b->hm_lay[c], b->hm_plans + b->hm_plan_off[c], ctx->status_d);
      view.image_err = nullptr;
      view.wait_limit_ns = ctx->wait_limit_ns;
      int launches = 0;
      if (e == cudaSuccess)
        e = launch_decode(nullptr, b->scratch + b->hm_scr_off[c], nullptr, view, s, &launches, nullptr,
                          b->hm_tun[c]);
      if (e == cudaSuccess) e = cudaEventRecord(evs[nc + c], s);
    }
    nvtxRangePop();
    nvtxRangePushA("gst copy out");
    for (int c = 0; c < nc && e == cudaSuccess; ++c) {
      const int i0 = b->hm_cut[c], i1 = b->hm_cut[c + 1];
      e = cudaStreamWaitEvent(so, evs[nc + c], 0);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(ho + out[i0], b->hm_out + out[i0], out[i1] - out[i0], cudaMemcpyDeviceToHost, so);
    }
    nvtxRangePop();
    if (e == cudaSuccess) e = cudaEventRecord(end_i, si);
    if (e == cudaSuccess) e = cudaEventRecord(end_c, sc[0]);
    if (e == cudaSuccess) e = cudaEventRecord(end_c2, sc[1]);
    if (e == cudaSuccess) e = cudaEventRecord(end_o, so);
    for (cudaEvent_t ev : {end_i, end_c, end_c2, end_o})
      if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev, 0);
    if (capturing_now) {
      const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
      if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) {
      if (b->hm_graph) cudaGraphExecDestroy(b->hm_graph);
      b->hm_graph = nullptr;
      e = cudaGraphInstantiate(&b->hm_graph, g, 0);
    }
    if (g) cudaGraphDestroy(g);
    for (auto ev : evs)
      if (ev) cudaEventDestroy(ev);
    if (cs) cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
      b->hm_graph = nullptr;
      return cuda_status(e);
    }
    b->hm_graph_cmp = h_cmp;
    b->hm_graph_out = h_out;
    b->hm_graph_tuning = tuning;
  }
  return cuda_status(cudaGraphLaunch(b->hm_graph, caller));
}

gst_status gst_set_option(gst_ctx *ctx, const char *name, int value) {
  if (!ctx || !name) return GST_E_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (strcmp(name, "rans_blocks_per_sm") == 0) {
    if (!valid_tuning(value, int(ctx->tuning.stage_words))) return GST_E_ARG;
    ctx->tuning.blocks_per_sm = value;
    ctx->tuning_explicit = true;
    return GST_OK;
  }
  if (strcmp(name, "rans_stage_words") == 0) {
    if (!valid_tuning(ctx->tuning.blocks_per_sm, value)) return GST_E_ARG;
    ctx->tuning.stage_words = uint32_t(value);
    ctx->tuning_explicit = true;
    return GST_OK;
  }
  if (strcmp(name, "persistent") == 0) {
    if (value != 0 && value != 1) return GST_E_ARG;
    ctx->tuning.persistent = value;
    ctx->tuning_explicit = true;
    return GST_OK;
  }
  if (strcmp(name, "persistent_wait_us") == 0) {
    if (value < 0 || value > 2000000) return GST_E_ARG;
    ctx->wait_limit_ns = uint64_t(value) * 1000u;
    return GST_OK;
  }
  if (strcmp(name, "auto_tuning") == 0) {  // back to the default configuration, chosen per launch size
    if (value != 1) return GST_E_ARG;
    ctx->tuning = GstTuning{};
    ctx->tuning_explicit = false;
    return GST_OK;
  }
  if (strcmp(name, "balance_rans_items") == 0) {
    if (value != 0 && value != 1) return GST_E_ARG;
    ctx->balance_items = value != 0;
    return GST_OK;
  }
  if (strcmp(name, "encode_hist_match") == 0) {
    if (value != 0 && value != 1) return GST_E_ARG;
    ctx->enc_hist_match = value != 0;
    return GST_OK;
  }
  if (strcmp(name, "inject_encode_stall") == 0) {
    if (value != 0 && value != 1) return GST_E_ARG;
    ctx->inject_encode_stall = value != 0;
    return GST_OK;
  }
  if (strcmp(name, "inject_drop_rans") == 0) {
    if (value != 0 && value != 1) return GST_E_ARG;
    ctx->inject_drop_rans = value != 0;
    return GST_OK;
  }
  return GST_E_ARG;
}

gst_status gst_batch_set_tuning(gst_batch *b, int blocks_per_sm, int stage_words, int persistent) {
  if (!b) return GST_E_ARG;
  if (blocks_per_sm == 0 && stage_words == 0) {  // back to the context's configuration
    b->tuned = false;
    return GST_OK;
  }
  if (!valid_tuning(blocks_per_sm, stage_words, persistent)) return GST_E_ARG;
  std::lock_guard<std::mutex> lock(b->ctx->mu);
  b->tuning.blocks_per_sm = blocks_per_sm;
  b->tuning.stage_words = uint32_t(stage_words);
  b->tuning.persistent = persistent;
  b->tuned = true;
  return GST_OK;
}

int gst_size_class(uint64_t blocks) { return size_class(blocks); }

gst_status gst_set_class_tuning(gst_ctx *ctx, int size_class_index, int blocks_per_sm, int stage_words,
                                int persistent) {
  if (!ctx || size_class_index < 0 || size_class_index >= kSizeClasses) return GST_E_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (blocks_per_sm == 0 && stage_words == 0) {  // clear: the class uses the context's configuration
    ctx->class_set[size_class_index] = false;
    return GST_OK;
  }
  if (!valid_tuning(blocks_per_sm, stage_words, persistent)) return GST_E_ARG;
  GstTuning t;
  t.blocks_per_sm = blocks_per_sm;
  t.stage_words = uint32_t(stage_words);
  t.persistent = persistent;
  ctx->class_tuning[size_class_index] = t;
  ctx->class_set[size_class_index] = true;
  return GST_OK;
}

gst_status gst_get_class_tuning(gst_ctx *ctx, int size_class_index, int *blocks_per_sm, int *stage_words,
                                int *persistent) {
  if (!ctx || size_class_index < 0 || size_class_index >= kSizeClasses || !blocks_per_sm || !stage_words ||
      !persistent)
    return GST_E_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  const GstTuning &t = ctx->class_set[size_class_index] ? ctx->class_tuning[size_class_index] : ctx->tuning;
  *blocks_per_sm = t.blocks_per_sm;
  *stage_words = int(t.stage_words);
  *persistent = t.persistent;
  return GST_OK;
}

gst_status gst_autotune_class(gst_ctx *ctx, const gst_header *hdrs, int n, const void *d_cmp, void *d_out,
                              void *stream, int iterations, int *size_class_out) {
  if (!ctx || !hdrs || n <= 0) return GST_E_ARG;
  gst_batch *b = nullptr;
  gst_status st = gst_batch_create(ctx, hdrs, n, &b);
  if (st != GST_OK) return st;
  int bps = 0, words = 0, pers = 0;
  st = gst_batch_autotune(b, d_cmp, d_out, stream, iterations, &bps, &words, &pers);
  const int c = size_class(uint64_t(b->layout.n_tiles) * 1024);
  gst_batch_destroy(b);
  if (st != GST_OK) return st;
  st = gst_set_class_tuning(ctx, c, bps, words, pers);
  if (st == GST_OK && size_class_out) *size_class_out = c;
  // The winner goes into the persisted table as well, where one is named.
  const char *table = std::getenv("GST_TUNING_TABLE");
  if (st == GST_OK && table && *table) st = gst_save_class_tuning(ctx, table);
  return st;
}

// ---------------------------------------------------------------------------
// The per-size-class tuning as a JSON table, so that the autotuner's choices
// outlive the process:
//   {"format": "gst_gb300 class tuning", "version": 1, "device": "<name>",
//    "classes": [{"class": c, "max_blocks": m, "blocks_per_sm": b,
//                 "stage_words": w, "persistent": p}, ...]}
// Only the classes that are set are written ("max_blocks" is informative:
// the class's upper bound in DXT1 blocks, 0 for the open-ended last one).
namespace {

std::string device_name(int device) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return "";
  std::string n;
  for (const char *c = prop.name; *c; ++c)
    if (*c != '"' && *c != '\\') n += *c;  // kept JSON-safe
  return n;
}

// The text after `"key":` (spaces skipped) in [at, end), or nullptr.
const char *json_value(const char *at, const char *end, const char *key) {
  const std::string k = std::string("\"") + key + "\"";
  const char *p = std::search(at, end, k.begin(), k.end());
  if (p == end) return nullptr;
  p += k.size();
  while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
  if (p == end || *p != ':') return nullptr;
  ++p;
  while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
  return p < end ? p : nullptr;
}

bool json_int(const char *at, const char *end, const char *key, long *out) {
  const char *p = json_value(at, end, key);
  if (!p) return false;
  char *q = nullptr;
  const long v = std::strtol(p, &q, 10);
  if (q == p || q > end) return false;
  *out = v;
  return true;
}

}  // namespace

gst_status gst_save_class_tuning(gst_ctx *ctx, const char *path) {
  if (!ctx || !path) return GST_E_ARG;
  std::string out = "{\"format\": \"gst_gb300 class tuning\", \"version\": 1, \"device\": \"" +
                    device_name(ctx->device) + "\",\n \"classes\": [";
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    bool first = true;
    for (int c = 0; c < kSizeClasses; ++c) {
      if (!ctx->class_set[c]) continue;
      const GstTuning &t = ctx->class_tuning[c];
      const unsigned long long max_blocks = c == kSizeClasses - 1 ? 0ull : (1ull << 14) << (2 * c);
      char line[256];
      std::snprintf(line, sizeof(line),
                    "%s\n  {\"class\": %d, \"max_blocks\": %llu, \"blocks_per_sm\": %d, \"stage_words\": %u, "
                    "\"persistent\": %d}",
                    first ? "" : ",", c, max_blocks, t.blocks_per_sm, t.stage_words, t.persistent);
      out += line;
      first = false;
    }
  }
  out += "\n ]}\n";
  // Written to a temporary file and renamed, so that a reader never sees half a table.
  const std::string tmp = std::string(path) + ".tmp";
  FILE *f = std::fopen(tmp.c_str(), "wb");
  if (!f) return GST_E_ARG;
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  if (std::fclose(f) != 0 || !ok || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return GST_E_ARG;
  }
  return GST_OK;
}

gst_status gst_load_class_tuning(gst_ctx *ctx, const char *path) {
  if (!ctx || !path) return GST_E_ARG;
  FILE *f = std::fopen(path, "rb");
  if (!f) return GST_E_ARG;
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0 && text.size() < (1u << 20)) text.append(buf, n);
  std::fclose(f);
  const char *b = text.data(), *e = b + text.size();
  const char *fmt = json_value(b, e, "format");
  const std::string want_fmt = "\"gst_gb300 class tuning\"";
  if (!fmt || size_t(e - fmt) < want_fmt.size() || std::string(fmt, want_fmt.size()) != want_fmt) return GST_E_FORMAT;
  long version = 0;
  if (!json_int(b, e, "version", &version) || version != 1) return GST_E_FORMAT;
  const char *dev = json_value(b, e, "device");
  const std::string want_dev = "\"" + device_name(ctx->device) + "\"";
  if (!dev || size_t(e - dev) < want_dev.size() || std::string(dev, want_dev.size()) != want_dev)
    return GST_E_ARG;  // measured on another kind of GPU: not applied
  const char *cls = json_value(b, e, "classes");
  if (!cls || *cls != '[') return GST_E_FORMAT;
  // Every entry is validated before any is applied.
  GstTuning t[kSizeClasses];
  bool set[kSizeClasses] = {};
  const char *p = cls + 1;
  for (;;) {
    const char *o = std::find(p, e, '{'), *close = std::find(p, e, ']');
    if (close < o) break;  // end of the list
    if (o == e) return GST_E_FORMAT;
    const char *oe = std::find(o, e, '}');
    if (oe == e) return GST_E_FORMAT;
    long c = -1, bps = 0, words = 0, pers = 0;
    if (!json_int(o, oe, "class", &c) || !json_int(o, oe, "blocks_per_sm", &bps) ||
        !json_int(o, oe, "stage_words", &words) || !json_int(o, oe, "persistent", &pers))
      return GST_E_FORMAT;
    if (c < 0 || c >= kSizeClasses || !valid_tuning(int(bps), int(words), int(pers))) return GST_E_FORMAT;
    t[c].blocks_per_sm = int(bps);
    t[c].stage_words = uint32_t(words);
    t[c].persistent = int(pers);
    set[c] = true;
    p = oe + 1;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  for (int c = 0; c < kSizeClasses; ++c) {
    ctx->class_set[c] = set[c];
    if (set[c]) ctx->class_tuning[c] = t[c];
  }
  return GST_OK;
}

gst_status gst_batch_autotune(gst_batch *b, const void *d_cmp, void *d_out, void *stream, int iterations,
                              int *blocks_per_sm, int *stage_words, int *persistent) {
  if (!b || !d_cmp || !d_out || iterations < 1) return GST_E_ARG;
  if ((reinterpret_cast<uintptr_t>(d_cmp) & 15) || (reinterpret_cast<uintptr_t>(d_out) & 7)) return GST_E_ARG;
  gst_ctx *ctx = b->ctx;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (capturing(st)) return GST_E_ARG;
  // Two kernels: CTAs of 128 threads per SM x staging depth, the deepest
  // stages that the shared memory of that many CTAs per SM holds and
  // shallower ones.  The persistent kernel (8 CTAs of 128 threads per SM):
  // its tile buffers hold 2040-word stages.
  static const GstTuning kCandidates[] = {
      {16, 520, 0}, {12, 520, 0}, {12, 1016, 0}, {8, 1528, 0}, {8, 2040, 0}, {8, 2816, 0}, {8, 4352, 0},
      {8, 1016, 1}, {8, 2040, 1},
  };
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  GstTuning best = batch_tuning(b);
  float best_ms = 0.f;
  bool found = false;
  for (const GstTuning &t : kCandidates) {
    if (e != cudaSuccess) break;
    e = batch_launch_locked(b, d_cmp, d_out, st, t, nullptr);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    for (int i = 0; i < iterations && e == cudaSuccess; ++i) e = batch_launch_locked(b, d_cmp, d_out, st, t, nullptr);
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && (!found || ms < best_ms)) {
      best = t;
      best_ms = ms;
      found = true;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_status(e);
  b->tuning = best;
  b->tuned = true;
  if (blocks_per_sm) *blocks_per_sm = best.blocks_per_sm;
  if (stage_words) *stage_words = int(best.stage_words);
  if (persistent) *persistent = best.persistent;
  return GST_OK;
}

gst_status gst_sync_status(gst_ctx *ctx, void *stream) {
  if (!ctx) return GST_E_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  return read_device_status(ctx, static_cast<cudaStream_t>(stream));
}

int gst_last_launch_count(gst_ctx *ctx) { return ctx ? ctx->last_launches : 0; }

gst_status gst_set_profiling(gst_ctx *ctx, int enable) {
  if (!ctx) return GST_E_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  if (enable && !ctx->ev[0]) {
    for (auto &e : ctx->ev) {
      cudaError_t err = cudaEventCreate(&e);
      if (err != cudaSuccess) return cuda_status(err);
    }
  }
  ctx->profiling = enable != 0;
  ctx->timed_kernels = 0;
  return GST_OK;
}

int gst_kernel_times(gst_ctx *ctx, float *ms, const char **names, int cap) {
  if (!ctx || !ms || cap <= 0) return 0;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  const int n = std::min(cap, ctx->timed_kernels);
  if (n == 0) return 0;
  if (cudaEventSynchronize(ctx->ev[n]) != cudaSuccess) return 0;
  for (int i = 0; i < n; ++i) {
    if (cudaEventElapsedTime(&ms[i], ctx->ev[i], ctx->ev[i + 1]) != cudaSuccess) return 0;
    if (names) names[i] = ctx->timed_names[i];
  }
  return n;
}

}  // extern "C"
