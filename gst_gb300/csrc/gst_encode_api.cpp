// gst_encode_api.cpp -- C ABI of the encoder stages (include/gst_encode.h):
// the call's plan (sections, units, histogram chunks, group-to-section map),
// its scratch and the four launches of gst_encode.cu.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "gst_encode.h"
#include "gst_host.h"

namespace gst {
namespace host {

struct EncodeState {
  int device = 0;
  int sm_count = 0;
  double *log2_d = nullptr;  // log2(n / (n + 1)), then log2(n / (n - 1)), n in [0, kEncLogTableLen)
  uint8_t *plan_d = nullptr;
  size_t plan_d_cap = 0;
  uint8_t *plan_h = nullptr;  // pinned staging of the plan
  size_t plan_h_cap = 0;
  uint8_t *scratch_d = nullptr;
  size_t scratch_cap = 0;
  cudaEvent_t done = nullptr;
  cudaStream_t last_stream = nullptr;
  bool used = false;
  int last_launches = 0;
  // host-to-host calls
  cudaStream_t own = nullptr;
  uint8_t *in_d = nullptr;
  size_t in_cap = 0;
  uint8_t *out_d = nullptr;
  size_t out_cap = 0;
  unsigned long long *offsets_d = nullptr;
  // endpoint stages (gst_prepare_symbols, gst_compress_dxt)
  uint8_t *prep_h = nullptr;  // pinned plan staging
  size_t prep_h_cap = 0;
  uint8_t *prep_d = nullptr;
  size_t prep_d_cap = 0;
  cudaEvent_t prep_done = nullptr;
  bool prep_used = false;
  uint8_t *blocks_d = nullptr;
  size_t blocks_cap = 0;
  uint32_t *pal_bytes_d = nullptr;
  // palette search (gst_reencode_blocks, gst_compress_rgb_dxt)
  uint8_t *re_h = nullptr;  // pinned descriptors
  size_t re_h_cap = 0;
  uint8_t *re_d = nullptr;  // descriptors, order, states, then each image's scores and maps
  size_t re_d_cap = 0;
  cudaEvent_t re_done = nullptr;
  bool re_used = false;
  uint8_t *rgb_d = nullptr;
  size_t rgb_cap = 0;
  uint8_t *blocks2_d = nullptr;
  size_t blocks2_cap = 0;
};

void destroy_encode_state(EncodeState *s) {
  if (!s) return;
  cudaFree(s->log2_d);
  cudaFree(s->plan_d);
  cudaFreeHost(s->plan_h);
  cudaFree(s->scratch_d);
  cudaFree(s->in_d);
  cudaFree(s->out_d);
  cudaFree(s->offsets_d);
  cudaFreeHost(s->prep_h);
  cudaFree(s->prep_d);
  cudaFree(s->blocks_d);
  cudaFree(s->pal_bytes_d);
  cudaFreeHost(s->re_h);
  cudaFree(s->re_d);
  cudaFree(s->rgb_d);
  cudaFree(s->blocks2_d);
  if (s->re_done) cudaEventDestroy(s->re_done);
  if (s->prep_done) cudaEventDestroy(s->prep_done);
  if (s->done) cudaEventDestroy(s->done);
  if (s->own) cudaStreamDestroy(s->own);
  delete s;
}

namespace {

// The rank table of the frequency correction: GetFreqChange
// (ans/histogram.cpp:25-29) takes log2 of n / (n + sign) with the C library's
// log2; the kernels multiply these exact values by the counts.
void fill_log2_tables(std::vector<double> *t) {
  t->assign(2 * kEncLogTableLen, 0.0);
  for (uint32_t n = 1; n < kEncLogTableLen; ++n)
    (*t)[n] = std::log2(static_cast<double>(n) / static_cast<double>(n + 1));
  for (uint32_t n = 2; n < kEncLogTableLen; ++n)
    (*t)[kEncLogTableLen + n] = std::log2(static_cast<double>(n) / static_cast<double>(n - 1));
}

gst_status get_state(gst_ctx *ctx, EncodeState **out) {
  EncodeState *&s = ctx_encode_state(ctx);
  if (!s) {
    EncodeState *n = new EncodeState();
    n->device = ctx_device(ctx);
    std::vector<double> t;
    fill_log2_tables(&t);
    cudaError_t e = cudaDeviceGetAttribute(&n->sm_count, cudaDevAttrMultiProcessorCount, n->device);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&n->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&n->prep_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&n->re_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void **>(&n->pal_bytes_d), sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&n->own, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void **>(&n->log2_d), t.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(n->log2_d, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMalloc(reinterpret_cast<void **>(&n->offsets_d), 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) {
      destroy_encode_state(n);
      return cuda_status(e);
    }
    s = n;
  }
  *out = s;
  return GST_OK;
}

gst_status grow_dev(uint8_t **p, size_t *cap, size_t need) {
  if (*cap >= need) return GST_OK;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const size_t sz = std::max(need, size_t(1) << 16);
  const cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), sz);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_status(e);
  }
  *cap = sz;
  return GST_OK;
}

gst_status grow_host(uint8_t **p, size_t *cap, size_t need) {
  if (*cap >= need) return GST_OK;
  cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  const size_t sz = std::max(need, size_t(1) << 16);
  const cudaError_t e = cudaMallocHost(reinterpret_cast<void **>(p), sz);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_status(e);
  }
  *cap = sz;
  return GST_OK;
}

constexpr uint64_t kMaxSectionSymbols = (1ull << 31) - kSymsPerGroup;  // counts sum in an int

// One unit of output: a ByteEncoder section or a GST stream of four sections.
struct UnitIn {
  bool stream;
  uint32_t width, height, palette_bytes;
  uint32_t first_section, n_sections;
};

struct SectionIn {
  const uint8_t *sym;
  uint64_t n;
};

uint64_t section_bound(uint64_t n) {
  const uint64_t G = n / kSymsPerGroup;
  return kFreqTableBytes + 4 * G + G * kEncMaxGroupBytes;
}

bool stream_dims_ok(uint32_t w, uint32_t h, uint32_t pal) {
  gst_header hd = {};
  hd.width = w;
  hd.height = h;
  hd.palette_bytes = pal;
  const uint64_t B = uint64_t(w / 4) * (h / 4);
  const uint64_t G[4] = {2 * B / kSymsPerGroup, 4 * B / kSymsPerGroup, pal / kSymsPerGroup, B / kSymsPerGroup};
  hd.y_cmp_sz = uint32_t(std::min<uint64_t>(G[0] * 132, 0xFFFFFFFCu));
  hd.chroma_cmp_sz = uint32_t(std::min<uint64_t>(G[1] * 132, 0xFFFFFFFCu));
  hd.palette_sz = uint32_t(std::min<uint64_t>(G[2] * 132, 0xFFFFFFFCu));
  hd.indices_sz = uint32_t(std::min<uint64_t>(G[3] * 132, 0xFFFFFFFCu));
  return check_header(hd) == GST_OK;
}

// Builds and launches one call's plan.
gst_status encode_locked(gst_ctx *ctx, EncodeState *st, const std::vector<SectionIn> &secs,
                         const std::vector<UnitIn> &units, uint8_t *d_out, size_t out_cap,
                         unsigned long long *d_offsets, cudaStream_t stream) {
  const uint32_t S = static_cast<uint32_t>(secs.size()), U = static_cast<uint32_t>(units.size());
  uint64_t G = 0, n_chunks = 0, bound = 0;
  for (const auto &s : secs) {
    if (!s.sym || s.n == 0 || s.n % kSymsPerGroup || s.n > kMaxSectionSymbols) return GST_E_ARG;
    if (reinterpret_cast<uintptr_t>(s.sym) % 16) return GST_E_ARG;
    G += s.n / kSymsPerGroup;
    n_chunks += (s.n + kEncHistChunk - 1) / kEncHistChunk;
  }
  for (const auto &u : units) bound += u.stream ? kHeaderBytes : 0;
  for (const auto &s : secs) bound += section_bound(s.n);
  if (G >= (1ull << 31) || !d_out || !d_offsets || out_cap < bound) return GST_E_ARG;
  if (reinterpret_cast<uintptr_t>(d_out) % 4 || reinterpret_cast<uintptr_t>(d_offsets) % 8) return GST_E_ARG;

  // plan layout
  const size_t off_sections = 0;
  const size_t off_units = align_up(off_sections + S * sizeof(EncSection), 16);
  const size_t off_chunks = align_up(off_units + U * sizeof(EncUnit), 16);
  const size_t off_gsec = align_up(off_chunks + n_chunks * sizeof(EncChunk), 16);
  const size_t plan_bytes = align_up(off_gsec + G * sizeof(uint32_t), 16);
  // scratch layout: zeroed part first
  const size_t s_counts = 0;
  const size_t s_status = align_up(s_counts + size_t(S) * 256 * 4, 256);
  const size_t s_ticket = align_up(s_status + G * 8, 256);
  const size_t s_zero = s_ticket + 16;
  const size_t s_tables = align_up(s_zero, 256);
  const size_t s_freqs = align_up(s_tables + size_t(S) * 256 * 16, 256);
  const size_t scratch_bytes = align_up(s_freqs + size_t(S) * 256 * 2, 256);

  if (st->used) {
    cudaError_t e = cudaEventSynchronize(st->done);  // staging and scratch of the previous call
    if (e != cudaSuccess) return cuda_status(e);
  }
  gst_status r = grow_host(&st->plan_h, &st->plan_h_cap, plan_bytes);
  if (r == GST_OK) r = grow_dev(&st->plan_d, &st->plan_d_cap, plan_bytes);
  if (r == GST_OK) r = grow_dev(&st->scratch_d, &st->scratch_cap, scratch_bytes);
  if (r != GST_OK) return r;

  uint8_t *ph = st->plan_h;
  memset(ph, 0, plan_bytes);
  EncSection *ps = reinterpret_cast<EncSection *>(ph + off_sections);
  EncUnit *pu = reinterpret_cast<EncUnit *>(ph + off_units);
  EncChunk *pc = reinterpret_cast<EncChunk *>(ph + off_chunks);
  uint32_t *pg = reinterpret_cast<uint32_t *>(ph + off_gsec);
  uint32_t g = 0, c = 0;
  for (uint32_t k = 0; k < S; ++k) {
    ps[k].sym = secs[k].sym;
    ps[k].n_groups = static_cast<uint32_t>(secs[k].n / kSymsPerGroup);
    ps[k].first_group = g;
    for (uint32_t j = 0; j < ps[k].n_groups; ++j) pg[g + j] = k;
    g += ps[k].n_groups;
    for (uint64_t at = 0; at < secs[k].n; at += kEncHistChunk)
      pc[c++] = {k, static_cast<uint32_t>(at), static_cast<uint32_t>(std::min<uint64_t>(kEncHistChunk, secs[k].n - at))};
  }
  uint64_t fixed_before = 0;
  for (uint32_t u = 0; u < U; ++u) {
    const UnitIn &in = units[u];
    EncUnit &eu = pu[u];
    eu.fixed_before = fixed_before;
    eu.first_section = in.first_section;
    eu.n_sections = in.n_sections;
    eu.first_group = ps[in.first_section].first_group;
    const EncSection &last = ps[in.first_section + in.n_sections - 1];
    eu.end_group = last.first_group + last.n_groups;
    eu.width = in.width;
    eu.height = in.height;
    eu.palette_bytes = in.palette_bytes;
    eu.is_stream = in.stream ? 1 : 0;
    uint64_t fixed = in.stream ? kHeaderBytes + 4 * kFreqTableBytes : 0;
    for (uint32_t q = 0; q < in.n_sections; ++q) {
      EncSection &s = ps[in.first_section + q];
      s.unit = u;
      if (in.stream) {
        fixed += 4ull * s.n_groups;
        s.grp_fixed = fixed_before + fixed;
        s.tbl_fixed = fixed_before + kHeaderBytes + q * kFreqTableBytes;
        s.tbl_group = eu.first_group;
      } else {
        s.tbl_fixed = fixed_before + fixed;
        s.tbl_group = s.first_group;
        fixed += kFreqTableBytes + 4ull * s.n_groups;
        s.grp_fixed = fixed_before + fixed;
      }
    }
    eu.fixed_bytes = fixed;
    fixed_before += fixed;
  }

  cudaError_t e = cudaMemcpyAsync(st->plan_d, ph, plan_bytes, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(st->scratch_d, 0, s_zero, stream);
  if (e != cudaSuccess) return cuda_status(e);
  EncPlanView v = {};
  v.sections = reinterpret_cast<const EncSection *>(st->plan_d + off_sections);
  v.units = reinterpret_cast<const EncUnit *>(st->plan_d + off_units);
  v.chunks = reinterpret_cast<const EncChunk *>(st->plan_d + off_chunks);
  v.group_section = reinterpret_cast<const uint32_t *>(st->plan_d + off_gsec);
  v.counts = reinterpret_cast<uint32_t *>(st->scratch_d + s_counts);
  v.status = reinterpret_cast<unsigned long long *>(st->scratch_d + s_status);
  v.ticket = reinterpret_cast<uint32_t *>(st->scratch_d + s_ticket);
  v.tables = reinterpret_cast<uint4 *>(st->scratch_d + s_tables);
  v.freqs = reinterpret_cast<uint16_t *>(st->scratch_d + s_freqs);
  v.log2_plus = st->log2_d;
  v.log2_minus = st->log2_d + kEncLogTableLen;
  v.out = d_out;
  v.offsets = d_offsets;
  v.err = ctx_status(ctx);
  v.wait_limit_ns = ctx_wait_limit_ns(ctx);
  v.stall_group = ctx_inject_encode_stall(ctx) && G > 1 ? 1u : ~0u;
  v.n_sections = S;
  v.n_units = U;
  v.n_groups = static_cast<uint32_t>(G);
  v.n_chunks = static_cast<uint32_t>(n_chunks);
  cudaEvent_t *ev = ctx_timing_events(ctx, false);
  e = launch_encode(v, st->sm_count, stream, false, &st->last_launches, ev, ctx_timed_names(ctx),
                    ctx_enc_hist_match(ctx));
  ctx_set_timed(ctx, ev ? st->last_launches : 0, st->last_launches);
  if (e != cudaSuccess) return cuda_status(e);
  cudaEventRecord(st->done, stream);
  st->used = true;
  st->last_stream = stream;
  return GST_OK;
}

uint64_t palette_capacity(uint32_t w, uint32_t h) {
  const uint64_t B = uint64_t(w / 4) * (h / 4);
  return (4 * B + kSymsPerGroup - 1) / kSymsPerGroup * kSymsPerGroup;
}

struct PrepIn {
  uint32_t width, height;
  const uint8_t *blocks;
  uint8_t *y, *chroma, *palette, *indices;
};

// Builds and launches the endpoint stages of one call.
// Builds and launches the endpoint stages of one call; with planes_only, the
// Y and chroma planes alone (palette, indices and d_palette_bytes unused).
gst_status prepare_locked(gst_ctx *ctx, EncodeState *st, const std::vector<PrepIn> &imgs, uint32_t *d_palette_bytes,
                          cudaStream_t stream, bool planes_only = false) {
  const uint32_t n = static_cast<uint32_t>(imgs.size());
  uint64_t tiles = 0, chunks = 0;
  for (const auto &im : imgs) {
    if (!stream_dims_ok(im.width, im.height, kSymsPerGroup)) return GST_E_ARG;
    if (!im.blocks || !im.y || !im.chroma || (!planes_only && (!im.palette || !im.indices))) return GST_E_ARG;
    if (reinterpret_cast<uintptr_t>(im.blocks) % 8) return GST_E_ARG;
    for (const uint8_t *q : {im.y, im.chroma, im.palette, im.indices})
      if (reinterpret_cast<uintptr_t>(q) % 16) return GST_E_ARG;
    const uint64_t B = uint64_t(im.width / 4) * (im.height / 4);
    tiles += B / 1024;
    if (!planes_only) chunks += (B + 8191) / 8192;
  }
  if (tiles >= (1u << 31)) return GST_E_ARG;
  if (!planes_only && (!d_palette_bytes || reinterpret_cast<uintptr_t>(d_palette_bytes) % 4)) return GST_E_ARG;
  const size_t off_chunks = align_up(n * sizeof(EncPrepImage), 16);
  const size_t off_counts = align_up(off_chunks + chunks * sizeof(EncPrepChunk), 16);
  const size_t bytes = align_up(off_counts + chunks * sizeof(uint32_t), 16);
  if (st->prep_used) {
    const cudaError_t e = cudaEventSynchronize(st->prep_done);
    if (e != cudaSuccess) return cuda_status(e);
  }
  gst_status r = grow_host(&st->prep_h, &st->prep_h_cap, bytes);
  if (r == GST_OK) r = grow_dev(&st->prep_d, &st->prep_d_cap, bytes);
  if (r != GST_OK) return r;
  memset(st->prep_h, 0, bytes);
  EncPrepImage *pi = reinterpret_cast<EncPrepImage *>(st->prep_h);
  EncPrepChunk *pc = reinterpret_cast<EncPrepChunk *>(st->prep_h + off_chunks);
  uint32_t t = 0, c = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const PrepIn &im = imgs[i];
    const uint32_t B = (im.width / 4) * (im.height / 4);
    pi[i] = {reinterpret_cast<const uint64_t *>(im.blocks), im.y, im.chroma, im.palette, im.indices,
             im.width, im.height, t, 0};
    t += B / 1024;
    if (planes_only) continue;
    const uint32_t first = c, count = (B + 8191) / 8192;
    for (uint32_t k = 0; k < count; ++k, ++c)
      pc[c] = {i, k * 8192u, std::min<uint32_t>(8192u, B - k * 8192u), first, first + count - 1};
  }
  cudaError_t e = cudaMemcpyAsync(st->prep_d, st->prep_h, bytes, cudaMemcpyHostToDevice, stream);
  cudaEvent_t *ev = ctx_timing_events(ctx, false);
  if (e == cudaSuccess)
    e = launch_prepare(reinterpret_cast<const EncPrepImage *>(st->prep_d), n, t,
                       reinterpret_cast<const EncPrepChunk *>(st->prep_d + off_chunks), c,
                       reinterpret_cast<uint32_t *>(st->prep_d + off_counts), d_palette_bytes, stream, ev,
                       ctx_timed_names(ctx));
  ctx_set_timed(ctx, ev ? 3 : 0, 3);
  if (e != cudaSuccess) return cuda_status(e);
  cudaEventRecord(st->prep_done, stream);
  st->prep_used = true;
  return GST_OK;
}

struct ReIn {
  uint32_t width, height;
  const uint8_t *rgb;
  const uint64_t *blocks;
  uint64_t *blocks_out;
  uint8_t *palette, *deltas;
  uint32_t *palette_bytes;
};

constexpr uint64_t kReMaxBlocks = 1ull << 24;  // a 16384 x 16384 image: 6.4 GB of scores

bool reencode_dims_ok(uint32_t w, uint32_t h) {
  return w && h && !(w & 3u) && !(h & 3u) && uint64_t(w / 4) * (h / 4) <= kReMaxBlocks;
}

// Builds and launches the palette search of one call (gst_reencode.cu).
gst_status reencode_locked(gst_ctx *ctx, EncodeState *st, const std::vector<ReIn> &imgs, cudaStream_t stream) {
  const uint32_t n = static_cast<uint32_t>(imgs.size());
  for (const ReIn &im : imgs) {
    if (!reencode_dims_ok(im.width, im.height)) return GST_E_ARG;
    if (!im.rgb || !im.blocks || !im.blocks_out || !im.palette || !im.deltas || !im.palette_bytes) return GST_E_ARG;
    if (reinterpret_cast<uintptr_t>(im.rgb) % 4 || reinterpret_cast<uintptr_t>(im.blocks) % 8 ||
        reinterpret_cast<uintptr_t>(im.blocks_out) % 8 || reinterpret_cast<uintptr_t>(im.palette) % 16 ||
        reinterpret_cast<uintptr_t>(im.palette_bytes) % 4)
      return GST_E_ARG;
  }
  const size_t off_order = align_up(n * sizeof(ReImage), 16);
  const size_t off_states = align_up(off_order + n * sizeof(uint32_t), 16);
  size_t off = align_up(off_states + n * sizeof(ReState), 256);
  std::vector<size_t> at(n);
  uint32_t max_blocks = 0;
  std::vector<uint32_t> chunks(n);
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t B = (imgs[i].width / 4) * (imgs[i].height / 4);
    max_blocks = std::max(max_blocks, B);
    chunks[i] = (B + kReChunk - 1) / kReChunk;
    at[i] = off;
    off = align_up(off + size_t(B) * kReRow, 256);
    off += 3 * align_up(size_t(B) * sizeof(uint32_t), 256);  // pal_src, pal_before, idx
    off += size_t(B) * kReInfo * 16;                         // info
    off += align_up(size_t(B) * kReGroupsPerBlock * 4, 256);  // masks
  }
  if (st->re_used) {
    const cudaError_t e = cudaEventSynchronize(st->re_done);
    if (e != cudaSuccess) return cuda_status(e);
  }
  gst_status r = grow_host(&st->re_h, &st->re_h_cap, off_states);
  if (r == GST_OK) r = grow_dev(&st->re_d, &st->re_d_cap, off);
  if (r != GST_OK) return r;
  ReImage *ri = reinterpret_cast<ReImage *>(st->re_h);
  uint32_t *order = reinterpret_cast<uint32_t *>(st->re_h + off_order);
  for (uint32_t i = 0; i < n; ++i) {
    const ReIn &im = imgs[i];
    const uint32_t B = (im.width / 4) * (im.height / 4);
    uint8_t *base = st->re_d + at[i];
    uint8_t *maps = st->re_d + align_up(at[i] + size_t(B) * kReRow, 256);
    ReImage &d = ri[i];
    memset(&d, 0, sizeof(d));
    d.rgb = im.rgb;
    d.blocks_in = im.blocks;
    d.blocks_out = im.blocks_out;
    d.palette = im.palette;
    d.deltas = im.deltas;
    d.palette_bytes = im.palette_bytes;
    d.scores = base;
    d.pal_src = reinterpret_cast<uint32_t *>(maps);
    d.pal_before = reinterpret_cast<uint32_t *>(maps + align_up(size_t(B) * 4, 256));
    d.idx = reinterpret_cast<uint32_t *>(maps + 2 * align_up(size_t(B) * 4, 256));
    d.info = reinterpret_cast<uint4 *>(maps + 3 * align_up(size_t(B) * 4, 256));
    d.masks = reinterpret_cast<uint32_t *>(maps + 3 * align_up(size_t(B) * 4, 256) + size_t(B) * kReInfo * 16);
    d.width = im.width;
    d.bw = im.width / 4;
    d.B = B;
    d.n_chunks = chunks[i];
    d.pal_cap = static_cast<uint32_t>(std::min<uint64_t>(palette_capacity(im.width, im.height), 0xFFFFFFFFu));
    order[i] = i;
  }
  std::stable_sort(order, order + n, [&](uint32_t a, uint32_t b) { return chunks[a] > chunks[b]; });
  std::vector<uint32_t> desc(n);
  for (uint32_t i = 0; i < n; ++i) desc[i] = chunks[order[i]];
  cudaError_t e = cudaMemcpyAsync(st->re_d, st->re_h, off_states, cudaMemcpyHostToDevice, stream);
  int nl = 0;
  if (e == cudaSuccess)
    e = launch_reencode(reinterpret_cast<const ReImage *>(st->re_d),
                        reinterpret_cast<const uint32_t *>(st->re_d + off_order),
                        reinterpret_cast<ReState *>(st->re_d + off_states), n, desc.data(), max_blocks,
                        ctx_status(ctx), stream, &nl);
  if (e != cudaSuccess) return cuda_status(e);
  st->last_launches = nl;
  cudaEventRecord(st->re_done, stream);
  st->re_used = true;
  return GST_OK;
}

}  // namespace
}  // namespace host
}  // namespace gst

using namespace gst;
using namespace gst::host;

extern "C" {

size_t gst_encode_section_bound(size_t n) {
  if (n == 0 || n % kSymsPerGroup) return 0;
  return static_cast<size_t>(section_bound(n));
}

size_t gst_encode_stream_bound(uint32_t width, uint32_t height, uint32_t palette_bytes) {
  if (!stream_dims_ok(width, height, palette_bytes)) return 0;
  const uint64_t B = uint64_t(width / 4) * (height / 4);
  return static_cast<size_t>(kHeaderBytes + section_bound(2 * B) + section_bound(4 * B) +
                             section_bound(palette_bytes) + section_bound(B));
}

gst_status gst_encode_bytes(gst_ctx *ctx, int n, const void *const *d_symbols, const size_t *n_symbols, void *d_out,
                            size_t out_cap, unsigned long long *d_offsets, void *stream) {
  if (!ctx || n <= 0 || !d_symbols || !n_symbols) return GST_E_ARG;
  std::vector<SectionIn> secs(n);
  std::vector<UnitIn> units(n);
  for (int i = 0; i < n; ++i) {
    secs[i] = {static_cast<const uint8_t *>(d_symbols[i]), n_symbols[i]};
    units[i] = {false, 0, 0, 0, static_cast<uint32_t>(i), 1};
  }
  std::lock_guard<std::mutex> lock(ctx_mutex(ctx));
  cudaSetDevice(ctx_device(ctx));
  EncodeState *st = nullptr;
  gst_status r = get_state(ctx, &st);
  if (r != GST_OK) return r;
  return encode_locked(ctx, st, secs, units, static_cast<uint8_t *>(d_out), out_cap, d_offsets,
                       static_cast<cudaStream_t>(stream));
}

gst_status gst_encode_streams(gst_ctx *ctx, const gst_stream_symbols *imgs, int n, void *d_out, size_t out_cap,
                              unsigned long long *d_offsets, void *stream) {
  if (!ctx || n <= 0 || !imgs) return GST_E_ARG;
  std::vector<SectionIn> secs;
  std::vector<UnitIn> units;
  secs.reserve(4 * size_t(n));
  for (int i = 0; i < n; ++i) {
    const gst_stream_symbols &im = imgs[i];
    if (!stream_dims_ok(im.width, im.height, im.palette_bytes)) return GST_E_ARG;
    const uint64_t B = uint64_t(im.width / 4) * (im.height / 4);
    units.push_back({true, im.width, im.height, im.palette_bytes, static_cast<uint32_t>(secs.size()), 4});
    secs.push_back({static_cast<const uint8_t *>(im.d_y), 2 * B});
    secs.push_back({static_cast<const uint8_t *>(im.d_chroma), 4 * B});
    secs.push_back({static_cast<const uint8_t *>(im.d_palette), im.palette_bytes});
    secs.push_back({static_cast<const uint8_t *>(im.d_indices), B});
  }
  std::lock_guard<std::mutex> lock(ctx_mutex(ctx));
  cudaSetDevice(ctx_device(ctx));
  EncodeState *st = nullptr;
  gst_status r = get_state(ctx, &st);
  if (r != GST_OK) return r;
  return encode_locked(ctx, st, secs, units, static_cast<uint8_t *>(d_out), out_cap, d_offsets,
                       static_cast<cudaStream_t>(stream));
}

gst_status gst_compress_symbols(gst_ctx *ctx, uint32_t width, uint32_t height, uint32_t palette_bytes,
                                const uint8_t *symbols, uint8_t *gst_out, size_t out_cap, size_t *out_len) {
  if (!ctx || !symbols || !gst_out || !out_len) return GST_E_ARG;
  if (!stream_dims_ok(width, height, palette_bytes)) return GST_E_ARG;
  const uint64_t B = uint64_t(width / 4) * (height / 4);
  const size_t nsym = static_cast<size_t>(7 * B + palette_bytes);
  const size_t bound = gst_encode_stream_bound(width, height, palette_bytes);
  std::lock_guard<std::mutex> lock(ctx_mutex(ctx));
  cudaSetDevice(ctx_device(ctx));
  EncodeState *st = nullptr;
  gst_status r = get_state(ctx, &st);
  if (r != GST_OK) return r;
  if (st->used) {
    const cudaError_t e = cudaEventSynchronize(st->done);
    if (e != cudaSuccess) return cuda_status(e);
  }
  r = grow_dev(&st->in_d, &st->in_cap, nsym);
  if (r == GST_OK) r = grow_dev(&st->out_d, &st->out_cap, bound);
  if (r != GST_OK) return r;
  cudaError_t e = cudaMemcpyAsync(st->in_d, symbols, nsym, cudaMemcpyHostToDevice, st->own);
  if (e != cudaSuccess) return cuda_status(e);
  const uint8_t *d = st->in_d;
  std::vector<SectionIn> secs = {{d, 2 * B}, {d + 2 * B, 4 * B}, {d + 6 * B, palette_bytes},
                                 {d + 6 * B + palette_bytes, B}};
  std::vector<UnitIn> units = {{true, width, height, palette_bytes, 0, 4}};
  r = encode_locked(ctx, st, secs, units, st->out_d, st->out_cap, st->offsets_d, st->own);
  if (r != GST_OK) return r;
  r = read_device_status(ctx, st->own);
  if (r != GST_OK) return r;
  unsigned long long off[2] = {0, 0};
  e = cudaMemcpy(off, st->offsets_d, sizeof(off), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  const size_t len = static_cast<size_t>(off[1] - off[0]);
  if (len > out_cap) return GST_E_ARG;
  e = cudaMemcpy(gst_out, st->out_d + off[0], len, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  *out_len = len;
  return GST_OK;
}

size_t gst_palette_capacity(uint32_t width, uint32_t height) {
  if (!stream_dims_ok(width, height, kSymsPerGroup)) return 0;
  return static_cast<size_t>(palette_capacity(width, height));
}

gst_status gst_prepare_symbols(gst_ctx *ctx, const gst_symbol_buffers *imgs, int n, uint32_t *d_palette_bytes,
                               void *stream) {
  if (!ctx || !imgs || n <= 0) return GST_E_ARG;
  std::vector<PrepIn> in(n);
  for (int i = 0; i < n; ++i)
    in[i] = {imgs[i].width, imgs[i].height, static_cast<const uint8_t *>(imgs[i].d_blocks),
             static_cast<uint8_t *>(imgs[i].d_y), static_cast<uint8_t *>(imgs[i].d_chroma),
             static_cast<uint8_t *>(imgs[i].d_palette), static_cast<uint8_t *>(imgs[i].d_indices)};
  std::lock_guard<std::mutex> lock(ctx_mutex(ctx));
  cudaSetDevice(ctx_device(ctx));
  EncodeState *st = nullptr;
  const gst_status r = get_state(ctx, &st);
  if (r != GST_OK) return r;
  return prepare_locked(ctx, st, in, d_palette_bytes, static_cast<cudaStream_t>(stream));
}

gst_status gst_compress_dxt(gst_ctx *ctx, uint32_t width, uint32_t height, const uint64_t *blocks, uint8_t *gst_out,
                            size_t out_cap, size_t *out_len) {
  if (!ctx || !blocks || !gst_out || !out_len) return GST_E_ARG;
  if (!stream_dims_ok(width, height, kSymsPerGroup)) return GST_E_ARG;
  const uint64_t B = uint64_t(width / 4) * (height / 4);
  const uint64_t pal_cap = palette_capacity(width, height);
  std::lock_guard<std::mutex> lock(ctx_mutex(ctx));
  cudaSetDevice(ctx_device(ctx));
  EncodeState *st = nullptr;
  gst_status r = get_state(ctx, &st);
  if (r != GST_OK) return r;
  for (cudaEvent_t ev : {st->done, st->prep_done}) {
    const cudaError_t e = cudaEventSynchronize(ev);
    if (e != cudaSuccess) return cuda_status(e);
  }
  // device symbol buffer: Y 2B | chroma 4B | indices B | palette (capacity)
  const size_t sym_bytes = static_cast<size_t>(7 * B + pal_cap);
  const size_t bound = gst_encode_stream_bound(width, height, static_cast<uint32_t>(std::min<uint64_t>(pal_cap, 0xFFFFE000u)));
  r = grow_dev(&st->blocks_d, &st->blocks_cap, static_cast<size_t>(8 * B));
  if (r == GST_OK) r = grow_dev(&st->in_d, &st->in_cap, sym_bytes);
  if (r == GST_OK) r = grow_dev(&st->out_d, &st->out_cap, bound);
  if (r != GST_OK) return r;
  cudaError_t e = cudaMemcpyAsync(st->blocks_d, blocks, static_cast<size_t>(8 * B), cudaMemcpyHostToDevice, st->own);
  if (e != cudaSuccess) return cuda_status(e);
  uint8_t *d = st->in_d;
  const std::vector<PrepIn> in = {{width, height, st->blocks_d, d, d + 2 * B, d + 7 * B, d + 6 * B}};
  r = prepare_locked(ctx, st, in, st->pal_bytes_d, st->own);
  if (r != GST_OK) return r;
  uint32_t pal_bytes = 0;
  e = cudaMemcpyAsync(&pal_bytes, st->pal_bytes_d, sizeof(pal_bytes), cudaMemcpyDeviceToHost, st->own);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st->own);
  if (e != cudaSuccess) return cuda_status(e);
  if (pal_bytes == 0 || pal_bytes > pal_cap) return GST_E_CUDA;
  std::vector<SectionIn> secs = {{d, 2 * B}, {d + 2 * B, 4 * B}, {d + 7 * B, pal_bytes}, {d + 6 * B, B}};
  std::vector<UnitIn> units = {{true, width, height, pal_bytes, 0, 4}};
  r = encode_locked(ctx, st, secs, units, st->out_d, st->out_cap, st->offsets_d, st->own);
  if (r != GST_OK) return r;
  r = read_device_status(ctx, st->own);
  if (r != GST_OK) return r;
  unsigned long long off[2] = {0, 0};
  e = cudaMemcpy(off, st->offsets_d, sizeof(off), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  const size_t len = static_cast<size_t>(off[1] - off[0]);
  if (len > out_cap) return GST_E_ARG;
  e = cudaMemcpy(gst_out, st->out_d + off[0], len, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  *out_len = len;
  return GST_OK;
}

gst_status gst_encode_normalize(gst_ctx *ctx, const uint32_t *counts, int n, uint32_t *freqs) {
  if (!ctx || !counts || !freqs || n <= 0 || n > 256) return GST_E_ARG;
  uint32_t c[256] = {0};
  bool any = false;
  for (int i = 0; i < n; ++i) {
    c[i] = counts[i];
    any = any || counts[i];
  }
  if (!any) return GST_E_ARG;
  std::lock_guard<std::mutex> lock(ctx_mutex(ctx));
  cudaSetDevice(ctx_device(ctx));
  EncodeState *st = nullptr;
  gst_status r = get_state(ctx, &st);
  if (r != GST_OK) return r;
  if (st->used) {
    const cudaError_t e = cudaEventSynchronize(st->done);
    if (e != cudaSuccess) return cuda_status(e);
  }
  r = grow_dev(&st->scratch_d, &st->scratch_cap, 256 * 4 + 256 * 16 + 256 * 2);
  if (r != GST_OK) return r;
  cudaError_t e = cudaMemcpyAsync(st->scratch_d, c, sizeof(c), cudaMemcpyHostToDevice, st->own);
  if (e != cudaSuccess) return cuda_status(e);
  EncPlanView v = {};
  v.counts = reinterpret_cast<uint32_t *>(st->scratch_d);
  v.tables = reinterpret_cast<uint4 *>(st->scratch_d + 256 * 4);
  v.freqs = reinterpret_cast<uint16_t *>(st->scratch_d + 256 * 4 + 256 * 16);
  v.log2_plus = st->log2_d;
  v.log2_minus = st->log2_d + kEncLogTableLen;
  v.err = ctx_status(ctx);
  v.stall_group = ~0u;
  v.n_sections = 1;
  e = launch_encode(v, st->sm_count, st->own, true, &st->last_launches);
  if (e != cudaSuccess) return cuda_status(e);
  r = read_device_status(ctx, st->own);
  if (r == GST_E_FORMAT) return GST_E_ARG;  // nothing could move (the reference asserts)
  if (r != GST_OK) return r;
  uint16_t f[256];
  e = cudaMemcpy(f, v.freqs, sizeof(f), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  for (int i = 0; i < n; ++i) freqs[i] = f[i];
  return GST_OK;
}

gst_status gst_reencode_blocks(gst_ctx *ctx, const gst_reencode_image *imgs, int n, void *stream) {
  if (!ctx || !imgs || n <= 0 || n > 65535) return GST_E_ARG;  // images are grid.y of every launch
  std::vector<ReIn> in(n);
  for (int i = 0; i < n; ++i)
    in[i] = {imgs[i].width,
             imgs[i].height,
             static_cast<const uint8_t *>(imgs[i].d_rgb),
             static_cast<const uint64_t *>(imgs[i].d_blocks),
             static_cast<uint64_t *>(imgs[i].d_blocks_out),
             static_cast<uint8_t *>(imgs[i].d_palette),
             static_cast<uint8_t *>(imgs[i].d_indices),
             imgs[i].d_palette_bytes};
  std::lock_guard<std::mutex> lock(ctx_mutex(ctx));
  cudaSetDevice(ctx_device(ctx));
  EncodeState *st = nullptr;
  const gst_status r = get_state(ctx, &st);
  if (r != GST_OK) return r;
  return reencode_locked(ctx, st, in, static_cast<cudaStream_t>(stream));
}

gst_status gst_prepare_planes(gst_ctx *ctx, const gst_symbol_buffers *imgs, int n, void *stream) {
  if (!ctx || !imgs || n <= 0) return GST_E_ARG;
  std::vector<PrepIn> in(n);
  for (int i = 0; i < n; ++i)
    in[i] = {imgs[i].width, imgs[i].height, static_cast<const uint8_t *>(imgs[i].d_blocks),
             static_cast<uint8_t *>(imgs[i].d_y), static_cast<uint8_t *>(imgs[i].d_chroma), nullptr, nullptr};
  std::lock_guard<std::mutex> lock(ctx_mutex(ctx));
  cudaSetDevice(ctx_device(ctx));
  EncodeState *st = nullptr;
  const gst_status r = get_state(ctx, &st);
  if (r != GST_OK) return r;
  return prepare_locked(ctx, st, in, nullptr, static_cast<cudaStream_t>(stream), true);
}

gst_status gst_compress_rgb_dxt(gst_ctx *ctx, uint32_t width, uint32_t height, const uint8_t *rgb,
                                const uint64_t *blocks, uint8_t *gst_out, size_t out_cap, size_t *out_len) {
  if (!ctx || !rgb || !blocks || !gst_out || !out_len) return GST_E_ARG;
  if (!stream_dims_ok(width, height, kSymsPerGroup) || !reencode_dims_ok(width, height)) return GST_E_ARG;
  const uint64_t B = uint64_t(width / 4) * (height / 4);
  const uint64_t pal_cap = palette_capacity(width, height);
  std::lock_guard<std::mutex> lock(ctx_mutex(ctx));
  cudaSetDevice(ctx_device(ctx));
  EncodeState *st = nullptr;
  gst_status r = get_state(ctx, &st);
  if (r != GST_OK) return r;
  for (cudaEvent_t ev : {st->done, st->prep_done, st->re_done}) {
    const cudaError_t e = cudaEventSynchronize(ev);
    if (e != cudaSuccess) return cuda_status(e);
  }
  // device symbol buffer: Y 2B | chroma 4B | indices B | palette (capacity)
  const size_t sym_bytes = static_cast<size_t>(7 * B + pal_cap);
  const size_t rgb_bytes = static_cast<size_t>(width) * height * 3;
  const size_t bound =
      gst_encode_stream_bound(width, height, static_cast<uint32_t>(std::min<uint64_t>(pal_cap, 0xFFFFE000u)));
  r = grow_dev(&st->blocks_d, &st->blocks_cap, static_cast<size_t>(8 * B));
  if (r == GST_OK) r = grow_dev(&st->blocks2_d, &st->blocks2_cap, static_cast<size_t>(8 * B));
  if (r == GST_OK) r = grow_dev(&st->rgb_d, &st->rgb_cap, rgb_bytes);
  if (r == GST_OK) r = grow_dev(&st->in_d, &st->in_cap, sym_bytes);
  if (r == GST_OK) r = grow_dev(&st->out_d, &st->out_cap, bound);
  if (r != GST_OK) return r;
  cudaError_t e = cudaMemcpyAsync(st->blocks_d, blocks, static_cast<size_t>(8 * B), cudaMemcpyHostToDevice, st->own);
  if (e == cudaSuccess) e = cudaMemcpyAsync(st->rgb_d, rgb, rgb_bytes, cudaMemcpyHostToDevice, st->own);
  if (e != cudaSuccess) return cuda_status(e);
  uint8_t *d = st->in_d;
  const std::vector<ReIn> re = {{width, height, st->rgb_d, reinterpret_cast<const uint64_t *>(st->blocks_d),
                                 reinterpret_cast<uint64_t *>(st->blocks2_d), d + 7 * B, d + 6 * B, st->pal_bytes_d}};
  r = reencode_locked(ctx, st, re, st->own);
  if (r != GST_OK) return r;
  const std::vector<PrepIn> in = {{width, height, st->blocks2_d, d, d + 2 * B, nullptr, nullptr}};
  r = prepare_locked(ctx, st, in, nullptr, st->own, true);
  if (r != GST_OK) return r;
  uint32_t pal_bytes = 0;
  e = cudaMemcpyAsync(&pal_bytes, st->pal_bytes_d, sizeof(pal_bytes), cudaMemcpyDeviceToHost, st->own);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st->own);
  if (e != cudaSuccess) return cuda_status(e);
  r = read_device_status(ctx, st->own);
  if (r != GST_OK) return r;
  if (pal_bytes == 0 || pal_bytes > pal_cap) return GST_E_CUDA;
  std::vector<SectionIn> secs = {{d, 2 * B}, {d + 2 * B, 4 * B}, {d + 7 * B, pal_bytes}, {d + 6 * B, B}};
  std::vector<UnitIn> units = {{true, width, height, pal_bytes, 0, 4}};
  r = encode_locked(ctx, st, secs, units, st->out_d, st->out_cap, st->offsets_d, st->own);
  if (r != GST_OK) return r;
  r = read_device_status(ctx, st->own);
  if (r != GST_OK) return r;
  unsigned long long off[2] = {0, 0};
  e = cudaMemcpy(off, st->offsets_d, sizeof(off), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  const size_t len = static_cast<size_t>(off[1] - off[0]);
  if (len > out_cap) return GST_E_ARG;
  e = cudaMemcpy(gst_out, st->out_d + off[0], len, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  *out_len = len;
  return GST_OK;
}

}  // extern "C"
