// gst_plan.h -- the per-call work plan the host builds and the kernels read.
//
// One decode call covers N images (the reference's LoadCompressedDXTs,
// codec/decoder.cpp:98-428), possibly of different sizes.  The host turns the
// N headers into:
//   * one GstImageDesc per image: where its frequency tables and sections are
//     in the compressed buffer (offsets as codec/decoder.cpp:132-149 computes
//     them), where its decoded symbols and index prefixes go in scratch, and
//     where its DXT1 blocks go in the output;
//   * the rANS work list: one item per (image, section, run of <= 4 groups of
//     32 x 256 symbols) -- a CTA of 4 warps, one warp per group;
//   * the tile work list: one item per (image, 32x32-block wavelet tile).
// The plan is copied to the device in one cudaMemcpyAsync; it also carries the
// per-image counters and error words, so the copy resets them for every call.
#pragma once

#include <stdint.h>

namespace gst {

constexpr uint32_t kTableSize = 2048;         // M = 2^11           ans/ans.h:73
constexpr uint32_t kSymsPerStream = 256;      //                    ans/ans.h:74
constexpr uint32_t kStreamsPerGroup = 32;     //                    ans/ans.h:75
constexpr uint32_t kSymsPerGroup = 8192;
constexpr uint32_t kGroupsPerRansCta = 4;
// rANS staging depth per warp, in 16-bit words (a multiple of 8, so that every
// warp's stage starts 16-byte aligned).  Sixteen steps read at most 512 words
// and a re-stage starts at most one word above the read pointer, so 520 words
// always cover the next sixteen steps; 2816 keeps seven CTAs per SM.
constexpr uint32_t kMinStageWords = 520, kMaxStageWords = 4352, kDefaultStageWords = 1016;

// Launch configuration of a decode.
constexpr int kSizeClasses = 7;  // launch size classes: up to 2^14 blocks, then x4 each, the last open-ended

struct GstTuning {
  int blocks_per_sm = 12;                      // rANS register budget: 8, 12 or 16 CTAs of 128 threads per SM
  uint32_t stage_words = kDefaultStageWords;  // staging depth
  int persistent = 0;                          // 1: one persistent kernel drains the whole plan
  bool operator==(const GstTuning &o) const {
    return blocks_per_sm == o.blocks_per_sm && stage_words == o.stage_words && persistent == o.persistent;
  }
  bool operator!=(const GstTuning &o) const { return !(*this == o); }
};
constexpr uint32_t kRansL = 1u << 15;         // k * M, k = 2^4      ans/ans_ocl_encode.cpp:15-16
constexpr uint32_t kFreqTableBytes = 512;
constexpr uint32_t kWaveletDim = 32;          //                    codec/codec_base.h:22

// Device error bits (GstPlanView::err).
constexpr uint32_t kErrTable = 1u;       // a frequency table does not sum to 2048
constexpr uint32_t kErrGroup = 2u;       // a group end offset is out of order or range
constexpr uint32_t kErrStream = 4u;      // a renormalisation read left its group
constexpr uint32_t kErrPalette = 8u;     // a palette index is outside the palette
constexpr uint32_t kErrTimeout = 16u;    // a bounded wait of the persistent kernel gave up
constexpr uint32_t kErrReencode = 32u;   // the palette search's decision and selection passes disagree

struct alignas(16) GstImageDesc {
  uint64_t freq_off;    // bytes from the compressed base to this image's 4 tables
  uint64_t body_off;    // bytes from the compressed base to its first section body
  uint64_t sym_off;     // scratch: decoded symbols, 8*B + palette_bytes (index section 2 B/block)
  uint64_t out_off;     // output: DXT1 blocks, 8*B bytes
  uint64_t chunk_off;   // scratch: int32 exclusive prefix per 32-block chunk, B/32
  uint64_t gsum_off;    // scratch: int32 index-group sums, then their exclusive prefix
  uint32_t sec_in[4];   // section body offsets from body_off (Y, chroma, palette, indices)
  uint32_t sec_len[4];  // section body bytes (header *_cmp_sz / *_sz)
  uint32_t sec_groups[4];
  uint32_t sec_out[4];  // decoded-symbol offsets from sym_off: 0, 2B, 6B, 6B + palette_bytes
  uint32_t bx, by;      // blocks across / down
  uint32_t palette_words;
  uint32_t tiles_x;     // bx / 32
};
static_assert(sizeof(GstImageDesc) == 128, "descriptor layout");

struct GstRansItem {
  uint32_t image;
  uint32_t section;      // 0 Y, 1 chroma, 2 palette, 3 indices
  uint32_t first_group;
  uint16_t ngroups;      // <= kGroupsPerRansCta
  uint16_t streams;      // interleaved streams per group, 1..32 (32 in GST streams)
};

struct GstTileItem {
  uint32_t image;
  uint32_t tile;
};

struct alignas(16) GstPlanHead {
  uint32_t n_images;
  uint32_t n_rans;
  uint32_t n_tiles;
  uint32_t reserved;
};

// Device-side view of an uploaded plan.
struct GstPlanView {
  uint32_t *err;  // the context's device status word (error bits, OR-ed)
  const GstImageDesc *images;
  const GstRansItem *rans;
  const GstTileItem *tiles;
  uint32_t *counters;   // one per image (index-group completion count)
  uint32_t *image_err;  // one per image (error bits), or null
  const uint32_t *rans_order;  // the rANS kernel's CTA b takes rans[rans_order[b]] (null: rans[b])
  // Persistent kernel (may be null otherwise): [0] work-queue head, [1] CTAs
  // finished, [4 + i] groups of image i decoded.  Every launch leaves them 0.
  uint32_t *sync;
  uint64_t wait_limit_ns;  // bound of a persistent tile's wait for its image (0: 2 s)
  uint32_t n_images;
  uint32_t rgb;  // 1: the tiles write RGB8 pixels (48 bytes per block) instead of DXT1
  uint32_t n_rans, n_tiles;
  uint32_t stage_words;  // rANS staging depth per warp, in 16-bit words
};

}  // namespace gst
