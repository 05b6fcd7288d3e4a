// gst_encode_plan.h -- device-visible plan of one GPU encode call (shared by
// gst_encode.cu and gst_encode_api.cpp).  Internal to the library.
//
// An encode call takes S sections of symbols (each a positive multiple of
// 8192 bytes) grouped into U units.  A unit is either one ByteEncoder section
// (codec/entropy.cpp:174-265: 512-byte frequency table, u32 group end offsets,
// groups) or one GST stream of four sections (codec/encoder.cpp:122-144:
// 28-byte header, the four frequency tables, then the four section bodies).
// Units are written back to back.  Every group of every section gets a global
// index in output order; a group's bytes land at
//     out + section.grp_fixed + (bytes of all groups before it),
// the last term coming from the encode kernel's decoupled look-back over group
// sizes, so the whole output is placed in one pass.
#pragma once

#include <stddef.h>
#include <stdint.h>
#include <vector_types.h>

namespace gst {

constexpr uint32_t kHeaderBytes = 28;         // GenTCHeader, codec/codec_base.h:9-20
constexpr uint32_t kEncMaxWords = 8192;       // 16-bit words per group: at most one per symbol
constexpr uint32_t kEncHistChunk = 32768;     // symbols per histogram CTA
constexpr uint32_t kEncLogTableLen = 2050;    // log2(n / (n +- 1)) for n in [0, 2049]
constexpr uint32_t kEncMaxGroupBytes = 2 * kEncMaxWords + 2 + 4 * 32;

struct EncSection {
  const uint8_t *sym;   // the section's symbols (16-byte aligned)
  uint64_t grp_fixed;   // fixed bytes before the section's first group (see above)
  uint64_t tbl_fixed;   // frequency table at out + tbl_fixed + (group bytes before group tbl_group)
  uint32_t n_groups;
  uint32_t first_group;
  uint32_t tbl_group;
  uint32_t unit;
};

struct EncUnit {
  uint64_t fixed_before;  // fixed bytes of all earlier units
  uint64_t fixed_bytes;   // this unit's own fixed bytes (header, tables, group offsets)
  uint32_t first_group, end_group;
  uint32_t first_section, n_sections;
  uint32_t width, height, palette_bytes;
  uint32_t is_stream;  // 1: GST stream of four sections; 0: one ByteEncoder section
};

struct EncChunk {
  uint32_t section, start, len;  // len: a multiple of 8192
};

// Endpoint stages (gst_prepare.cu): one image's DXT1 blocks in, its four
// symbol sections out.
struct EncPrepImage {
  const uint64_t *blocks;  // width * height / 16 blocks, raster order
  uint8_t *y, *chroma, *palette, *indices;
  uint32_t width, height;
  uint32_t first_tile;  // tiles of earlier images
  uint32_t pad;
};

// Index palette search (DXTImage::Reencode, codec/dxt_image.cpp:510-624).
// Blocks are decided kReChunk at a time: every block of a chunk is first
// scored against the window at the chunk's start (the last 127 palette
// words) and against the chunk's earlier blocks, then one warp walks the
// chunk in order and decides which blocks append their word.
constexpr uint32_t kReWindow = 127;    // palette words a block may reuse (dxt_image.cpp:509, 562)
constexpr uint32_t kReThreshold = 35;  // largest error increase + 1 of a reuse (dxt_image.cpp:508, 597)
constexpr uint32_t kReChunk = 256;
constexpr uint32_t kReRow = 128 + kReChunk;  // score row: window slots 0..126, a pad byte, chunk slots
constexpr uint32_t kReInfo = 6;              // uint4 per block of ReImage::info
constexpr uint32_t kReGroupsPerBlock = 4 + kReChunk / 32;  // 32-slot groups of a score row

struct ReImage {
  const uint8_t *rgb;        // width * height * 3 bytes, 4-byte aligned
  const uint64_t *blocks_in;  // the given blocks, raster order
  uint64_t *blocks_out;       // the blocks after the search
  uint8_t *palette;           // palette words (capacity pal_cap bytes), 16-byte aligned
  uint8_t *deltas;            // B index deltas + 128
  uint32_t *palette_bytes;    // the padded palette size (device u32)
  uint8_t *scores;            // B rows of kReRow bytes: min(max(error increase, 0), 35), 35 = not usable
  uint32_t *pal_src;          // palette index -> the block that appended it
  uint32_t *pal_before;       // block -> palette size before it
  uint32_t *idx;              // block -> its palette index
  uint32_t *masks;            // per block kReGroupsPerBlock words: bit s of word g = slot 32g + s scores
                              // below 35 (window slots in words 0-3, chunk slots in words 4-11)
  uint4 *info;                // per block kReInfo uint4: its 16 pixels (0x00BBGGRR), then {word,
                              // asq, bsq, ab} and {1 / (asq bsq - ab ab), error as given, 0, 0}
  uint32_t width, bw, B, n_chunks;
  uint32_t pal_cap;
  uint32_t pad[3];
};

struct ReState {  // per image, device
  uint32_t P;       // palette words so far
  uint32_t arrive;  // scoring CTAs of the current step that are done
  uint32_t pad[2];
};

struct EncPrepChunk {  // 8192 blocks (or the image's rest) in raster order
  uint32_t image, start, len;
  uint32_t first_chunk, last_chunk;  // the image's chunks
};

// Look-back status word of a group: flag in bits 62-63, byte count below.
constexpr uint64_t kEncFlagAggregate = 1ull << 62;
constexpr uint64_t kEncFlagInclusive = 2ull << 62;
constexpr uint64_t kEncValueMask = (1ull << 62) - 1;

struct EncPlanView {
  const EncSection *sections;
  const EncUnit *units;
  const EncChunk *chunks;
  const uint32_t *group_section;
  // scratch, zeroed before each call: counts, status, ticket
  uint32_t *counts;               // [S][256]
  unsigned long long *status;     // [G]
  uint32_t *ticket;
  // scratch written by the kernels
  uint4 *tables;                  // [S][256] encode entries
  uint16_t *freqs;                // [S][256] normalised frequencies
  const double *log2_plus;        // log2(n / (n + 1)), n in [0, 2049]
  const double *log2_minus;       // log2(n / (n - 1)), n in [0, 2049] (n = 0, 1 unused)
  uint8_t *out;
  unsigned long long *offsets;    // [U + 1]: unit starts, then the total
  uint32_t *err;
  uint64_t wait_limit_ns;
  uint32_t n_sections, n_units, n_groups, n_chunks;
  uint32_t stall_group;  // fault injection for tests: this group never publishes its size (~0u: none)
};

}  // namespace gst
