/*
 * gst_encode.h -- C ABI of the GB300 GST encoder stages (symbols -> GST
 * sections and streams).  Same library and context as gst_decoder.h.
 *
 * The reference runs these stages on the host, one section at a time:
 *
 *   reference                                       this header
 *   ----------------------------------------------  -------------------------
 *   ans::ocl::NormalizeFrequencies                  gst_encode_normalize
 *     (ans/ans_ocl_encode.cpp:6-8 = ans::GenerateHistogram at M = 2048,
 *     ans/histogram.cpp:40-121)
 *   ByteEncoder::EncodeBytes::Run                   gst_encode_bytes
 *     (codec/entropy.cpp:174-265: byte counts, normalisation,
 *     ans::EncodeInterleaved ans/encode.cpp:224-259 per 8192-symbol group,
 *     group end offsets)
 *   the section and stream assembly of              gst_encode_streams,
 *     GenTC::CompressDXTImage                       gst_compress_symbols
 *     (codec/encoder.cpp:69-145, after the
 *     wavelet and palette stages)
 *
 * Outputs are byte-identical to the reference's.  All sections of a call are
 * encoded by the same four kernel launches (counts, normalisation, rANS
 * encode, tables and offsets); units (sections or streams) are written back
 * to back from d_out and their start offsets, then the total, go to
 * d_offsets (device memory, n + 1 unsigned 64-bit values).  Symbol buffers
 * must be 16-byte aligned and hold a positive multiple of 8192 bytes (below
 * 2^31 per section); d_out must be 4-byte and d_offsets 8-byte aligned;
 * anything else returns GST_E_ARG before a launch.  The
 * calls are asynchronous on `stream` (a cudaStream_t passed as void*); a
 * bounded wait that gave up on the device is reported as GST_E_TIMEOUT by
 * gst_sync_status.  There is no CPU path: without a GPU the calls fail with
 * GST_E_CUDA.
 */
#ifndef GST_ENCODE_H
#define GST_ENCODE_H

#include <stddef.h>
#include <stdint.h>

#include "gst_decoder.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Upper bound of one encoded section of n symbols: 512 + 4G + G * 16514
 * bytes for G = n / 8192 groups (at most one 16-bit word per symbol, a
 * 2-byte pad and 32 final states per group).  0 if n is not a positive
 * multiple of 8192. */
size_t gst_encode_section_bound(size_t n_symbols);

/* Upper bound of one GST stream: the 28-byte header and the four sections
 * (Y planes 2B, chroma planes 4B, palette, index deltas B; B = w * h / 16).
 * 0 for dimensions the decoder would reject. */
size_t gst_encode_stream_bound(uint32_t width, uint32_t height, uint32_t palette_bytes);

/* ByteEncoder::EncodeBytes for n sections: section i is n_symbols[i] bytes
 * at d_symbols[i] (device).  d_offsets[i] receives section i's start in
 * d_out, d_offsets[n] the total; out_cap must cover the sum of the bounds. */
gst_status gst_encode_bytes(gst_ctx *ctx, int n, const void *const *d_symbols, const size_t *n_symbols, void *d_out,
                            size_t out_cap, unsigned long long *d_offsets, void *stream);

/* The four symbol sections of one image (device pointers), in the layout of
 * the decoder's decompressed-symbol buffer (codec/decoder.cpp:441-461). */
typedef struct gst_stream_symbols {
  uint32_t width, height;
  uint32_t palette_bytes; /* the padded palette: a multiple of 8192 */
  uint32_t reserved;      /* 0 */
  const void *d_y;        /* 2B bytes: the two Y planes           */
  const void *d_chroma;   /* 4B bytes: Co1, Cg1, Co2, Cg2 planes  */
  const void *d_palette;  /* palette_bytes                        */
  const void *d_indices;  /* B bytes: palette-index deltas + 128   */
} gst_stream_symbols;

/* GST streams of n images (codec/encoder.cpp:122-144): d_offsets[i] receives
 * stream i's start in d_out, d_offsets[n] the total; out_cap must cover the
 * sum of gst_encode_stream_bound. */
gst_status gst_encode_streams(gst_ctx *ctx, const gst_stream_symbols *imgs, int n, void *d_out, size_t out_cap,
                              unsigned long long *d_offsets, void *stream);

/* Blocking host-to-host form for one image: `symbols` holds 7B +
 * palette_bytes bytes in the decompressed-symbol layout (Y planes, chroma
 * planes, palette, index deltas); the stream goes to gst_out (out_cap at
 * least gst_encode_stream_bound) and its length to *out_len. */
gst_status gst_compress_symbols(gst_ctx *ctx, uint32_t width, uint32_t height, uint32_t palette_bytes,
                                const uint8_t *symbols, uint8_t *gst_out, size_t out_cap, size_t *out_len);

/* --- endpoint stages: DXT1 blocks -> symbol sections ----------------------
 *
 *   reference                                       this header
 *   ----------------------------------------------  -------------------------
 *   RunDXTEndpointPipeline + RGB565toYCoCg667 +     gst_prepare_symbols
 *     ImageSplit (codec/encoder.cpp:20-98;
 *     FWavelet2D, codec/image_processing.h:267-333)
 *   DXTImage::Reencode's index palette              gst_prepare_symbols (a
 *     (codec/dxt_image.cpp:510-624)                 different, parallel rule)
 *   GenTC::CompressDXTImage                         gst_compress_dxt
 *     (codec/encoder.cpp:39-180)
 *
 * The Y and chroma sections are the reference's, byte for byte.  The index
 * palette is not the reference's least-squares search (sequential over the
 * blocks, in floating point): a block whose 32-bit index word equals the
 * previous block's (raster order) reuses its entry, any other block appends
 * its word.  Blocks keep their endpoints and words, so the stream decodes to
 * the given blocks wherever their wavelet coefficients fit in 8 bits (they
 * wrap as in the reference otherwise). */

/* One image: w*h/16 DXT1 blocks in (8-byte aligned device memory, raster
 * order, {u16 ep1, u16 ep2, u32 indices}), its sections out (16-byte aligned
 * device memory). */
typedef struct gst_symbol_buffers {
  uint32_t width, height;
  const void *d_blocks;
  void *d_y;       /* 2B bytes                                    */
  void *d_chroma;  /* 4B bytes                                    */
  void *d_palette; /* gst_palette_capacity(width, height) bytes   */
  void *d_indices; /* B bytes                                     */
} gst_symbol_buffers;

/* 4B bytes rounded up to 8192: room for a palette of one word per block. */
size_t gst_palette_capacity(uint32_t width, uint32_t height);

/* The endpoint stages for n images; d_palette_bytes[i] (device u32) receives
 * image i's palette bytes (padded to a multiple of 8192), the palette_bytes of
 * its gst_stream_symbols. */
gst_status gst_prepare_symbols(gst_ctx *ctx, const gst_symbol_buffers *imgs, int n, uint32_t *d_palette_bytes,
                               void *stream);

/* Blocking host-to-host form for one image: DXT1 blocks -> GST stream
 * (out_cap at least gst_encode_stream_bound(width, height,
 * gst_palette_capacity(width, height))). */
gst_status gst_compress_dxt(gst_ctx *ctx, uint32_t width, uint32_t height, const uint64_t *blocks, uint8_t *gst_out,
                            size_t out_cap, size_t *out_len);

/* The Y and chroma sections alone (gst_prepare_symbols without the palette
 * stage; d_palette and d_indices are not used), for blocks whose palette and
 * index deltas come from gst_reencode_blocks. */
gst_status gst_prepare_planes(gst_ctx *ctx, const gst_symbol_buffers *imgs, int n, void *stream);

/* --- the reference's index palette search ----------------------------------
 *
 *   reference                                       this header
 *   ----------------------------------------------  -------------------------
 *   DXTImage::Reencode (codec/dxt_image.cpp:         gst_reencode_blocks
 *     510-624), run by the DXTImage(width, height,
 *     rgb, dxt) constructor (:455-468)
 *   GenTC::CompressDXTImage of that image           gst_compress_rgb_dxt
 *     (codec/encoder.cpp:39-180)
 *
 * Byte for byte the reference's results: each block, in raster order, tries
 * the last min(127, palette size) palette words, most recent first, refitting
 * its 16 source pixels to the word (least-squares endpoints snapped to
 * 5:6:5); the first refit that does not raise the block's error, else the one
 * of least raise, is taken if the raise is below 35, and the block then
 * carries the refit endpoints and that word; any other block keeps its own
 * endpoints and appends its word.  Float arithmetic is the reference's as
 * compiled for x86-64 (no fused multiply-add; a float -> int conversion of
 * NaN or of a value outside int32 gives INT32_MIN).
 *
 * The search is sequential through the palette, so one call decides 256
 * blocks of every image per kernel launch: an image of B blocks takes
 * ceil(B / 256) launches, and images of a call run side by side.  It keeps
 * 540 bytes of scratch per block on the device (the context's, grown as
 * needed). */

/* One image: w, h multiples of 4, at most 2^24 blocks. */
typedef struct gst_reencode_image {
  uint32_t width, height;
  const void *d_rgb;        /* w*h*3 bytes RGB8, row-major, 4-byte aligned        */
  const void *d_blocks;     /* w*h/16 DXT1 blocks (raster order), 8-byte aligned  */
  void *d_blocks_out;       /* w*h/16 blocks after the search, 8-byte aligned     */
  void *d_palette;          /* palette words, 4B rounded up to 8192 bytes, 16-byte aligned */
  void *d_indices;          /* B index deltas + 128                                */
  uint32_t *d_palette_bytes; /* device u32: the palette's bytes padded to 8192     */
} gst_reencode_image;

/* n <= 65535 images per call. */
gst_status gst_reencode_blocks(gst_ctx *ctx, const gst_reencode_image *imgs, int n, void *stream);

/* Blocking host-to-host form: RGB8 source (w*h*3 bytes) and its DXT1 blocks
 * -> the GST stream of the reference's CompressDXTImage(DXTImage(w, h, rgb,
 * dxt)); out_cap at least gst_encode_stream_bound(width, height,
 * gst_palette_capacity(width, height)). */
gst_status gst_compress_rgb_dxt(gst_ctx *ctx, uint32_t width, uint32_t height, const uint8_t *rgb,
                                const uint64_t *blocks, uint8_t *gst_out, size_t out_cap, size_t *out_len);

/* ans::ocl::NormalizeFrequencies on the GPU (blocking, host arrays): n <= 256
 * byte counts -> n frequencies summing to 2048.  GST_E_ARG when every count is
 * zero (the reference asserts). */
gst_status gst_encode_normalize(gst_ctx *ctx, const uint32_t *counts, int n, uint32_t *freqs);

#ifdef __cplusplus
}
#endif
#endif
