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

/* ans::ocl::NormalizeFrequencies on the GPU (blocking, host arrays): n <= 256
 * byte counts -> n frequencies summing to 2048.  GST_E_ARG when every count is
 * zero (the reference asserts). */
gst_status gst_encode_normalize(gst_ctx *ctx, const uint32_t *counts, int n, uint32_t *freqs);

#ifdef __cplusplus
}
#endif
#endif
