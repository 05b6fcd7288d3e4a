/*
 * gst_oracle.h -- CPU oracle for the GST decode path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's GPU decoder (GammaUNC/GST): the five
 * OpenCL kernels ans/build_table.cl, ans/ans_decode.cl, codec/inverse_wavelet.cl,
 * codec/decode_indices.cl, codec/assemble.cl and their driver codec/decoder.cpp.
 * Each function names the reference lines it follows.  Only the tests, the
 * smoke check and the CPU-baseline leg of bench.py may call it, and only as the
 * checker or the timed CPU baseline; the product never links it.
 *
 * It also restates the encoder stages that the GPU encoder runs
 * (ans/histogram.cpp, ans/encode.cpp, codec/entropy.cpp, codec/encoder.cpp).
 *
 * Parity is pinned (tests/test_oracle.py) against:
 *   - the reference encoder's DXTImage::PhysicalBlocks() on the streams it
 *     wrote (codec/test/codec_test.cpp:36-48), committed as tests/golden/;
 *   - the reference's own ans::DecodeInterleaved and GenTC::InverseWavelet2D,
 *     compiled from the reference sources by oracle/build_ref.sh;
 *   - the known answers of ans/ans_ocl_test.cpp and codec/test/wavelet_test.cpp;
 *   - for the encoder stages, the reference's own ans::GenerateHistogram and
 *     ByteEncoder outputs (tests/golden/golden.json) and its encoder's streams.
 */
#ifndef GST_ORACLE_H
#define GST_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (same values as the product's gst_status). */
#define GSTO_OK 0
#define GSTO_E_ARG 1
#define GSTO_E_FORMAT 2

/* Constants of the format: ans/ans.h:72-76, codec/codec_base.h:22. */
#define GSTO_TABLE_SIZE 2048       /* M = 2^11 */
#define GSTO_TABLE_LOG 11
#define GSTO_SYMS_PER_STREAM 256
#define GSTO_STREAMS_PER_GROUP 32
#define GSTO_SYMS_PER_GROUP (GSTO_SYMS_PER_STREAM * GSTO_STREAMS_PER_GROUP)
#define GSTO_RANS_L (1u << 15)     /* k * M = 2^4 * 2^11 */
#define GSTO_HEADER_BYTES 28
#define GSTO_FREQ_BYTES 512

/* codec/codec_base.h:9-20, seven little-endian u32 words. */
typedef struct gsto_header {
  uint32_t width, height, palette_bytes, y_cmp_sz, chroma_cmp_sz, palette_sz, indices_sz;
} gsto_header;

/* Scan modes for the palette-index prefix sum. */
#define GSTO_SCAN_REFERENCE 0 /* emulate decode_indices + collect_indices stage by stage */
#define GSTO_SCAN_EXACT 1     /* plain inclusive prefix sum                               */

/* Header parse + validation of the whole stream (sizes, tables, group offsets). */
int gsto_parse_header(const uint8_t *gst, size_t n, gsto_header *hdr);

/* build_table.cl:12-83 for one table: exclusive Blelloch scan of the 256 u16
 * frequencies, then the kernel's 11-step search per slot.  Outputs per slot. */
void gsto_build_table(const uint16_t freqs[256], uint16_t freq[2048], uint16_t cum[2048],
                      uint8_t sym[2048]);

/* Straightforward table: slot s belongs to the symbol x with cum[x] <= s < cum[x]+freq[x]. */
void gsto_build_table_direct(const uint16_t freqs[256], uint16_t freq[2048], uint16_t cum[2048],
                             uint8_t sym[2048]);

/* ans_decode.cl:25-74 (ans_decode_single) for one group of `num_streams`
 * interleaved streams, 256 symbols each.  `data` is the section (its u32 group
 * end-offset table first); `group` selects the end offset.  Renormalisation
 * reads must stay in the group's word region, from `lo_bytes` (the group's
 * first byte) up to its final states; a read outside it (only a malformed
 * stream makes one) sets the return value to GSTO_E_FORMAT and reads 0.
 * out[(lane) * 256 + 255 - i] = symbol decoded at step i. */
int gsto_rans_decode_group(const uint8_t *data, size_t data_len, uint32_t group,
                           const uint16_t freq[2048], const uint16_t cum[2048],
                           const uint8_t sym[2048], int num_streams, size_t lo_bytes,
                           uint8_t *out);

/* inverse_wavelet.cl:69-192 for one 32x32 block: byte-128, five levels of the
 * integer 5/3 inverse lifting (rows then columns) in int32, char store.
 * in: 1024 bytes block-linear (row-major); out: 1024 int8 row-major. */
void gsto_inverse_wavelet_block(const uint8_t *in, int8_t *out);

/* The 1-D/2-D reversible 5/3 inverse at one level (dim x dim, int32), the same
 * arithmetic as the kernel, exposed for the wavelet known-answer tests. */
void gsto_inverse_wavelet_level(int32_t *blk, int stride, int dim);

/* decode_indices.cl + collect_indices driven as decoder.cpp:302-393 does
 * (mode GSTO_SCAN_REFERENCE), or the exact prefix sum (GSTO_SCAN_EXACT).
 * deltas: n bytes (value+128); out: n int32 palette indices. */
void gsto_scan_indices(const uint8_t *deltas, uint32_t n, int32_t *out, int mode);

/* assemble.cl:39-62: YCoCg (6,6,7 bit, signed char planes) -> RGB565. */
uint16_t gsto_ycocg_to_565(int y, int co, int cg);

/* Whole decode of one GST stream into w*h/2 bytes of DXT1 (assemble_dxt layout).
 * nthreads <= 1 runs single-threaded.  Returns a status code. */
int gsto_decode(const uint8_t *gst, size_t n, uint8_t *dxt_out, size_t out_cap, int scan_mode,
                int nthreads);

/* The same decode to 8-bit RGB (codec/assemble.cl:83-129, the reference's
 * LoadRGB): width*height*3 bytes, raster order, 3 bytes per pixel. */
int gsto_decode_rgb(const uint8_t *gst, size_t n, uint8_t *rgb_out, size_t out_cap, int scan_mode, int nthreads);

/* The same decode, stopping after the rANS stage: writes the reference's
 * decompressed-symbol buffer (Y planes, chroma planes, palette, index deltas,
 * decoder.cpp:441-461 layout) of 7*B + palette_bytes bytes. */
int gsto_decode_symbols(const uint8_t *gst, size_t n, uint8_t *symbols, size_t cap, int nthreads);

/* Decode of a batch: n_streams concatenated streams of arbitrary sizes; outputs
 * are written back to back in input order. */
int gsto_decode_batch(const uint8_t *const *gst, const size_t *lens, int n_streams,
                      uint8_t *dxt_out, size_t out_cap, int scan_mode, int nthreads);

/* --- encoder stages (the checker of the GPU encoder) ----------------------- */

/* ans/histogram.cpp:40-121 (ans::GenerateHistogram) for n counts and target sum
 * M: the float-scaled first guess per symbol, then the heap correction that
 * moves the sum to M one unit at a time, cheapest rank first.  Equal ranks
 * resolve in the order of the C++ library's binary heap (std::make_heap /
 * std::pop_heap / std::push_heap with std::greater), the sift procedure of the
 * SGI STL that GCC's libstdc++ keeps; it is restated here in C.  Ranks use the
 * C library's log2, as the reference does.  Returns GSTO_E_ARG for M <= 0 or
 * all-zero counts (the reference asserts). */
int gsto_normalize(const uint32_t *counts, int n, int M, uint32_t *out);

/* codec/entropy.cpp:174-265 (ByteEncoder::EncodeBytes) with ans/encode.cpp:56-69
 * and 224-259 (rANS_Encoder::Encode, ans::EncodeInterleaved) at the OpenCL
 * settings of ans/ans_ocl_encode.cpp (M = 2^11, k = 2^4, b = 2^16), 32 streams
 * of 256 symbols per group: the 512-byte frequency table, the u32 group end
 * offsets, then the groups.  n must be a positive multiple of 8192.  A section
 * holding only byte 0 (the reference's encoder refuses a one-entry frequency
 * vector, ans/ans_utils.h:43-47) encodes with F[0] = 2048. */
int gsto_encode_section(const uint8_t *in, size_t n, uint8_t *out, size_t cap, size_t *out_len);

/* Upper bound of gsto_encode_section's output for n symbols. */
size_t gsto_encode_section_bound(size_t n);

/* codec/encoder.cpp:122-144: one GST stream from its four symbol sections
 * (Y planes 2B, chroma planes 4B, palette padded to palette_bytes, index
 * deltas B; B = w*h/16). */
int gsto_encode_stream(uint32_t w, uint32_t h, uint32_t palette_bytes, const uint8_t *y, const uint8_t *chroma,
                       const uint8_t *palette, const uint8_t *indices, uint8_t *out, size_t cap, size_t *out_len);

/* The endpoint stages of GenTC::CompressDXTImage (codec/encoder.cpp:20-98):
 * per block, RGB565 endpoints -> YCoCg667 (codec/image_processing.cpp:10-27,
 * RGB565toYCoCg667), the six planes split (ImageSplit), each 32x32 tile
 * transformed by five levels of the forward 5/3 wavelet, columns then rows
 * per level (codec/image_processing.h:267-333 FWavelet2D with
 * codec/wavelet.cpp:37-157, int16 storage, truncating division, mirrored
 * edges), then MakeUnsigned / Linearize / RearrangeStream / ReducePrecision:
 * byte = (coefficient + 128) mod 256, tile-major, row-major within a tile.
 * Writes the Y section (Y1 then Y2 planes, 2B bytes) and the chroma section
 * (Co1, Cg1, Co2, Cg2, 4B bytes) of B = w*h/16 DXT1 blocks (u64, raster
 * order).  Returns the number of coefficients outside [-128, 127] (those wrap,
 * as in the reference encoder). */
uint64_t gsto_endpoint_planes(uint32_t w, uint32_t h, const uint64_t *blocks, uint8_t *y, uint8_t *chroma);

/* The run index palette of the GPU pipeline (this project's rule in place of
 * the reference's sequential least-squares search, codec/dxt_image.cpp:510-624):
 * a block whose index word equals the previous block's reuses its entry,
 * otherwise the word is appended.  Writes the palette words (LE, padded with
 * zeros to a multiple of 8192 bytes) and B index deltas (+128: 128 or 129),
 * and returns the padded palette bytes; pal_cap must be at least 4B rounded up
 * to 8192. */
uint32_t gsto_run_palette(uint32_t w, uint32_t h, const uint64_t *blocks, uint8_t *palette, size_t pal_cap,
                          uint8_t *deltas);

/* DXTImage::Reencode (codec/dxt_image.cpp:510-624): the reference's index
 * palette search over the blocks in raster order.  Each block (its 16 RGB8
 * pixels from `rgb`, w*h*3 bytes) tries the last min(127, palette size)
 * palette words, most recent first: the pixels are refitted to the word
 * (least-squares endpoints snapped to 5:6:5), a refit whose endpoints would
 * swap is skipped, and the first refit whose error does not exceed the given
 * block's ends the search; otherwise the smallest error increase wins.  An
 * increase below 35 reuses that word (blocks_out gets the refit block),
 * anything else appends the block's own word (blocks_out = blocks_in).
 * Writes the palette (padded with zeros to a multiple of 8192 bytes) and the
 * B index deltas (+128); returns the padded palette bytes, 0 if pal_cap is
 * below 4B rounded up to 8192. */
uint32_t gsto_reencode(uint32_t w, uint32_t h, const uint8_t *rgb, const uint64_t *blocks_in, uint64_t *blocks_out,
                       uint8_t *palette, size_t pal_cap, uint8_t *deltas);

/* One refit of the Reencode search: 16 RGB8 pixels (row-major in the block)
 * refitted to index word `word` -> the error (dxt_image.cpp:266-285), *ok and
 * the refit endpoints. */
int gsto_reencode_candidate(const uint8_t px[48], uint32_t word, int *ok, uint16_t *ep1, uint16_t *ep2);

/* ans_decode.cl:97-143 section lookup (ans_decode_multiple), for tests: returns
 * the section x the work-group at `wg` is assigned to by the kernel's search. */
uint32_t gsto_section_search(const uint32_t *output_offsets, uint32_t num_offsets, uint32_t wg);

#ifdef __cplusplus
}
#endif
#endif
