/*
 * gst_encoder.h -- the project's GST stream producer (host-side C++).
 *
 * Makes the decoder's inputs: seeded synthetic RGB images, a DXT1 block
 * compressor with an index palette, and the GST stream writer.  The stream
 * writer follows the reference encoder's format stages exactly
 * (codec/encoder.cpp:39-180: RGB565 -> YCoCg667, per-plane 32x32 five-level
 * 5/3 forward wavelet, +128, block-linear order; codec/entropy.cpp:174-265
 * sections; ans/histogram.cpp:40-121 frequency normalisation;
 * ans/encode.cpp:56-69,224-259 interleaved rANS).  Its sections are checked
 * byte for byte against the reference's ByteEncoder in the tests.  The DXT1
 * block compressor and palette search are this project's own (the reference
 * uses stb_dxt and a least-squares endpoint refit), so whole streams differ
 * from the reference encoder's while keeping its format and statistics.
 */
#ifndef GST_ENCODER_H
#define GST_ENCODER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Seeded synthetic RGB8 image (w*h*3 bytes): four random-direction linear
 * gradients + three octaves of value noise (periods 64/32/16 px, amplitude 40)
 * + 20 random rectangles of uniform random colour, clamped to [0, 255].  When
 * checker_frac > 0, about that fraction of the area is replaced by rectangles
 * of two-colour checkerboards with 1-8 px cells.  Integer arithmetic only, so
 * the bytes are the same on every host. */
int gst_synth_image(uint32_t w, uint32_t h, uint64_t seed, double checker_frac, uint8_t *rgb);

/* RGB8 image -> GST stream.  *out is malloc'd (free with gst_encoder_free).
 * blocks (w*h/2 bytes, may be NULL) receives the DXT1 blocks the stream
 * decodes to; wavelet_clips (may be NULL) receives the number of wavelet
 * coefficients that did not fit in 8 bits.  Those wrap, as in the reference
 * encoder, so their tiles' endpoints differ from the compressor's; `blocks`
 * then holds the endpoints the stream really carries.  Returns 0 on success. */
int gst_encode_rgb(uint32_t w, uint32_t h, const uint8_t *rgb, uint8_t **out, size_t *out_len,
                   uint8_t *blocks, uint64_t *wavelet_clips, int nthreads);

/* The block compressor alone: RGB8 image -> w*h/16 DXT1 blocks (8-byte
 * aligned, raster order), before any palette search; w and h multiples of 4.
 * Returns 0 on success. */
int gst_compress_blocks(uint32_t w, uint32_t h, const uint8_t *rgb, uint8_t *blocks, int nthreads);

/* DXT1 blocks (w*h/2 bytes, raster order) -> GST stream, with the index
 * palette built from the given blocks' interpolation words. */
int gst_encode_dxt(uint32_t w, uint32_t h, const uint8_t *rgb, const uint8_t *dxt, uint8_t **out,
                   size_t *out_len, uint8_t *blocks, uint64_t *wavelet_clips);

/* One rANS section in the reference's ByteEncoder format (512-byte frequency
 * header, u32 group end offsets, groups).  n must be a multiple of 8192. */
int gst_encode_section(const uint8_t *in, size_t n, uint8_t **out, size_t *out_len, int nthreads);

/* Frequency normalisation to a total of M (ans/histogram.cpp:40-121). */
int gst_normalize_frequencies(const uint32_t *counts, size_t n, int M, uint32_t *out);

void gst_encoder_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
