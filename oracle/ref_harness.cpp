// Test infrastructure only.  A thin C harness over the reference's own CPU
// code (GammaUNC/GST), compiled from the reference sources by build_ref.sh into
// oracle/_ref/libgstref.so.  The tests use it to pin the C oracle (oracle/gst_oracle.c)
// and to generate golden fixtures; the product never links it.
//
// Entry points and the reference code each one calls:
//   gstref_compress_rgb / gstref_compress_file
//       GenTC::DXTImage + GenTC::CompressDXT           codec/encoder.cpp:39-195
//       (the stream) and DXTImage::PhysicalBlocks      codec/dxt_image.h:72-74
//   gstref_encode_bytes   ByteEncoder::EncodeBytes     codec/entropy.cpp:174-265
//   gstref_decode_interleaved  ans::DecodeInterleaved  ans/decode.cpp:240-292
//   gstref_generate_histogram  ans::GenerateHistogram  ans/histogram.cpp:40-121
//   gstref_inverse_wavelet2d   GenTC::InverseWavelet2D codec/wavelet.cpp:133-155
//   gstref_encode_interleaved  ans::EncodeInterleaved     ans/encode.cpp:224-259
//   gstref_stb_blocks     CompressRGB's stb_dxt blocks     codec/dxt_image.cpp:362-384
//   gstref_reencode       DXTImage(w, h, rgb, dxt) = DXTImage::Reencode
//                         codec/dxt_image.cpp:455-468, 510-624 (+ CompressDXT)
//   gstref_rans_encode_single  rANS encoder at the OpenCL decoder's settings
//                              (ans/ans_ocl_encode.cpp:10-18, ans/encode.cpp:56-69)
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "ans.h"
#include "bits.h"
#include "histogram.h"
#include "dxt_image.h"
#include "encoder.h"
#include "entropy.h"
#include "wavelet.h"
#include "stb_dxt.h"

namespace {
int copy_out(const std::vector<uint8_t> &v, uint8_t *out, size_t cap, size_t *out_len) {
  *out_len = v.size();
  if (v.size() > cap) return -1;
  if (!v.empty()) memcpy(out, v.data(), v.size());
  return 0;
}

int compress_image(const GenTC::DXTImage &img, uint8_t *stream, size_t cap, size_t *stream_len,
                   uint8_t *blocks) {
  std::vector<uint8_t> s = GenTC::CompressDXT(img);
  const auto &pb = img.PhysicalBlocks();
  if (blocks) memcpy(blocks, pb.data(), pb.size() * sizeof(pb[0]));
  return copy_out(s, stream, cap, stream_len);
}
}  // namespace

extern "C" {

// RGB8 image (w*h*3 bytes) -> GST stream and the encoder's DXT1 blocks (w*h/2 bytes).
int gstref_compress_rgb(int w, int h, const uint8_t *rgb, uint8_t *stream, size_t cap,
                        size_t *stream_len, uint8_t *blocks) {
  GenTC::DXTImage img(w, h, rgb);
  return compress_image(img, stream, cap, stream_len, blocks);
}

// Image file (anything stb_image loads) -> GST stream + DXT1 blocks; *w, *h receive the size.
int gstref_compress_file(const char *fn, uint8_t *stream, size_t cap, size_t *stream_len,
                         uint8_t *blocks, size_t blocks_cap, int *w, int *h) {
  GenTC::DXTImage img(fn, nullptr);
  *w = img.Width();
  *h = img.Height();
  if (static_cast<size_t>(img.Width()) * img.Height() / 2 > blocks_cap) return -2;
  return compress_image(img, stream, cap, stream_len, blocks);
}

int gstref_encode_bytes(const uint8_t *in, size_t n, uint8_t *out, size_t cap, size_t *out_len) {
  std::unique_ptr<std::vector<uint8_t> > v(new std::vector<uint8_t>(in, in + n));
  auto enc = GenTC::ByteEncoder::Encoder(ans::ocl::kNumEncodedSymbols);
  auto r = enc->Run(v);
  return copy_out(*r, out, cap, out_len);
}

int gstref_decode_interleaved(const uint8_t *data, size_t n, size_t num_symbols,
                              const uint32_t *F, size_t nF, size_t num_streams, uint8_t *out) {
  std::vector<uint8_t> d(data, data + n);
  std::vector<uint32_t> f(F, F + nF);
  std::vector<uint8_t> r = ans::DecodeInterleaved(d, num_symbols, ans::ocl::GetOpenCLOptions(f),
                                                  num_streams);
  if (r.size() != num_symbols) return -1;
  memcpy(out, r.data(), num_symbols);
  return 0;
}

int gstref_generate_histogram(const uint32_t *counts, size_t n, int M, uint32_t *out) {
  std::vector<uint32_t> c(counts, counts + n);
  std::vector<uint32_t> h = ans::GenerateHistogram(c, M);
  if (h.size() != n) return -1;
  memcpy(out, h.data(), n * sizeof(uint32_t));
  return 0;
}

// dim x dim block, row-major int16, one level of the inverse 2-D wavelet.
void gstref_inverse_wavelet2d(const int16_t *src, int16_t *dst, size_t dim) {
  std::vector<int16_t> s(src, src + dim * dim);
  GenTC::InverseWavelet2D(s.data(), dim * sizeof(int16_t), dst, dim * sizeof(int16_t), dim);
}

// Encodes `n` symbols with one rANS encoder at the GPU decoder's settings
// (b = 2^16, k = 2^4, M = 2^11, frequencies normalised from F).  Writes the
// 16-bit renormalisation words to `out` (cap bytes) and the final state.
int gstref_rans_encode_single(const uint32_t *F, size_t nF, const uint8_t *symbols, size_t n,
                              uint8_t *out, size_t cap, size_t *out_len, uint32_t *final_state) {
  std::vector<uint32_t> f(F, F + nF);
  std::unique_ptr<ans::Encoder> enc = ans::Encoder::Create(ans::ocl::GetOpenCLOptions(f));
  std::vector<uint8_t> buf(2 * n + 16, 0);
  size_t written = 0;
  for (size_t i = 0; i < n; ++i) {
    ans::BitWriter w(buf.data() + written);
    enc->Encode(symbols[i], &w);
    written += w.BytesWritten();
  }
  buf.resize(written);
  *final_state = enc->GetState();
  return copy_out(buf, out, cap, out_len);
}

// ans::EncodeInterleaved at the GPU decoder's settings: `n` symbols laid out
// stream-major (stream s holds symbols[s * n/num_streams ...]); output is the
// renormalisation words followed by the num_streams final states.
int gstref_encode_interleaved(const uint32_t *F, size_t nF, const uint8_t *symbols, size_t n,
                              size_t num_streams, uint8_t *out, size_t cap, size_t *out_len) {
  std::vector<uint32_t> f(F, F + nF);
  std::vector<uint8_t> s(symbols, symbols + n);
  std::vector<uint8_t> r = ans::EncodeInterleaved(s, ans::ocl::GetOpenCLOptions(f), num_streams);
  return copy_out(r, out, cap, out_len);
}

// The reference encoder's DXT1 blocks before its palette search: each 4x4
// block as RGBA (alpha 255) through stb_compress_dxt_block in high-quality
// mode, as CompressRGB does (codec/dxt_image.cpp:362-384, 520-529).
void gstref_stb_blocks(int w, int h, const uint8_t *rgb, uint8_t *blocks) {
  for (int by = 0; by < h / 4; ++by)
    for (int bx = 0; bx < w / 4; ++bx) {
      unsigned char block[64];
      for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 4; ++i) {
          const uint8_t *p = rgb + ((size_t)(4 * by + j) * w + 4 * bx + i) * 3;
          unsigned char *q = block + (j * 4 + i) * 4;
          q[0] = p[0];
          q[1] = p[1];
          q[2] = p[2];
          q[3] = 0xFF;
        }
      stb_compress_dxt_block(blocks + 8 * ((size_t)by * (w / 4) + bx), block, 0, STB_DXT_HIGHQUAL);
    }
}

// GenTC::DXTImage(width, height, rgb, dxt) runs DXTImage::Reencode over the
// given blocks (codec/dxt_image.cpp:455-468, 510-624): the blocks after the
// search, the palette words and the index deltas; and, when stream is not
// null, CompressDXT of that image (codec/encoder.cpp:39-195).
int gstref_reencode(int w, int h, const uint8_t *rgb, const uint8_t *dxt, uint8_t *blocks_out, uint8_t *palette,
                    size_t pal_cap, size_t *pal_len, uint8_t *deltas, uint8_t *stream, size_t cap,
                    size_t *stream_len) {
  const size_t nblk = static_cast<size_t>(w / 4) * (h / 4);
  std::vector<uint8_t> px(rgb, rgb + static_cast<size_t>(w) * h * 3);
  std::vector<uint8_t> blocks(dxt, dxt + 8 * nblk);
  GenTC::DXTImage img(w, h, px, blocks);
  const auto &pb = img.PhysicalBlocks();
  memcpy(blocks_out, pb.data(), pb.size() * sizeof(pb[0]));
  const std::vector<uint8_t> &d = img.IndexDiffs();
  if (d.size() != nblk) return -3;
  memcpy(deltas, d.data(), nblk);
  if (copy_out(img.PaletteData(), palette, pal_cap, pal_len) != 0) return -1;
  if (!stream) return 0;
  return copy_out(GenTC::CompressDXT(img), stream, cap, stream_len);
}

}  // extern "C"
