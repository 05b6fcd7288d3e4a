// gst_prepare.cu -- sm_103a kernels of the encoder's endpoint stages: DXT1
// blocks -> the four symbol sections of a GST stream (the input of the
// entropy stages in gst_encode.cu).
//
//  gst_fwd_tile_kernel  GenTC::CompressDXTImage's endpoint pipeline
//     (codec/encoder.cpp:20-98): per 32x32-block tile, RGB565 endpoints ->
//     YCoCg667 (codec/image_processing.cpp:10-27), six planes, five levels
//     of the forward 5/3 wavelet with columns then rows per level
//     (codec/image_processing.h:267-333, codec/wavelet.cpp:37-157: int16
//     storage, truncating division, mirrored edges), and the byte planes
//     (coefficient + 128, tile-major).  One CTA per tile, one thread per
//     line of the six planes; the tile stays in shared memory.  It mirrors
//     the decoder's tile kernel.
//
//  gst_fwd_count_kernel / gst_fwd_palette_kernel  the index palette: a
//     block whose index word equals the previous block's reuses its entry,
//     otherwise its word is appended (index deltas +128 are 128 or 129).
//     This replaces the reference's sequential least-squares search
//     (codec/dxt_image.cpp:510-624) with a rule that parallelises: 8192-block
//     chunks count their new words, then each chunk sums the counts of the
//     chunks before it in its image and writes its entries at ballot
//     positions.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gst_encode_plan.h"
#include "gst_plan.h"

namespace gst {
namespace {

constexpr int kTileThreads = 192;  // 6 planes x 32 lines
constexpr int kChunkBlocks = 8192;
constexpr int kChunkThreads = 256;
constexpr int kLineStride = 33;    // int32 words: conflict-free rows and columns

__device__ __forceinline__ void ycocg667(uint32_t c, int &y, int &co, int &cg) {
  const int r = static_cast<int>(c >> 11), g = static_cast<int>((c >> 5) & 63), b = static_cast<int>(c & 31);
  co = r - b;
  const int t = r + b + (b >> 4);
  cg = g - t;
  y = t + cg / 2;
}

// NormalizeIndex (codec/wavelet.cpp:37-41): mirrored index in [0, len).
__device__ __forceinline__ int mirror(int idx, int len) {
  const int v = idx - (idx >= len ? idx - len + 2 : 0);
  return v < 0 ? -v : v;
}

// ForwardWavelet1D (codec/wavelet.cpp:56-88) on one line of `len` int16
// values held as int32 at p[0], p[step], ...: odd samples become details,
// even samples smoothed averages, both wrapped to int16 as the reference
// stores them.
template <int L>
__device__ __forceinline__ void forward_line(int *p, int step) {
  int s[L], d[L];
#pragma unroll
  for (int k = 0; k < L; ++k) s[k] = p[k * step];
  constexpr int mid = L - L / 2;
#pragma unroll
  for (int i = 1; i < L; i += 2)
    d[mid + i / 2] = static_cast<int16_t>(s[i] - (s[mirror(i - 1, L)] + s[mirror(i + 1, L)]) / 2);
#pragma unroll
  for (int i = 0; i < L; i += 2)
    d[i / 2] = static_cast<int16_t>(s[i] + (d[mid + mirror(i - 1, L) / 2] + d[mid + mirror(i + 1, L) / 2] + 2) / 4);
#pragma unroll
  for (int k = 0; k < L; ++k) p[k * step] = d[k];
}

template <int L>
__device__ __forceinline__ void forward_level(int *planes, int t) {
  const int plane = t / 32, line = t % 32;
  int *pl = planes + plane * 32 * kLineStride;
  if (line < L) forward_line<L>(pl + line, kLineStride);  // column `line`
  __syncthreads();
  if (line < L) forward_line<L>(pl + line * kLineStride, 1);  // row `line`
  __syncthreads();
}

// One tile of one image: tiles of an image in raster order, images back to
// back (EncPrepImage::first_tile).
__global__ void __launch_bounds__(kTileThreads) gst_fwd_tile_kernel(const EncPrepImage *__restrict__ images,
                                                                    uint32_t n_images) {
  __shared__ int planes[6 * 32 * kLineStride];
  // the image of this tile: the last with first_tile <= blockIdx.x
  uint32_t lo = 0, hi = n_images;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (images[mid].first_tile <= blockIdx.x)
      lo = mid;
    else
      hi = mid;
  }
  const uint32_t im = lo;
  const EncPrepImage &img = images[im];
  const uint32_t tile = blockIdx.x - img.first_tile;
  const uint32_t bx = img.width / 4, tiles_x = bx / 32;
  const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
  const int t = threadIdx.x;
  const uint64_t *blk = img.blocks + (static_cast<size_t>(ty) * 32) * bx + static_cast<size_t>(tx) * 32;
  for (int i = t; i < 1024; i += kTileThreads) {
    const uint64_t b = __ldg(reinterpret_cast<const unsigned long long *>(blk) + static_cast<size_t>(i / 32) * bx +
                             (i % 32));
    int v[6];
    ycocg667(static_cast<uint32_t>(b & 0xFFFF), v[0], v[1], v[2]);
    ycocg667(static_cast<uint32_t>((b >> 16) & 0xFFFF), v[3], v[4], v[5]);
    const int at = (i / 32) * kLineStride + i % 32;
#pragma unroll
    for (int p = 0; p < 6; ++p) planes[p * 32 * kLineStride + at] = v[p];
  }
  __syncthreads();
  forward_level<32>(planes, t);
  forward_level<16>(planes, t);
  forward_level<8>(planes, t);
  forward_level<4>(planes, t);
  forward_level<2>(planes, t);
  // Y section: Y1, Y2; chroma section: Co1, Cg1, Co2, Cg2 (encoder.cpp:86-98).
  const size_t B = static_cast<size_t>(bx) * (img.height / 4);
  for (int q = t; q < 6 * 256; q += kTileThreads) {
    const int p = q / 256, k = 4 * (q % 256);
    const int *src = planes + p * 32 * kLineStride + (k / 32) * kLineStride + k % 32;
    const uint32_t word = (static_cast<uint32_t>(src[0] + 128) & 0xFF) |
                          ((static_cast<uint32_t>(src[1] + 128) & 0xFF) << 8) |
                          ((static_cast<uint32_t>(src[2] + 128) & 0xFF) << 16) |
                          ((static_cast<uint32_t>(src[3] + 128) & 0xFF) << 24);
    uint8_t *base = p == 0 ? img.y : p == 3 ? img.y + B : img.chroma + (p == 1 ? 0 : p == 2 ? B : p == 4 ? 2 * B : 3 * B);
    reinterpret_cast<uint32_t *>(base + static_cast<size_t>(tile) * 1024)[k / 4] = word;
  }
}

__device__ __forceinline__ uint32_t index_word(const uint64_t *blocks, size_t b) {
  return static_cast<uint32_t>(__ldg(reinterpret_cast<const unsigned long long *>(blocks) + b) >> 32);
}

// New-word flags of block b (its word differs from the previous block's).
__device__ __forceinline__ uint32_t fresh(const uint64_t *blocks, size_t b) {
  return b == 0 || index_word(blocks, b) != index_word(blocks, b - 1);
}

__device__ __forceinline__ int cta_sum(int v, int *red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  v = 0;
#pragma unroll
  for (int w = 0; w < kChunkThreads / 32; ++w) v += red[w];
  __syncthreads();
  return v;
}

// Chunk c covers blocks [start, start + len) of image `image`.
__global__ void __launch_bounds__(kChunkThreads) gst_fwd_count_kernel(const EncPrepImage *__restrict__ images,
                                                                      const EncPrepChunk *__restrict__ chunks,
                                                                      uint32_t *__restrict__ counts) {
  __shared__ int red[kChunkThreads / 32];
  const EncPrepChunk ch = chunks[blockIdx.x];
  const uint64_t *blocks = images[ch.image].blocks;
  int n = 0;
  for (uint32_t k = threadIdx.x; k < ch.len; k += kChunkThreads) n += fresh(blocks, size_t(ch.start) + k);
  n = cta_sum(n, red);
  if (threadIdx.x == 0) counts[blockIdx.x] = static_cast<uint32_t>(n);
}

// Each warp takes 1024 consecutive blocks of the chunk, 32 per step (lane =
// block): the previous block's word comes from the lane below (one load for
// lane 0), new-word positions from a ballot.  Pass 1 counts per warp; after a
// scan of the warp counts, pass 2 writes the palette words and index deltas.
__global__ void __launch_bounds__(kChunkThreads) gst_fwd_palette_kernel(const EncPrepImage *__restrict__ images,
                                                                        const EncPrepChunk *__restrict__ chunks,
                                                                        const uint32_t *__restrict__ counts,
                                                                        uint32_t *__restrict__ palette_bytes) {
  constexpr int kWarps = kChunkThreads / 32;
  constexpr int kPerWarp = kChunkBlocks / kWarps;
  __shared__ int red[kWarps];
  __shared__ int warp_base[kWarps];
  __shared__ uint32_t total;
  const EncPrepChunk ch = chunks[blockIdx.x];
  const EncPrepImage &img = images[ch.image];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1;
  // entries written by the chunks before this one in its image
  int before = 0;
  for (uint32_t c = ch.first_chunk + threadIdx.x; c < blockIdx.x; c += kChunkThreads) before += counts[c];
  before = cta_sum(before, red);
  const uint32_t lo = warp * kPerWarp, hi = min(lo + kPerWarp, ch.len);
  auto flags = [&](uint32_t at, uint32_t &word) -> uint32_t {  // ballot of new words in blocks at .. at + 31
    const size_t b = size_t(ch.start) + at + lane;
    const bool in = at + lane < hi;
    word = in ? index_word(img.blocks, b) : 0u;
    uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, word, 1);
    if (lane == 0) prev = b > 0 ? index_word(img.blocks, b - 1) : ~word;
    return __ballot_sync(0xFFFFFFFFu, in && (b == 0 || word != prev));
  };
  int n = 0;
  for (uint32_t at = lo; at < hi; at += 32) {
    uint32_t word;
    n += __popc(flags(at, word));
  }
  if (lane == 0) warp_base[warp] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = before;
    for (int w = 0; w < kWarps; ++w) {
      const int c = warp_base[w];
      warp_base[w] = run;
      run += c;
    }
    total = 4u * static_cast<uint32_t>(run);
  }
  __syncthreads();
  int base = warp_base[warp];
  uint32_t *pal = reinterpret_cast<uint32_t *>(img.palette);
  for (uint32_t at = lo; at < hi; at += 32) {
    uint32_t word;
    const uint32_t m = flags(at, word);
    const size_t b = size_t(ch.start) + at + lane;
    if (m >> lane & 1) pal[base + __popc(m & lt)] = word;
    if (at + lane < hi) img.indices[b] = static_cast<uint8_t>(128 + (b > 0 ? (m >> lane & 1) : 0));
    base += __popc(m);
  }
  if (blockIdx.x == ch.last_chunk) {
    // the image's last chunk: its palette size, and zeros up to the padded end
    const uint32_t end = (total + kSymsPerGroup - 1) / kSymsPerGroup * kSymsPerGroup;
    for (uint32_t q = total + threadIdx.x; q < end; q += kChunkThreads) img.palette[q] = 0;
    if (threadIdx.x == 0) palette_bytes[ch.image] = end;
  }
}

}  // namespace

// Enqueues the endpoint stages of one plan.
// With `ev` non-null, records ev[0] before the first kernel and ev[i + 1]
// after kernel i, whose name goes to names[i] (instrumentation).
cudaError_t launch_prepare(const EncPrepImage *d_images, uint32_t n_images, uint32_t n_tiles,
                           const EncPrepChunk *d_chunks, uint32_t n_chunks, uint32_t *d_counts,
                           uint32_t *d_palette_bytes, cudaStream_t stream, cudaEvent_t *ev, const char **names) {
  if (ev) cudaEventRecord(ev[0], stream);
  gst_fwd_tile_kernel<<<n_tiles, kTileThreads, 0, stream>>>(d_images, n_images);
  if (ev) cudaEventRecord(ev[1], stream);
  if (n_chunks == 0) {  // the planes only: palette and deltas come from elsewhere
    if (ev) {
      cudaEventRecord(ev[2], stream);
      cudaEventRecord(ev[3], stream);
    }
    if (names) names[0] = "gst_fwd_tile_kernel", names[1] = names[2] = "";
    return cudaGetLastError();
  }
  gst_fwd_count_kernel<<<n_chunks, kChunkThreads, 0, stream>>>(d_images, d_chunks, d_counts);
  if (ev) cudaEventRecord(ev[2], stream);
  gst_fwd_palette_kernel<<<n_chunks, kChunkThreads, 0, stream>>>(d_images, d_chunks, d_counts, d_palette_bytes);
  if (ev) cudaEventRecord(ev[3], stream);
  if (names) {
    names[0] = "gst_fwd_tile_kernel";
    names[1] = "gst_fwd_count_kernel";
    names[2] = "gst_fwd_palette_kernel";
  }
  return cudaGetLastError();
}

}  // namespace gst
