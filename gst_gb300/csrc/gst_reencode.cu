// gst_reencode.cu -- the reference's index palette search (DXTImage::Reencode,
// codec/dxt_image.cpp:510-624) on the GPU, with identical results.
//
// The search runs over the blocks in raster order.  Block b tries the last
// min(127, palette size) palette words, most recent first: its 16 pixels are
// refitted to the word (least-squares endpoints snapped to 5:6:5,
// RecalculateEndpoints :301-359), a refit whose endpoints would swap is
// skipped, the first refit that does not raise the block's error ends the
// loop, otherwise the least raise wins; a raise below 35 reuses the word, any
// other block appends its own word.  Only the palette makes it sequential: a
// refit's error does not depend on any decision.  So the work splits into
//
//   gst_re_info_kernel    per block: its pixels, the sums of the normal
//       equations of its own word (block-independent) and its error as given;
//   gst_re_score_kernel   one step per kReChunk blocks of every image: scores
//       each block of the chunk against the window at the chunk's start and
//       against the chunk's earlier blocks (one warp per block and 32 words,
//       one refit per lane); the last scoring CTA of an image then walks the
//       chunk: one warp decides, block after block, whether the block's
//       window holds a usable word (bit masks: a chain of register operations
//       per block, warp votes once more than 127 blocks of the chunk appended),
//       and the CTA appends the words of the blocks that found none;
//   gst_re_select_kernel  each block's word: the first of least score in
//       recency order (what the reference's loop with its early exit picks),
//       and the refit of the block's endpoints to it;
//   gst_re_finish_kernel  index deltas and the palette's zero padding.
//
// A score is min(max(error raise, 0), 35), 35 also for a refit that would
// swap its endpoints: the loop stops at the first raise <= 0, and a raise of
// 35 or more is never used, so that byte keeps every decision.
//
// Float arithmetic restates the reference's as compiled for x86-64 (SSE, no
// fused multiply-add): each product, sum and quotient is rounded on its own
// (__fmul_rn, __fadd_rn, __fsub_rn and __fdiv_rn are never contracted), and
// the float -> int32 conversion gives INT32_MIN for NaN and out-of-range
// values, as cvttss2si does.
#include <cstdint>

#include <cuda_runtime.h>

#include "gst_encode_plan.h"
#include "gst_plan.h"

namespace gst {
namespace {

constexpr uint32_t kReWarps = 8;                   // warps per scoring CTA
constexpr uint32_t kReThreads = 32 * kReWarps;     // = kReChunk: the walker has a thread per block
constexpr uint32_t kReGroups = kReGroupsPerBlock;  // 32-slot groups per block: 4 window, 8 chunk
constexpr uint32_t kReMaskWords = kReChunk / 32;
static_assert(kReThreads == kReChunk, "the walker's first pass has one thread per block of the chunk");

// fl(2/3) and fl(1/3): (3 - order) / 3 and order / 3 for the middle orders
// (dxt_image.cpp:314-323).
__device__ __forceinline__ float two_thirds() { return __int_as_float(0x3F2AAAABu); }
__device__ __forceinline__ float one_third() { return __int_as_float(0x3EAAAAABu); }

__device__ __forceinline__ int32_t f2i_x86(float q) {
  return (q >= -2147483648.0f && q < 2147483648.0f) ? __float2int_rz(q) : INT32_MIN;
}

__device__ __forceinline__ uint32_t clamp255(int32_t v) { return static_cast<uint32_t>(v < 0 ? 0 : v > 255 ? 255 : v); }

// ToFiveBits (bits = 5) / ToSixBits (bits = 6), dxt_image.cpp:82-130.
__device__ __forceinline__ uint32_t snap_channel(uint32_t x, uint32_t bits) {
  const uint32_t mask = bits == 5 ? 0xF8u : 0xFCu, step = bits == 5 ? 4u : 2u;
  uint32_t base = x & mask, high = base + step, low = base ? base - step : 0u;
  base |= base >> bits;
  high |= high >> bits;
  low |= low >> bits;
  const uint32_t db = __usad(x, base, 0u), dh = __usad(x, high, 0u), dl = __usad(x, low, 0u);
  return db <= dh ? (db < dl ? base : low) : high;
}

// Packed 0x00BBGGRR of a 5:6:5 colour (Decode565, dxt_image.cpp:53-72).
__device__ __forceinline__ uint32_t unpack565(uint32_t v) {
  const uint32_t r = v >> 11, g = (v >> 5) & 0x3Fu, b = v & 0x1Fu;
  return ((r << 3) | (r >> 2)) | (((g << 2) | (g >> 4)) << 8) | (((b << 3) | (b >> 2)) << 16);
}

__device__ __forceinline__ uint32_t ch(uint32_t c, int k) { return (c >> (8 * k)) & 0xFFu; }

// (a * (div - num) + b * num) / div per channel (LerpChannels, dxt_image.cpp:44-51).
__device__ __forceinline__ uint32_t lerp_packed(uint32_t a, uint32_t b, uint32_t num, uint32_t div) {
  uint32_t out = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) out |= ((ch(a, k) * (div - num) + ch(b, k) * num) / div) << (8 * k);
  return out;
}

// Sum of squared channel differences of the 16 pixels against the palette
// entries the word selects, / 48 (CompressedBlock::Error, :266-285).
__device__ __forceinline__ uint32_t block_error(const uint32_t (&px)[16], uint32_t p0, uint32_t p1, uint32_t p2,
                                                uint32_t p3, uint32_t word) {
  uint32_t err = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint32_t k = (word >> (2 * i)) & 3u;
    const uint32_t lo = (k & 1u) ? p1 : p0, hi = (k & 1u) ? p3 : p2;
    const uint32_t d = __vabsdiffu4(px[i], (k & 2u) ? hi : lo);
    err = __dp4a(d, d, err);
  }
  return err / 48u;
}

// Error of the block as given: PhysicalToLogical's palette (:144-170), the
// three-colour one with black when ep1 <= ep2.
__device__ __forceinline__ uint32_t given_error(const uint32_t (&px)[16], uint64_t blk) {
  const uint32_t e1 = static_cast<uint32_t>(blk) & 0xFFFFu, e2 = static_cast<uint32_t>(blk >> 16) & 0xFFFFu;
  const uint32_t a = unpack565(e1), b = unpack565(e2);
  const bool three = e1 <= e2;
  const uint32_t p2 = three ? lerp_packed(a, b, 1, 2) : lerp_packed(a, b, 1, 3);
  const uint32_t p3 = three ? 0u : lerp_packed(a, b, 2, 3);
  return block_error(px, a, b, p2, p3, static_cast<uint32_t>(blk >> 32));
}

// Sums of the normal equations that depend on the word alone, and the
// reciprocal of their determinant (RecalculateEndpoints, :301-333).
struct WordSums {
  float asq, bsq, ab, inv;
};

__device__ __forceinline__ void index_weights(uint32_t k, float *a, float *b) {
  // order 0, 3, 1, 2 for k = 0..3: a = (3 - order) / 3, b = order / 3
  *a = k == 0 ? 1.0f : k == 1 ? 0.0f : k == 2 ? two_thirds() : one_third();
  *b = k == 0 ? 0.0f : k == 1 ? 1.0f : k == 2 ? one_third() : two_thirds();
}

__device__ __forceinline__ WordSums word_sums(uint32_t word) {
  float asq = 0.0f, bsq = 0.0f, ab = 0.0f;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    float a, b;
    index_weights((word >> (2 * i)) & 3u, &a, &b);
    asq = __fadd_rn(asq, __fmul_rn(a, a));
    bsq = __fadd_rn(bsq, __fmul_rn(b, b));
    ab = __fadd_rn(ab, __fmul_rn(a, b));
  }
  return {asq, bsq, ab, __fdiv_rn(1.0f, __fsub_rn(__fmul_rn(asq, bsq), __fmul_rn(ab, ab)))};
}

// The block refitted to `word` (AssignIndices + RecalculateEndpoints,
// :295-359): returns the error; *ep receives ep1 | ep2 << 16 as 5:6:5 and
// *ok whether they keep the word as is (ep1 > ep2; otherwise
// LogicalToPhysical would swap them and flip the word, :576-584).
__device__ __forceinline__ uint32_t refit(const uint32_t (&px)[16], uint32_t word, const WordSums &w, uint32_t *ep,
                                          bool *ok) {
  float ax[3] = {0.0f, 0.0f, 0.0f}, bx[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    float a, b;
    index_weights((word >> (2 * i)) & 3u, &a, &b);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = static_cast<float>(ch(px[i], c));
      ax[c] = __fadd_rn(ax[c], __fmul_rn(v, a));
      bx[c] = __fadd_rn(bx[c], __fmul_rn(v, b));
    }
  }
  uint32_t c1 = 0, c2 = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float p1 = __fmul_rn(w.inv, __fsub_rn(__fmul_rn(ax[c], w.bsq), __fmul_rn(bx[c], w.ab)));
    const float p2 = __fmul_rn(w.inv, __fsub_rn(__fmul_rn(bx[c], w.asq), __fmul_rn(ax[c], w.ab)));
    const uint32_t bits = c == 1 ? 6u : 5u;
    c1 |= snap_channel(clamp255(f2i_x86(__fadd_rn(p1, 0.5f))), bits) << (8 * c);
    c2 |= snap_channel(clamp255(f2i_x86(__fadd_rn(p2, 0.5f))), bits) << (8 * c);
  }
  const uint32_t e1 = ((ch(c1, 0) & 0xF8u) << 8) | ((ch(c1, 1) & 0xFCu) << 3) | (ch(c1, 2) >> 3);
  const uint32_t e2 = ((ch(c2, 0) & 0xF8u) << 8) | ((ch(c2, 1) & 0xFCu) << 3) | (ch(c2, 2) >> 3);
  *ep = e1 | (e2 << 16);
  *ok = e1 > e2;
  return block_error(px, c1, c2, lerp_packed(c1, c2, 1, 3), lerp_packed(c1, c2, 2, 3), word);
}

// The 16 pixels of block b, row-major in the block, packed 0x00BBGGRR.  Rows
// of the image start 4-byte aligned (width is a multiple of 4).
__device__ __forceinline__ void load_pixels(const ReImage &im, uint32_t b, uint32_t (&px)[16]) {
  const uint32_t bx = b % im.bw, by = b / im.bw;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint32_t *q = reinterpret_cast<const uint32_t *>(im.rgb + (static_cast<size_t>(4 * by + r) * im.width +
                                                                     4 * bx) * 3);
    const uint32_t w0 = __ldg(q), w1 = __ldg(q + 1), w2 = __ldg(q + 2);
    px[4 * r + 0] = w0 & 0xFFFFFFu;
    px[4 * r + 1] = __byte_perm(w0, w1, 0x0543u) & 0xFFFFFFu;
    px[4 * r + 2] = __byte_perm(w1, w2, 0x0432u) & 0xFFFFFFu;
    px[4 * r + 3] = w2 >> 8;
  }
}

__device__ __forceinline__ void info_pixels(const uint4 *info, uint32_t (&px)[16]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint4 v = info[q];
    px[4 * q] = v.x;
    px[4 * q + 1] = v.y;
    px[4 * q + 2] = v.z;
    px[4 * q + 3] = v.w;
  }
}

__device__ __forceinline__ WordSums info_sums(const uint4 *info, uint32_t *word) {
  const uint4 a = info[4], b = info[5];
  *word = a.x;
  return {__uint_as_float(a.y), __uint_as_float(a.z), __uint_as_float(a.w), __uint_as_float(b.x)};
}

__device__ __forceinline__ uint32_t score_of(uint32_t err, uint32_t given, bool ok) {
  const int32_t d = static_cast<int32_t>(err) - static_cast<int32_t>(given);
  return !ok ? kReThreshold : d <= 0 ? 0u : d >= static_cast<int32_t>(kReThreshold) ? kReThreshold : uint32_t(d);
}

// Per block, once per call: its pixels, the sums of its own word (what any
// later block refitting to that word needs) and its error as given.
__global__ void __launch_bounds__(256) gst_re_info_kernel(const ReImage *__restrict__ imgs) {
  const ReImage &im = imgs[blockIdx.y];
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= im.B) return;
  uint32_t px[16];
  load_pixels(im, b, px);
  const uint64_t blk = im.blocks_in[b];
  const uint32_t word = static_cast<uint32_t>(blk >> 32);
  const WordSums w = word_sums(word);
  uint4 *o = im.info + static_cast<size_t>(b) * kReInfo;
#pragma unroll
  for (int q = 0; q < 4; ++q) o[q] = make_uint4(px[4 * q], px[4 * q + 1], px[4 * q + 2], px[4 * q + 3]);
  o[4] = make_uint4(word, __float_as_uint(w.asq), __float_as_uint(w.bsq), __float_as_uint(w.ab));
  o[5] = make_uint4(__float_as_uint(w.inv), given_error(px, blk), 0u, 0u);
}

// The decisions of one chunk (K blocks from c0, palette size P at its start),
// by the CTA that finished its scoring last.  Block j appends its word iff no
// word of its window scores below 35: window slot r < min(Wn, 127 - c) of the
// chunk's start (c = blocks of the chunk appended before j) or an appended
// chunk block among the last 127 appended.
__device__ void walk_chunk(const ReImage &im, ReState *st, uint32_t c0, uint32_t K, uint32_t P) {
  __shared__ uint32_t usable[kReMaskWords][kReChunk];  // word w, block j: chunk slots 32w.. < j below 35
  // meta[j]: bits 0-7 127 - (first window slot below 35), 0 if none: the
  // window still holds that word while fewer blocks of the chunk appended;
  // bit 31: a usable appended block in the 32-block words before j's
  __shared__ uint32_t meta[kReChunk];
  __shared__ uint32_t own_word[kReChunk];  // the blocks' own index words
  __shared__ uint32_t app[kReMaskWords];  // appended blocks of the chunk, bit j
  __shared__ uint16_t app_pos[kReChunk];  // their positions in order (once more than 127)
  const uint32_t t = threadIdx.x;
  const uint32_t Wn = min(P, kReWindow);
  if (t < K) {
    // the scorers' ballots; words of groups that had no valid slot were not written
    const uint4 *mk = reinterpret_cast<const uint4 *>(im.masks + static_cast<size_t>(c0 + t) * kReGroups);
    const uint4 q0 = __ldcg(mk), q1 = __ldcg(mk + 1), q2 = __ldcg(mk + 2);
    own_word[t] = static_cast<uint32_t>(im.blocks_in[c0 + t] >> 32);
    const uint32_t win[4] = {q0.x, q0.y, q0.z, q0.w};
    const uint32_t chk[8] = {q1.x, q1.y, q1.z, q1.w, q2.x, q2.y, q2.z, q2.w};
    uint32_t first = 255;
#pragma unroll
    for (int q = 3; q >= 0; --q)
      if (32 * q < Wn && win[q]) first = 32 * q + __ffs(win[q]) - 1;
    meta[t] = first < Wn ? kReWindow - first : 0u;
#pragma unroll
    for (uint32_t w = 0; w < kReMaskWords; ++w) usable[w][t] = 32 * w < t ? chk[w] : 0u;
  }
  if (t < kReMaskWords) app[t] = 0;
  __syncthreads();
  if (t < 32) {
    const uint32_t lane = t;
    const uint32_t nw = (K + 31) / 32;
    uint32_t c = 0;   // appended so far in this chunk
    uint32_t w = 0;   // word of the next block to decide
    uint32_t j0 = 0;  // next block to decide
    // Fast path, 32 blocks at a time while no appended chunk block has left
    // the window (c <= 127 before each decision): the hits in the finished
    // words are found in parallel; the 32 decisions are then a chain of
    // register operations.  A word in which the 128th append happens keeps
    // its decisions up to that block; the slow path takes the rest.
    for (; w < nw && c <= kReWindow; ++w) {
      {
        const uint32_t j = 32 * w + lane;
        uint32_t low = 0;
#pragma unroll
        for (uint32_t v = 0; v < kReMaskWords; ++v)
          if (v < w) low |= usable[v][j] & app[v];
        if (j >= K || low) meta[j] |= 1u << 31;  // past the chunk: never appends
      }
      __syncwarp();
      uint32_t g[32], m[32];
#pragma unroll
      for (uint32_t i = 0; i < 32; ++i) {
        g[i] = usable[w][32 * w + i];
        m[i] = meta[32 * w + i];
      }
      uint32_t A = 0;
      const uint32_t c_start = c;
#pragma unroll
      for (uint32_t i = 0; i < 32; ++i) {
        const bool hit = (m[i] >> 31) != 0u || (g[i] & A) != 0u || c < (m[i] & 0xFFu);
        A |= static_cast<uint32_t>(!hit) << i;
        c += !hit;
      }
      j0 = min(32 * w + 32, K);
      if (c > kReWindow) {
        // the (128 - c_start)-th append of this word is the last decision kept
        uint32_t mm = A;
        for (uint32_t k = 1; k < kReWindow + 1 - c_start; ++k) mm &= mm - 1u;
        const uint32_t pos = static_cast<uint32_t>(__ffs(mm)) - 1u;
        A &= pos == 31 ? 0xFFFFFFFFu : (2u << pos) - 1u;
        c = kReWindow + 1;
        j0 = 32 * w + pos + 1;
      }
      if (lane == 0) app[w] = A;
      __syncwarp();
      if (c > kReWindow) {
        ++w;
        break;
      }
    }
    if (j0 < K) {
      // Slow path: appended chunk blocks may leave the window (c > 127).
      // Lane l keeps the appended bits of word l; app_pos lists the appended
      // positions.
      if (lane == 0) {
        uint32_t n = 0;
        for (uint32_t v = 0; v < kReMaskWords; ++v)
          for (uint32_t mm = app[v]; mm; mm &= mm - 1) app_pos[n++] = static_cast<uint16_t>(32 * v + __ffs(mm) - 1);
      }
      __syncwarp();
      uint32_t A = lane < kReMaskWords ? app[lane] : 0u;
      uint32_t first_kept = c > kReWindow ? app_pos[c - kReWindow] : 0u;
      for (uint32_t j = j0; j < K; ++j) {
        const uint32_t g = lane < kReMaskWords ? usable[lane][j] : 0u;
        const uint32_t keep = first_kept <= 32 * lane ? 0xFFFFFFFFu
                              : first_kept >= 32 * lane + 32 ? 0u
                                                             : 0xFFFFFFFFu << (first_kept - 32 * lane);
        const bool hit_new = __any_sync(0xFFFFFFFFu, (g & A & keep) != 0u);
        const bool hit_old = c < (meta[j] & 0xFFu);
        if (!(hit_new || hit_old)) {
          if (lane == (j >> 5)) A |= 1u << (j & 31u);
          if (lane == 0) app_pos[c] = static_cast<uint16_t>(j);
          ++c;
          if (c > kReWindow) {
            __syncwarp();
            first_kept = app_pos[c - kReWindow];
          }
        }
      }
      if (lane < kReMaskWords) app[lane] = A;
    }
  }
  __syncthreads();
  if (t < K) {
    const uint32_t wj = t >> 5, bit = 1u << (t & 31u);
    uint32_t before = __popc(app[wj] & (bit - 1u));
    for (uint32_t v = 0; v < wj; ++v) before += __popc(app[v]);
    const uint32_t b = c0 + t, k = P + before;
    im.pal_before[b] = k;
    if (app[wj] & bit) {
      im.pal_src[k] = b;
      reinterpret_cast<uint32_t *>(im.palette)[k] = own_word[t];
    }
  }
  if (t == 0) {
    uint32_t total = 0;
    for (uint32_t v = 0; v < kReMaskWords; ++v) total += __popc(app[v]);
    st->P = P + total;
    st->arrive = 0;
  }
}

// One step: chunk `step` of every image that has one.  blockIdx.y walks the
// images in order of decreasing chunk count (order), so the images still
// going are the first gridDim.y.
// Five CTAs per SM (48 registers, no spills): 74 ms for the 64-image batch's
// search against 81 ms at four (60 registers); six spill.
__global__ void __launch_bounds__(kReThreads, 5) gst_re_score_kernel(const ReImage *__restrict__ imgs,
                                                                  const uint32_t *__restrict__ order,
                                                                  ReState *__restrict__ states, uint32_t step) {
  const uint32_t id = order[blockIdx.y];
  const ReImage &im = imgs[id];
  ReState *st = states + id;
  const uint32_t c0 = step * kReChunk;
  if (c0 >= im.B) return;
  const uint32_t K = min(kReChunk, im.B - c0);
  const uint32_t n_items = K * kReGroups;
  const uint32_t n_ctas = (n_items + kReWarps - 1) / kReWarps;
  if (blockIdx.x >= n_ctas) return;  // not counted below
  const uint32_t P = st->P;  // set by the previous step's walker (an earlier launch)
  const uint32_t Wn = min(P, kReWindow);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint32_t item = blockIdx.x * kReWarps + warp;
  if (item < n_items) {
    const uint32_t j = item / kReGroups, g = item - j * kReGroups;
    const bool win = g < 4;
    const uint32_t base = win ? 32 * g : 32 * (g - 4);
    const uint32_t lim = win ? Wn : j;  // window slots below Wn; chunk slots before j
    if (base < lim) {
      const uint32_t b = c0 + j, s = base + lane;
      const bool valid = s < lim;
      // the candidate word's block: the palette entry's source, or chunk block s
      const uint32_t src = !valid ? b : win ? im.pal_src[P - 1 - s] : c0 + s;
      uint32_t word;
      const WordSums ws = info_sums(im.info + static_cast<size_t>(src) * kReInfo, &word);
      const uint4 *bi = im.info + static_cast<size_t>(b) * kReInfo;
      uint32_t px[16];
      info_pixels(bi, px);
      const uint32_t given = bi[5].y;
      uint32_t ep;
      bool ok;
      const uint32_t err = refit(px, word, ws, &ep, &ok);
      const uint32_t sc = score_of(err, given, ok);
      if (valid) im.scores[static_cast<size_t>(b) * kReRow + (win ? s : 128 + s)] = uint8_t(sc);
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, valid && sc < kReThreshold);
      if (lane == 0) im.masks[static_cast<size_t>(b) * kReGroups + g] = m;
    }
  }
  __shared__ uint32_t last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&st->arrive, 1u) == n_ctas - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  walk_chunk(im, st, c0, K, P);
}

// Each block's word and refit (one warp per block).  A block whose window
// holds no score below 35 keeps its own block and word.
__global__ void __launch_bounds__(256) gst_re_select_kernel(const ReImage *__restrict__ imgs,
                                                            const ReState *__restrict__ states,
                                                            uint32_t *__restrict__ status) {
  const ReImage &im = imgs[blockIdx.y];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t b = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (b >= im.B) return;
  const uint32_t Pb = im.pal_before[b];
  const uint32_t c0 = b - b % kReChunk;
  const uint32_t Ps = im.pal_before[c0];
  const uint32_t Pn = b + 1 < im.B ? im.pal_before[b + 1] : states[blockIdx.y].P;
  const uint8_t *row = im.scores + static_cast<size_t>(b) * kReRow;
  const uint32_t n = min(Pb, kReWindow);
  uint32_t key = 0xFFFFFFFFu;
  for (uint32_t r = lane; r < n; r += 32) {  // r = recency: palette index Pb - 1 - r
    const uint32_t idx = Pb - 1 - r;
    const uint32_t sc = idx >= Ps ? row[128 + (im.pal_src[idx] - c0)] : row[Ps - 1 - idx];
    key = min(key, (sc << 8) | r);
  }
  key = __reduce_min_sync(0xFFFFFFFFu, key);
  const bool reuse = key < (kReThreshold << 8);
  if (lane != 0) return;
  if (reuse == (Pn != Pb)) atomicOr(status, kErrReencode);  // the walker appended iff nothing was usable
  uint64_t out = im.blocks_in[b];
  uint32_t idx = Pb;
  if (reuse) {
    idx = Pb - 1 - (key & 0xFFu);
    uint32_t word;
    const WordSums ws = info_sums(im.info + static_cast<size_t>(im.pal_src[idx]) * kReInfo, &word);
    uint32_t px[16];
    info_pixels(im.info + static_cast<size_t>(b) * kReInfo, px);
    uint32_t ep;
    bool ok;
    refit(px, word, ws, &ep, &ok);
    out = static_cast<uint64_t>(ep) | (static_cast<uint64_t>(word) << 32);
  }
  im.blocks_out[b] = out;
  im.idx[b] = idx;
}

__global__ void __launch_bounds__(256) gst_re_finish_kernel(const ReImage *__restrict__ imgs,
                                                            const ReState *__restrict__ states) {
  const ReImage &im = imgs[blockIdx.y];
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < im.B) im.deltas[t] = static_cast<uint8_t>(im.idx[t] - (t ? im.idx[t - 1] : 0u) + 128u);
  const uint32_t P = states[blockIdx.y].P;
  const uint32_t padded = (4 * P + kSymsPerGroup - 1) / kSymsPerGroup * kSymsPerGroup;
  if (4 * (P + t) < padded) reinterpret_cast<uint32_t *>(im.palette)[P + t] = 0u;
  if (t == 0) *im.palette_bytes = padded;
}

}  // namespace

// d_order: image ids by decreasing chunk count; chunks_desc: those counts
// (host).  d_states are cleared here.  One scoring launch per step, then the
// selection and the deltas.
cudaError_t launch_reencode(const ReImage *d_imgs, const uint32_t *d_order, ReState *d_states, uint32_t n_images,
                            const uint32_t *chunks_desc, uint32_t max_blocks, uint32_t *d_status, cudaStream_t stream,
                            int *launches) {
  cudaError_t e = cudaMemsetAsync(d_states, 0, sizeof(ReState) * n_images, stream);
  if (e != cudaSuccess || n_images == 0) return e;
  const uint32_t ctas = (kReChunk * kReGroups + kReWarps - 1) / kReWarps;
  gst_re_info_kernel<<<dim3((max_blocks + 255) / 256, n_images), 256, 0, stream>>>(d_imgs);
  uint32_t active = n_images;
  int nl = 1;
  for (uint32_t s = 0; s < chunks_desc[0]; ++s) {
    while (active > 0 && chunks_desc[active - 1] <= s) --active;
    gst_re_score_kernel<<<dim3(ctas, active), kReThreads, 0, stream>>>(d_imgs, d_order, d_states, s);
    ++nl;
  }
  gst_re_select_kernel<<<dim3((max_blocks + 7) / 8, n_images), 256, 0, stream>>>(d_imgs, d_states, d_status);
  const uint32_t fin = max_blocks > 2048 ? max_blocks : 2048;  // covers the palette padding (< 2048 words)
  gst_re_finish_kernel<<<dim3((fin + 255) / 256, n_images), 256, 0, stream>>>(d_imgs, d_states);
  if (launches) *launches = nl + 2;
  return cudaGetLastError();
}

}  // namespace gst
