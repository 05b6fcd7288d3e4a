// gst_kernels.cu -- sm_103a kernels of the GST decode path.
//
// Two kernels replace the reference's five OpenCL programs and their ~2S+4
// launches per batch (codec/decoder.cpp:164-417):
//
//  gst_rans_kernel  (ans/build_table.cl + ans/ans_decode.cl + the group sums of
//                    codec/decode_indices.cl)
//     One CTA = 8 warps = up to 8 rANS groups of one section.  The CTA builds
//     the section's 2048-slot decode table in shared memory (one packed u32 per
//     slot), then each warp decodes one group of 32 interleaved streams x 256
//     symbols: the 32 lanes are the 32 streams, a warp ballot + popcount gives
//     each renormalising lane its read offset (the reference uses local-memory
//     atomics and two barriers per symbol, ans_decode.cl:126-145).  Symbols go
//     out 16 at a time as 128-bit stores.  Warps of the index section also
//     produce the palette-index prefix sums at 32-block granularity; the last
//     index warp of an image turns the per-group sums into group prefixes
//     (threadfence-reduction pattern, no waiting).
//
//  gst_tile_kernel  (codec/inverse_wavelet.cl + codec/decode_indices.cl's
//                    per-block scan + codec/assemble.cl)
//     One CTA per 32x32-block tile of one image: loads the tile's six endpoint
//     planes, runs the five-level integer 5/3 inverse wavelet in shared memory,
//     converts YCoCg667 to RGB565, finishes the palette-index prefix sum with a
//     warp scan, gathers the palette word and writes whole 8-byte DXT1 blocks
//     (a warp writes 256 contiguous bytes).  Decoded endpoint planes and
//     indices never go back to HBM.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gst_plan.h"

namespace gst {

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ void flag_error(uint32_t *err, uint32_t bits) { atomicOr(err, bits); }

// ---------------------------------------------------------------------------
// Decode table (ans/build_table.cl:12-83).  Slot s in [0, 2048) belongs to the
// symbol x with cum[x] <= s < cum[x] + freq[x]; the table stores
// freq | (s - cum) << 12 | x << 23 so that one lookup gives the next state,
// x' = (x >> 11) * freq + (s - cum), equal to the reference's
// (x >> 11) * freq - cum + s in u32 arithmetic.  Requires blockDim.x == 256.
// Returns false (block-uniformly) if the frequencies do not sum to 2048.
__device__ bool build_decode_table(const uint16_t *__restrict__ freqs, uint32_t *tbl, uint32_t *cum_s,
                                   uint32_t *f_s, uint32_t *wsum) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t f = freqs[t];
  uint32_t v = f;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, v, d);
    if (lane >= d) v += n;
  }
  if (lane == 31) wsum[warp] = v;
  __syncthreads();
  uint32_t woff = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) woff += (w < warp) ? wsum[w] : 0u;
  const uint32_t excl = woff + v - f;
  cum_s[t] = excl;
  f_s[t] = f;
  if (t == 255) cum_s[256] = excl + f;
  __syncthreads();
  if (cum_s[256] != kTableSize) return false;
  for (uint32_t s = t; s < kTableSize; s += 256) {
    uint32_t x = 0;
#pragma unroll
    for (uint32_t step = 128; step >= 1; step >>= 1)
      if (cum_s[x + step] <= s) x += step;
    tbl[s] = f_s[x] | ((s - cum_s[x]) << 12) | (x << 23);
  }
  __syncthreads();
  return true;
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) gst_rans_kernel(const uint8_t *__restrict__ cmp,
                                                       uint8_t *__restrict__ scratch, GstPlanView plan) {
  __shared__ uint32_t tbl[kTableSize];
  __shared__ uint32_t cum_s[257];
  __shared__ uint32_t f_s[256];
  __shared__ uint32_t wsum[8];

  const GstRansItem it = plan.rans[blockIdx.x];
  const GstImageDesc &im = plan.images[it.image];
  uint32_t *err = &plan.head->err;
  const uint16_t *freqs = reinterpret_cast<const uint16_t *>(cmp + im.freq_off + kFreqTableBytes * it.section);
  const bool table_ok = build_decode_table(freqs, tbl, cum_s, f_s, wsum);
  if (!table_ok && threadIdx.x == 0) flag_error(err, kErrTable);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (static_cast<uint32_t>(warp) >= it.ngroups) return;
  const uint32_t g = it.first_group + warp;
  const uint32_t G = im.sec_groups[it.section];
  const uint32_t len = im.sec_len[it.section];
  const uint8_t *sec = cmp + im.body_off + im.sec_in[it.section];
  const uint32_t *ends = reinterpret_cast<const uint32_t *>(sec);
  const uint32_t hi = ends[g];
  const uint32_t lo = g == 0 ? 4u * G : ends[g - 1];
  const uint32_t ns = it.streams;
  const bool active = static_cast<uint32_t>(lane) < ns;
  const bool group_ok = table_ok && (hi & 3u) == 0 && hi <= len && lo <= len && hi >= lo + 4u * ns;
  const bool is_index = it.section == 3;

  int32_t suf[8];
  uint32_t total_sym = 0;
  if (group_ok) {
    const uint32_t top = hi - 4u * ns;  // the group's final states sit at [top, hi)
    uint32_t x = active ? reinterpret_cast<const uint32_t *>(sec + top)[lane] : kRansL;
    const uint16_t *words = reinterpret_cast<const uint16_t *>(sec);
    const uint32_t lo16 = lo >> 1, top16 = top >> 1;
    uint32_t ptr = top16;
    uint32_t bad = 0;
    const uint32_t lt = lanemask_lt();
    uint8_t *out = scratch + im.sym_off + im.sec_out[it.section] + static_cast<size_t>(g) * ns * kSymsPerStream +
                   static_cast<size_t>(lane) * kSymsPerStream;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      uint32_t w[4] = {0u, 0u, 0u, 0u};
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const uint32_t e = tbl[x & (kTableSize - 1)];
        x = (x >> 11) * (e & 0xFFFu) + ((e >> 12) & 0x7FFu);
        const uint32_t sym = e >> 23;
        const bool need = active && x < kRansL;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, need);
        const uint32_t total = __popc(m);
        if (need) {
          // ans_decode.cl:133-140: lanes that renormalise read consecutive
          // 16-bit words below the read pointer, lowest lane lowest address.
          const uint32_t idx = ptr - total + __popc(m & lt);
          uint32_t v = 0;
          if (idx - lo16 < top16 - lo16) v = __ldg(words + idx);
          else bad = 1;
          x = (x << 16) | v;
        }
        ptr -= total;
        w[3 - j / 4] = (w[3 - j / 4] << 8) | sym;
        total_sym += sym;
      }
      // Steps 16k..16k+15 are positions 255-16k .. 240-16k of this stream
      // (ans_decode.cl:154-155 writes the symbols in reverse).
      if (active) *reinterpret_cast<uint4 *>(out + 240 - 16 * k) = make_uint4(w[0], w[1], w[2], w[3]);
      if (is_index && (k & 1)) suf[k >> 1] = static_cast<int32_t>(total_sym) - 128 * 32 * ((k >> 1) + 1);
    }
    if (__any_sync(0xFFFFFFFFu, bad) && lane == 0) flag_error(err, kErrStream);
  } else if (lane == 0 && table_ok) {
    flag_error(err, kErrGroup);
  }

  if (!is_index) return;
  // Palette-index prefix sums (codec/decode_indices.cl computes them with a
  // multi-pass 128-wide scan; here: per 32-block chunk within the group, and
  // per group below).
  const int32_t T = group_ok ? suf[7] : 0;  // this lane's 256 deltas
  int32_t incl = T;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, d);
    if (lane >= d) incl += n;
  }
  if (group_ok) {
    const int32_t lane_off = incl - T;
    int32_t pre[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) pre[c] = lane_off + T - suf[7 - c];
    int32_t *chunk = reinterpret_cast<int32_t *>(scratch + im.chunk_off) + static_cast<size_t>(g) * 256 + lane * 8;
    reinterpret_cast<int4 *>(chunk)[0] = make_int4(pre[0], pre[1], pre[2], pre[3]);
    reinterpret_cast<int4 *>(chunk)[1] = make_int4(pre[4], pre[5], pre[6], pre[7]);
  }
  int32_t *gsum = reinterpret_cast<int32_t *>(scratch + im.gsum_off);
  uint32_t last = 0;
  if (lane == 31) {
    gsum[g] = incl;
    __threadfence();
    last = atomicAdd(&plan.counters[it.image], 1u) == G - 1;
  }
  last = __shfl_sync(0xFFFFFFFFu, last, 31);
  if (!last) return;
  __threadfence();
  // Exclusive prefix of the G group sums, one warp, 32 at a time.
  int32_t carry = 0;
  for (uint32_t base = 0; base < G; base += 32) {
    const uint32_t i = base + lane;
    const int32_t s = i < G ? __ldcg(gsum + i) : 0;
    int32_t v = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int32_t n = __shfl_up_sync(0xFFFFFFFFu, v, d);
      if (lane >= d) v += n;
    }
    if (i < G) gsum[G + i] = carry + v - s;
    carry += __shfl_sync(0xFFFFFFFFu, v, 31);
  }
}

// ---------------------------------------------------------------------------
// Inverse 5/3 lifting of one line of length L in place, with the arithmetic of
// inverse_wavelet.cl:28-64 (NormalizeIndex mirroring; C division).
template <int L>
__device__ __forceinline__ void inv53_line(int32_t *p, int step) {
  constexpr int mid = L / 2;
  int32_t s[L], d[L];
#pragma unroll
  for (int k = 0; k < L; ++k) s[k] = p[k * step];
#pragma unroll
  for (int x = 0; x < mid; ++x) {
    const int prev = mid + (x > 0 ? x - 1 : 0);  // mid + NormalizeIndex(2x-1, L)/2
    const int next = mid + x;                    // mid + NormalizeIndex(2x+1, L)/2
    d[2 * x] = s[x] - (s[prev] + s[next] + 2) / 4;
  }
#pragma unroll
  for (int x = 0; x < mid; ++x) {
    const int nx = (2 * x + 2 < L) ? 2 * x + 2 : L - 2;  // NormalizeIndex(2x+2, L)
    d[2 * x + 1] = s[mid + x] + (d[2 * x] + d[nx]) / 2;
  }
#pragma unroll
  for (int k = 0; k < L; ++k) p[k * step] = d[k];
}

constexpr int kPlanePitch = 33;  // row pitch in words: rows and columns both bank-conflict free
constexpr int kPlaneWords = 32 * kPlanePitch;

// One level over the top-left L x L of all six planes: rows, then columns.
template <int L>
__device__ __forceinline__ void inv53_level(int32_t *pl) {
  const int t = threadIdx.x;
  if (t < 6 * L) {
    const int p = t / L, r = t % L;
    inv53_line<L>(pl + p * kPlaneWords + r * kPlanePitch, 1);
  }
  __syncthreads();
  if (t < 6 * L) {
    const int p = t / L, c = t % L;
    inv53_line<L>(pl + p * kPlaneWords + c, kPlanePitch);
  }
  __syncthreads();
}

// assemble.cl:39-62: YCoCg667 -> RGB565 on int values of signed chars.
__device__ __forceinline__ uint32_t ycocg_to_565(int y, int co, int cg) {
  const int t = y - cg / 2;
  const int g = cg + t;
  const int b = (t - co) / 2;
  const int r = b + co;
  return ((static_cast<uint32_t>(r) << 11) | (static_cast<uint32_t>(g) << 5) | static_cast<uint32_t>(b)) & 0xFFFFu;
}

__global__ void __launch_bounds__(256) gst_tile_kernel(const uint8_t *__restrict__ scratch, uint8_t *__restrict__ out,
                                                       GstPlanView plan) {
  __shared__ int32_t pl[6 * kPlaneWords];
  const GstTileItem it = plan.tiles[blockIdx.x];
  const GstImageDesc &im = plan.images[it.image];
  const size_t B = static_cast<size_t>(im.bx) * im.by;
  const uint32_t tx = it.tile % im.tiles_x, ty = it.tile / im.tiles_x;
  const uint8_t *sym = scratch + im.sym_off;

  // The tile's 1024 coefficients of plane p are the tile-th 1024-byte run of
  // the plane (inverse_wavelet.cl:79-104); planes Y1 Y2 Co1 Cg1 Co2 Cg2 are
  // consecutive B-byte runs of the decoded Y and chroma sections.
  for (int i = threadIdx.x; i < 6 * 256; i += 256) {
    const int p = i >> 8, wi = i & 255;
    const uint32_t v = __ldg(reinterpret_cast<const uint32_t *>(sym + p * B + static_cast<size_t>(it.tile) * 1024) + wi);
    int32_t *dst = pl + p * kPlaneWords + (wi >> 3) * kPlanePitch + (wi & 7) * 4;
    dst[0] = static_cast<int32_t>(v & 0xFFu) - 128;
    dst[1] = static_cast<int32_t>((v >> 8) & 0xFFu) - 128;
    dst[2] = static_cast<int32_t>((v >> 16) & 0xFFu) - 128;
    dst[3] = static_cast<int32_t>(v >> 24) - 128;
  }
  __syncthreads();
  inv53_level<2>(pl);
  inv53_level<4>(pl);
  inv53_level<8>(pl);
  inv53_level<16>(pl);
  inv53_level<32>(pl);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int32_t *chunk_pref = reinterpret_cast<const int32_t *>(scratch + im.chunk_off);
  const int32_t *gpref = reinterpret_cast<const int32_t *>(scratch + im.gsum_off) + im.sec_groups[3];
  const uint8_t *deltas = sym + im.sec_out[3];
  const uint32_t *pal = reinterpret_cast<const uint32_t *>(sym + im.sec_out[2]);
  bool bad = false;
#pragma unroll
  for (int rr = 0; rr < 4; ++rr) {
    const int r = warp + 8 * rr;
    const uint32_t p0 = (ty * 32 + r) * im.bx + tx * 32;  // first block of this row segment
    const uint32_t p = p0 + lane;
    uint32_t d = static_cast<uint32_t>(__ldg(deltas + p)) - 128u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, d, o);
      if (lane >= o) d += n;
    }
    const uint32_t idx = static_cast<uint32_t>(gpref[p0 >> 13]) + static_cast<uint32_t>(chunk_pref[p0 >> 5]) + d;
    uint32_t word = 0;
    if (idx < im.palette_words) word = __ldg(pal + idx);
    else bad = true;
    const int32_t *row = pl + r * kPlanePitch + lane;
    const int y1 = static_cast<int8_t>(row[0]), y2 = static_cast<int8_t>(row[kPlaneWords]);
    const int co1 = static_cast<int8_t>(row[2 * kPlaneWords]), cg1 = static_cast<int8_t>(row[3 * kPlaneWords]);
    const int co2 = static_cast<int8_t>(row[4 * kPlaneWords]), cg2 = static_cast<int8_t>(row[5 * kPlaneWords]);
    const uint32_t ep1 = ycocg_to_565(y1, co1, cg1), ep2 = ycocg_to_565(y2, co2, cg2);
    *reinterpret_cast<uint2 *>(out + im.out_off + static_cast<size_t>(p) * 8) = make_uint2(ep1 | (ep2 << 16), word);
  }
  if (__any_sync(0xFFFFFFFFu, bad) && lane == 0) flag_error(&plan.head->err, kErrPalette);
}

// Enqueues the decode of one plan.  With `ev` non-null, records ev[0] before
// the first kernel and ev[i + 1] after kernel i (instrumentation).
cudaError_t launch_decode(const uint8_t *d_cmp, uint8_t *d_scratch, uint8_t *d_out, const GstPlanView &plan,
                          cudaStream_t stream, int *launches, cudaEvent_t *ev) {
  *launches = 0;
  if (ev) cudaEventRecord(ev[0], stream);
  if (plan.n_rans) {
    gst_rans_kernel<<<plan.n_rans, 256, 0, stream>>>(d_cmp, d_scratch, plan);
    ++*launches;
    if (ev) cudaEventRecord(ev[*launches], stream);
  }
  if (plan.n_tiles) {
    gst_tile_kernel<<<plan.n_tiles, 256, 0, stream>>>(d_scratch, d_out, plan);
    ++*launches;
    if (ev) cudaEventRecord(ev[*launches], stream);
  }
  return cudaGetLastError();
}

const char *kernel_name(int i) { return i == 0 ? "gst_rans_kernel" : "gst_tile_kernel"; }

}  // namespace gst
