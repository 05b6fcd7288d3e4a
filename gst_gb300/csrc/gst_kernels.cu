// gst_kernels.cu -- sm_103a kernels of the GST decode path.
//
// Two kernels replace the reference's five OpenCL programs and their ~2S+4
// launches per batch (codec/decoder.cpp:164-417):
//
//  gst_rans_kernel  (ans/build_table.cl + ans/ans_decode.cl + the group sums of
//                    codec/decode_indices.cl)
//     One CTA = 4 warps = up to 4 rANS groups of one section (small CTAs keep
//     the groups of a batch spread evenly over the SMs).  The CTA builds the
//     section's 2048-slot decode table in shared memory (one packed u32 per
//     slot), then each warp decodes one group of 32 interleaved streams x 256
//     symbols: the 32 lanes are the 32 streams, a warp ballot + popcount gives
//     each renormalising lane its read offset (the reference uses local-memory
//     atomics and two barriers per symbol, ans_decode.cl:43-65).  Symbols go
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

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>

#include "gst_host.h"
#include "gst_plan.h"

namespace gst {

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Error bits go to the call's status word and, where the plan has them, to the
// image's own word (so that a batch can report per image).
// Barrier `id` over `n` threads (a multiple of 32): id 0 over the whole CTA is
// __syncthreads; the persistent kernel's two rANS halves use ids 1 and 2.
__device__ __forceinline__ void bar_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

__device__ __forceinline__ void flag_error(uint32_t *err, uint32_t *image_err, uint32_t bits) {
  atomicOr(err, bits);
  if (image_err) atomicOr(image_err, bits);
}

// ---------------------------------------------------------------------------
// Decode table (ans/build_table.cl:12-83).  Slot s in [0, 2048) belongs to the
// symbol x with cum[x] <= s < cum[x] + freq[x]; the table stores
// x | (s - cum) << 8 | freq << 19 (8, 11 and 12 bits) so that one lookup
// gives the next state, x' = (x >> 11) * freq + (s - cum), equal to the
// reference's (x >> 11) * freq - cum + s in u32 arithmetic, and the symbol as
// the entry's low byte.  Both shifted fields come out of the entry with one
// independent shift each (entry >> 19 = freq, entry >> 8 = freq * 2048 +
// s - cum), so the state update is one dependent step shorter than with a
// masked field.
//
// Built without searching: each symbol with freq > 0 marks its first slot,
// and since those first slots increase with x, a running maximum of the marks
// over the slots gives every slot's symbol.  Entry = (freq << 19 | x) -
// (cum << 8) + (s << 8), from one per-symbol word.  Run by 128 threads (t = 0..127) that
// synchronise on named barrier BAR; `work` is 3 KB of shared scratch
// (per-symbol words, slot marks) that is free again on return.  Returns false
// (uniformly over the 128 threads) if the frequencies do not sum to 2048.
template <int BAR>
__device__ bool build_decode_table(const uint16_t *__restrict__ freqs, uint32_t *tbl, uint32_t *wred,
                                   uint8_t *work, int t) {
  const int lane = t & 31, warp = t >> 5;
  uint32_t *sym_word = reinterpret_cast<uint32_t *>(work);  // 256
  uint8_t *marks = work + 1024;                             // 2048
  reinterpret_cast<uint4 *>(marks)[t] = make_uint4(0, 0, 0, 0);
  const uint32_t f0 = freqs[2 * t], f1 = freqs[2 * t + 1];
  uint32_t v = f0 + f1;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, v, d);
    if (lane >= d) v += n;
  }
  if (lane == 31) wred[warp] = v;
  bar_sync(BAR, 128);
  uint32_t woff = 0;
#pragma unroll
  for (int w = 0; w < 4; ++w) woff += (w < warp) ? wred[w] : 0u;
  const uint32_t total = wred[0] + wred[1] + wred[2] + wred[3];
  const uint32_t c0 = woff + v - f0 - f1, c1 = c0 + f0;
  const uint32_t x0 = 2 * t, x1 = 2 * t + 1;
  sym_word[x0] = ((f0 << 19) | x0) - (c0 << 8);
  sym_word[x1] = ((f1 << 19) | x1) - (c1 << 8);
  if (total == kTableSize) {  // then every marked slot c < cum + freq <= 2048
    if (f0) marks[c0] = static_cast<uint8_t>(x0);
    if (f1) marks[c1] = static_cast<uint8_t>(x1);
  }
  bar_sync(BAR, 128);
  if (total != kTableSize) return false;
  // Thread t owns slots [16t, 16t + 16): running maximum within, then an
  // exclusive maximum over the preceding threads.
  const uint4 mk = reinterpret_cast<const uint4 *>(marks)[t];
  const uint32_t mw[4] = {mk.x, mk.y, mk.z, mk.w};
  uint32_t own[16], run = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    run = max(run, (mw[k >> 2] >> (8 * (k & 3))) & 0xFFu);
    own[k] = run;
  }
  uint32_t incl = run;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, d);
    if (lane >= d) incl = max(incl, n);
  }
  if (lane == 31) wred[4 + warp] = incl;
  uint32_t excl = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
  if (lane == 0) excl = 0;
  bar_sync(BAR, 128);
#pragma unroll
  for (int w = 0; w < 3; ++w)
    if (w < warp) excl = max(excl, wred[4 + w]);
  uint32_t e[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) e[k] = sym_word[max(own[k], excl)] + (static_cast<uint32_t>(16 * t + k) << 8);
  uint4 *dst = reinterpret_cast<uint4 *>(tbl) + 4 * t;
  dst[0] = make_uint4(e[0], e[1], e[2], e[3]);
  dst[1] = make_uint4(e[4], e[5], e[6], e[7]);
  dst[2] = make_uint4(e[8], e[9], e[10], e[11]);
  dst[3] = make_uint4(e[12], e[13], e[14], e[15]);
  bar_sync(BAR, 128);
  return true;
}

// ---------------------------------------------------------------------------
// rANS kernel shared memory: the decode table, the table-build scratch, and one
// staging buffer per warp holding the renormalisation words the warp is about
// to read, so that the serial decode chain reads shared memory, not HBM.
// The stage holds `stage_words` 16-bit words per warp (a launch parameter, the
// "staging depth" tuning knob), each warp's stage padded by 8 words of slack
// for the 16-byte alignment of the copy.
// The table build's 3 KB of scratch lives in the (not yet used) stages.
struct alignas(16) RansHead {
  uint32_t tbl[kTableSize];
  uint32_t wred[8];
};
constexpr size_t kStageOffset = (sizeof(RansHead) + 15) & ~size_t(15);
__host__ __device__ constexpr size_t rans_smem_bytes(uint32_t stage_words) {
  return kStageOffset + size_t(kGroupsPerRansCta) * (stage_words + 8) * 2;
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Warp-cooperative copy of the 4-aligned byte range [a, b) into `buf`, where
// buf[0] corresponds to the 16-byte-aligned address at or below a.  The bulk
// goes as 16-byte cp.async copies, the unaligned ends as 4-byte ones; nothing
// outside [a, b) is read.
__device__ __forceinline__ void stage_range(uint8_t *buf, const uint8_t *a, const uint8_t *b, int lane) {
  const uintptr_t ua = reinterpret_cast<uintptr_t>(a), ub = reinterpret_cast<uintptr_t>(b);
  const uintptr_t origin = ua & ~uintptr_t(15);
  uintptr_t m0 = (ua + 15) & ~uintptr_t(15), m1 = ub & ~uintptr_t(15);
  if (m0 >= m1) m0 = m1 = ub;  // no whole 16-byte chunk: all 4-byte copies
  const int head = static_cast<int>((m0 - ua) >> 2), tail = static_cast<int>((ub - m1) >> 2);
  if (lane < head) cp_async4(buf + (ua + 4 * lane - origin), reinterpret_cast<const void *>(ua + 4 * lane));
  if (lane < tail) cp_async4(buf + (m1 + 4 * lane - origin), reinterpret_cast<const void *>(m1 + 4 * lane));
  const int chunks = static_cast<int>((m1 - m0) >> 4);
  for (int c = lane; c < chunks; c += 32)
    cp_async16(buf + (m0 + 16 * c - origin), reinterpret_cast<const void *>(m0 + 16 * c));
  cp_async_wait_all();
  __syncwarp();
}

__device__ __forceinline__ uint32_t lds_u32(uint32_t a) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ uint32_t lds_u16(uint32_t a) {
  uint16_t v;
  asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(a));
  return v;
}

// Integer multiply-adds, kept as such so that they issue to the FMA pipe and
// leave the integer ALU pipe to the shifts, logic and warp votes.
__device__ __forceinline__ uint32_t mad_lo(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
__device__ __forceinline__ uint32_t mad_hi(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("mad.hi.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
__device__ __forceinline__ uint32_t mul_hi(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("mul.hi.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

// Decodes one group: ns <= 32 interleaved streams of 256 symbols whose final
// states sit at [top, hi) and whose renormalisation words fill [lo, top) of
// the section `sec` (ans_decode.cl:25-74).  Lane l is stream l, its 256
// symbols go to out[0..255].  When INDEX (the palette-index deltas
// d = symbol - 128), out instead receives 256 int16: for position k of the
// stream, the sum of d over the positions after k within k's 32-position
// chunk (decode order runs backwards, so that is the chunk's running sum when
// k is decoded); and suf[m] returns the sum of d over the last 32(m + 1)
// positions.
//
// The top stage_words words of [lo, top) are staged in shared memory; every 16
// steps, if the next 16 steps could read below the staged words, the warp
// re-stages the stage_words words below its read pointer (a warp-uniform test;
// groups that fit never re-stage).
//
// One step, with q = x >> 11 and the table entry e of slot x mod 2048:
//   x' = q * freq + (s - cum), computed as (q - 2048) * (e >> 19) + (e >> 8)
//   (e >> 8 = freq * 2048 + s - cum: the freq * 2048 term cancels), and the
//   slot's byte offset 4x - 8192 q as multiply-adds.  Renormalising lanes read consecutive
//   words below the read pointer, the lowest lane the lowest address
//   (ans_decode.cl:50-57): lane l's word lies popc(renormalising lanes >= l)
//   words below the pointer, and only those lanes load it from the stage.
// For a valid stream the read pointer never goes below the staged words; a
// malformed one is caught at the end of a 16-step run (the pointer is then
// clamped so that every read stays inside the CTA's shared memory) or by the
// final pointer.
template <bool INDEX>
__device__ __forceinline__ bool decode_group(const uint8_t *__restrict__ sec, uint32_t lo, uint32_t top,
                                             const uint32_t *__restrict__ tbl, uint16_t *stage, uint32_t stage_words,
                                             int lane, bool active, uint8_t *__restrict__ out, int32_t suf[8]) {


  const int lo16 = static_cast<int>(lo >> 1);
  uint32_t stage_lo = (top - lo > 2u * stage_words) ? top - 2u * stage_words : lo;
  stage_range(reinterpret_cast<uint8_t *>(stage), sec + stage_lo, sec + top, lane);
  // stage[0] holds the word at sec + stage_lo rounded down to 16 bytes, so
  // word idx of the section is stage[idx - sbase16].
  int sbase16 = static_cast<int>(stage_lo >> 1) -
                static_cast<int>((reinterpret_cast<uintptr_t>(sec + stage_lo) & 15) >> 1);
  uint32_t x = active ? reinterpret_cast<const uint32_t *>(sec + top)[lane] : kRansL;
  int ptr = static_cast<int>(top >> 1);      // word index of the section
  const uint32_t stage_s = static_cast<uint32_t>(__cvta_generic_to_shared(stage));
  const uint32_t tbl_c = static_cast<uint32_t>(__cvta_generic_to_shared(tbl)) - (1u << 24);
  uint32_t s2 = stage_s + 2u * (ptr - sbase16);  // shared address of word ptr in the stage
  const uint32_t ge = ~lanemask_lt();
  bool bad = false;
  int32_t crun = 0, tot = 0;  // INDEX: running sum within the chunk, and over the chunks done
  int32_t s0 = 0, s1 = 0, s2_ = 0, s3 = 0, s4 = 0, s5 = 0, s6 = 0, s7 = 0;
  uint4 even_run = make_uint4(0, 0, 0, 0);  // symbols of the last even run, stored with the next odd one
#pragma unroll 2
  for (int k = 0; k < 16; ++k) {
    if (ptr - 16 * 32 < static_cast<int>(stage_lo >> 1) && static_cast<int>(stage_lo) > static_cast<int>(lo) &&
        ptr > lo16) {
      // Every later read is below ptr: stage the words just below it.
      const uint32_t new_top = (2u * static_cast<uint32_t>(ptr) + 3u) & ~3u;
      stage_lo = (new_top - lo > 2u * stage_words) ? new_top - 2u * stage_words : lo;
      stage_range(reinterpret_cast<uint8_t *>(stage), sec + stage_lo, sec + new_top, lane);
      sbase16 = static_cast<int>(stage_lo >> 1) -
                static_cast<int>((reinterpret_cast<uintptr_t>(sec + stage_lo) & 15) >> 1);
      s2 = stage_s + 2u * (ptr - sbase16);
    }
    if (static_cast<int>(s2 - stage_s) < 0) {  // only a malformed stream gets here
      bad = true;
      s2 = stage_s;
    }
    uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;
    uint32_t ew[8];  // INDEX: 16 int16 partial sums, slot 15 - j for step j
    if (INDEX && !(k & 1)) crun = 0;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const uint32_t qm = mad_hi(x, 1u << 21, 0u - 2048u);            // q - 2048
      const uint32_t ea = mad_lo(qm, 0u - 8192u, mad_lo(x, 4u, tbl_c));  // table + 4 (x mod 2048)
      const uint32_t e = lds_u32(ea);
      x = mad_lo(e >> 19, qm, e >> 8);
      const bool need = active && x < kRansL;
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, need);
      if (need) {
        const uint32_t depth2 = 2u * static_cast<uint32_t>(__popc(m & ge));
        const uint32_t v = lds_u16(s2 - depth2);
        x = mad_lo(x, 65536u, v);
      }
      s2 = mad_lo(static_cast<uint32_t>(__popc(m)), 0u - 2u, s2);
      // Steps 16k..16k+15 are positions 255-16k .. 240-16k of this stream
      // (ans_decode.cl:71-72 stores the symbols in reverse).
      if constexpr (INDEX) {
        const uint32_t part = static_cast<uint32_t>(crun) & 0xFFFFu;
        crun += static_cast<int32_t>(e & 0xFFu) - 128;
        if (j & 1) ew[7 - (j >> 1)] |= part;  // slot 15 - j, even: low half
        else ew[7 - (j >> 1)] = part << 16;   // odd slot: high half
      } else {
        if (j < 4) w3 = __byte_perm(w3, e, 0x2104);
        else if (j < 8) w2 = __byte_perm(w2, e, 0x2104);
        else if (j < 12) w1 = __byte_perm(w1, e, 0x2104);
        else w0 = __byte_perm(w0, e, 0x2104);
      }
    }
    ptr = static_cast<int>((s2 - stage_s) >> 1) + sbase16;
    if constexpr (INDEX) {
      if (active) {
        uint4 *o = reinterpret_cast<uint4 *>(out + 2 * (240 - 16 * k));
        o[0] = make_uint4(ew[0], ew[1], ew[2], ew[3]);
        o[1] = make_uint4(ew[4], ew[5], ew[6], ew[7]);
      }
    } else if (!(k & 1)) {
      even_run = make_uint4(w0, w1, w2, w3);
    } else if (active) {
      // Runs k - 1 and k fill positions 224 - 16(k - 1) .. 255 - 16(k - 1),
      // one aligned 32-byte sector: written whole, so that no sector of the
      // output reaches L2 in two halves.
      uint4 *o = reinterpret_cast<uint4 *>(out + 240 - 16 * k);
      o[0] = make_uint4(w0, w1, w2, w3);
      o[1] = even_run;
    }
    if (INDEX && (k & 1)) {
      const int mm = k >> 1;
      tot += crun;
      const int32_t v = tot;
      s0 = mm == 0 ? v : s0;
      s1 = mm == 1 ? v : s1;
      s2_ = mm == 2 ? v : s2_;
      s3 = mm == 3 ? v : s3;
      s4 = mm == 4 ? v : s4;
      s5 = mm == 5 ? v : s5;
      s6 = mm == 6 ? v : s6;
      s7 = mm == 7 ? v : s7;
    }
  }
  if (INDEX) {
    suf[0] = s0; suf[1] = s1; suf[2] = s2_; suf[3] = s3;
    suf[4] = s4; suf[5] = s5; suf[6] = s6; suf[7] = s7;
  }
  // The lowest word read is the final pointer.
  return __any_sync(0xFFFFFFFFu, bad || ptr < lo16);
}

// Group g of `section`, decoded by one warp with `ns` streams (lanes) against
// the table in `tbl`, staging through `stage`.  `counter` counts the image's
// finished index groups; image_err (may be null) is the image's error word.
__device__ __forceinline__ void rans_group(const uint8_t *__restrict__ cmp, uint8_t *__restrict__ scratch,
                                           uint32_t *err, uint32_t *image_err, uint32_t *counter,
                                           const GstImageDesc &im, uint32_t section, uint32_t g, uint32_t ns,
                                           bool table_ok, const uint32_t *tbl, uint16_t *stage,
                                           uint32_t stage_words) {
  const int lane = threadIdx.x & 31;
  const uint32_t G = im.sec_groups[section];
  const uint32_t len = im.sec_len[section];
  const uint8_t *sec = cmp + im.body_off + im.sec_in[section];
  const uint32_t *ends = reinterpret_cast<const uint32_t *>(sec);
  const uint32_t hi = ends[g];
  const uint32_t lo = g == 0 ? 4u * G : ends[g - 1];
  const bool active = static_cast<uint32_t>(lane) < ns;
  const bool group_ok = table_ok && (hi & 3u) == 0 && (lo & 3u) == 0 && hi <= len && lo <= len &&
                        hi >= lo + 4u * ns;
  const bool is_index = section == 3;
  // Index sections store 2 bytes per position (decode_group<true>).
  const size_t pos = static_cast<size_t>(g) * ns * kSymsPerStream + static_cast<size_t>(lane) * kSymsPerStream;
  uint8_t *out = scratch + im.sym_off + im.sec_out[section] + (is_index ? 2 * pos : pos);

  int32_t suf[8];
  if (group_ok) {
    const uint32_t top = hi - 4u * ns;  // the group's final states sit at [top, hi)
    const bool bad = is_index ? decode_group<true>(sec, lo, top, tbl, stage, stage_words, lane, active, out, suf)
                              : decode_group<false>(sec, lo, top, tbl, stage, stage_words, lane, active, out, suf);
    if (bad && lane == 0) flag_error(err, image_err, kErrStream);
  } else if (lane == 0 && table_ok) {
    flag_error(err, image_err, kErrGroup);
  }

  if (!is_index) return;
  // Palette-index prefix sums (codec/decode_indices.cl computes them with a
  // multi-pass 128-wide scan; here: the prefix through the end of each
  // 32-block chunk within the group, and per group below; a block's index is
  // then group prefix + chunk prefix - its partial sum from decode_group).
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
    for (int c = 0; c < 8; ++c) pre[c] = lane_off + T - (c < 7 ? suf[6 - c] : 0);
    int32_t *chunk = reinterpret_cast<int32_t *>(scratch + im.chunk_off) + static_cast<size_t>(g) * 256 + lane * 8;
    reinterpret_cast<int4 *>(chunk)[0] = make_int4(pre[0], pre[1], pre[2], pre[3]);
    reinterpret_cast<int4 *>(chunk)[1] = make_int4(pre[4], pre[5], pre[6], pre[7]);
  }
  int32_t *gsum = reinterpret_cast<int32_t *>(scratch + im.gsum_off);
  uint32_t last = 0;
  if (lane == 31) {
    gsum[g] = incl;
    __threadfence();
    last = atomicAdd(counter, 1u) == G - 1;
  }
  last = __shfl_sync(0xFFFFFFFFu, last, 31);
  if (!last) return;
  __threadfence();
  // Every index group of this image is done: re-arm the counter so that a
  // resident plan can be launched again without a re-upload.
  if (lane == 0) *counter = 0;
  // Exclusive prefix of the G group sums, one warp, 32 at a time.
  int32_t carry = 0;
  for (uint32_t base = 0; base < G; base += 32) {
    const uint32_t i = base + lane;
    const int32_t sv = i < G ? __ldcg(gsum + i) : 0;
    int32_t v = sv;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int32_t n = __shfl_up_sync(0xFFFFFFFFu, v, d);
      if (lane >= d) v += n;
    }
    if (i < G) gsum[G + i] = carry + v - sv;
    carry += __shfl_sync(0xFFFFFFFFu, v, 31);
  }
}

// One rANS work item: ngroups <= 4 groups of one section, group first_group + w
// decoded by warp w of a group of 128 threads (t = 0..127) that owns the
// shared memory at `smem` (rans_smem_bytes(stage_words)) and named barrier
// BAR; all of them return.
template <int BAR>
__device__ __forceinline__ void rans_item(const uint8_t *__restrict__ cmp, uint8_t *__restrict__ scratch,
                                          uint32_t *err, uint32_t *image_err, uint32_t *counter,
                                          const GstImageDesc &im, uint32_t section, uint32_t first_group,
                                          uint32_t ngroups, uint32_t ns, uint32_t stage_words, uint8_t *smem,
                                          int t) {
  RansHead &sm = *reinterpret_cast<RansHead *>(smem);
  const uint16_t *freqs = reinterpret_cast<const uint16_t *>(cmp + im.freq_off + kFreqTableBytes * section);
  const bool table_ok = build_decode_table<BAR>(freqs, sm.tbl, sm.wred, smem + kStageOffset, t);
  if (!table_ok && t == 0) flag_error(err, image_err, kErrTable);
  const uint32_t warp = static_cast<uint32_t>(t) >> 5;
  if (warp < ngroups) {
    uint16_t *stage = reinterpret_cast<uint16_t *>(smem + kStageOffset) + warp * (stage_words + 8);
    rans_group(cmp, scratch, err, image_err, counter, im, section, first_group + warp, ns, table_ok, sm.tbl, stage,
               stage_words);
  }
}

// MINB: CTAs of 128 threads per SM that the register allocation must allow
// (the "blocks per SM" tuning knob: 8 leaves 64 registers, 12 about 40,
// 16 fills the SM with 64 warps at 32).
// Programmatic dependent launch.  The rANS kernel lets the tile kernel queued
// right behind it launch as soon as every rANS CTA has started; tile CTAs then
// wait in griddepcontrol.wait until the rANS grid has completed and its writes
// are visible.  Tile CTAs can only become resident after every rANS CTA has
// started, so they never hold resources a rANS CTA still needs.  Launched
// without the attribute, the wait returns at once.
__device__ __forceinline__ void pdl_release_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait_prerequisites() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <int MINB>
__global__ void __launch_bounds__(128, MINB) gst_rans_kernel(const uint8_t *__restrict__ cmp,
                                                             uint8_t *__restrict__ scratch, GstPlanView plan) {
  pdl_release_dependents();
  extern __shared__ __align__(16) uint8_t smem_raw[];
  const GstRansItem it = plan.rans[plan.rans_order ? plan.rans_order[blockIdx.x] : blockIdx.x];
  rans_item<0>(cmp, scratch, plan.err, plan.image_err ? plan.image_err + it.image : nullptr,
               plan.counters + it.image, plan.images[it.image], it.section, it.first_group, it.ngroups, it.streams,
               plan.stage_words, smem_raw, threadIdx.x);
}

// ---------------------------------------------------------------------------
// Byte (SEL & 7) of w sign-extended to 32 bits: a byte permute whose upper
// selector nibbles have the sign-replicate bit set (prmt's default mode).
template <uint32_t SEL>
__device__ __forceinline__ int32_t sext_byte(uint32_t w) {
  uint32_t d;
  asm("prmt.b32 %0, %1, 0, %2;" : "=r"(d) : "r"(w), "n"(SEL));
  return static_cast<int32_t>(d);
}

// Inverse 5/3 lifting of one line of length L in place, with the arithmetic of
// inverse_wavelet.cl:28-64 (NormalizeIndex mirroring; C division).
template <int L>
__device__ __forceinline__ void inv53_lift(const int32_t (&s)[L], int32_t (&d)[L]) {
  constexpr int mid = L / 2;
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
}

template <int L>
__device__ __forceinline__ void inv53_line(int32_t *p, int step) {
  int32_t s[L], d[L];
#pragma unroll
  for (int k = 0; k < L; ++k) s[k] = p[k * step];
  inv53_lift<L>(s, d);
#pragma unroll
  for (int k = 0; k < L; ++k) p[k * step] = d[k];
}

// A row of L coefficients (8-byte aligned: even pitch, even plane stride),
// moved two at a time.
template <int L>
__device__ __forceinline__ void inv53_row(int32_t *p) {
  int32_t s[L], d[L];
  int2 *q = reinterpret_cast<int2 *>(p);
#pragma unroll
  for (int k = 0; k < L / 2; ++k) {
    const int2 v = q[k];
    s[2 * k] = v.x;
    s[2 * k + 1] = v.y;
  }
  inv53_lift<L>(s, d);
#pragma unroll
  for (int k = 0; k < L / 2; ++k) q[k] = make_int2(d[2 * k], d[2 * k + 1]);
}

// A row segment of N values from registers to (8-byte aligned) shared memory.
template <int N>
__device__ __forceinline__ void store_row(int32_t *p, const int32_t *v) {
  int2 *q = reinterpret_cast<int2 *>(p);
#pragma unroll
  for (int k = 0; k < N / 2; ++k) q[k] = make_int2(v[2 * k], v[2 * k + 1]);
}

// The 16 coefficients (byte - 128) of a 16-byte chunk: the byte with its top
// bit flipped, sign-extended by one byte permute.
__device__ __forceinline__ void unpack16(uint4 cv, int32_t *dst) {
  const uint32_t w[4] = {cv.x ^ 0x80808080u, cv.y ^ 0x80808080u, cv.z ^ 0x80808080u, cv.w ^ 0x80808080u};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    dst[4 * k + 0] = sext_byte<0x8880u>(w[k]);
    dst[4 * k + 1] = sext_byte<0x9991u>(w[k]);
    dst[4 * k + 2] = sext_byte<0xAAA2u>(w[k]);
    dst[4 * k + 3] = sext_byte<0xBBB3u>(w[k]);
  }
}

// Row pitch in words: even, so that a thread moves its row two words at a
// time (8-byte accesses by 16 rows of a half-warp start on 16 different even
// banks), and columns stay bank-conflict free (a warp's 32 columns of one row
// are consecutive words).
constexpr int kPlanePitch = 34;
// Planes 16 banks apart, so that half-warps working on two planes at once do
// not collide.
constexpr int kPlaneWords = 32 * kPlanePitch + 16;

// One level over the top-left L x L of all six planes: rows, then columns;
// NT threads take the 6L lines of each pass.
template <int L, int NT>
__device__ __forceinline__ void inv53_level(int32_t *pl) {
#pragma unroll
  for (int t = threadIdx.x; t < 6 * L; t += NT) {
    const int p = t / L, r = t % L;
    inv53_row<L>(pl + p * kPlaneWords + r * kPlanePitch);
  }
  __syncthreads();
#pragma unroll
  for (int t = threadIdx.x; t < 6 * L; t += NT) {
    const int p = t / L, c = t % L;
    inv53_line<L>(pl + p * kPlaneWords + c, kPlanePitch);
  }
  __syncthreads();
}

// The same over the first NG threads of the CTA only (threadIdx.x < NG), which
// synchronise on named barrier BAR.
template <int L, int NG, int BAR>
__device__ __forceinline__ void inv53_level_group(int32_t *pl) {
#pragma unroll
  for (int t = threadIdx.x; t < 6 * L; t += NG) {
    const int p = t / L, r = t % L;
    inv53_row<L>(pl + p * kPlaneWords + r * kPlanePitch);
  }
  bar_sync(BAR, NG);
#pragma unroll
  for (int t = threadIdx.x; t < 6 * L; t += NG) {
    const int p = t / L, c = t % L;
    inv53_line<L>(pl + p * kPlaneWords + c, kPlanePitch);
  }
  bar_sync(BAR, NG);
}

// assemble.cl:39-62: YCoCg667 -> RGB565 on int values of signed chars.  The
// reference's ushort endpoint is the low 16 bits of the result (the caller
// keeps only those).
__device__ __forceinline__ uint32_t ycocg_to_565(int y, int co, int cg) {
  const int t = y - cg / 2;
  const int g = cg + t;
  const int b = (t - co) / 2;
  const int r = b + co;
  return (static_cast<uint32_t>(r) << 11) | (static_cast<uint32_t>(g) << 5) | static_cast<uint32_t>(b);
}

// assemble.cl:83-129 (assemble_rgb): an endpoint as 8-bit R, G, B by bit
// replication of its 5:6:5 integers, packed as bytes 0-2 of a word (each the
// low 8 bits of the reference's int).
__device__ __forceinline__ void ycocg_to_rgb8(int y, int co, int cg, int c[3]) {
  const int t = y - cg / 2;
  const int g = cg + t;
  const int b = (t - co) / 2;
  const int r = b + co;
  c[0] = static_cast<int>(static_cast<uint32_t>(r) << 3) | (r >> 2);
  c[1] = static_cast<int>(static_cast<uint32_t>(g) << 2) | (g >> 4);
  c[2] = static_cast<int>(static_cast<uint32_t>(b) << 3) | (b >> 2);
}
__device__ __forceinline__ uint32_t pack_rgb8(int r, int g, int b) {
  return (static_cast<uint32_t>(r) & 0xFFu) | ((static_cast<uint32_t>(g) & 0xFFu) << 8) |
         ((static_cast<uint32_t>(b) & 0xFFu) << 16);
}

// Writes the 4x4 RGB8 pixels of one block (48 bytes over four pixel rows of
// `pitch` bytes): the reference's four-colour palette, endpoints, then
// (2a + b) / 3 and (a + 2b) / 3 in C integer division, selected by 2-bit
// fields of `word`, low bits first, raster order within the block.
__device__ __forceinline__ void store_rgb_block(uint8_t *o, size_t pitch, int y1, int co1, int cg1, int y2, int co2,
                                                int cg2, uint32_t word) {
  int a[3], b[3];
  ycocg_to_rgb8(y1, co1, cg1, a);
  ycocg_to_rgb8(y2, co2, cg2, b);
  const uint32_t c0 = pack_rgb8(a[0], a[1], a[2]), c1 = pack_rgb8(b[0], b[1], b[2]);
  const uint32_t c2 = pack_rgb8((2 * a[0] + b[0]) / 3, (2 * a[1] + b[1]) / 3, (2 * a[2] + b[2]) / 3);
  const uint32_t c3 = pack_rgb8((a[0] + 2 * b[0]) / 3, (a[1] + 2 * b[1]) / 3, (a[2] + 2 * b[2]) / 3);
  auto pick = [&](uint32_t s) { return (s & 2u) ? ((s & 1u) ? c3 : c2) : ((s & 1u) ? c1 : c0); };
#pragma unroll
  for (int py = 0; py < 4; ++py) {
    const uint32_t q0 = pick(word), q1 = pick(word >> 2), q2 = pick(word >> 4), q3 = pick(word >> 6);
    word >>= 8;
    uint32_t *dst = reinterpret_cast<uint32_t *>(o + pitch * py);
    dst[0] = __byte_perm(q0, q1, 0x4210);  // r0 g0 b0 r1
    dst[1] = __byte_perm(q1, q2, 0x5421);  // g1 b1 r2 g2
    dst[2] = __byte_perm(q2, q3, 0x6542);  // b2 r3 g3 b3
  }
}

// Loads of decoded symbols: through the read-only path when another kernel
// wrote them (COH false), coherently at L2 when CTAs of the same kernel did.
template <bool COH, typename T>
__device__ __forceinline__ T ld_sym(const T *p) {
  if constexpr (COH) return __ldcg(p);
  else return __ldg(p);
}

constexpr size_t kTileSmemBytes = 6 * kPlaneWords * sizeof(int32_t);

// One 32x32-block tile of one image with NT threads; `pl` is kTileSmemBytes
// of shared memory.  Writes DXT1 blocks, or with RGB the blocks' RGB8 pixels
// (LoadRGB).  All threads return.
template <int NT, bool COH, bool RGB = false>
__device__ __forceinline__ void tile_work(const uint8_t *__restrict__ scratch, uint8_t *__restrict__ out,
                                          uint32_t *err, uint32_t *image_err, const GstImageDesc &im,
                                          uint32_t tile, int32_t *pl) {
  constexpr int kWarps = NT / 32;
  constexpr int kRows = 32 / kWarps;            // block rows a warp assembles
  // With at least 192 threads every thread owns at most one coefficient row
  // and keeps it in registers until level 32; with fewer, the coefficients
  // all go to shared memory first (two rows per thread would spill).
  constexpr bool kRegRows = NT >= 192;
  constexpr int kOwn = kRegRows ? 1 : (384 + NT - 1) / NT;  // rows owned, or 16-byte chunks loaded
  const size_t B = static_cast<size_t>(im.bx) * im.by;
  const uint32_t tx = tile % im.tiles_x, ty = tile / im.tiles_x;
  const uint8_t *sym = scratch + im.sym_off;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

  // 1. The tile's 1024 coefficients of plane p are the tile-th 1024-byte run of
  //    the plane (inverse_wavelet.cl:79-104); planes Y1 Y2 Co1 Cg1 Co2 Cg2 are
  //    consecutive B-byte runs of the decoded Y and chroma sections.  A thread
  //    owns whole coefficient rows (line l: plane 2 (w mod 3) + lane / 16, row
  //    16 (w / 3) + lane mod 16, w = l / 32, so "row < 16" is warp-uniform) and
  //    keeps their 32 bytes in registers: only rows < 16, columns < 16 -- the
  //    part levels 2..16 work on -- go to shared memory before level 32.
  const uint8_t *tile_base = sym + static_cast<size_t>(tile) * 1024;
  uint4 raw_lo[kOwn], raw_hi[kOwn];
#pragma unroll
  for (int k = 0; k < kOwn; ++k) {
    const int l = t + k * NT;
    raw_lo[k] = raw_hi[k] = make_uint4(0, 0, 0, 0);
    if (kRegRows && l < 192) {
      const int w = l >> 5, ln = l & 31;
      const int p = 2 * (w % 3) + (ln >> 4), r = 16 * (w / 3) + (ln & 15);
      const uint4 *row = reinterpret_cast<const uint4 *>(tile_base + p * B + r * 32);
      raw_lo[k] = ld_sym<COH>(row);
      raw_hi[k] = ld_sym<COH>(row + 1);
    } else if (!kRegRows && l < 384) {  // chunk l: plane l / 64, row (l % 64) / 2, half l % 2
      raw_lo[k] = ld_sym<COH>(reinterpret_cast<const uint4 *>(tile_base + (l >> 6) * B) + (l & 63));
    }
  }

  // 3. (fewer than 192 threads) All coefficients to int32 shared memory
  //    (pitch kPlanePitch), byte - 128.
  if constexpr (!kRegRows) {
#pragma unroll
    for (int k = 0; k < kOwn; ++k) {
      const int l = t + k * NT;
      if (l < 384) {
        int32_t v[16];
        unpack16(raw_lo[k], v);
        const int q = l & 63;
        int32_t *dst = pl + (l >> 6) * kPlaneWords + (q >> 1) * kPlanePitch + (q & 1) * 16;
        store_row<16>(dst, v);
      }
    }
  }

  // 5. Five levels of the inverse 5/3 wavelet.
  if constexpr (!kRegRows) {
    __syncthreads();
    inv53_level<2, NT>(pl);
    inv53_level<4, NT>(pl);
    inv53_level<8, NT>(pl);
    inv53_level<16, NT>(pl);
    inv53_level<32, NT>(pl);
  } else {
    // Levels 2..16 touch only the top-left 16x16 of each plane, rows 0..15,
    // whose owners are warps 0-2: they run those levels among themselves
    // (named barrier 1) and then level 32's row pass of their rows.  Rows
    // 16..31 (warps 3-5) are untouched coefficients until level 32, so their
    // owners run level 32's row pass at once, straight from registers, while
    // the small levels run.  Then level 32's column pass over the CTA.
    int32_t sv[32], dv[32];
    if (t < 96) {
      const int p = 2 * warp + (lane >> 4), r = lane & 15;
      int32_t *row = pl + p * kPlaneWords + r * kPlanePitch;
      unpack16(raw_lo[0], sv);
      store_row<16>(row, sv);
      bar_sync(1, 96);
      inv53_level_group<2, 96, 1>(pl);
      inv53_level_group<4, 96, 1>(pl);
      inv53_level_group<8, 96, 1>(pl);
      inv53_level_group<16, 96, 1>(pl);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int2 v = reinterpret_cast<const int2 *>(row)[j];
        sv[2 * j] = v.x;
        sv[2 * j + 1] = v.y;
      }
      unpack16(raw_hi[0], sv + 16);
      inv53_lift<32>(sv, dv);
      store_row<32>(row, dv);
    } else if (t < 192) {
      const int w = warp - 3, p = 2 * w + (lane >> 4), r = 16 + (lane & 15);
      int32_t *row = pl + p * kPlaneWords + r * kPlanePitch;
      unpack16(raw_lo[0], sv);
      unpack16(raw_hi[0], sv + 16);
      inv53_lift<32>(sv, dv);
      store_row<32>(row, dv);
    }
    __syncthreads();
#pragma unroll
    for (int c = threadIdx.x; c < 6 * 32; c += NT) inv53_line<32>(pl + (c >> 5) * kPlaneWords + (c & 31), kPlanePitch);
    __syncthreads();
  }

  // 2. Palette indices of the rows this thread assembles (rows warp + kWarps i,
  //    column lane): group prefix + prefix through the block's 32-block chunk
  //    - the sum of the deltas after the block in its chunk.  Loaded after the
  //    wavelet, so that nothing of them is live through it.
  const int32_t *chunk_pref = reinterpret_cast<const int32_t *>(scratch + im.chunk_off);
  const int32_t *gpref = reinterpret_cast<const int32_t *>(scratch + im.gsum_off) + im.sec_groups[3];
  const int16_t *partial = reinterpret_cast<const int16_t *>(sym + im.sec_out[3]);
  uint32_t d[kRows], base[kRows];
#pragma unroll
  for (int i = 0; i < kRows; ++i) {
    const uint32_t p0 = (ty * 32 + warp + kWarps * i) * im.bx + tx * 32;  // first block of the row segment
    d[i] = static_cast<uint32_t>(static_cast<int32_t>(ld_sym<COH>(partial + p0 + lane)));
    base[i] = static_cast<uint32_t>(ld_sym<COH>(gpref + (p0 >> 13))) +
              static_cast<uint32_t>(ld_sym<COH>(chunk_pref + (p0 >> 5)));
  }

  // 4. The palette gathers.
  const uint32_t *pal = reinterpret_cast<const uint32_t *>(sym + im.sec_out[2]);
  uint32_t word[kRows];
  bool bad = false;
#pragma unroll
  for (int i = 0; i < kRows; ++i) {
    const uint32_t idx = base[i] - d[i];
    word[i] = 0;
    if (idx < im.palette_words) word[i] = ld_sym<COH>(pal + idx);
    else bad = true;
  }

  // 6. YCoCg667 -> RGB565 endpoints and whole 8-byte DXT1 blocks (or the
  //    blocks' pixels).
#pragma unroll
  for (int i = 0; i < kRows; ++i) {
    const int r = warp + kWarps * i;
    const uint32_t p = (ty * 32 + r) * im.bx + tx * 32 + lane;
    // Each value as the reference's signed char: the low byte of the int32
    // coefficient, loaded sign-extended.
    const int8_t *row = reinterpret_cast<const int8_t *>(pl + r * kPlanePitch + lane);
    constexpr int kPB = 4 * kPlaneWords;  // plane stride in bytes
    const int y1 = row[0], y2 = row[kPB];
    const int co1 = row[2 * kPB], cg1 = row[3 * kPB];
    const int co2 = row[4 * kPB], cg2 = row[5 * kPB];
    if constexpr (RGB) {
      const size_t pitch = static_cast<size_t>(im.bx) * 12;  // W * 3 bytes
      uint8_t *o = out + im.out_off + pitch * 4 * (ty * 32 + r) + 12 * static_cast<size_t>(tx * 32 + lane);
      store_rgb_block(o, pitch, y1, co1, cg1, y2, co2, cg2, word[i]);
    } else {
      // The low 16 bits of each endpoint, packed by one byte permute.
      const uint32_t ep = __byte_perm(ycocg_to_565(y1, co1, cg1), ycocg_to_565(y2, co2, cg2), 0x5410);
      *reinterpret_cast<uint2 *>(out + im.out_off + static_cast<size_t>(p) * 8) = make_uint2(ep, word[i]);
    }
  }
  if (__any_sync(0xFFFFFFFFu, bad) && lane == 0) flag_error(err, image_err, kErrPalette);
}

template <bool RGB>
__global__ void __launch_bounds__(256, 8) gst_tile_kernel(const uint8_t *__restrict__ scratch, uint8_t *__restrict__ out,
                                                       GstPlanView plan) {
  __shared__ __align__(16) int32_t pl[6 * kPlaneWords];  // 8-byte row accesses
  const GstTileItem it = plan.tiles[blockIdx.x];
  pdl_wait_prerequisites();  // the rANS kernel's symbols (launched right behind it: see launch_decode)
  tile_work<256, false, RGB>(scratch, out, plan.err, plan.image_err ? plan.image_err + it.image : nullptr,
                             plan.images[it.image], it.tile, pl);
}

// ---------------------------------------------------------------------------
// Persistent form: one launch of CTAs that drain the whole plan as a work
// queue -- first every rANS item, then every tile -- so that tiles of images
// whose groups are done run beside the remaining rANS work instead of after
// the last of it.  A tile item waits (bounded) until its image's groups are
// all decoded.  Every item a tile can wait for was taken from the queue
// before the tile and is held by a running CTA that never waits, so the
// waits end whether or not all CTAs are resident.  The last CTA to finish
// re-arms the queue and the counters, so a resident plan can be relaunched.
// (CTAs of 256 threads taking rANS items in pairs measured slower: at 48
// registers they spill, at 64 only four fit per SM.)
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // default: a tile waits at most 2 s for its image
constexpr uint32_t kWaitLimitSpins = 1u << 24;   // and at most this many polls
constexpr int kPersistentThreads = 128;

__host__ __device__ constexpr size_t persistent_smem_bytes(uint32_t stage_words) {
  return rans_smem_bytes(stage_words) > kTileSmemBytes ? rans_smem_bytes(stage_words) : kTileSmemBytes;
}

__global__ void __launch_bounds__(kPersistentThreads, 8) gst_persistent_kernel(const uint8_t *__restrict__ cmp,
                                                                               uint8_t *__restrict__ scratch,
                                                                               uint8_t *__restrict__ out,
                                                                               GstPlanView plan) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  __shared__ uint32_t item_s, ok_s;
  uint32_t *queue = plan.sync, *exits = plan.sync + 1, *ready = plan.sync + 4;
  const uint32_t n_items = plan.n_rans + plan.n_tiles;
  for (;;) {
    __syncthreads();  // the previous item is done with shared memory and item_s
    if (threadIdx.x == 0) item_s = atomicAdd(queue, 1u);
    __syncthreads();
    const uint32_t item = item_s;
    if (item >= n_items) break;
    if (item < plan.n_rans) {
      const GstRansItem it = plan.rans[item];
      rans_item<0>(cmp, scratch, plan.err, plan.image_err ? plan.image_err + it.image : nullptr,
                   plan.counters + it.image, plan.images[it.image], it.section, it.first_group, it.ngroups,
                   it.streams, plan.stage_words, smem_raw, threadIdx.x);
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ready + it.image, static_cast<uint32_t>(it.ngroups));
      }
    } else {
      const GstTileItem it = plan.tiles[item - plan.n_rans];
      const GstImageDesc &im = plan.images[it.image];
      uint32_t *image_err = plan.image_err ? plan.image_err + it.image : nullptr;
      if (threadIdx.x == 0) {
        const uint32_t need = im.sec_groups[0] + im.sec_groups[1] + im.sec_groups[2] + im.sec_groups[3];
        uint32_t ok = 1;
        if (ld_acquire(ready + it.image) < need) {
          const uint64_t t0 = global_ns();
          const uint64_t limit = plan.wait_limit_ns ? plan.wait_limit_ns : kWaitLimitNs;
          for (uint32_t spin = 0;; ++spin) {
            __nanosleep(256);
            if (ld_acquire(ready + it.image) >= need) break;
            if (spin > kWaitLimitSpins || global_ns() - t0 > limit) {
              ok = 0;
              flag_error(plan.err, image_err, kErrTimeout);
              break;
            }
          }
        }
        ok_s = ok;
      }
      __syncthreads();
      if (ok_s)
        tile_work<kPersistentThreads, true>(scratch, out, plan.err, image_err, im, it.tile,
                                            reinterpret_cast<int32_t *>(smem_raw));
    }
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(exits, 1u) == gridDim.x - 1) {
      for (uint32_t i = 0; i < plan.n_images; ++i) ready[i] = 0;
      *queue = 0;
      *exits = 0;
      __threadfence();
    }
  }
}

// Enqueues the decode of one plan.  With `ev` non-null, records ev[0] before
// the first kernel and ev[i + 1] after kernel i (instrumentation).  `tuning`
// selects the form (two kernels, or the persistent kernel where the plan has
// its sync words), the rANS kernel's register budget and the staging depth.
uint32_t rans_wave_capacity(const GstTuning &t) {
  if (t.persistent || t.stage_words < kMinStageWords || t.stage_words > kMaxStageWords) return 0;
  const int minb = t.blocks_per_sm >= 14 ? 16 : t.blocks_per_sm >= 10 ? 12 : 8;  // as launch_decode picks
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  const uint64_t key = (uint64_t(dev) << 40) | (uint64_t(minb) << 32) | t.stage_words;
  static std::mutex mu;
  static std::map<uint64_t, uint32_t> cache;
  {
    std::lock_guard<std::mutex> lock(mu);
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  int sms = 0, per_sm = 0;
  const size_t smem = rans_smem_bytes(t.stage_words);
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) {
    if (minb == 16) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gst_rans_kernel<16>, 128, smem);
    else if (minb == 12) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gst_rans_kernel<12>, 128, smem);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gst_rans_kernel<8>, 128, smem);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();  // a failed query leaves the layout unbalanced, nothing else
    return 0;
  }
  const uint32_t cap = uint32_t(std::max(0, sms * per_sm));
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = cap;
  return cap;
}

cudaError_t launch_decode(const uint8_t *d_cmp, uint8_t *d_scratch, uint8_t *d_out, GstPlanView plan,
                          cudaStream_t stream, int *launches, cudaEvent_t *ev, const GstTuning &tuning,
                          const char **names) {
  *launches = 0;
  static std::atomic<bool> configured{false};  // per process; the attribute applies to every device context
  if (!configured.load(std::memory_order_acquire)) {
    const int bytes = static_cast<int>(rans_smem_bytes(kMaxStageWords));
    cudaError_t e = cudaFuncSetAttribute(gst_rans_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(gst_rans_kernel<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(gst_rans_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(gst_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(persistent_smem_bytes(kMaxStageWords)));
    if (e != cudaSuccess) return e;
    configured.store(true, std::memory_order_release);  // setting the attributes twice is harmless
  }
  if (tuning.stage_words < kMinStageWords || tuning.stage_words > kMaxStageWords || (tuning.stage_words & 7))
    return cudaErrorInvalidValue;
  plan.stage_words = tuning.stage_words;
  if (ev) cudaEventRecord(ev[0], stream);
  if (tuning.persistent && plan.sync && !plan.rgb && plan.n_rans + plan.n_tiles > 0) {
    NvtxRange range("gst persistent decode");
    const size_t smem = persistent_smem_bytes(plan.stage_words);
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gst_persistent_kernel, kPersistentThreads, smem);
    if (e != cudaSuccess) return e;
    const uint32_t grid = std::min<uint32_t>(plan.n_rans + plan.n_tiles, uint32_t(std::max(1, sms * per_sm)));
    gst_persistent_kernel<<<grid, kPersistentThreads, smem, stream>>>(d_cmp, d_scratch, d_out, plan);
    if (names) names[*launches] = "gst_persistent_kernel";
    ++*launches;
    if (ev) cudaEventRecord(ev[*launches], stream);
    return cudaGetLastError();
  }
  if (plan.n_rans) {
    NvtxRange range("gst rANS");
    const size_t smem = rans_smem_bytes(plan.stage_words);
    if (tuning.blocks_per_sm >= 14) gst_rans_kernel<16><<<plan.n_rans, 128, smem, stream>>>(d_cmp, d_scratch, plan);
    else if (tuning.blocks_per_sm >= 10) gst_rans_kernel<12><<<plan.n_rans, 128, smem, stream>>>(d_cmp, d_scratch, plan);
    else gst_rans_kernel<8><<<plan.n_rans, 128, smem, stream>>>(d_cmp, d_scratch, plan);
    if (names) names[*launches] = "gst_rans_kernel";
    ++*launches;
    if (ev) cudaEventRecord(ev[*launches], stream);
  }
  if (plan.n_tiles) {
    NvtxRange range(plan.rgb ? "gst tile (RGB)" : "gst tile");
    // Right behind the rANS kernel (no event between them) the tile kernel is
    // a programmatic dependent launch: its launch and CTA setup overlap the
    // rANS tail, and griddepcontrol.wait orders its reads after the symbols.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(plan.n_tiles);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    const bool pdl = plan.n_rans && !ev;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    const uint8_t *scratch = d_scratch;
    const cudaError_t e = plan.rgb ? cudaLaunchKernelEx(&cfg, gst_tile_kernel<true>, scratch, d_out, plan)
                                   : cudaLaunchKernelEx(&cfg, gst_tile_kernel<false>, scratch, d_out, plan);
    if (e != cudaSuccess) return e;
    if (names) names[*launches] = plan.rgb ? "gst_tile_rgb_kernel" : "gst_tile_kernel";
    ++*launches;
    if (ev) cudaEventRecord(ev[*launches], stream);
  }
  return cudaGetLastError();
}


}  // namespace gst

namespace gst {

// ===========================================================================
// One-image decode that allocates nothing: gst_load_compressed_dxt_static.
//
// Who needs it: callers that must not allocate device memory at decode time.
// cudaMalloc and cudaFree can synchronise the whole device, which a render or
// texture-streaming thread with a per-frame time budget cannot afford; and
// some engines hand out all device memory from their own fixed pools and
// forbid anyone else to allocate.  Such callers cannot create a gst_ctx
// (it allocates its scratch, plan buffers and events), so this entry point
// needs no context: its scratch is g_static_scratch below, a file-scope device
// array that is part of this library's image and is held by every GPU that
// loads the library until the process exits.
//
// Limits and rules (also stated in include/gst_decoder.h):
//  * kStaticScratchBytes (4 MiB) bounds the image: 256 + 8*B + palette_bytes
//    + B/8 + 8*B/8192 bytes must fit (B = w*h/16); that is at most 2048x2048
//    with a typical palette.  Larger images are rejected with GST_E_ARG before
//    anything is enqueued.
//  * Malformed payloads are reported only through device_status: with it null
//    the kernels' error bits stay in the array and the call returns GST_OK.
//  * Every call uses the same array and leaves its contents behind.  Each call
//    clears, on its stream, the words that must start at zero (the device
//    status word and the index-group counter); the rest is fully rewritten
//    before it is read.  Calls whose work overlaps on the GPU (different
//    streams without ordering between them, or several host threads) race on
//    the array: serialise them, e.g. by using one stream.
//  * The first call on each device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current) and sets the rANS
//    kernel's shared-memory attribute; make that first call before any stream
//    capture on that device.
//  * It calls no cudaMalloc, cudaFree or other allocating routine.
// No counterpart in the reference, whose decoder allocates its scratch per call
// or from PreallocateDecompressor (codec/decoder.cpp:98-130, 478-485).
constexpr size_t kStaticScratchBytes = size_t(4) << 20;
constexpr size_t kStaticHeaderBytes = 256;  // [status word][index-group counter], then image scratch
static __device__ __align__(256) uint8_t g_static_scratch[kStaticScratchBytes];

// gst_rans_kernel for a single image whose descriptor arrives by value; the
// work item is derived from blockIdx (ceil(G/4) CTAs per section, in section
// order).  `base` is g_static_scratch: [status][counter] then the image scratch.
__global__ void __launch_bounds__(128) gst_rans_static_kernel(const uint8_t *__restrict__ cmp, uint8_t *base,
                                                              GstImageDesc im) {
  uint32_t b = blockIdx.x, section = 0;
  for (; section < 3; ++section) {
    const uint32_t c = (im.sec_groups[section] + kGroupsPerRansCta - 1) / kGroupsPerRansCta;
    if (b < c) break;
    b -= c;
  }
  const uint32_t first = b * kGroupsPerRansCta;
  const uint32_t ngroups = min(kGroupsPerRansCta, im.sec_groups[section] - first);
  extern __shared__ __align__(16) uint8_t smem_raw[];
  uint32_t *err = reinterpret_cast<uint32_t *>(base);
  rans_item<0>(cmp, base + kStaticHeaderBytes, err, nullptr, err + 1, im, section, first, ngroups,
               kStreamsPerGroup, kDefaultStageWords, smem_raw, threadIdx.x);
}

// gst_tile_kernel for a single image whose descriptor arrives by value; the
// tile is blockIdx.x.
__global__ void __launch_bounds__(256) gst_tile_static_kernel(const uint8_t *base, uint8_t *__restrict__ out,
                                                              GstImageDesc im) {
  __shared__ __align__(16) int32_t pl[6 * kPlaneWords];  // 8-byte row accesses
  uint32_t *err = reinterpret_cast<uint32_t *>(const_cast<uint8_t *>(base));
  tile_work<256, false>(base + kStaticHeaderBytes, out, err, nullptr, im, blockIdx.x, pl);
}

}  // namespace gst

// Host side of the static-scratch decode.
#include <mutex>

#include "gst_decoder.h"
#include "gst_host.h"

namespace {

constexpr int kMaxStaticDevices = 64;
std::mutex g_static_mu;
void *g_static_ptr[kMaxStaticDevices] = {};  // device address of g_static_scratch, per device

// Once per device, with it current: the array's device address and the rANS
// kernel's shared-memory attribute.  The array's name is only a host-side
// stand-in; kernels must be given this address.
gst_status static_setup(int device, uint8_t **base) {
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (device < 0 || device >= kMaxStaticDevices) return GST_E_ARG;
  if (!g_static_ptr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, gst::g_static_scratch);
    if (e != cudaSuccess || !p) return GST_E_CUDA;
    e = cudaFuncSetAttribute(gst::gst_rans_static_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(gst::rans_smem_bytes(gst::kDefaultStageWords)));
    if (e != cudaSuccess) return GST_E_CUDA;
    g_static_ptr[device] = p;
  }
  *base = static_cast<uint8_t *>(g_static_ptr[device]);
  return GST_OK;
}

}  // namespace

extern "C" gst_status gst_load_compressed_dxt_static(const gst_header *hdr, const void *d_cmp, void *d_out,
                                                     void *stream, uint32_t *device_status) {
  using namespace gst;
  if (!hdr || !d_cmp || !d_out) return GST_E_ARG;
  if ((reinterpret_cast<uintptr_t>(d_cmp) & 15) || (reinterpret_cast<uintptr_t>(d_out) & 7)) return GST_E_ARG;
  const gst_header &h = *hdr;
  // The header rules every decode call applies (gst_parse_header's).
  if (host::check_header(h) != GST_OK) return GST_E_FORMAT;
  const uint64_t B = uint64_t(h.width) * h.height / 16;
  const uint32_t lens[4] = {h.y_cmp_sz, h.chroma_cmp_sz, h.palette_sz, h.indices_sz};
  const uint64_t syms[4] = {2 * B, 4 * B, h.palette_bytes, B};
  // Scratch inside the static array: symbols, chunk prefixes, group sums.
  auto up = [](uint64_t x) { return (x + 255) / 256 * 256; };
  const uint64_t sym_bytes = up(8 * B + h.palette_bytes), chunk_bytes = up(B / 32 * 4);
  const uint64_t gsum_bytes = up(2 * (B / kSymsPerGroup) * 4);
  if (kStaticHeaderBytes + sym_bytes + chunk_bytes + gsum_bytes > kStaticScratchBytes) return GST_E_ARG;

  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return GST_E_CUDA;
  uint8_t *base = nullptr;
  gst_status st = static_setup(device, &base);
  if (st != GST_OK) return st;

  GstImageDesc im = {};
  im.freq_off = 512;  // the reference's layout for one image: offsets page, tables, sections
  im.body_off = 512 + 4 * kFreqTableBytes;
  im.sym_off = 0;
  im.chunk_off = sym_bytes;
  im.gsum_off = sym_bytes + chunk_bytes;
  im.out_off = 0;
  uint32_t in = 0, o = 0, rans_ctas = 0;
  for (int s = 0; s < 4; ++s) {
    im.sec_in[s] = in;
    im.sec_len[s] = lens[s];
    im.sec_groups[s] = uint32_t(syms[s] / kSymsPerGroup);
    im.sec_out[s] = o;
    in += lens[s];
    o += uint32_t(syms[s]);
    rans_ctas += (im.sec_groups[s] + kGroupsPerRansCta - 1) / kGroupsPerRansCta;
  }
  im.bx = h.width / 4;
  im.by = h.height / 4;
  im.palette_words = h.palette_bytes / 4;
  im.tiles_x = im.bx / kWaveletDim;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Words that must start at zero: the status word and the index-group counter.
  // Each call below reports its own error (a launch through cudaLaunchKernelEx
  // returns the launch's status), so an error left pending by unrelated earlier
  // work is neither cleared nor reported as this call's.
  if (cudaMemsetAsync(base, 0, 8, s) != cudaSuccess) return GST_E_CUDA;
  cudaLaunchConfig_t cfg = {};
  cfg.stream = s;
  cfg.gridDim = dim3(rans_ctas);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = rans_smem_bytes(kDefaultStageWords);
  const uint8_t *cmp = static_cast<const uint8_t *>(d_cmp);
  if (cudaLaunchKernelEx(&cfg, gst_rans_static_kernel, cmp, base, im) != cudaSuccess) return GST_E_CUDA;
  cfg.gridDim = dim3(uint32_t(B / 1024));
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  const uint8_t *cbase = base;
  if (cudaLaunchKernelEx(&cfg, gst_tile_static_kernel, cbase, static_cast<uint8_t *>(d_out), im) != cudaSuccess)
    return GST_E_CUDA;
  if (device_status) {
    if (cudaStreamSynchronize(s) != cudaSuccess) return GST_E_CUDA;
    uint32_t bits = 0;
    if (cudaMemcpy(&bits, base, sizeof(bits), cudaMemcpyDeviceToHost) != cudaSuccess) return GST_E_CUDA;
    *device_status = bits;
  }
  return GST_OK;
}
