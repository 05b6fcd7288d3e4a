// gst_encode.cu -- sm_103a kernels of the GST encoder stages: the reference's
// ByteEncoder::EncodeBytes (codec/entropy.cpp:174-265) over any number of
// sections in four launches.
//
//  gst_enc_histogram_kernel  byte counts per section (entropy.cpp:176-179):
//     one CTA per 32 KB chunk, warp-private shared histograms, one shared
//     atomic per byte, one global atomic per bin per CTA.  (Merging the lanes
//     that hold the same byte with a match-any first, which avoids
//     serialising on the most frequent bin, measured 3.5-4x slower on these
//     sections; it remains as option encode_hist_match.)
//
//  gst_enc_normalize_kernel  ans::GenerateHistogram (ans/histogram.cpp:40-121)
//     at M = 2048, one CTA per section, thread i = symbol i.  The first guess
//     is the reference's float/double arithmetic.  The correction: the
//     reference pops the cheapest rank from a binary heap |correction| times,
//     re-inserting the symbol's next rank.  Each symbol's ranks strictly
//     increase, so the heap pops ranks in nondecreasing order and the result
//     is fixed by ranks alone except where equal ranks straddle the last pop.
//     The kernel pops in rounds: every element below a threshold T is popped
//     at once when their number fits in the correction left, T galloping
//     along the sequence of the symbol holding the minimum.  Only a tie group
//     larger than the correction left needs the heap's own tie order; then
//     thread 0 replays the heap exactly (libstdc++'s make_heap / pop_heap /
//     push_heap sift procedure).  Ranks are log2(n / (n +- 1)) * count with
//     log2 from a host-built table (the C library's log2, as the reference
//     calls it) and IEEE double products; they are compared as ordered
//     64-bit keys.
//
//  gst_enc_rans_kernel  ans::EncodeInterleaved (ans/encode.cpp:224-259) with
//     rANS_Encoder::Encode (:56-69) at M = 2^11, k = 2^4, b = 2^16: one warp
//     per 8192-symbol group, lane = stream.  Division by the frequency is a
//     multiply-high by a per-symbol reciprocal (exact for states < 2^31, the
//     encoder's range).  A renormalising lane's word goes to shared memory at
//     the position a warp ballot gives it, in the reference's emission order
//     (step by step, streams in order).  Groups are taken by a ticket counter
//     in output order; each warp publishes its group's byte count and finds
//     the bytes before it with a decoupled look-back over its predecessors'
//     published counts, then writes its words and final states straight to
//     their place in the output.  Waits are bounded.
//
//  gst_enc_finish_kernel  the frequency tables, group end offsets and GST
//     stream headers (codec/encoder.cpp:122-144), whose places depend on the
//     compressed sizes.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "gst_encode_plan.h"
#include "gst_plan.h"

namespace gst {
namespace {

constexpr int kHistThreads = 256;
constexpr int kNormThreads = 256;
constexpr int kFinishThreads = 256;
constexpr int kEncWarps = 1;  // one warp per CTA: measured faster than 2 or 4 (more independent CTAs per SM)
constexpr uint64_t kEncWaitLimitNs = 2000000000ull;
constexpr uint32_t kEncWaitSpins = 1u << 24;
constexpr unsigned long long kKeyInf = ~0ull;

__device__ __forceinline__ uint32_t enc_lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
__device__ __forceinline__ uint64_t enc_global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// ---------------------------------------------------------------------------
// Byte counts (codec/entropy.cpp:176-179).
template <bool MATCH>
__device__ __forceinline__ void count_word(uint32_t *h, uint32_t w, int lane) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t b = (w >> (8 * k)) & 0xFF;
    if (MATCH) {
      const uint32_t same = __match_any_sync(0xFFFFFFFFu, b);
      if (lane == __ffs(same) - 1) atomicAdd(&h[b], __popc(same));
    } else {
      atomicAdd(&h[b], 1u);
    }
  }
}

template <bool MATCH>
__global__ void __launch_bounds__(kHistThreads) gst_enc_histogram_kernel(EncPlanView p) {
  __shared__ uint32_t hist[kHistThreads / 32][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < (kHistThreads / 32) * 256; i += kHistThreads) (&hist[0][0])[i] = 0;
  __syncthreads();
  const EncChunk ch = p.chunks[blockIdx.x];
  const uint4 *src = reinterpret_cast<const uint4 *>(p.sections[ch.section].sym + ch.start);
  uint32_t *h = hist[warp];
  const uint32_t n16 = ch.len / 16;  // a multiple of 512: every thread runs the same iterations
  for (uint32_t v = threadIdx.x; v < n16; v += 2 * kHistThreads) {
    const uint4 a = __ldg(src + v);
    const uint4 b = __ldg(src + v + kHistThreads);
    count_word<MATCH>(h, a.x, lane);
    count_word<MATCH>(h, a.y, lane);
    count_word<MATCH>(h, a.z, lane);
    count_word<MATCH>(h, a.w, lane);
    count_word<MATCH>(h, b.x, lane);
    count_word<MATCH>(h, b.y, lane);
    count_word<MATCH>(h, b.z, lane);
    count_word<MATCH>(h, b.w, lane);
  }
  __syncthreads();
  uint32_t sum = 0;
#pragma unroll
  for (int w = 0; w < kHistThreads / 32; ++w) sum += hist[w][threadIdx.x];
  if (sum) atomicAdd(&p.counts[ch.section * 256 + threadIdx.x], sum);
}

// ---------------------------------------------------------------------------
// Frequency normalisation (ans/histogram.cpp:40-121).
constexpr int kWin = 8;

// Minimum of the heads with its tie count, first symbol and the second
// smallest distinct head.
struct HeadMin {
  unsigned long long m1, m2;
  int t, i0;
};

struct NormShared {
  double L[kEncLogTableLen];  // the rank table of the correction's sign
  HeadMin hm[kNormThreads / 32];
  int i0n;  // the minimum symbol's frequency
  double i0c;  // and count
  int red32[kNormThreads / 32];
  int ibcast;
  int corr;       // the correction (histogram.cpp:65)
  int stop;       // the rounds finished without the heap replay
  int replayed;   // the rounds met a tie group larger than the correction left
  uint32_t cnt[256];
  int first[256];  // first guess
  int fin[256];    // result of the heap replay
  unsigned long long heap_key[256];
  int heap_sym[256];
  unsigned long long key0[256];  // each candidate's rank at its first guess
};

// Barrier of the 256 round threads (the replay warp does not take part).
__device__ __forceinline__ void round_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kNormThreads) : "memory"); }

__device__ __forceinline__ int block_sum32(int v, NormShared &s) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) s.red32[threadIdx.x >> 5] = v;
  round_sync();
  v = 0;
#pragma unroll
  for (int w = 0; w < kNormThreads / 32; ++w) v += s.red32[w];
  round_sync();
  return v;
}

__device__ __forceinline__ uint32_t block_sum_u32(uint32_t v, NormShared &s) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) s.red32[threadIdx.x >> 5] = static_cast<int>(v);
  round_sync();
  v = 0;
#pragma unroll
  for (int w = 0; w < kNormThreads / 32; ++w) v += static_cast<uint32_t>(s.red32[w]);
  round_sync();
  return v;
}

__device__ __forceinline__ HeadMin merge_heads(HeadMin a, HeadMin b) {
  HeadMin r;
  if (a.m1 < b.m1) {
    r = a;
    r.m2 = b.m1 < a.m2 ? b.m1 : a.m2;
  } else if (b.m1 < a.m1) {
    r = b;
    r.m2 = a.m1 < b.m2 ? a.m1 : b.m2;
  } else {
    r.m1 = a.m1;
    r.m2 = a.m2 < b.m2 ? a.m2 : b.m2;
    r.t = a.t + b.t;
    r.i0 = a.i0 < b.i0 ? a.i0 : b.i0;
  }
  return r;
}

__device__ __forceinline__ HeadMin block_heads(unsigned long long head, NormShared &s) {
  HeadMin h = {head, kKeyInf, 1, static_cast<int>(threadIdx.x)};
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    HeadMin u;
    u.m1 = __shfl_xor_sync(0xFFFFFFFFu, h.m1, o);
    u.m2 = __shfl_xor_sync(0xFFFFFFFFu, h.m2, o);
    u.t = __shfl_xor_sync(0xFFFFFFFFu, h.t, o);
    u.i0 = __shfl_xor_sync(0xFFFFFFFFu, h.i0, o);
    h = merge_heads(h, u);
  }
  if ((threadIdx.x & 31) == 0) s.hm[threadIdx.x >> 5] = h;
  round_sync();
  h = s.hm[0];
#pragma unroll
  for (int w = 1; w < kNormThreads / 32; ++w) h = merge_heads(h, s.hm[w]);
  round_sync();
  return h;
}

// Inclusive scan of one int per thread (256 threads).
__device__ __forceinline__ int block_scan32(int v, NormShared &s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) s.red32[warp] = v;
  round_sync();
  int before = 0;
  for (int w = 0; w < warp; ++w) before += s.red32[w];
  round_sync();
  return v + before;
}

// Ordered key of the rank of a symbol with `count` at frequency n:
// GetFreqChange (ans/histogram.cpp:25-29) = log2(n / (n + sign)) * count,
// as a u64 that orders like the double; kKeyInf where the symbol cannot move
// (sign -1 and n <= 1, histogram.cpp:86-91 and :109).
__device__ __forceinline__ unsigned long long rank_key(const double *L, int sign, int n, double count) {
  if ((sign < 0 && n <= 1) || n < 0 || n >= static_cast<int>(kEncLogTableLen)) return kKeyInf;
  const double r = __dmul_rn(L[n], count);
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(r));
  return sign < 0 ? b : ~b;  // sign +1: every rank is negative, so the bit order reverses
}

// Number of consecutive ranks of this symbol, from frequency n on, below T
// (at most cap), when the first c0 of them are known to be below T:
// exponential then binary search over its increasing ranks.
__device__ __forceinline__ int count_from(const double *L, int sign, int n, double count, unsigned long long T,
                                          int cap, int c0) {
  if (c0 >= cap) return cap;
  if (rank_key(L, sign, n + sign * c0, count) >= T) return c0;
  int good = c0, bad = cap;
  for (int step = 1; c0 + step < cap; step *= 2) {
    if (rank_key(L, sign, n + sign * (c0 + step), count) < T) {
      good = c0 + step;
    } else {
      bad = c0 + step;
      break;
    }
  }
  while (bad - good > 1) {
    const int mid = (good + bad) >> 1;
    if (rank_key(L, sign, n + sign * mid, count) < T)
      good = mid;
    else
      bad = mid;
  }
  return bad;
}

// The C++ library's binary heap with std::greater (a min-heap): GCC's
// libstdc++ __push_heap / __adjust_heap, the SGI STL sift procedure.
__device__ void heap_sift_up(unsigned long long *key, int *sym, int hole, int top, unsigned long long vk, int vs) {
  int parent = (hole - 1) / 2;
  while (hole > top && key[parent] > vk) {
    key[hole] = key[parent];
    sym[hole] = sym[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  key[hole] = vk;
  sym[hole] = vs;
}

__device__ void heap_adjust(unsigned long long *key, int *sym, int hole, int len, unsigned long long vk, int vs) {
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (key[child] > key[child - 1]) child--;
    key[hole] = key[child];
    sym[hole] = sym[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    key[hole] = key[child - 1];
    sym[hole] = sym[child - 1];
    hole = child - 1;
  }
  heap_sift_up(key, sym, hole, top, vk, vs);
}

// ans/histogram.cpp:78-117 replayed exactly (thread 0).
// Runs in its own warp beside the rounds; returns early once the rounds have
// finished without needing it (s.stop).
__device__ void heap_replay(NormShared &s, const double *L, int sign, int correction, uint32_t *err) {
  const volatile int *stop = &s.stop;
  int len = 0;
  for (int i = 0; i < 256; ++i) {
    s.fin[i] = s.first[i];
    if (s.cnt[i] && (s.first[i] > 1 || correction > 0)) {
      s.heap_key[len] = s.key0[i];  // evaluated by the round threads
      s.heap_sym[len] = i;
      ++len;
    }
  }
  if (len >= 2) {
    for (int parent = (len - 2) / 2;; --parent) {
      if (*stop) return;
      heap_adjust(s.heap_key, s.heap_sym, parent, len, s.heap_key[parent], s.heap_sym[parent]);
      if (parent == 0) break;
    }
  }
  while (correction != 0) {
    if (*stop) return;
    if (len == 0) {
      atomicOr(err, kErrTable);
      return;
    }
    // pop_heap: the minimum goes to the back
    if (len > 1) {
      const unsigned long long vk = s.heap_key[len - 1];
      const int vs = s.heap_sym[len - 1];
      s.heap_key[len - 1] = s.heap_key[0];
      s.heap_sym[len - 1] = s.heap_sym[0];
      heap_adjust(s.heap_key, s.heap_sym, 0, len - 1, vk, vs);
    }
    const int i = s.heap_sym[--len];
    s.fin[i] += sign;
    correction -= sign;
    if (s.fin[i] > 1 || sign == 1) {
      s.heap_key[len] = rank_key(L, sign, s.fin[i], static_cast<double>(static_cast<int>(s.cnt[i])));
      s.heap_sym[len] = i;
      ++len;
      heap_sift_up(s.heap_key, s.heap_sym, len - 1, 0, s.heap_key[len - 1], s.heap_sym[len - 1]);
    }
  }
}

// 256 round threads (thread i = symbol i) and one replay warp.
__global__ void __launch_bounds__(kNormThreads + 32) gst_enc_normalize_kernel(EncPlanView p) {
  __shared__ NormShared s;
  const int i = threadIdx.x;
  const uint32_t k = blockIdx.x;
  const bool rounds = i < kNormThreads;
  uint32_t c = 0;
  int n = 0;
  if (rounds) {
    c = p.counts[k * 256 + i];
    s.cnt[i] = c;
    // fold_sum (histogram.cpp:31-33): uint32 sum, then int
    const int sum = static_cast<int>(block_sum_u32(c, s));
    // first guess (histogram.cpp:52-63): uint32 product, float quotient, double test
    if (c) {
      const uint32_t scaled = c * kTableSize;
      const double fs = static_cast<double>(__fdiv_rn(__uint2float_rn(scaled), __int2float_rn(sum)));
      const int down = static_cast<int>(fs);
      const int v = (__dmul_rn(fs, fs) <= static_cast<double>(down * (down + 1))) ? down : down + 1;
      n = v > 1 ? v : 1;
    }
    s.first[i] = n;
    const int correction = static_cast<int>(kTableSize) - block_sum32(n, s);
    if (i == 0) {
      s.corr = correction;
      s.stop = 0;
      s.replayed = 0;
    }
    if (correction != 0) {
      const double *Lg = correction > 0 ? p.log2_plus : p.log2_minus;
      for (uint32_t j = i; j < kEncLogTableLen; j += kNormThreads) s.L[j] = __ldg(Lg + j);
      round_sync();
      // every candidate's first rank, for the rounds and the heap replay
      const int sign = correction > 0 ? 1 : -1;
      const bool cand = c != 0 && (n > 1 || correction > 0);
      s.key0[i] = cand ? rank_key(s.L, sign, n, static_cast<double>(static_cast<int>(c))) : kKeyInf;
    }
  }
  __syncthreads();
  const int correction = s.corr;
  if (correction != 0) {
    const int sign = correction > 0 ? 1 : -1;
    const double *L = s.L;
    if (!rounds) {
      // The heap replay starts at once beside the rounds: its result is used
      // only if they meet a tie group larger than the correction left.
      if (i == kNormThreads) heap_replay(s, L, sign, correction, p.err);
    } else {
      const bool cand = c != 0 && (n > 1 || correction > 0);
      const double cd = static_cast<double>(static_cast<int>(c));
      int left = correction > 0 ? correction : -correction;
      bool replay = false;
      // This symbol's next kWin ranks, evaluated together (independent
      // products) the first time a round needs them; counts below a threshold
      // within them are integer compares.  FP64 products are few on this
      // part, so only symbols whose head lies below a threshold evaluate any.
      // Beyond the window the count is searched between what earlier
      // thresholds showed: count(tlo) = clo, count(thi) = chi.
      unsigned long long win[kWin];
      bool have_win = false;
      unsigned long long head = s.key0[i];
      unsigned long long tlo = kKeyInf, thi = 0;
      int clo = 0, chi = 0;
      auto below = [&](unsigned long long T, int cap) -> int {
        if (head >= T) return 0;
        if (!have_win) {
#pragma unroll
          for (int q = 0; q < kWin; ++q) win[q] = rank_key(L, sign, n + sign * q, cd);
          have_win = true;
        }
        int b = 0;
#pragma unroll
        for (int q = 0; q < kWin; ++q) b += win[q] < T ? 1 : 0;
        if (b < kWin || cap <= kWin) return b < cap ? b : cap;
        const int lo = (T >= tlo && clo > kWin) ? clo : kWin;
        const int hi = (T <= thi && chi < cap) ? chi : cap;
        return lo >= hi ? hi : count_from(L, sign, n, cd, T, hi, lo);
      };
      auto advance = [&](int by) {  // a symbol whose frequency moved re-evaluates its ranks
        if (by) {
          n += sign * by;
          head = cand ? rank_key(L, sign, n, cd) : kKeyInf;
          have_win = false;
          tlo = kKeyInf;
          thi = 0;
        }
      };
      auto probe = [&](unsigned long long T) -> bool {  // do the ranks below T fit in `left`?
        const int b = below(T, left + 1);
        const bool fits = block_sum32(b, s) <= left;
        if (fits) {
          tlo = T;
          clo = b;
        } else {
          thi = T;
          chi = b;
        }
        return fits;
      };
      while (left > 0) {
        const HeadMin hm = block_heads(head, s);
        const unsigned long long m1 = hm.m1;
        if (m1 == kKeyInf) {  // nothing can move (the reference asserts)
          if (i == 0) atomicOr(p.err, kErrTable);
          break;
        }
        const bool tied = head == m1;
        const int t = hm.t, i0 = hm.i0;
        if (i == i0) {
          s.i0n = n;
          s.i0c = cd;
          // A unique minimum: every rank of i0 below the second smallest
          // head comes before any other rank; a run of two or more is popped
          // at once (at most `left`).  Shorter runs (sequences taking turns)
          // go to the galloping below, which pops the interleaved stretch.
          s.ibcast = t == 1 ? below(hm.m2, left) : 0;
        }
        round_sync();
        const int cnt = s.ibcast, n0 = s.i0n;
        const double c0 = s.i0c;
        round_sync();
        if (t == 1 && (cnt >= 2 || cnt == left)) {
          if (i == i0) advance(cnt);
          left -= cnt;
          continue;
        }
        // Largest j such that the ranks below T(j), the j-th next rank of
        // symbol i0, number at most `left` (all of them are then popped).
        int best = 0, bad = 0;
        for (int j = 1;; j *= 2) {
          if (j > left) {
            bad = j;
            break;
          }
          const unsigned long long T = rank_key(L, sign, n0 + sign * j, c0);
          if (!probe(T)) {
            bad = j;
            break;
          }
          best = j;
          if (T == kKeyInf) break;
        }
        if (bad) {
          while (bad - best > 1) {
            const int mid = (best + bad) >> 1;
            if (probe(rank_key(L, sign, n0 + sign * mid, c0)))
              best = mid;
            else
              bad = mid;
          }
        }
        if (best == 0) {
          // Ranks below the second rank of i0 exceed what is left: pop the
          // tie group at the minimum if it fits, else its order decides.
          if (t > left) {
            replay = true;
            break;
          }
          advance(tied ? 1 : 0);
          left -= t;
          continue;
        }
        const int adv = below(rank_key(L, sign, n0 + sign * best, c0), left + 1);
        left -= block_sum32(adv, s);
        advance(adv);
      }
      if (i == 0) {
        if (replay)
          s.replayed = 1;
        else
          *reinterpret_cast<volatile int *>(&s.stop) = 1;
      }
    }
  }
  __syncthreads();
  if (!rounds) return;
  if (correction != 0 && s.replayed) n = s.fin[i];
  // Encode entry: the reciprocal m = ceil(2^(31 + l) / F), l = ceil(log2 F),
  // gives floor(x / F) = umulhi(2x, m) >> l for every x < 2^31.
  const uint32_t F = static_cast<uint32_t>(n);
  const int C = block_scan32(n, s) - n;
  uint4 e = make_uint4(0, 0, 0, 0);
  if (F) {
    const uint32_t l = F > 1 ? 32 - __clz(F - 1) : 0;
    const uint32_t m = static_cast<uint32_t>(((1ull << (31 + l)) + F - 1) / F);
    e = make_uint4(m, F << 20, kTableSize - F, (static_cast<uint32_t>(C) << 5) | l);
  }
  p.tables[k * 256 + i] = e;
  p.freqs[k * 256 + i] = static_cast<uint16_t>(F);
}

// ---------------------------------------------------------------------------
// Interleaved rANS encode of one group per warp, placed by decoupled look-back.
__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}

// Publishes group g's byte count and returns the bytes of all groups before it.
__device__ unsigned long long enc_lookback(const EncPlanView &p, uint32_t g, uint32_t bytes, int lane) {
  const bool publish = g != p.stall_group;
  if (lane == 0 && publish) st_relaxed(p.status + g, (g == 0 ? kEncFlagInclusive : kEncFlagAggregate) | bytes);
  if (g == 0) return 0;
  unsigned long long excl = 0;
  long long end = static_cast<long long>(g) - 1;
  const uint64_t t0 = enc_global_ns();
  const uint64_t limit = p.wait_limit_ns ? p.wait_limit_ns : kEncWaitLimitNs;
  uint32_t spins = 0;
  for (;;) {
    const long long idx = end - lane;
    unsigned long long v = idx >= 0 ? ld_relaxed(p.status + idx) : kEncFlagInclusive;
    while (__any_sync(0xFFFFFFFFu, (v >> 62) == 0)) {
      __nanosleep(64);
      if ((v >> 62) == 0) v = ld_relaxed(p.status + idx);
      const bool give_up =
          __shfl_sync(0xFFFFFFFFu, ++spins > kEncWaitSpins || enc_global_ns() - t0 > limit, 0);
      if (give_up) {
        if (lane == 0) atomicOr(p.err, kErrTimeout);
        if ((v >> 62) == 0) v = kEncFlagInclusive;  // the output is void; end the wait
      }
    }
    const uint32_t incl = __ballot_sync(0xFFFFFFFFu, (v >> 62) == 2);
    const int stop = incl ? __ffs(incl) - 1 : 31;
    excl += warp_sum64(lane <= stop ? (v & kEncValueMask) : 0);
    if (incl) break;
    end -= 32;
  }
  if (lane == 0 && publish) st_relaxed(p.status + g, kEncFlagInclusive | (excl + bytes));
  return excl;
}

// One pass of the interleaved encoder over a group (encode.cpp:56-69 per
// lane, lanes in order per step).  STORE: each renormalising lane writes its
// word to w16 at the position the warp ballot gives it (the reference's
// emission order); otherwise only the word count is kept.
__device__ __forceinline__ uint4 ld_nc_v4(const uint4 *p) {
  uint4 v;
  asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

// floor(a / 2^(c mod 32)): the funnel shift takes the shift from the low five
// bits of the packed table word (C << 5 | l).
__device__ __forceinline__ uint32_t shr_wrap(uint32_t a, uint32_t c) {
  uint32_t d;
  asm("shf.r.wrap.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(0u), "r"(c));
  return d;
}

// One pass of the interleaved encoder over a group (encode.cpp:56-69 per
// lane, lanes in order per step).  STORE: each renormalising lane writes its
// word to w16 at the position the warp ballot gives it (the reference's
// emission order) and nw_out is the warp's word count; otherwise nw_out is
// this lane's own word count.
template <bool STORE>
__device__ __forceinline__ void encode_pass(const uint4 *__restrict__ src, const uint4 *tab, uint32_t lt,
                                            uint16_t *__restrict__ w16, uint32_t &x_out, uint32_t &nw_out) {
  uint32_t x = kRansL, nw = 0;
  uint4 q = ld_nc_v4(src);
  for (int j = 0; j < static_cast<int>(kSymsPerStream / 16); ++j) {
    const uint4 nxt = ld_nc_v4(src + (j + 1 < static_cast<int>(kSymsPerStream / 16) ? j + 1 : j));
    const uint32_t w4[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      const uint32_t s = (w4[b >> 2] >> (8 * (b & 3))) & 0xFF;
      const uint4 e = tab[s];
      // renormalise (encode.cpp:59-64): at most one word, x < 2^31
      const bool r = x >= e.y;
      if (STORE) {
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, r);
        if (r) w16[nw + __popc(m & lt)] = static_cast<uint16_t>(x);
        nw += __popc(m);
      } else {
        nw += r ? 1u : 0u;
      }
      if (r) x >>= 16;
      // x' = (x / F) * M + C + x % F = x + q * (M - F) + C (encode.cpp:67)
      const uint32_t qd = shr_wrap(__umulhi(x + x, e.x), e.w);
      x = x + qd * e.z + (e.w >> 5);
    }
    q = nxt;
  }
  x_out = x;
  nw_out = nw;
}

// Each group is encoded twice: the first pass only counts its 16-bit words,
// so the group's byte count is published (and the look-back resolved) before
// the second pass writes the words straight to their place in the output.
// No per-warp word buffer: shared memory holds only the warp's encode table,
// which keeps many warps resident to hide the per-step latency.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) gst_enc_rans_kernel(EncPlanView p) {
  __shared__ uint4 s_tab[WARPS][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint4 *tab = s_tab[warp];
  const uint32_t lt = enc_lanemask_lt();
  uint32_t cur = 0xFFFFFFFFu;
  for (;;) {
    uint32_t g = 0;
    if (lane == 0) g = atomicAdd(p.ticket, 1u);
    g = __shfl_sync(0xFFFFFFFFu, g, 0);
    if (g >= p.n_groups) break;
    const uint32_t k = p.group_section[g];
    const EncSection &sec = p.sections[k];
    if (k != cur) {
      __syncwarp();
      for (int e = lane; e < 256; e += 32) tab[e] = p.tables[k * 256 + e];
      __syncwarp();
      cur = k;
    }
    const uint4 *src = reinterpret_cast<const uint4 *>(sec.sym + static_cast<size_t>(g - sec.first_group) * kSymsPerGroup +
                                                       lane * kSymsPerStream);
    uint32_t x, nw;
    encode_pass<false>(src, tab, lt, nullptr, x, nw);
#pragma unroll
    for (int o = 16; o; o >>= 1) nw += __shfl_xor_sync(0xFFFFFFFFu, nw, o);
    // Group bytes: [2 zero bytes if the word count is odd][words][32 states]
    // (entropy.cpp:213-229 and encode.cpp:248-256).
    const uint32_t odd = nw & 1;
    const uint32_t bytes = 2 * (nw + odd) + 4 * kStreamsPerGroup;
    const unsigned long long before = enc_lookback(p, g, bytes, lane);
    uint8_t *dst = p.out + sec.grp_fixed + before;
    if (odd && lane == 0) *reinterpret_cast<uint16_t *>(dst) = 0;
    uint32_t nw2;
    encode_pass<true>(src, tab, lt, reinterpret_cast<uint16_t *>(dst + 2 * odd), x, nw2);
    reinterpret_cast<uint32_t *>(dst + 2 * (nw + odd))[lane] = x;
  }
}

// ---------------------------------------------------------------------------
// Tables, group end offsets, stream headers and unit offsets.
__global__ void __launch_bounds__(kFinishThreads) gst_enc_finish_kernel(EncPlanView p) {
  const uint32_t k = blockIdx.x;
  const EncSection sec = p.sections[k];
  const EncUnit u = p.units[sec.unit];
  auto incl = [&](uint32_t g) -> unsigned long long {
    const unsigned long long v = p.status[g];
    if ((v >> 62) != 2) atomicOr(p.err, kErrTimeout);
    return v & kEncValueMask;
  };
  auto excl = [&](uint32_t g) -> unsigned long long { return g ? incl(g - 1) : 0ull; };
  const unsigned long long first = excl(sec.first_group);
  uint32_t *tbl = reinterpret_cast<uint32_t *>(p.out + sec.tbl_fixed + excl(sec.tbl_group));
  if (threadIdx.x < 128) {
    const uint16_t *f = p.freqs + k * 256 + 2 * threadIdx.x;
    tbl[threadIdx.x] = static_cast<uint32_t>(f[0]) | (static_cast<uint32_t>(f[1]) << 16);
  }
  uint32_t *offs = reinterpret_cast<uint32_t *>(p.out + sec.grp_fixed - 4ull * sec.n_groups + first);
  for (uint32_t j = threadIdx.x; j < sec.n_groups; j += kFinishThreads)
    offs[j] = static_cast<uint32_t>(4ull * sec.n_groups + incl(sec.first_group + j) - first);
  if (threadIdx.x == 0 && k == u.first_section) {
    const unsigned long long start = u.fixed_before + excl(u.first_group);
    p.offsets[sec.unit] = start;
    if (u.is_stream) {
      uint32_t *hdr = reinterpret_cast<uint32_t *>(p.out + start);
      hdr[0] = u.width;
      hdr[1] = u.height;
      hdr[2] = u.palette_bytes;
      for (uint32_t q = 0; q < u.n_sections; ++q) {
        const EncSection &s = p.sections[u.first_section + q];
        hdr[3 + q] = static_cast<uint32_t>(4ull * s.n_groups + incl(s.first_group + s.n_groups - 1) -
                                           excl(s.first_group));
      }
    }
    if (sec.unit == p.n_units - 1) p.offsets[p.n_units] = u.fixed_before + u.fixed_bytes + incl(p.n_groups - 1);
  }
}

std::atomic<int> g_rans_blocks_per_sm{0};  // occupancy of the encode kernel, computed once per process

}  // namespace

// Enqueues the encoder kernels of one plan.  normalize_only: the counts are
// already in place (gst_encode_normalize); only the normalisation runs.  With
// `ev` non-null, records ev[0] before the first kernel and ev[i + 1] after
// kernel i, whose name goes to names[i] (instrumentation).
cudaError_t launch_encode(const EncPlanView &v, int sm_count, cudaStream_t stream, bool normalize_only,
                          int *launches, cudaEvent_t *ev, const char **names, bool hist_match) {
  int n = 0;
  auto mark = [&](const char *name) {
    if (names) names[n] = name;
    ++n;
    if (ev) cudaEventRecord(ev[n], stream);
  };
  if (ev) cudaEventRecord(ev[0], stream);
  if (!normalize_only) {
    if (hist_match)
      gst_enc_histogram_kernel<true><<<v.n_chunks, kHistThreads, 0, stream>>>(v);
    else
      gst_enc_histogram_kernel<false><<<v.n_chunks, kHistThreads, 0, stream>>>(v);
    mark("gst_enc_histogram_kernel");
  }
  gst_enc_normalize_kernel<<<v.n_sections, kNormThreads + 32, 0, stream>>>(v);
  mark("gst_enc_normalize_kernel");
  if (!normalize_only) {
    int per_sm = g_rans_blocks_per_sm.load(std::memory_order_relaxed);
    if (per_sm == 0) {
      int b = 0;
      const cudaError_t e =
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, gst_enc_rans_kernel<kEncWarps>, kEncWarps * 32, 0);
      if (e != cudaSuccess) return e;
      per_sm = b > 0 ? b : 1;
      g_rans_blocks_per_sm.store(per_sm, std::memory_order_relaxed);
    }
    const uint32_t need = (v.n_groups + kEncWarps - 1) / kEncWarps;
    const uint32_t fill = static_cast<uint32_t>(per_sm * sm_count);
    gst_enc_rans_kernel<kEncWarps><<<need < fill ? need : fill, kEncWarps * 32, 0, stream>>>(v);
    mark("gst_enc_rans_kernel");
    gst_enc_finish_kernel<<<v.n_sections, kFinishThreads, 0, stream>>>(v);
    mark("gst_enc_finish_kernel");
  }
  if (launches) *launches = n;
  return cudaGetLastError();
}

}  // namespace gst
