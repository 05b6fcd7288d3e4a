// gst_encode.cu -- sm_103a kernels of the GST encoder stages: the reference's
// ByteEncoder::EncodeBytes (codec/entropy.cpp:174-265) over any number of
// sections in four launches.
//
//  gst_enc_histogram_kernel  byte counts per section (entropy.cpp:176-179):
//     one CTA per 32 KB chunk, warp-private shared histograms; lanes holding
//     the same byte are merged with a match-any before one shared atomic, so
//     skewed sections (most bytes 128) do not serialise on one bin.
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

#include "gst_encode_plan.h"
#include "gst_plan.h"

namespace gst {
namespace {

constexpr int kHistThreads = 256;
constexpr int kNormThreads = 256;
constexpr int kFinishThreads = 256;
constexpr int kEncWarps = 2;
constexpr size_t kEncSmemPerWarp = 256 * sizeof(uint4) + kEncMaxWords * sizeof(uint16_t);
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
__device__ __forceinline__ void count_word(uint32_t *h, uint32_t w, int lane) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t b = (w >> (8 * k)) & 0xFF;
    const uint32_t same = __match_any_sync(0xFFFFFFFFu, b);
    if (lane == __ffs(same) - 1) atomicAdd(&h[b], __popc(same));
  }
}

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
    count_word(h, a.x, lane);
    count_word(h, a.y, lane);
    count_word(h, a.z, lane);
    count_word(h, a.w, lane);
    count_word(h, b.x, lane);
    count_word(h, b.y, lane);
    count_word(h, b.z, lane);
    count_word(h, b.w, lane);
  }
  __syncthreads();
  uint32_t sum = 0;
#pragma unroll
  for (int w = 0; w < kHistThreads / 32; ++w) sum += hist[w][threadIdx.x];
  if (sum) atomicAdd(&p.counts[ch.section * 256 + threadIdx.x], sum);
}

// ---------------------------------------------------------------------------
// Frequency normalisation (ans/histogram.cpp:40-121).
struct NormShared {
  unsigned long long red64[kNormThreads / 32];
  int red32[kNormThreads / 32];
  unsigned long long bcast;
  uint32_t cnt[256];
  int first[256];  // first guess
  int fin[256];    // result of the heap replay
  unsigned long long heap_key[256];
  int heap_sym[256];
};

__device__ __forceinline__ unsigned long long block_min64(unsigned long long v, NormShared &s) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const unsigned long long u = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = u < v ? u : v;
  }
  if ((threadIdx.x & 31) == 0) s.red64[threadIdx.x >> 5] = v;
  __syncthreads();
  v = s.red64[0];
#pragma unroll
  for (int w = 1; w < kNormThreads / 32; ++w) v = s.red64[w] < v ? s.red64[w] : v;
  __syncthreads();
  return v;
}

__device__ __forceinline__ int block_sum32(int v, NormShared &s) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) s.red32[threadIdx.x >> 5] = v;
  __syncthreads();
  v = 0;
#pragma unroll
  for (int w = 0; w < kNormThreads / 32; ++w) v += s.red32[w];
  __syncthreads();
  return v;
}

__device__ __forceinline__ uint32_t block_sum_u32(uint32_t v, NormShared &s) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) s.red32[threadIdx.x >> 5] = static_cast<int>(v);
  __syncthreads();
  v = 0;
#pragma unroll
  for (int w = 0; w < kNormThreads / 32; ++w) v += static_cast<uint32_t>(s.red32[w]);
  __syncthreads();
  return v;
}

__device__ __forceinline__ int block_min32(int v, NormShared &s) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  if ((threadIdx.x & 31) == 0) s.red32[threadIdx.x >> 5] = v;
  __syncthreads();
  v = s.red32[0];
#pragma unroll
  for (int w = 1; w < kNormThreads / 32; ++w) v = min(v, s.red32[w]);
  __syncthreads();
  return v;
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
  __syncthreads();
  int before = 0;
  for (int w = 0; w < warp; ++w) before += s.red32[w];
  __syncthreads();
  return v + before;
}

// Ordered key of the rank of a symbol with `count` at frequency n:
// GetFreqChange (ans/histogram.cpp:25-29) = log2(n / (n + sign)) * count,
// as a u64 that orders like the double; kKeyInf where the symbol cannot move
// (sign -1 and n <= 1, histogram.cpp:86-91 and :109).
__device__ __forceinline__ unsigned long long rank_key(const double *L, int sign, int n, double count) {
  if ((sign < 0 && n <= 1) || n < 0 || n >= static_cast<int>(kEncLogTableLen)) return kKeyInf;
  const double r = __dmul_rn(__ldg(L + n), count);
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(r));
  return sign < 0 ? b : ~b;  // sign +1: every rank is negative, so the bit order reverses
}

// Number of consecutive ranks of this symbol, from frequency n on, below T
// (at most cap): exponential then binary search over its increasing ranks.
__device__ __forceinline__ int count_below(const double *L, int sign, int n, double count, unsigned long long T,
                                           int cap) {
  if (rank_key(L, sign, n, count) >= T) return 0;
  int good = 0, bad = cap;
  for (int c = 1; c < cap; c *= 2) {
    if (rank_key(L, sign, n + sign * c, count) < T) {
      good = c;
    } else {
      bad = c;
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
__device__ void heap_replay(NormShared &s, const double *L, int sign, int correction, uint32_t *err) {
  int len = 0;
  for (int i = 0; i < 256; ++i) {
    s.fin[i] = s.first[i];
    if (s.cnt[i] && (s.first[i] > 1 || correction > 0)) {
      s.heap_key[len] = rank_key(L, sign, s.first[i], static_cast<double>(static_cast<int>(s.cnt[i])));
      s.heap_sym[len] = i;
      ++len;
    }
  }
  if (len >= 2) {
    for (int parent = (len - 2) / 2;; --parent) {
      heap_adjust(s.heap_key, s.heap_sym, parent, len, s.heap_key[parent], s.heap_sym[parent]);
      if (parent == 0) break;
    }
  }
  while (correction != 0) {
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

__global__ void __launch_bounds__(kNormThreads) gst_enc_normalize_kernel(EncPlanView p) {
  __shared__ NormShared s;
  const int i = threadIdx.x;
  const uint32_t k = blockIdx.x;
  const uint32_t c = p.counts[k * 256 + i];
  s.cnt[i] = c;
  // fold_sum (histogram.cpp:31-33): uint32 sum, then int
  const int sum = static_cast<int>(block_sum_u32(c, s));
  // first guess (histogram.cpp:52-63): uint32 product, float quotient, double test
  int n = 0;
  if (c) {
    const uint32_t scaled = c * kTableSize;
    const double fs = static_cast<double>(__fdiv_rn(__uint2float_rn(scaled), __int2float_rn(sum)));
    const int down = static_cast<int>(fs);
    const int v = (__dmul_rn(fs, fs) <= static_cast<double>(down * (down + 1))) ? down : down + 1;
    n = v > 1 ? v : 1;
  }
  s.first[i] = n;
  const int correction = static_cast<int>(kTableSize) - block_sum32(n, s);
  if (correction != 0) {
    const int sign = correction > 0 ? 1 : -1;
    const double *L = sign > 0 ? p.log2_plus : p.log2_minus;
    const bool cand = c != 0 && (n > 1 || correction > 0);
    const double cd = static_cast<double>(static_cast<int>(c));
    int left = correction > 0 ? correction : -correction;
    bool replay = false;
    while (left > 0) {
      const unsigned long long head = cand ? rank_key(L, sign, n, cd) : kKeyInf;
      const unsigned long long m1 = block_min64(head, s);
      if (m1 == kKeyInf) {  // nothing can move (the reference asserts)
        if (i == 0) atomicOr(p.err, kErrTable);
        break;
      }
      const bool tied = head == m1;
      const int t = block_sum32(tied ? 1 : 0, s);
      const int i0 = block_min32(tied ? i : 256, s);
      // Largest j such that the ranks below T(j) = the j-th next rank of
      // symbol i0 number at most `left` (all of them are then popped).
      int best = 0, bad = 0;
      for (int j = 1;; j *= 2) {
        if (j > left) {
          bad = j;
          break;
        }
        if (i == i0) s.bcast = rank_key(L, sign, n + sign * j, cd);
        __syncthreads();
        const unsigned long long T = s.bcast;
        __syncthreads();
        const int tot = block_sum32(cand && head < T ? count_below(L, sign, n, cd, T, left + 1) : 0, s);
        if (tot > left) {
          bad = j;
          break;
        }
        best = j;
        if (T == kKeyInf) break;
      }
      if (bad) {
        while (bad - best > 1) {
          const int mid = (best + bad) >> 1;
          if (i == i0) s.bcast = rank_key(L, sign, n + sign * mid, cd);
          __syncthreads();
          const unsigned long long T = s.bcast;
          __syncthreads();
          const int tot = block_sum32(cand && head < T ? count_below(L, sign, n, cd, T, left + 1) : 0, s);
          if (tot <= left)
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
        if (tied) n += sign;
        left -= t;
        continue;
      }
      if (i == i0) s.bcast = rank_key(L, sign, n + sign * best, cd);
      __syncthreads();
      const unsigned long long T = s.bcast;
      __syncthreads();
      const int adv = cand && head < T ? count_below(L, sign, n, cd, T, left + 1) : 0;
      n += sign * adv;
      left -= block_sum32(adv, s);
    }
    if (replay) {
      if (i == 0) heap_replay(s, L, sign, correction, p.err);
      __syncthreads();
      n = s.fin[i];
    }
  }
  // Encode entry: the reciprocal m = ceil(2^(31 + l) / F), l = ceil(log2 F),
  // gives floor(x / F) = umulhi(2x, m) >> l for every x < 2^31.
  const uint32_t F = static_cast<uint32_t>(n);
  const int C = block_scan32(n, s) - n;
  uint4 e = make_uint4(0, 0, 0, 0);
  if (F) {
    const uint32_t l = F > 1 ? 32 - __clz(F - 1) : 0;
    const uint32_t m = static_cast<uint32_t>(((1ull << (31 + l)) + F - 1) / F);
    e = make_uint4(m, F << 20, kTableSize - F, static_cast<uint32_t>(C) | (l << 16));
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
  if (lane == 0) st_relaxed(p.status + g, (g == 0 ? kEncFlagInclusive : kEncFlagAggregate) | bytes);
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
  if (lane == 0) st_relaxed(p.status + g, kEncFlagInclusive | (excl + bytes));
  return excl;
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) gst_enc_rans_kernel(EncPlanView p) {
  extern __shared__ __align__(16) uint8_t enc_smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint4 *tab = reinterpret_cast<uint4 *>(enc_smem + warp * kEncSmemPerWarp);
  uint16_t *words = reinterpret_cast<uint16_t *>(enc_smem + warp * kEncSmemPerWarp + 256 * sizeof(uint4));
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
      for (int e = lane; e < 256; e += 32) tab[e] = p.tables[k * 256 + e];
      __syncwarp();
      cur = k;
    }
    const uint4 *src = reinterpret_cast<const uint4 *>(sec.sym + static_cast<size_t>(g - sec.first_group) * kSymsPerGroup +
                                                       lane * kSymsPerStream);
    uint32_t x = kRansL, nw = 0;
    uint4 q = __ldg(src);
    for (int j = 0; j < static_cast<int>(kSymsPerStream / 16); ++j) {
      const uint4 nxt = __ldg(src + (j + 1 < static_cast<int>(kSymsPerStream / 16) ? j + 1 : j));
      const uint32_t w4[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int b = 0; b < 16; ++b) {
        const uint32_t s = (w4[b >> 2] >> (8 * (b & 3))) & 0xFF;
        const uint4 e = tab[s];
        // renormalise (encode.cpp:59-64): at most one word, x < 2^31
        const bool r = x >= e.y;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, r);
        if (r) {
          words[nw + __popc(m & lt)] = static_cast<uint16_t>(x);
          x >>= 16;
        }
        nw += __popc(m);
        // x' = (x / F) * M + C + x % F = x + q * (M - F) + C (encode.cpp:67)
        const uint32_t qd = __umulhi(x + x, e.x) >> (e.w >> 16);
        x = x + qd * e.z + (e.w & 0xFFFF);
      }
      q = nxt;
    }
    // Group bytes: [2 zero bytes if the word count is odd][words][32 states]
    // (entropy.cpp:213-229 and encode.cpp:248-256).
    const uint32_t odd = nw & 1;
    const uint32_t bytes = 2 * (nw + odd) + 4 * kStreamsPerGroup;
    const unsigned long long before = enc_lookback(p, g, bytes, lane);
    uint32_t *d32 = reinterpret_cast<uint32_t *>(p.out + sec.grp_fixed + before);
    __syncwarp();
    const uint32_t n32 = (nw + odd) >> 1;
    for (uint32_t w = lane; w < n32; w += 32) {
      const int lo = 2 * static_cast<int>(w) - static_cast<int>(odd);
      const uint32_t wlo = lo >= 0 ? words[lo] : 0u;
      d32[w] = wlo | (static_cast<uint32_t>(words[lo + 1]) << 16);
    }
    d32[n32 + lane] = x;
    __syncwarp();
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

int g_rans_blocks_per_sm = 0;

}  // namespace

size_t encode_rans_smem_bytes() { return kEncWarps * kEncSmemPerWarp; }

// Enqueues the encoder kernels of one plan.  normalize_only: the counts are
// already in place (gst_encode_normalize); only the normalisation runs.
cudaError_t launch_encode(const EncPlanView &v, int sm_count, cudaStream_t stream, bool normalize_only,
                          int *launches) {
  int n = 0;
  if (!normalize_only) {
    gst_enc_histogram_kernel<<<v.n_chunks, kHistThreads, 0, stream>>>(v);
    ++n;
  }
  gst_enc_normalize_kernel<<<v.n_sections, kNormThreads, 0, stream>>>(v);
  ++n;
  if (!normalize_only) {
    const size_t smem = encode_rans_smem_bytes();
    if (g_rans_blocks_per_sm == 0) {
      cudaError_t e = cudaFuncSetAttribute(gst_enc_rans_kernel<kEncWarps>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem));
      if (e != cudaSuccess) return e;
      int b = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, gst_enc_rans_kernel<kEncWarps>, kEncWarps * 32, smem);
      if (e != cudaSuccess) return e;
      g_rans_blocks_per_sm = b > 0 ? b : 1;
    }
    const uint32_t need = (v.n_groups + kEncWarps - 1) / kEncWarps;
    const uint32_t fill = static_cast<uint32_t>(g_rans_blocks_per_sm * sm_count);
    gst_enc_rans_kernel<kEncWarps><<<need < fill ? need : fill, kEncWarps * 32, smem, stream>>>(v);
    gst_enc_finish_kernel<<<v.n_sections, kFinishThreads, 0, stream>>>(v);
    n += 2;
  }
  if (launches) *launches = n;
  return cudaGetLastError();
}

}  // namespace gst
