// gst_encoder.cpp -- the project's GST stream producer (host side).
//
// Format stages restate the reference encoder (GammaUNC/GST) exactly, in this
// project's own code:
//   RGB565 -> YCoCg667                 codec/image_processing.cpp:10-27
//   32x32 five-level 5/3 forward       codec/image_processing.h:291-330,
//     wavelet, +128, block-linear        codec/wavelet.cpp:56-157,
//                                        codec/entropy.h:216-263
//   plane order Y1 Y2 | Co1 Cg1 Co2 Cg2 codec/encoder.cpp:86-98
//   palette padded to 8192 bytes       codec/encoder.cpp:100-108
//   index deltas +128                  codec/dxt_image.cpp:605-619
//   section format                     codec/entropy.cpp:174-265
//   frequency normalisation            ans/histogram.cpp:40-121
//   interleaved rANS (b=2^16,k=2^4,M=2^11) ans/encode.cpp:56-69,224-259
// The DXT1 block compressor and the palette search are this project's own.
#include "gst_encoder.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr uint32_t kTableSize = 2048;
constexpr uint32_t kSymsPerStream = 256;
constexpr uint32_t kStreams = 32;
constexpr uint32_t kSymsPerGroup = kSymsPerStream * kStreams;
constexpr int kPaletteLookback = 127;
constexpr int kReuseThreshold = 35;

template <typename F>
void parallel_for(uint32_t count, int nthreads, F fn) {
  if (nthreads <= 1 || count < 2) {
    fn(0u, count);
    return;
  }
  nthreads = std::min<int>(nthreads, static_cast<int>(count));
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) {
    const uint32_t lo = static_cast<uint32_t>(uint64_t(count) * t / nthreads);
    const uint32_t hi = static_cast<uint32_t>(uint64_t(count) * (t + 1) / nthreads);
    th.emplace_back([=] { fn(lo, hi); });
  }
  for (auto &t : th) t.join();
}

// ---------------------------------------------------------------------------
// PRNG: splitmix64 seeding a xoshiro256** generator (Blackman & Vigna).
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    for (auto &w : s) {
      seed += 0x9E3779B97F4A7C15ull;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      w = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  // Uniform integer in [lo, hi].
  int64_t range(int64_t lo, int64_t hi) {
    return lo + static_cast<int64_t>(next() % static_cast<uint64_t>(hi - lo + 1));
  }
};

uint64_t hash64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xFF51AFD7ED558CCDull;
  x ^= x >> 33;
  x *= 0xC4CEB9FE1A85EC53ull;
  x ^= x >> 33;
  return x;
}

// ---------------------------------------------------------------------------
// Synthetic image.
struct Gradient {
  int64_t ux, uy, pmin, pspan;
  int64_t slope[3], offset[3];
};

struct RectPaint {
  uint32_t x0, y0, x1, y1;
  uint8_t c0[3], c1[3];
  uint32_t cell;  // 0: solid colour c0; else checkerboard of c0/c1 with this cell size
};

// Value noise: lattice values in [-1024, 1024] hashed from (seed, octave,
// channel, ix, iy); smoothstep weights in 16.16 fixed point.
int64_t lattice(uint64_t seed, int oct, int ch, int64_t ix, int64_t iy) {
  const uint64_t h = hash64(seed ^ hash64((uint64_t(oct) << 56) ^ (uint64_t(ch) << 48) ^
                                          (uint64_t(ix & 0xFFFFFF) << 24) ^ uint64_t(iy & 0xFFFFFF)));
  return static_cast<int64_t>(h % 2049) - 1024;
}

int64_t smooth16(int64_t t) {  // t in [0, 65536): 3t^2 - 2t^3 in 16.16
  return (t * t / 65536) * (3 * 65536 - 2 * t) / 65536;
}

int64_t value_noise(uint64_t seed, int oct, int period, int ch, int64_t x, int64_t y) {
  const int64_t ix = x / period, iy = y / period;
  const int64_t tx = smooth16((x % period) * 65536 / period);
  const int64_t ty = smooth16((y % period) * 65536 / period);
  const int64_t v00 = lattice(seed, oct, ch, ix, iy), v10 = lattice(seed, oct, ch, ix + 1, iy);
  const int64_t v01 = lattice(seed, oct, ch, ix, iy + 1), v11 = lattice(seed, oct, ch, ix + 1, iy + 1);
  const int64_t a = v00 * (65536 - tx) + v10 * tx;  // 1024 * 2^16 scale
  const int64_t b = v01 * (65536 - tx) + v11 * tx;
  return (a / 65536) * (65536 - ty) / 65536 + (b / 65536) * ty / 65536;  // [-1024, 1024]
}

}  // namespace

extern "C" int gst_synth_image(uint32_t w, uint32_t h, uint64_t seed, double checker_frac,
                               uint8_t *rgb) {
  if (!rgb || w == 0 || h == 0) return 1;
  Rng rng(seed);
  Gradient g[4];
  for (auto &gr : g) {
    gr.ux = rng.range(-4096, 4096);
    gr.uy = rng.range(-4096, 4096);
    if (gr.ux == 0 && gr.uy == 0) gr.ux = 1;
    const int64_t c[4] = {0, gr.ux * (w - 1), gr.uy * (h - 1), gr.ux * (w - 1) + gr.uy * (h - 1)};
    gr.pmin = *std::min_element(c, c + 4);
    gr.pspan = std::max<int64_t>(1, *std::max_element(c, c + 4) - gr.pmin);
    for (int ch = 0; ch < 3; ++ch) {
      gr.slope[ch] = rng.range(-48, 47);
      gr.offset[ch] = rng.range(0, 47);
    }
  }
  std::vector<RectPaint> rects;
  for (int i = 0; i < 20; ++i) {
    RectPaint r{};
    const uint32_t rw = static_cast<uint32_t>(rng.range(std::max<int64_t>(1, w / 32), std::max<int64_t>(1, w / 4)));
    const uint32_t rh = static_cast<uint32_t>(rng.range(std::max<int64_t>(1, h / 32), std::max<int64_t>(1, h / 4)));
    r.x0 = static_cast<uint32_t>(rng.range(0, w - 1));
    r.y0 = static_cast<uint32_t>(rng.range(0, h - 1));
    r.x1 = std::min(w, r.x0 + rw);
    r.y1 = std::min(h, r.y0 + rh);
    for (int ch = 0; ch < 3; ++ch) r.c0[ch] = static_cast<uint8_t>(rng.range(0, 255));
    r.cell = 0;
    rects.push_back(r);
  }
  if (checker_frac > 0) {
    const double target = checker_frac * double(w) * double(h);
    double area = 0;
    while (area < target) {
      RectPaint r{};
      const uint32_t rw = static_cast<uint32_t>(rng.range(std::max<int64_t>(8, w / 64), std::max<int64_t>(8, w / 12)));
      const uint32_t rh = static_cast<uint32_t>(rng.range(std::max<int64_t>(8, h / 64), std::max<int64_t>(8, h / 12)));
      r.x0 = static_cast<uint32_t>(rng.range(0, w - 1));
      r.y0 = static_cast<uint32_t>(rng.range(0, h - 1));
      r.x1 = std::min(w, r.x0 + rw);
      r.y1 = std::min(h, r.y0 + rh);
      for (int ch = 0; ch < 3; ++ch) {
        r.c0[ch] = static_cast<uint8_t>(rng.range(0, 255));
        r.c1[ch] = static_cast<uint8_t>(rng.range(0, 255));
      }
      r.cell = static_cast<uint32_t>(rng.range(1, 8));
      area += double(r.x1 - r.x0) * double(r.y1 - r.y0);
      rects.push_back(r);
    }
  }
  const uint64_t nseed = rng.next();
  const int periods[3] = {64, 32, 16};
  const int64_t weights[3] = {4, 2, 1};  // 1, 1/2, 1/4 normalised by 7/4
  std::vector<int> base(3 * size_t(w) * h);
  parallel_for(h, 8, [&](uint32_t lo, uint32_t hi) {
    for (uint32_t y = lo; y < hi; ++y) {
      for (uint32_t x = 0; x < w; ++x) {
        for (int ch = 0; ch < 3; ++ch) {
          int64_t v = 0;
          for (const auto &gr : g) {
            const int64_t t = (gr.ux * x + gr.uy * y - gr.pmin) * 4096 / gr.pspan;  // [0, 4096]
            v += gr.offset[ch] + gr.slope[ch] * t / 4096;
          }
          int64_t n = 0;
          for (int o = 0; o < 3; ++o) n += weights[o] * value_noise(nseed, o, periods[o], ch, x, y);
          v += n * 20 / (7 * 1024);  // amplitude 40 peak to peak
          base[(size_t(y) * w + x) * 3 + ch] = static_cast<int>(v);
        }
      }
    }
  });
  for (const auto &r : rects) {
    for (uint32_t y = r.y0; y < r.y1; ++y) {
      for (uint32_t x = r.x0; x < r.x1; ++x) {
        const bool second = r.cell && (((x - r.x0) / r.cell + (y - r.y0) / r.cell) & 1);
        for (int ch = 0; ch < 3; ++ch) {
          int &px = base[(size_t(y) * w + x) * 3 + ch];
          if (r.cell) px = second ? r.c1[ch] : r.c0[ch];
          else px = r.c0[ch] + (px - 96) / 4;  // solid colour keeps a little of the texture
        }
      }
    }
  }
  for (size_t i = 0; i < base.size(); ++i) rgb[i] = static_cast<uint8_t>(std::min(255, std::max(0, base[i])));
  return 0;
}

namespace {

// ---------------------------------------------------------------------------
// DXT1 block compressor (this project's own): principal axis by power
// iteration, extreme projections as endpoints, nearest-colour indices in the
// four-colour mode (colour0 > colour1), one least-squares endpoint refinement.
struct Rgb8 {
  int r, g, b;
};

Rgb8 expand565(uint16_t c) {
  const int r = c >> 11, g = (c >> 5) & 63, b = c & 31;
  return {(r << 3) | (r >> 2), (g << 2) | (g >> 4), (b << 3) | (b >> 2)};
}

uint16_t quant565(double r, double g, double b) {
  auto q = [](double v, int maxv) {
    const int i = static_cast<int>(std::floor(std::min(255.0, std::max(0.0, v)) * maxv / 255.0 + 0.5));
    return std::min(maxv, std::max(0, i));
  };
  return static_cast<uint16_t>((q(r, 31) << 11) | (q(g, 63) << 5) | q(b, 31));
}

void palette4(uint16_t c0, uint16_t c1, Rgb8 p[4]) {
  p[0] = expand565(c0);
  p[1] = expand565(c1);
  p[2] = {(2 * p[0].r + p[1].r) / 3, (2 * p[0].g + p[1].g) / 3, (2 * p[0].b + p[1].b) / 3};
  p[3] = {(p[0].r + 2 * p[1].r) / 3, (p[0].g + 2 * p[1].g) / 3, (p[0].b + 2 * p[1].b) / 3};
}

int dist2(const Rgb8 &a, const uint8_t *px) {
  const int dr = a.r - px[0], dg = a.g - px[1], db = a.b - px[2];
  return dr * dr + dg * dg + db * db;
}

uint32_t assign_indices(const uint8_t px[48], const Rgb8 p[4], int *err) {
  uint32_t word = 0;
  int total = 0;
  for (int i = 0; i < 16; ++i) {
    int best = 0, bd = dist2(p[0], px + 3 * i);
    for (int k = 1; k < 4; ++k) {
      const int d = dist2(p[k], px + 3 * i);
      if (d < bd) {
        bd = d;
        best = k;
      }
    }
    total += bd;
    word |= uint32_t(best) << (2 * i);
  }
  *err = total;
  return word;
}

uint64_t make_block(uint16_t c0, uint16_t c1, uint32_t word) {
  return uint64_t(c0) | (uint64_t(c1) << 16) | (uint64_t(word) << 32);
}

// Orders the endpoints for the four-colour mode; equal endpoints give word 0.
uint64_t finish_block(uint16_t c0, uint16_t c1, const uint8_t px[48], int *err) {
  if (c0 == c1) {
    Rgb8 p[4];
    palette4(c0, c1, p);
    int e = 0;
    for (int i = 0; i < 16; ++i) e += dist2(p[0], px + 3 * i);
    *err = e;
    return make_block(c0, c1, 0);
  }
  if (c0 < c1) std::swap(c0, c1);
  Rgb8 p[4];
  palette4(c0, c1, p);
  const uint32_t word = assign_indices(px, p, err);
  return make_block(c0, c1, word);
}

uint64_t compress_block(const uint8_t px[48]) {
  double mean[3] = {0, 0, 0};
  for (int i = 0; i < 16; ++i)
    for (int c = 0; c < 3; ++c) mean[c] += px[3 * i + c];
  for (double &m : mean) m /= 16.0;
  double cov[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 16; ++i) {
    const double r = px[3 * i] - mean[0], g = px[3 * i + 1] - mean[1], b = px[3 * i + 2] - mean[2];
    cov[0] += r * r;
    cov[1] += r * g;
    cov[2] += r * b;
    cov[3] += g * g;
    cov[4] += g * b;
    cov[5] += b * b;
  }
  double v[3] = {1.0, 0.7, 0.3};
  for (int it = 0; it < 4; ++it) {
    const double x = cov[0] * v[0] + cov[1] * v[1] + cov[2] * v[2];
    const double y = cov[1] * v[0] + cov[3] * v[1] + cov[4] * v[2];
    const double z = cov[2] * v[0] + cov[4] * v[1] + cov[5] * v[2];
    const double m = std::max(std::fabs(x), std::max(std::fabs(y), std::fabs(z)));
    if (m < 1e-9) break;
    v[0] = x / m;
    v[1] = y / m;
    v[2] = z / m;
  }
  int imin = 0, imax = 0;
  double pmin = 1e300, pmax = -1e300;
  for (int i = 0; i < 16; ++i) {
    const double p = px[3 * i] * v[0] + px[3 * i + 1] * v[1] + px[3 * i + 2] * v[2];
    if (p < pmin) {
      pmin = p;
      imin = i;
    }
    if (p > pmax) {
      pmax = p;
      imax = i;
    }
  }
  uint16_t c0 = quant565(px[3 * imax], px[3 * imax + 1], px[3 * imax + 2]);
  uint16_t c1 = quant565(px[3 * imin], px[3 * imin + 1], px[3 * imin + 2]);
  int err = 0;
  uint64_t best = finish_block(c0, c1, px, &err);
  // One least-squares refit of the endpoints from the chosen indices.
  const uint32_t word = uint32_t(best >> 32);
  if (word != 0) {
    static const double wt[4] = {1.0, 0.0, 2.0 / 3.0, 1.0 / 3.0};  // weight of colour0
    double aa = 0, bb = 0, ab = 0, ax[3] = {0, 0, 0}, bx[3] = {0, 0, 0};
    for (int i = 0; i < 16; ++i) {
      const double a = wt[(word >> (2 * i)) & 3], b = 1.0 - a;
      aa += a * a;
      bb += b * b;
      ab += a * b;
      for (int c = 0; c < 3; ++c) {
        ax[c] += a * px[3 * i + c];
        bx[c] += b * px[3 * i + c];
      }
    }
    const double det = aa * bb - ab * ab;
    if (std::fabs(det) > 1e-9) {
      double e0[3], e1[3];
      for (int c = 0; c < 3; ++c) {
        e0[c] = (ax[c] * bb - bx[c] * ab) / det;
        e1[c] = (bx[c] * aa - ax[c] * ab) / det;
      }
      int err2 = 0;
      const uint64_t cand = finish_block(quant565(e0[0], e0[1], e0[2]), quant565(e1[0], e1[1], e1[2]), px, &err2);
      if (err2 < err) best = cand;
    }
  }
  return best;
}

void block_pixels(const uint8_t *rgb, uint32_t w, uint32_t bx, uint32_t by, uint8_t px[48]) {
  for (int y = 0; y < 4; ++y)
    memcpy(px + 12 * y, rgb + ((size_t(by) * 4 + y) * w + size_t(bx) * 4) * 3, 12);
}

// The reference's block error metric (codec/dxt_image.cpp:255-275): mean of
// squared channel differences, integer-divided by 48.
int block_error_from_dists(const int d[16][4], uint32_t word) {
  int e = 0;
  for (int i = 0; i < 16; ++i) e += d[i][(word >> (2 * i)) & 3];
  return e / 48;
}

// ---------------------------------------------------------------------------
// Frequency normalisation (ans/histogram.cpp:40-121, Bloom's heap correction).
struct RankedSymbol {
  int symbol;
  double rank;
  bool operator>(const RankedSymbol &o) const { return rank > o.rank; }
};

double freq_change(int count, int new_count, int sign) {
  return std::log2(static_cast<double>(new_count) / static_cast<double>(new_count + sign)) *
         static_cast<double>(count);
}

std::vector<uint32_t> normalize_counts(const std::vector<uint32_t> &counts, int M) {
  std::vector<uint32_t> hist;
  hist.reserve(counts.size());
  uint32_t usum = 0;
  for (uint32_t c : counts) usum += c;
  const int sum = static_cast<int>(usum);
  for (uint32_t c : counts) {
    if (c == 0) {
      hist.push_back(0);
      continue;
    }
    const uint32_t scaled = c * static_cast<uint32_t>(M);  // uint32 product, as the reference
    const double from_scaled = static_cast<float>(scaled) / static_cast<float>(sum);
    const int down = static_cast<int>(from_scaled);
    hist.push_back(static_cast<uint32_t>(
        std::max(1, (from_scaled * from_scaled <= down * (down + 1)) ? down : down + 1)));
  }
  uint32_t hsum = 0;
  for (uint32_t v : hist) hsum += v;
  int correction = M - static_cast<int>(hsum);
  if (correction == 0 || correction == M) return hist;
  const int sign = correction > 0 ? 1 : -1;
  std::vector<RankedSymbol> heap;
  for (size_t i = 0; i < counts.size(); ++i) {
    if (counts[i] == 0) continue;
    if (hist[i] > 1 || correction > 0)
      heap.push_back({static_cast<int>(i), freq_change(static_cast<int>(counts[i]),
                                                       static_cast<int>(hist[i]), sign)});
  }
  std::make_heap(heap.begin(), heap.end(), std::greater<RankedSymbol>());
  while (correction != 0 && !heap.empty()) {
    std::pop_heap(heap.begin(), heap.end(), std::greater<RankedSymbol>());
    const RankedSymbol s = heap.back();
    heap.pop_back();
    const int i = s.symbol;
    hist[i] = static_cast<uint32_t>(static_cast<int>(hist[i]) + sign);
    correction -= sign;
    if (hist[i] > 1 || sign == 1) {
      heap.push_back({i, freq_change(static_cast<int>(counts[i]), static_cast<int>(hist[i]), sign)});
      std::push_heap(heap.begin(), heap.end(), std::greater<RankedSymbol>());
    }
  }
  return hist;
}

// ---------------------------------------------------------------------------
// Interleaved rANS over one 8192-symbol group (ans/encode.cpp:56-69, 224-259).
void encode_group(const uint8_t *sym, const std::vector<uint32_t> &F, const std::vector<uint32_t> &C,
                  std::vector<uint8_t> *out) {
  uint32_t state[kStreams];
  for (auto &s : state) s = 16u * kTableSize;
  std::vector<uint16_t> words;
  words.reserve(kSymsPerGroup);
  for (uint32_t i = 0; i < kSymsPerStream; ++i) {
    for (uint32_t s = 0; s < kStreams; ++s) {
      const uint32_t x = sym[s * kSymsPerStream + i];
      uint32_t st = state[s];
      const uint32_t upper = F[x] << 20;  // b * k * F
      while (st >= upper) {
        words.push_back(static_cast<uint16_t>(st & 0xFFFF));
        st >>= 16;
      }
      state[s] = (st / F[x]) * kTableSize + C[x] + (st % F[x]);
    }
  }
  size_t nbytes = words.size() * 2 + 4 * kStreams;
  const size_t pad = (nbytes & 3) ? 2 : 0;
  out->assign(nbytes + pad, 0);
  uint8_t *p = out->data() + pad;
  for (uint16_t w : words) {
    *p++ = static_cast<uint8_t>(w);
    *p++ = static_cast<uint8_t>(w >> 8);
  }
  for (uint32_t s = 0; s < kStreams; ++s) {
    for (int k = 0; k < 4; ++k) *p++ = static_cast<uint8_t>(state[s] >> (8 * k));
  }
}

int encode_section(const uint8_t *in, size_t n, std::vector<uint8_t> *result, int nthreads) {
  if (n == 0 || n % kSymsPerGroup) return 1;
  std::vector<uint32_t> counts(256, 0);
  for (size_t i = 0; i < n; ++i) counts[in[i]]++;
  size_t nz = 0;
  for (size_t i = 0; i < 256; ++i)
    if (counts[i]) nz = i + 1;
  counts.resize(std::max<size_t>(nz, 2));
  std::vector<uint32_t> F = normalize_counts(counts, kTableSize);
  std::vector<uint32_t> C(F.size(), 0);
  for (size_t i = 1; i < F.size(); ++i) C[i] = C[i - 1] + F[i - 1];
  const uint32_t G = static_cast<uint32_t>(n / kSymsPerGroup);
  std::vector<std::vector<uint8_t> > groups(G);
  parallel_for(G, nthreads, [&](uint32_t lo, uint32_t hi) {
    for (uint32_t g = lo; g < hi; ++g) encode_group(in + size_t(g) * kSymsPerGroup, F, C, &groups[g]);
  });
  size_t total = 512 + 4 * size_t(G);
  for (const auto &g : groups) total += g.size();
  result->assign((total + 3) / 4 * 4, 0);
  uint8_t *p = result->data();
  for (size_t i = 0; i < 256; ++i) {
    const uint32_t f = i < F.size() ? F[i] : 0;
    p[2 * i] = static_cast<uint8_t>(f);
    p[2 * i + 1] = static_cast<uint8_t>(f >> 8);
  }
  uint32_t off = 4 * G;
  uint8_t *body = p + 512;
  size_t pos = 4 * size_t(G);
  for (uint32_t g = 0; g < G; ++g) {
    off += static_cast<uint32_t>(groups[g].size());
    for (int k = 0; k < 4; ++k) body[4 * g + k] = static_cast<uint8_t>(off >> (8 * k));
    memcpy(body + pos, groups[g].data(), groups[g].size());
    pos += groups[g].size();
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Endpoint planes: RGB565 -> YCoCg667 (codec/image_processing.cpp:10-27).
void rgb565_to_ycocg667(uint16_t c, int *y, int *co, int *cg) {
  const int r = c >> 11, g = (c >> 5) & 63, b = c & 31;
  *co = r - b;
  const int t = r + b + (b >> 4);
  *cg = g - t;
  *y = t + (*cg / 2);
}

int normalize_index(int idx, int range) {  // codec/wavelet.cpp:37-41
  const int v = idx - static_cast<int>(idx >= range) * (idx - range + 2);
  return v < 0 ? -v : v;
}

// codec/wavelet.cpp:56-88, int16 storage.
void forward_1d(const int16_t *src, int16_t *dst, int len) {
  const int mid = len - len / 2;
  for (int i = 1; i < len; i += 2) {
    const int next = normalize_index(i + 1, len), prev = normalize_index(i - 1, len);
    dst[mid + i / 2] = static_cast<int16_t>(src[i] - (src[prev] + src[next]) / 2);
  }
  for (int i = 0; i < len; i += 2) {
    const int next = mid + normalize_index(i + 1, len) / 2, prev = mid + normalize_index(i - 1, len) / 2;
    dst[i / 2] = static_cast<int16_t>(src[i] + (dst[prev] + dst[next] + 2) / 4);
  }
}

// codec/wavelet.cpp:123-157 on the top-left dim x dim of a 32x32 block:
// columns first, then rows.
void forward_2d(int16_t *blk, int dim) {
  int16_t line[32], out[32];
  for (int x = 0; x < dim; ++x) {
    for (int y = 0; y < dim; ++y) line[y] = blk[y * 32 + x];
    forward_1d(line, out, dim);
    for (int y = 0; y < dim; ++y) blk[y * 32 + x] = out[y];
  }
  for (int y = 0; y < dim; ++y) {
    forward_1d(blk + y * 32, out, dim);
    memcpy(blk + y * 32, out, sizeof(int16_t) * dim);
  }
}

// The decoder's inverse (int32 intermediates, C division, char result), used
// only for tiles whose coefficients did not fit in 8 bits: it tells which
// endpoints such a stream really decodes to.
void inverse_1d_i32(int32_t *v, int stride, int len) {
  const int mid = len / 2;
  int32_t s[32], d[32];
  for (int k = 0; k < len; ++k) s[k] = v[k * stride];
  for (int x = 0; x < mid; ++x) {
    const int prev = mid + normalize_index(2 * x - 1, len) / 2, next = mid + normalize_index(2 * x + 1, len) / 2;
    d[2 * x] = s[x] - (s[prev] + s[next] + 2) / 4;
  }
  for (int x = 0; x < mid; ++x)
    d[2 * x + 1] = s[mid + x] + (d[normalize_index(2 * x, len)] + d[normalize_index(2 * x + 2, len)]) / 2;
  for (int k = 0; k < len; ++k) v[k * stride] = d[k];
}

void decode_tile(const uint8_t *bytes, int8_t *out) {
  int32_t b[1024];
  for (int i = 0; i < 1024; ++i) b[i] = int32_t(bytes[i]) - 128;
  for (int len = 2; len <= 32; len *= 2) {
    for (int r = 0; r < len; ++r) inverse_1d_i32(b + r * 32, 1, len);
    for (int c = 0; c < len; ++c) inverse_1d_i32(b + c, 32, len);
  }
  for (int i = 0; i < 1024; ++i) out[i] = static_cast<int8_t>(static_cast<uint8_t>(uint32_t(b[i]) & 0xFF));
}

uint16_t ycocg_to_565(int y, int co, int cg) {  // the decoder's arithmetic
  const int t = y - cg / 2, g = cg + t, b = (t - co) / 2, r = b + co;
  return static_cast<uint16_t>((uint32_t(r) << 11) | (uint32_t(g) << 5) | uint32_t(b));
}

// One plane (bx x by values) -> block-linear bytes, +128, counting clips.
void plane_to_stream(const std::vector<int> &plane, uint32_t bx, uint32_t by, uint8_t *out,
                     uint64_t *clips, std::vector<uint8_t> *tile_clipped) {
  const uint32_t tx_n = bx / 32, ty_n = by / 32;
  for (uint32_t ty = 0; ty < ty_n; ++ty) {
    for (uint32_t tx = 0; tx < tx_n; ++tx) {
      int16_t blk[1024];
      for (int y = 0; y < 32; ++y)
        for (int x = 0; x < 32; ++x) blk[y * 32 + x] = static_cast<int16_t>(plane[(size_t(ty) * 32 + y) * bx + tx * 32 + x]);
      for (int dim = 32; dim > 1; dim /= 2) forward_2d(blk, dim);
      uint8_t *dst = out + (size_t(ty) * tx_n + tx) * 1024;
      for (int i = 0; i < 1024; ++i) {
        if (blk[i] < -128 || blk[i] > 127) {
          ++*clips;
          (*tile_clipped)[size_t(ty) * tx_n + tx] = 1;
        }
        dst[i] = static_cast<uint8_t>(static_cast<int8_t>(blk[i]) + 128);
      }
    }
  }
}

int write_stream(uint32_t w, uint32_t h, std::vector<uint64_t> &blocks,
                 const std::vector<uint32_t> &palette, const std::vector<uint8_t> &index_deltas,
                 uint8_t **out, size_t *out_len, uint64_t *clips_out, int nthreads) {
  const uint32_t bx = w / 4, by = h / 4;
  const size_t B = size_t(bx) * by;
  std::vector<int> planes[6];  // Y1 Co1 Cg1 Y2 Co2 Cg2
  for (auto &p : planes) p.resize(B);
  for (size_t i = 0; i < B; ++i) {
    const uint16_t e1 = static_cast<uint16_t>(blocks[i]), e2 = static_cast<uint16_t>(blocks[i] >> 16);
    rgb565_to_ycocg667(e1, &planes[0][i], &planes[1][i], &planes[2][i]);
    rgb565_to_ycocg667(e2, &planes[3][i], &planes[4][i], &planes[5][i]);
  }
  std::vector<uint8_t> ybuf(2 * B), cbuf(4 * B);
  uint64_t clips[6] = {0, 0, 0, 0, 0, 0};
  // Y section: Y1, Y2.  Chroma section: Co1, Cg1, Co2, Cg2 (codec/encoder.cpp:86-98).
  uint8_t *dst[6] = {ybuf.data(), cbuf.data(), cbuf.data() + B, ybuf.data() + B, cbuf.data() + 2 * B,
                     cbuf.data() + 3 * B};
  const uint32_t tiles_x = bx / 32, tiles = tiles_x * (by / 32);
  std::vector<uint8_t> clipped[6];
  for (auto &c : clipped) c.assign(tiles, 0);
  parallel_for(6, nthreads, [&](uint32_t lo, uint32_t hi) {
    for (uint32_t p = lo; p < hi; ++p) plane_to_stream(planes[p], bx, by, dst[p], &clips[p], &clipped[p]);
  });
  uint64_t clips_total = 0;
  for (uint64_t c : clips) clips_total += c;
  if (clips_out) *clips_out = clips_total;
  // Coefficients that did not fit in 8 bits wrap, as in the reference encoder;
  // report the endpoints such tiles really decode to.
  for (uint32_t t = 0; t < tiles && clips_total; ++t) {
    bool any = false;
    for (auto &c : clipped) any = any || c[t];
    if (!any) continue;
    int8_t dec[6][1024];
    for (int p = 0; p < 6; ++p) decode_tile(dst[p] + size_t(t) * 1024, dec[p]);
    const uint32_t tx = t % tiles_x, ty = t / tiles_x;
    for (int i = 0; i < 1024; ++i) {
      const size_t bi = (size_t(ty) * 32 + i / 32) * bx + tx * 32 + i % 32;
      const uint16_t e1 = ycocg_to_565(dec[0][i], dec[1][i], dec[2][i]);
      const uint16_t e2 = ycocg_to_565(dec[3][i], dec[4][i], dec[5][i]);
      blocks[bi] = (blocks[bi] & 0xFFFFFFFF00000000ull) | uint64_t(e1) | (uint64_t(e2) << 16);
    }
  }
  std::vector<uint8_t> pal_bytes(palette.size() * 4);
  for (size_t i = 0; i < palette.size(); ++i)
    for (int k = 0; k < 4; ++k) pal_bytes[4 * i + k] = static_cast<uint8_t>(palette[i] >> (8 * k));
  pal_bytes.resize((pal_bytes.size() + kSymsPerGroup - 1) / kSymsPerGroup * kSymsPerGroup, 0);
  std::vector<uint8_t> sec[4];
  if (encode_section(ybuf.data(), ybuf.size(), &sec[0], nthreads) ||
      encode_section(cbuf.data(), cbuf.size(), &sec[1], nthreads) ||
      encode_section(pal_bytes.data(), pal_bytes.size(), &sec[2], nthreads) ||
      encode_section(index_deltas.data(), index_deltas.size(), &sec[3], nthreads))
    return 3;
  uint32_t hdr[7] = {w, h, static_cast<uint32_t>(pal_bytes.size()), static_cast<uint32_t>(sec[0].size() - 512),
                     static_cast<uint32_t>(sec[1].size() - 512), static_cast<uint32_t>(sec[2].size() - 512),
                     static_cast<uint32_t>(sec[3].size() - 512)};
  size_t total = 28;
  for (auto &s : sec) total += s.size();
  uint8_t *buf = static_cast<uint8_t *>(malloc(total));
  if (!buf) return 4;
  for (int i = 0; i < 7; ++i)
    for (int k = 0; k < 4; ++k) buf[4 * i + k] = static_cast<uint8_t>(hdr[i] >> (8 * k));
  size_t pos = 28;
  for (auto &s : sec) {
    memcpy(buf + pos, s.data(), 512);
    pos += 512;
  }
  for (auto &s : sec) {
    memcpy(buf + pos, s.data() + 512, s.size() - 512);
    pos += s.size() - 512;
  }
  *out = buf;
  *out_len = total;
  return 0;
}

bool dims_ok(uint32_t w, uint32_t h) {
  return w && h && w % 128 == 0 && h % 128 == 0 && (uint64_t(w) * h) % (16u * 256u * 32u) == 0 &&
         uint64_t(w) * h / 16 < (1u << 28);
}

// Index palette (this project's own search, after the idea of
// codec/dxt_image.cpp:510-624): each block may reuse one of the last 127
// palette words if its error grows by less than 35; the block keeps its own
// endpoints.  Returns palette words and +128 index deltas; rewrites `blocks`.
void build_palette(const uint8_t *rgb, uint32_t w, uint32_t h, std::vector<uint64_t> *blocks,
                   std::vector<uint32_t> *palette, std::vector<uint8_t> *deltas) {
  const uint32_t bx = w / 4, by = h / 4;
  int last = 0;
  deltas->resize(size_t(bx) * by);
  for (uint32_t j = 0; j < by; ++j) {
    for (uint32_t i = 0; i < bx; ++i) {
      const size_t bi = size_t(j) * bx + i;
      uint64_t &blk = (*blocks)[bi];
      int this_index;
      if (rgb) {
        uint8_t px[48];
        block_pixels(rgb, w, i, j, px);
        Rgb8 p[4];
        const uint16_t c0 = static_cast<uint16_t>(blk), c1 = static_cast<uint16_t>(blk >> 16);
        palette4(c0, c1, p);
        if (c0 <= c1) p[3] = {0, 0, 0};  // three-colour mode palette (codec/dxt_image.cpp:186-193)
        if (c0 <= c1) p[2] = {(p[0].r + p[1].r) / 2, (p[0].g + p[1].g) / 2, (p[0].b + p[1].b) / 2};
        int d[16][4];
        for (int q = 0; q < 16; ++q)
          for (int k = 0; k < 4; ++k) d[q][k] = dist2(p[k], px + 3 * q);
        const int own = block_error_from_dists(d, uint32_t(blk >> 32));
        int best = 1 << 30;
        size_t best_j = 0;
        const size_t look = std::min<size_t>(kPaletteLookback, palette->size());
        for (size_t k = 0; k < look; ++k) {
          const uint32_t word = (*palette)[palette->size() - 1 - k];
          const int diff = block_error_from_dists(d, word) - own;
          if (diff < best) {
            best = diff;
            best_j = k;
            if (diff <= 0) break;
          }
        }
        if (best < kReuseThreshold) {
          const uint32_t word = (*palette)[palette->size() - 1 - best_j];
          blk = (blk & 0xFFFFFFFFull) | (uint64_t(word) << 32);
          this_index = static_cast<int>(palette->size() - 1 - best_j);
        } else {
          this_index = static_cast<int>(palette->size());
          palette->push_back(uint32_t(blk >> 32));
        }
      } else {
        // No source pixels: reuse only exact matches among the last 127 words.
        const uint32_t word = uint32_t(blk >> 32);
        const size_t look = std::min<size_t>(kPaletteLookback, palette->size());
        size_t k = 0;
        for (; k < look; ++k)
          if ((*palette)[palette->size() - 1 - k] == word) break;
        if (k < look) this_index = static_cast<int>(palette->size() - 1 - k);
        else {
          this_index = static_cast<int>(palette->size());
          palette->push_back(word);
        }
      }
      (*deltas)[bi] = static_cast<uint8_t>(this_index - last + 128);
      last = this_index;
    }
  }
}

int encode_blocks(uint32_t w, uint32_t h, const uint8_t *rgb, std::vector<uint64_t> &blocks,
                  uint8_t **out, size_t *out_len, uint8_t *blocks_out, uint64_t *clips, int nthreads) {
  std::vector<uint32_t> palette;
  std::vector<uint8_t> deltas;
  build_palette(rgb, w, h, &blocks, &palette, &deltas);
  const int rc = write_stream(w, h, blocks, palette, deltas, out, out_len, clips, nthreads);
  if (rc == 0 && blocks_out) memcpy(blocks_out, blocks.data(), blocks.size() * 8);
  return rc;
}

}  // namespace

extern "C" int gst_encode_rgb(uint32_t w, uint32_t h, const uint8_t *rgb, uint8_t **out, size_t *out_len,
                              uint8_t *blocks_out, uint64_t *clips, int nthreads) {
  if (!rgb || !out || !out_len || !dims_ok(w, h)) return 1;
  const uint32_t bx = w / 4, by = h / 4;
  std::vector<uint64_t> blocks(size_t(bx) * by);
  parallel_for(by, nthreads, [&](uint32_t lo, uint32_t hi) {
    uint8_t px[48];
    for (uint32_t j = lo; j < hi; ++j)
      for (uint32_t i = 0; i < bx; ++i) {
        block_pixels(rgb, w, i, j, px);
        blocks[size_t(j) * bx + i] = compress_block(px);
      }
  });
  return encode_blocks(w, h, rgb, blocks, out, out_len, blocks_out, clips, nthreads);
}

extern "C" int gst_compress_blocks(uint32_t w, uint32_t h, const uint8_t *rgb, uint8_t *blocks_out, int nthreads) {
  if (!rgb || !blocks_out || !w || !h || (w & 3) || (h & 3)) return 1;
  const uint32_t bx = w / 4, by = h / 4;
  uint64_t *blocks = reinterpret_cast<uint64_t *>(blocks_out);
  parallel_for(by, nthreads, [&](uint32_t lo, uint32_t hi) {
    uint8_t px[48];
    for (uint32_t j = lo; j < hi; ++j)
      for (uint32_t i = 0; i < bx; ++i) {
        block_pixels(rgb, w, i, j, px);
        blocks[size_t(j) * bx + i] = compress_block(px);
      }
  });
  return 0;
}

extern "C" int gst_encode_dxt(uint32_t w, uint32_t h, const uint8_t *rgb, const uint8_t *dxt, uint8_t **out,
                              size_t *out_len, uint8_t *blocks_out, uint64_t *clips) {
  if (!dxt || !out || !out_len || !dims_ok(w, h)) return 1;
  std::vector<uint64_t> blocks(size_t(w / 4) * (h / 4));
  memcpy(blocks.data(), dxt, blocks.size() * 8);
  return encode_blocks(w, h, rgb, blocks, out, out_len, blocks_out, clips, 1);
}

extern "C" int gst_encode_section(const uint8_t *in, size_t n, uint8_t **out, size_t *out_len, int nthreads) {
  if (!in || !out || !out_len) return 1;
  std::vector<uint8_t> r;
  if (encode_section(in, n, &r, nthreads)) return 2;
  uint8_t *buf = static_cast<uint8_t *>(malloc(r.size()));
  if (!buf) return 4;
  memcpy(buf, r.data(), r.size());
  *out = buf;
  *out_len = r.size();
  return 0;
}

extern "C" int gst_normalize_frequencies(const uint32_t *counts, size_t n, int M, uint32_t *out) {
  if (!counts || !out || M <= 0) return 1;
  std::vector<uint32_t> c(counts, counts + n);
  std::vector<uint32_t> h = normalize_counts(c, M);
  memcpy(out, h.data(), n * sizeof(uint32_t));
  return 0;
}

extern "C" void gst_encoder_free(void *p) { free(p); }
