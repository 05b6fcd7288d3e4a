/*
 * gst_oracle.c -- CPU oracle for the GST decode path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's OpenCL decoder (GammaUNC/GST).  It
 * is the checker for the CUDA path and the timed CPU baseline; the product
 * never links it.  Every function follows the reference lines named beside it,
 * with the reference's integer semantics: uint32 state arithmetic, int32
 * wavelet intermediates, C truncating division, char stores, ushort packing.
 */
#include "gst_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static uint32_t rd32(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static uint16_t rd16(const uint8_t *p) { return (uint16_t)(p[0] | (p[1] << 8)); }
static void wr16(uint8_t *p, uint16_t v) {
  p[0] = (uint8_t)v;
  p[1] = (uint8_t)(v >> 8);
}
static void wr32(uint8_t *p, uint32_t v) {
  p[0] = (uint8_t)v;
  p[1] = (uint8_t)(v >> 8);
  p[2] = (uint8_t)(v >> 16);
  p[3] = (uint8_t)(v >> 24);
}
static int popc32(uint32_t x) { return __builtin_popcount(x); }

/* ------------------------------------------------------------------------- */
/* Stream geometry: codec/decoder.cpp:430-461 (offsets), codec/encoder.cpp:122-144
 * (header, four 512-byte frequency tables, then the sections Y, chroma,
 * palette, indices), codec/entropy.cpp:174-265 (section body: u32 group end
 * offsets, then groups). */
typedef struct {
  uint32_t in_off;  /* byte offset of the section body from the end of the freq tables */
  uint32_t in_len;  /* section body bytes (header *_sz field) */
  uint32_t nsyms;   /* decoded symbols */
  uint32_t ngroups; /* nsyms / 8192 */
  uint32_t out_off; /* offset in the decompressed-symbol buffer */
} gsto_section;

static void section_layout(const gsto_header *h, gsto_section s[4]) {
  const uint32_t B = (h->width / 4) * (h->height / 4);
  const uint32_t lens[4] = {h->y_cmp_sz, h->chroma_cmp_sz, h->palette_sz, h->indices_sz};
  const uint32_t syms[4] = {2 * B, 4 * B, h->palette_bytes, B};
  uint32_t in = 0, out = 0;
  for (int i = 0; i < 4; ++i) {
    s[i].in_off = in;
    s[i].in_len = lens[i];
    s[i].nsyms = syms[i];
    s[i].ngroups = syms[i] / GSTO_SYMS_PER_GROUP;
    s[i].out_off = out;
    in += lens[i];
    out += syms[i];
  }
}

int gsto_parse_header(const uint8_t *gst, size_t n, gsto_header *hdr) {
  if (!gst || !hdr) return GSTO_E_ARG;
  if (n < GSTO_HEADER_BYTES + 4 * GSTO_FREQ_BYTES) return GSTO_E_FORMAT;
  uint32_t w[7];
  for (int i = 0; i < 7; ++i) w[i] = rd32(gst + 4 * i);
  hdr->width = w[0];
  hdr->height = w[1];
  hdr->palette_bytes = w[2];
  hdr->y_cmp_sz = w[3];
  hdr->chroma_cmp_sz = w[4];
  hdr->palette_sz = w[5];
  hdr->indices_sz = w[6];
  /* README.md:67-71 dimension rules; blocks < 2^28 keeps every offset in u32. */
  if (hdr->width == 0 || hdr->height == 0) return GSTO_E_FORMAT;
  if (hdr->width % 128 || hdr->height % 128) return GSTO_E_FORMAT;
  const uint64_t px = (uint64_t)hdr->width * hdr->height;
  if (px % (16u * 256u * 32u)) return GSTO_E_FORMAT;
  const uint64_t B = px / 16;
  if (B >= (1u << 28)) return GSTO_E_FORMAT;
  if (hdr->palette_bytes == 0 || hdr->palette_bytes % GSTO_SYMS_PER_GROUP) return GSTO_E_FORMAT;
  if (7 * B + hdr->palette_bytes >= (1ull << 32)) return GSTO_E_FORMAT;
  gsto_section s[4];
  section_layout(hdr, s);
  uint64_t total = GSTO_HEADER_BYTES + 4 * GSTO_FREQ_BYTES;
  for (int i = 0; i < 4; ++i) total += s[i].in_len;
  if (total > n) return GSTO_E_FORMAT;
  const uint8_t *freqs = gst + GSTO_HEADER_BYTES;
  const uint8_t *body = freqs + 4 * GSTO_FREQ_BYTES;
  for (int i = 0; i < 4; ++i) {
    uint32_t sum = 0;
    for (int k = 0; k < 256; ++k) sum += rd16(freqs + i * GSTO_FREQ_BYTES + 2 * k);
    if (sum != GSTO_TABLE_SIZE) return GSTO_E_FORMAT;
    const uint32_t G = s[i].ngroups;
    if (s[i].in_len % 4) return GSTO_E_FORMAT;
    if ((uint64_t)G * 4 + (uint64_t)G * 128 > s[i].in_len) return GSTO_E_FORMAT;
    const uint8_t *sec = body + s[i].in_off;
    uint32_t prev = 4 * G;
    for (uint32_t g = 0; g < G; ++g) {
      const uint32_t e = rd32(sec + 4 * g);
      if (e % 4 || e < prev + 4 * GSTO_STREAMS_PER_GROUP || e > s[i].in_len) return GSTO_E_FORMAT;
      prev = e;
    }
  }
  return GSTO_OK;
}

/* ------------------------------------------------------------------------- */
/* build_table.cl:12-83 */
static void blelloch_exclusive_u16(uint16_t c[256]) {
  uint32_t offset = 1;
  for (uint32_t d = 256 >> 1; d > 0; d >>= 1) { /* :29-37 */
    for (uint32_t lid = 0; lid < d; ++lid) {
      const uint32_t ai = offset * (2 * lid + 1) - 1, bi = offset * (2 * lid + 2) - 1;
      c[bi] = (uint16_t)(c[bi] + c[ai]);
    }
    offset *= 2;
  }
  c[255] = 0; /* :39-41 */
  for (uint32_t d = 1; d < 256; d *= 2) { /* :43-54 */
    offset >>= 1;
    for (uint32_t lid = 0; lid < d; ++lid) {
      const uint32_t ai = offset * (2 * lid + 1) - 1, bi = offset * (2 * lid + 2) - 1;
      const uint32_t t = c[ai];
      c[ai] = c[bi];
      c[bi] = (uint16_t)(c[bi] + t);
    }
  }
}

void gsto_build_table(const uint16_t freqs[256], uint16_t freq[2048], uint16_t cum[2048],
                      uint8_t sym[2048]) {
  uint16_t c[256];
  memcpy(c, freqs, sizeof(c));
  blelloch_exclusive_u16(c);
  for (uint32_t id = 0; id < GSTO_TABLE_SIZE; ++id) { /* :61-75, the kernel's 11-step search */
    uint32_t low = 0, high = 255, x = (high + low) / 2;
    for (int i = 0; i < GSTO_TABLE_LOG; ++i) {
      const uint32_t too_high = (uint32_t)(id < c[x & 255]);
      const uint32_t too_low = (uint32_t)(x < 255 && c[(x + 1) & 255] <= id);
      const uint32_t lo1 = (low + 1 > x) ? low + 1 : x;
      const uint32_t hi1 = (high - 1 < x) ? high - 1 : x;
      low = too_low * lo1 + (1 - too_low) * low;
      high = too_high * hi1 + (1 - too_high) * high;
      x = (high + low) / 2;
    }
    x &= 255;
    freq[id] = freqs[x]; /* :78-82 */
    cum[id] = c[x];
    sym[id] = (uint8_t)x;
  }
}

void gsto_build_table_direct(const uint16_t freqs[256], uint16_t freq[2048], uint16_t cum[2048],
                             uint8_t sym[2048]) {
  uint32_t c = 0;
  for (uint32_t x = 0; x < 256; ++x) {
    for (uint32_t k = 0; k < freqs[x] && c + k < GSTO_TABLE_SIZE; ++k) {
      freq[c + k] = freqs[x];
      cum[c + k] = (uint16_t)c;
      sym[c + k] = (uint8_t)x;
    }
    c += freqs[x];
  }
}

/* ------------------------------------------------------------------------- */
/* ans_decode.cl:25-74 (ans_decode_single); constants :3-8. */
int gsto_rans_decode_group(const uint8_t *data, size_t data_len, uint32_t group,
                           const uint16_t freq[2048], const uint16_t cum[2048],
                           const uint8_t sym[2048], int num_streams, size_t lo_bytes,
                           uint8_t *out) {
  if (num_streams < 1 || num_streams > 32) return GSTO_E_ARG;
  if ((size_t)group * 4 + 4 > data_len) return GSTO_E_FORMAT;
  int status = GSTO_OK;
  const uint32_t offset = rd32(data + 4 * group); /* :113 */
  const uint32_t ns = (uint32_t)num_streams;
  if (offset < 4 * ns || offset > data_len) return GSTO_E_FORMAT;
  uint32_t st[32];
  for (uint32_t l = 0; l < ns; ++l) st[l] = rd32(data + offset - 4 * ns + 4 * l); /* :114 */
  uint32_t next = (offset - ns * 4) / 2;                                       /* :115 */
  for (int i = 0; i < GSTO_SYMS_PER_STREAM; ++i) {
    uint32_t mask = 0;
    uint8_t s_out[32];
    for (uint32_t l = 0; l < ns; ++l) { /* :121-129 */
      const uint32_t slot = st[l] & (GSTO_TABLE_SIZE - 1);
      st[l] = (st[l] >> GSTO_TABLE_LOG) * freq[slot] - cum[slot] + slot;
      s_out[l] = sym[slot];
      mask |= (uint32_t)(st[l] < GSTO_RANS_L) << l;
    }
    const uint32_t total = (uint32_t)popc32(mask); /* :134 */
    for (uint32_t l = 0; l < ns; ++l) {            /* :135-140 */
      if (!((mask >> l) & 1)) continue;
      const uint32_t rank = (uint32_t)popc32(mask & ((1u << l) - 1));
      const uint32_t idx = next - total + rank;
      uint16_t v = 0;
      /* Reads stay inside the group's word region [lo_bytes, offset - 4*ns);
       * a valid stream never leaves it. */
      if ((uint64_t)idx * 2 < lo_bytes || (uint64_t)idx * 2 + 2 > (uint64_t)offset - 4 * ns) {
        status = GSTO_E_FORMAT;
      } else {
        v = rd16(data + 2 * (size_t)idx);
      }
      st[l] = (st[l] << 16) | v;
    }
    next -= total; /* :148 */
    for (uint32_t l = 0; l < ns; ++l) out[l * GSTO_SYMS_PER_STREAM + GSTO_SYMS_PER_STREAM - 1 - i] = s_out[l];
  }
  return status;
}

/* ------------------------------------------------------------------------- */
/* inverse_wavelet.cl:14-64 (NormalizeIndex, InverseWaveletEven/Odd) */
static int normalize_index(int idx, int range) {
  const int v = idx - (int)(idx >= range) * (idx - range + 2);
  return v < 0 ? -v : v;
}

/* One level (len = dim): the row pass then the column pass, as the kernel's
 * two transposing half-passes do (:117-172). */
void gsto_inverse_wavelet_level(int32_t *blk, int stride, int dim) {
  const int mid = dim / 2;
  int32_t src[32], dst[32];
  for (int pass = 0; pass < 2; ++pass) {
    for (int line = 0; line < dim; ++line) {
      for (int k = 0; k < dim; ++k) src[k] = pass == 0 ? blk[line * stride + k] : blk[k * stride + line];
      for (int x = 0; x < mid; ++x) { /* Even */
        const int prev = mid + normalize_index(2 * x - 1, dim) / 2;
        const int next = mid + normalize_index(2 * x + 1, dim) / 2;
        dst[2 * x] = src[x] - (src[prev] + src[next] + 2) / 4;
      }
      for (int x = 0; x < mid; ++x) { /* Odd */
        const int prev = normalize_index(2 * x, dim);
        const int next = normalize_index(2 * x + 2, dim);
        dst[2 * x + 1] = src[mid + x] + (dst[prev] + dst[next]) / 2;
      }
      for (int k = 0; k < dim; ++k) {
        if (pass == 0) blk[line * stride + k] = dst[k];
        else blk[k * stride + line] = dst[k];
      }
    }
  }
}

void gsto_inverse_wavelet_block(const uint8_t *in, int8_t *out) {
  int32_t b[1024];
  for (int i = 0; i < 1024; ++i) b[i] = (int32_t)in[i] - 128; /* :93-104 */
  for (int len = 2; len <= 32; len *= 2) gsto_inverse_wavelet_level(b, 32, len);
  for (int i = 0; i < 1024; ++i) out[i] = (int8_t)(uint8_t)((uint32_t)b[i] & 0xFF); /* :188-190 */
}

/* ------------------------------------------------------------------------- */
/* decode_indices.cl:6-84 driven by decoder.cpp:302-393. */
static void local_scan128(uint32_t s[128], uint32_t lsize) {
  uint32_t offset = 1; /* :225-236 */
  for (uint32_t i = 128 >> 1; i > 0; i >>= 1) {
    for (uint32_t tid = 0; tid < i && tid < lsize; ++tid) {
      const uint32_t a = offset * (2 * tid + 1) - 1, b = offset * (2 * tid + 2) - 1;
      s[b] += s[a];
    }
    offset *= 2;
  }
  offset >>= 1; /* :238-248 */
  for (uint32_t d = 2; d < 128; d *= 2) {
    offset >>= 1;
    for (uint32_t tid = 1; tid < d && tid < lsize; ++tid) {
      if (offset == 0) continue;
      const uint32_t a = offset * (2 * tid) - 1, b = offset * (2 * tid + 1) - 1;
      s[b] += s[a];
    }
  }
}

static void scan_reference(const uint8_t *deltas, uint32_t n, int32_t *out_i) {
  uint32_t *out = (uint32_t *)out_i;
  int stage = -1;
  for (;;) { /* decoder.cpp:311-356 */
    stage++;
    const uint32_t num = n >> (stage * 7);
    if (num == 0) break;
    const uint32_t gsize = num < 128 ? num : ((num + 127) / 128) * 128;
    const uint32_t lsize = num < 128 ? num : 128;
    const uint32_t idx_offset = 1u << (stage * 7);
    /* Work-groups run one after another in id order (one legal interleaving;
     * for the sizes where the kernel's writes alias, decode_indices.cl:58-63
     * gives no ordering guarantee). */
    for (uint32_t g0 = 0; g0 < gsize; g0 += lsize) {
      uint32_t s[128];
      for (uint32_t k = 0; k < 128; ++k) s[k] = 0xA5A5A5A5u; /* local memory not written by the kernel */
      for (uint32_t lid = 0; lid < lsize; ++lid) {
        const uint32_t gid = g0 + lid;
        const uint32_t gidx = idx_offset * (gid + 1) - 1, pgidx = idx_offset * gid - 1;
        if (stage == 0) s[lid] = (uint32_t)((int32_t)deltas[gid] - 128);
        else if (gidx < n) s[lid] = out[gidx];
        else if (pgidx < n) s[lid] = out[n - 1];
        else s[lid] = 0;
      }
      local_scan128(s, lsize);
      for (uint32_t lid = 0; lid < lsize; ++lid) {
        const uint32_t gid = g0 + lid;
        const uint32_t gidx = idx_offset * (gid + 1) - 1, pgidx = idx_offset * gid - 1;
        if (stage == 0 || gidx < n) out[gidx] = s[lid];
        else if (pgidx < n && gidx >= n) out[n - 1] = s[lid];
      }
    }
  }
  while (stage > 0) { /* decoder.cpp:358-393, collect_indices :66-84 */
    const int sh = (stage - 1) * 7;
    const uint32_t num = n >> (sh > 0 ? sh : 0);
    const uint32_t gsize = ((num + 127) / 128) * 128;
    const uint32_t offset = 1u << (stage * 7), next_offset = 1u << ((stage - 1) * 7);
    for (uint32_t gid = 0; gid < gsize; ++gid) {
      const uint32_t group = gid / 128, lid = gid % 128;
      const uint32_t gidx = offset * group - 1, tidx = next_offset * (gid + 1) - 1;
      if (tidx < n - 1 && gidx < n - 1 && group > 0 && lid != 127) out[tidx] += out[gidx];
    }
    stage--;
  }
}

void gsto_scan_indices(const uint8_t *deltas, uint32_t n, int32_t *out, int mode) {
  if (n == 0) return;
  if (mode == GSTO_SCAN_REFERENCE && n % 128 == 0) {
    scan_reference(deltas, n, out);
    return;
  }
  uint32_t acc = 0;
  for (uint32_t i = 0; i < n; ++i) {
    acc += (uint32_t)((int32_t)deltas[i] - 128);
    out[i] = (int32_t)acc;
  }
}

/* ------------------------------------------------------------------------- */
/* assemble.cl:39-62 */
uint16_t gsto_ycocg_to_565(int y, int co, int cg) {
  const int t = y - (cg / 2);
  const int g = cg + t;
  const int b = (t - co) / 2;
  const int r = b + co;
  const uint32_t p = ((uint32_t)r << 11) | ((uint32_t)g << 5) | (uint32_t)b;
  return (uint16_t)p;
}

/* ------------------------------------------------------------------------- */
/* Parallel-for over [0, count) with a static split (pthreads). */
typedef void (*range_fn)(void *ctx, uint32_t lo, uint32_t hi, int *status);
typedef struct {
  range_fn fn;
  void *ctx;
  uint32_t lo, hi;
  int status;
} pf_job;

static void *pf_thread(void *arg) {
  pf_job *j = (pf_job *)arg;
  j->fn(j->ctx, j->lo, j->hi, &j->status);
  return NULL;
}

static int parallel_for(uint32_t count, int nthreads, range_fn fn, void *ctx) {
  if (nthreads < 1) nthreads = 1;
  if ((uint32_t)nthreads > count) nthreads = count ? (int)count : 1;
  if (nthreads == 1) {
    int st = GSTO_OK;
    fn(ctx, 0, count, &st);
    return st;
  }
  pthread_t th[256];
  pf_job jobs[256];
  if (nthreads > 256) nthreads = 256;
  for (int t = 0; t < nthreads; ++t) {
    jobs[t].fn = fn;
    jobs[t].ctx = ctx;
    jobs[t].lo = (uint32_t)((uint64_t)count * t / nthreads);
    jobs[t].hi = (uint32_t)((uint64_t)count * (t + 1) / nthreads);
    jobs[t].status = GSTO_OK;
    pthread_create(&th[t], NULL, pf_thread, &jobs[t]);
  }
  int st = GSTO_OK;
  for (int t = 0; t < nthreads; ++t) {
    pthread_join(th[t], NULL);
    if (jobs[t].status != GSTO_OK) st = jobs[t].status;
  }
  return st;
}

typedef struct {
  const uint8_t *gst;
  gsto_header hdr;
  gsto_section sec[4];
  uint16_t freq[4][2048], cum[4][2048];
  uint8_t sym[4][2048];
  uint32_t group_base[5]; /* first flat group id per section */
  uint8_t *symbols;       /* 7B + palette_bytes */
  int8_t *planes;         /* 6 x B raster */
  int32_t *indices;       /* B */
  uint8_t *dxt;
  uint8_t *rgb; /* when set, assemble_rgb output (W*H*3) instead of DXT1 */
  uint32_t B, bx, by;
} decode_ctx;

static void rans_range(void *vctx, uint32_t lo, uint32_t hi, int *status) {
  decode_ctx *c = (decode_ctx *)vctx;
  const uint8_t *body = c->gst + GSTO_HEADER_BYTES + 4 * GSTO_FREQ_BYTES;
  for (uint32_t fg = lo; fg < hi; ++fg) {
    int s = 0;
    while (fg >= c->group_base[s + 1]) ++s;
    const uint32_t g = fg - c->group_base[s];
    const uint8_t *sec = body + c->sec[s].in_off;
    const size_t lo_bytes = g == 0 ? 4u * c->sec[s].ngroups : rd32(sec + 4 * (g - 1));
    const int st = gsto_rans_decode_group(sec, c->sec[s].in_len, g, c->freq[s], c->cum[s], c->sym[s],
                                          GSTO_STREAMS_PER_GROUP, lo_bytes,
                                          c->symbols + c->sec[s].out_off + (size_t)g * GSTO_SYMS_PER_GROUP);
    if (st != GSTO_OK) *status = st;
  }
}

/* inverse_wavelet.cl:69-192 over all planes and 32x32 tiles; the block of tile
 * (tx, ty) is the (ty * tiles_x + tx)-th 1024-byte run of the plane (:94-95)
 * and lands at rows ty*32.., columns tx*32.. of the raster plane (:175-191). */
static void wavelet_range(void *vctx, uint32_t lo, uint32_t hi, int *status) {
  (void)status;
  decode_ctx *c = (decode_ctx *)vctx;
  const uint32_t tiles_x = c->bx / 32, tiles = (c->bx / 32) * (c->by / 32);
  int8_t blk[1024];
  for (uint32_t item = lo; item < hi; ++item) {
    const uint32_t p = item / tiles, t = item % tiles;
    const uint32_t tx = t % tiles_x, ty = t / tiles_x;
    gsto_inverse_wavelet_block(c->symbols + (size_t)p * c->B + (size_t)t * 1024, blk);
    int8_t *plane = c->planes + (size_t)p * c->B;
    for (uint32_t r = 0; r < 32; ++r)
      memcpy(plane + (size_t)(ty * 32 + r) * c->bx + tx * 32, blk + r * 32, 32);
  }
}

/* assemble.cl:64-81 (assemble_dxt), rows [lo, hi) of blocks. */
static void assemble_range(void *vctx, uint32_t lo, uint32_t hi, int *status) {
  decode_ctx *c = (decode_ctx *)vctx;
  const uint8_t *palette = c->symbols + c->sec[2].out_off;
  const uint32_t nwords = c->hdr.palette_bytes / 4;
  const int8_t *Y1 = c->planes, *Y2 = c->planes + c->B, *Co1 = c->planes + 2 * (size_t)c->B,
               *Cg1 = c->planes + 3 * (size_t)c->B, *Co2 = c->planes + 4 * (size_t)c->B,
               *Cg2 = c->planes + 5 * (size_t)c->B;
  for (uint32_t i = lo * c->bx; i < hi * c->bx; ++i) {
    const uint16_t ep1 = gsto_ycocg_to_565(Y1[i], Co1[i], Cg1[i]);
    const uint16_t ep2 = gsto_ycocg_to_565(Y2[i], Co2[i], Cg2[i]);
    const uint32_t idx = (uint32_t)c->indices[i];
    uint32_t word = 0;
    if (idx < nwords) word = rd32(palette + 4 * (size_t)idx);
    else *status = GSTO_E_FORMAT;
    wr16(c->dxt + 8 * (size_t)i, ep1);
    wr16(c->dxt + 8 * (size_t)i + 2, ep2);
    wr32(c->dxt + 8 * (size_t)i + 4, word);
  }
}

/* assemble.cl:39-45 (YCoCgToRGB) and :83-129 (assemble_rgb), rows [lo, hi)
 * of blocks: the two endpoints to 5:6:5 integers, widened to 8 bits by bit
 * replication, two interpolated colours (2a + b) / 3 and (a + 2b) / 3 in C
 * integer division (four-colour mode only), and each pixel's 2-bit selector
 * from the palette word, low bits first in raster order within the block.
 * Every channel is stored as its low 8 bits. */
static void ycocg_to_rgb(int y, int co, int cg, int rgb[3]) {
  const int t = y - (cg / 2);
  const int g = cg + t;
  const int b = (t - co) / 2;
  const int r = b + co;
  rgb[0] = (int)((uint32_t)r << 3) | (r >> 2);
  rgb[1] = (int)((uint32_t)g << 2) | (g >> 4);
  rgb[2] = (int)((uint32_t)b << 3) | (b >> 2);
}

static void assemble_rgb_range(void *vctx, uint32_t lo, uint32_t hi, int *status) {
  decode_ctx *c = (decode_ctx *)vctx;
  const uint8_t *palette = c->symbols + c->sec[2].out_off;
  const uint32_t nwords = c->hdr.palette_bytes / 4;
  const size_t B = c->B;
  const int8_t *P = c->planes;
  const size_t W = c->hdr.width;
  for (uint32_t by = lo; by < hi; ++by) {
    for (uint32_t bx = 0; bx < c->bx; ++bx) {
      const size_t i = (size_t)by * c->bx + bx;
      int pal[4][3];
      ycocg_to_rgb(P[i], P[2 * B + i], P[3 * B + i], pal[0]);
      ycocg_to_rgb(P[B + i], P[4 * B + i], P[5 * B + i], pal[1]);
      for (int k = 0; k < 3; ++k) {
        pal[2][k] = (2 * pal[0][k] + pal[1][k]) / 3;
        pal[3][k] = (pal[0][k] + 2 * pal[1][k]) / 3;
      }
      const uint32_t idx = (uint32_t)c->indices[i];
      uint32_t word = 0;
      if (idx < nwords) word = rd32(palette + 4 * (size_t)idx);
      else *status = GSTO_E_FORMAT;
      for (int p = 0; p < 16; ++p) {
        const int *col = pal[word & 3];
        const size_t x = 4 * (size_t)bx + (p % 4), y = 4 * (size_t)by + (p / 4);
        uint8_t *o = c->rgb + 3 * (W * y + x);
        o[0] = (uint8_t)col[0];
        o[1] = (uint8_t)col[1];
        o[2] = (uint8_t)col[2];
        word >>= 2;
      }
    }
  }
}

static int setup_ctx(decode_ctx *c, const uint8_t *gst, size_t n) {
  int st = gsto_parse_header(gst, n, &c->hdr);
  if (st != GSTO_OK) return st;
  c->gst = gst;
  section_layout(&c->hdr, c->sec);
  c->bx = c->hdr.width / 4;
  c->by = c->hdr.height / 4;
  c->B = c->bx * c->by;
  c->group_base[0] = 0;
  for (int s = 0; s < 4; ++s) {
    uint16_t f[256];
    for (int k = 0; k < 256; ++k) f[k] = rd16(gst + GSTO_HEADER_BYTES + s * GSTO_FREQ_BYTES + 2 * k);
    gsto_build_table(f, c->freq[s], c->cum[s], c->sym[s]);
    c->group_base[s + 1] = c->group_base[s] + c->sec[s].ngroups;
  }
  return GSTO_OK;
}

int gsto_decode_symbols(const uint8_t *gst, size_t n, uint8_t *symbols, size_t cap, int nthreads) {
  decode_ctx *c = (decode_ctx *)calloc(1, sizeof(decode_ctx));
  if (!c) return GSTO_E_ARG;
  int st = setup_ctx(c, gst, n);
  if (st == GSTO_OK) {
    const size_t need = 7 * (size_t)c->B + c->hdr.palette_bytes;
    if (!symbols || cap < need) st = GSTO_E_ARG;
    else {
      c->symbols = symbols;
      st = parallel_for(c->group_base[4], nthreads, rans_range, c);
    }
  }
  free(c);
  return st;
}

static int decode_image(const uint8_t *gst, size_t n, uint8_t *out, size_t out_cap, int scan_mode, int nthreads,
                        int rgb) {
  decode_ctx *c = (decode_ctx *)calloc(1, sizeof(decode_ctx));
  if (!c) return GSTO_E_ARG;
  int st = setup_ctx(c, gst, n);
  if (st != GSTO_OK) {
    free(c);
    return st;
  }
  if (!out || out_cap < (rgb ? 48 : 8) * (size_t)c->B) {
    free(c);
    return GSTO_E_ARG;
  }
  if (rgb) c->rgb = out;
  else c->dxt = out;
  c->symbols = (uint8_t *)malloc(7 * (size_t)c->B + c->hdr.palette_bytes);
  c->planes = (int8_t *)malloc(6 * (size_t)c->B);
  c->indices = (int32_t *)malloc(4 * (size_t)c->B);
  if (!c->symbols || !c->planes || !c->indices) {
    st = GSTO_E_ARG;
  } else {
    int s1 = parallel_for(c->group_base[4], nthreads, rans_range, c);
    parallel_for(6 * (c->bx / 32) * (c->by / 32), nthreads, wavelet_range, c);
    gsto_scan_indices(c->symbols + c->sec[3].out_off, c->B, c->indices, scan_mode);
    int s2 = parallel_for(c->by, nthreads, rgb ? assemble_rgb_range : assemble_range, c);
    st = s1 != GSTO_OK ? s1 : s2;
  }
  free(c->symbols);
  free(c->planes);
  free(c->indices);
  free(c);
  return st;
}

int gsto_decode(const uint8_t *gst, size_t n, uint8_t *dxt_out, size_t out_cap, int scan_mode, int nthreads) {
  return decode_image(gst, n, dxt_out, out_cap, scan_mode, nthreads, 0);
}

int gsto_decode_rgb(const uint8_t *gst, size_t n, uint8_t *rgb_out, size_t out_cap, int scan_mode, int nthreads) {
  return decode_image(gst, n, rgb_out, out_cap, scan_mode, nthreads, 1);
}

int gsto_decode_batch(const uint8_t *const *gst, const size_t *lens, int n_streams,
                      uint8_t *dxt_out, size_t out_cap, int scan_mode, int nthreads) {
  size_t off = 0;
  int status = GSTO_OK;
  for (int i = 0; i < n_streams; ++i) {
    gsto_header h;
    int st = gsto_parse_header(gst[i], lens[i], &h);
    if (st != GSTO_OK) return st;
    const size_t sz = (size_t)h.width * h.height / 2;
    if (off + sz > out_cap) return GSTO_E_ARG;
    st = gsto_decode(gst[i], lens[i], dxt_out + off, sz, scan_mode, nthreads);
    if (st == GSTO_E_ARG) return st;
    if (st != GSTO_OK) status = st;
    off += sz;
  }
  return status;
}

/* ans_decode.cl:104-121 (the binary search of ans_decode_multiple) */
uint32_t gsto_section_search(const uint32_t *oo, uint32_t num_offsets, uint32_t wg) {
  const uint32_t id = wg * GSTO_STREAMS_PER_GROUP * GSTO_SYMS_PER_STREAM;
  uint32_t low = 0, high = num_offsets - 1, x = (high + low) / 2;
  const uint32_t iters = 32 - (uint32_t)__builtin_clz(high - low + 1);
  for (uint32_t i = 0; i < iters; ++i) {
    const uint32_t too_high = (uint32_t)(id < oo[x]);
    const uint32_t too_low = (uint32_t)(x < (num_offsets - 1) && oo[x + 1] <= id);
    const uint32_t lo1 = (low + 1 > x) ? low + 1 : x;
    const uint32_t hi1 = (high - 1 < x) ? high - 1 : x;
    low = too_low * lo1 + (1 - too_low) * low;
    high = too_high * hi1 + (1 - too_high) * high;
    x = (high + low) >> 1;
  }
  return x;
}

/* ========================================================================= */
/* Encoder stages.                                                           */

/* A candidate of the frequency correction: ans/histogram.cpp:10-19 (Symbol). */
typedef struct {
  int symbol;
  double rank;
} gsto_ranked;

/* The binary heap of the C++ library with comparator std::greater<Symbol>
 * (a min-heap on rank), as GCC's libstdc++ implements it (bits/stl_heap.h:
 * __push_heap, __adjust_heap, __make_heap, __pop_heap -- the SGI STL sift
 * procedure).  The tie order of ans/histogram.cpp:84-110 depends on it. */
static void heap_sift_up(gsto_ranked *h, long hole, long top, gsto_ranked v) {
  long parent = (hole - 1) / 2;
  while (hole > top && h[parent].rank > v.rank) {
    h[hole] = h[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  h[hole] = v;
}

static void heap_adjust(gsto_ranked *h, long hole, long len, gsto_ranked v) {
  const long top = hole;
  long child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (h[child].rank > h[child - 1].rank) child--; /* on equal ranks the right child moves up */
    h[hole] = h[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    h[hole] = h[child - 1];
    hole = child - 1;
  }
  heap_sift_up(h, hole, top, v);
}

static void heap_make(gsto_ranked *h, long len) {
  if (len < 2) return;
  for (long parent = (len - 2) / 2;; --parent) {
    heap_adjust(h, parent, len, h[parent]);
    if (parent == 0) return;
  }
}

/* Moves the minimum to h[len-1]; the heap keeps len-1 entries. */
static void heap_pop(gsto_ranked *h, long len) {
  if (len < 2) return;
  const gsto_ranked v = h[len - 1];
  h[len - 1] = h[0];
  heap_adjust(h, 0, len - 1, v);
}

/* h[len-1] joins the heap of len-1 entries. */
static void heap_push(gsto_ranked *h, long len) { heap_sift_up(h, len - 1, 0, h[len - 1]); }

/* ans/histogram.cpp:25-29 (GetFreqChange). */
static double freq_change(int count, int new_count, int sign) {
  return log2((double)new_count / (double)(new_count + sign)) * (double)count;
}

/* ans/histogram.cpp:40-121 */
int gsto_normalize(const uint32_t *counts, int n, int M, uint32_t *out) {
  if (M <= 0 || n < 0 || (n > 0 && (!counts || !out))) return GSTO_E_ARG;
  uint32_t usum = 0; /* fold_sum: std::accumulate in uint32, then int */
  for (int i = 0; i < n; ++i) usum += counts[i];
  const int sum = (int)usum;
  for (int i = 0; i < n; ++i) {
    if (counts[i] == 0) {
      out[i] = 0;
      continue;
    }
    const uint32_t scaled = counts[i] * (uint32_t)M; /* uint32 product, wraps as the reference's */
    const double from_scaled = (double)((float)scaled / (float)sum);
    const int down = (int)from_scaled;
    const int v = (from_scaled * from_scaled <= (double)(down * (down + 1))) ? down : down + 1;
    out[i] = (uint32_t)(v > 1 ? v : 1);
  }
  uint32_t hsum = 0;
  for (int i = 0; i < n; ++i) hsum += out[i];
  int correction = M - (int)hsum;
  if (correction == 0) return GSTO_OK;
  if (correction == M) return GSTO_E_ARG;
  const int sign = correction > 0 ? 1 : -1;
  gsto_ranked *h = (gsto_ranked *)malloc(sizeof(gsto_ranked) * (size_t)(n > 0 ? n : 1));
  if (!h) return GSTO_E_ARG;
  long len = 0;
  for (int i = 0; i < n; ++i) {
    if (counts[i] == 0) continue;
    if (out[i] > 1 || correction > 0) {
      h[len].symbol = i;
      h[len].rank = freq_change((int)counts[i], (int)out[i], sign);
      ++len;
    }
  }
  heap_make(h, len);
  int status = GSTO_OK;
  while (correction != 0) {
    if (len == 0) {
      status = GSTO_E_ARG;
      break;
    }
    heap_pop(h, len);
    const int i = h[--len].symbol;
    out[i] = (uint32_t)((int)out[i] + sign);
    correction -= sign;
    if (out[i] > 1 || sign == 1) {
      h[len].symbol = i;
      h[len].rank = freq_change((int)counts[i], (int)out[i], sign);
      heap_push(h, ++len);
    }
  }
  free(h);
  return status;
}

size_t gsto_encode_section_bound(size_t n) {
  const size_t G = n / GSTO_SYMS_PER_GROUP;
  /* at most one 16-bit word per symbol (the state drops below 2^15 after
   * one shift, ans/encode.cpp:62-66), a 2-byte pad and the 32 states */
  return GSTO_FREQ_BYTES + 4 * G + G * (2 * GSTO_SYMS_PER_GROUP + 2 + 4 * GSTO_STREAMS_PER_GROUP);
}

/* ans/encode.cpp:224-259 over one group (EncodeInterleaved with 32 encoders of
 * ans/encode.cpp:39-69), then codec/entropy.cpp:213-229's 4-byte alignment
 * (two zero bytes in front).  Returns the group's byte count. */
static size_t encode_group(const uint8_t *sym, const uint32_t F[256], const uint32_t C[256], uint8_t *out,
                           uint16_t *words) {
  uint32_t state[GSTO_STREAMS_PER_GROUP];
  for (int s = 0; s < GSTO_STREAMS_PER_GROUP; ++s) state[s] = GSTO_RANS_L; /* k * M */
  size_t nw = 0;
  for (int i = 0; i < GSTO_SYMS_PER_STREAM; ++i) {
    for (int s = 0; s < GSTO_STREAMS_PER_GROUP; ++s) {
      const uint32_t x = sym[s * GSTO_SYMS_PER_STREAM + i];
      uint32_t st = state[s];
      const uint32_t upper = (1u << 16) * 16u * F[x]; /* b * k * F */
      while (st >= upper) {
        words[nw++] = (uint16_t)(st & 0xFFFF);
        st >>= 16;
      }
      state[s] = (st / F[x]) * GSTO_TABLE_SIZE + C[x] + (st % F[x]);
    }
  }
  const size_t pad = (nw & 1) ? 2 : 0;
  uint8_t *p = out;
  if (pad) {
    p[0] = p[1] = 0;
    p += 2;
  }
  for (size_t k = 0; k < nw; ++k, p += 2) wr16(p, words[k]);
  for (int s = 0; s < GSTO_STREAMS_PER_GROUP; ++s, p += 4) wr32(p, state[s]);
  return (size_t)(p - out);
}

/* codec/entropy.cpp:174-265 */
int gsto_encode_section(const uint8_t *in, size_t n, uint8_t *out, size_t cap, size_t *out_len) {
  if (!in || !out || !out_len || n == 0 || n % GSTO_SYMS_PER_GROUP) return GSTO_E_ARG;
  if (n > 0xFFFFFFFFu || cap < gsto_encode_section_bound(n)) return GSTO_E_ARG;
  uint32_t counts[256] = {0};
  for (size_t i = 0; i < n; ++i) counts[in[i]]++;
  int nz = 0;
  for (int i = 0; i < 256; ++i)
    if (counts[i]) nz = i + 1;
  uint32_t F[256] = {0}, C[256] = {0};
  if (gsto_normalize(counts, nz, GSTO_TABLE_SIZE, F) != GSTO_OK) return GSTO_E_ARG;
  for (int i = 1; i < 256; ++i) C[i] = C[i - 1] + F[i - 1];
  const size_t G = n / GSTO_SYMS_PER_GROUP;
  for (int i = 0; i < 256; ++i) wr16(out + 2 * i, (uint16_t)F[i]);
  uint8_t *offs = out + GSTO_FREQ_BYTES;
  uint8_t *p = offs + 4 * G;
  uint16_t *words = (uint16_t *)malloc(sizeof(uint16_t) * GSTO_SYMS_PER_GROUP);
  if (!words) return GSTO_E_ARG;
  uint32_t cum = (uint32_t)(4 * G);
  for (size_t g = 0; g < G; ++g) {
    const size_t sz = encode_group(in + g * GSTO_SYMS_PER_GROUP, F, C, p, words);
    cum += (uint32_t)sz;
    wr32(offs + 4 * g, cum);
    p += sz;
  }
  free(words);
  *out_len = (size_t)(p - out); /* already a multiple of 4 (entropy.cpp:261-262) */
  return GSTO_OK;
}

/* codec/encoder.cpp:122-144 */
int gsto_encode_stream(uint32_t w, uint32_t h, uint32_t palette_bytes, const uint8_t *y, const uint8_t *chroma,
                       const uint8_t *palette, const uint8_t *indices, uint8_t *out, size_t cap, size_t *out_len) {
  if (!out || !out_len || w == 0 || h == 0 || w % 4 || h % 4) return GSTO_E_ARG;
  const size_t B = (size_t)(w / 4) * (h / 4);
  const uint8_t *src[4] = {y, chroma, palette, indices};
  const size_t nsym[4] = {2 * B, 4 * B, palette_bytes, B};
  size_t need = GSTO_HEADER_BYTES;
  for (int k = 0; k < 4; ++k) {
    if (!src[k] || nsym[k] == 0 || nsym[k] % GSTO_SYMS_PER_GROUP) return GSTO_E_ARG;
    need += gsto_encode_section_bound(nsym[k]);
  }
  if (cap < need) return GSTO_E_ARG;
  uint8_t *tmp = (uint8_t *)malloc(gsto_encode_section_bound(4 * B > palette_bytes ? 4 * B : palette_bytes));
  if (!tmp) return GSTO_E_ARG;
  uint32_t sizes[4];
  uint8_t *body = out + GSTO_HEADER_BYTES + 4 * GSTO_FREQ_BYTES;
  for (int k = 0; k < 4; ++k) {
    size_t len = 0;
    const int st = gsto_encode_section(src[k], nsym[k], tmp, gsto_encode_section_bound(nsym[k]), &len);
    if (st != GSTO_OK) {
      free(tmp);
      return st;
    }
    memcpy(out + GSTO_HEADER_BYTES + k * GSTO_FREQ_BYTES, tmp, GSTO_FREQ_BYTES);
    memcpy(body, tmp + GSTO_FREQ_BYTES, len - GSTO_FREQ_BYTES);
    body += len - GSTO_FREQ_BYTES;
    sizes[k] = (uint32_t)(len - GSTO_FREQ_BYTES);
  }
  free(tmp);
  const uint32_t hdr[7] = {w, h, palette_bytes, sizes[0], sizes[1], sizes[2], sizes[3]};
  for (int i = 0; i < 7; ++i) wr32(out + 4 * i, hdr[i]);
  *out_len = (size_t)(body - out);
  return GSTO_OK;
}

/* ------------------------------------------------------------------------- */
/* Endpoint stages of the encoder.                                           */

/* codec/image_processing.cpp:10-27 */
static void rgb565_to_ycocg667(uint16_t c, int *y, int *co, int *cg) {
  const int r = c >> 11, g = (c >> 5) & 63, b = c & 31;
  *co = r - b;
  const int t = r + b + (b >> 4);
  *cg = g - t;
  *y = t + (*cg / 2);
}

/* codec/wavelet.cpp:56-88 (ForwardWavelet1D), int16 storage */
static void forward_line(const int16_t *src, int16_t *dst, int len) {
  const int mid = len - len / 2;
  for (int i = 1; i < len; i += 2) {
    const int prev = normalize_index(i - 1, len), next = normalize_index(i + 1, len);
    dst[mid + i / 2] = (int16_t)(src[i] - (src[prev] + src[next]) / 2);
  }
  for (int i = 0; i < len; i += 2) {
    const int prev = mid + normalize_index(i - 1, len) / 2, next = mid + normalize_index(i + 1, len) / 2;
    dst[i / 2] = (int16_t)(src[i] + (dst[prev] + dst[next] + 2) / 4);
  }
}

/* codec/wavelet.cpp:123-157 (ForwardWavelet2D) on the top-left dim x dim of a
 * 32x32 tile: every column, then every row. */
static void forward_level(int16_t *blk, int dim) {
  int16_t line[32], out[32];
  for (int x = 0; x < dim; ++x) {
    for (int y = 0; y < dim; ++y) line[y] = blk[y * 32 + x];
    forward_line(line, out, dim);
    for (int y = 0; y < dim; ++y) blk[y * 32 + x] = out[y];
  }
  for (int y = 0; y < dim; ++y) {
    forward_line(blk + y * 32, out, dim);
    memcpy(blk + y * 32, out, sizeof(int16_t) * (size_t)dim);
  }
}

uint64_t gsto_endpoint_planes(uint32_t w, uint32_t h, const uint64_t *blocks, uint8_t *y, uint8_t *chroma) {
  const uint32_t bx = w / 4, by = h / 4, tx_n = bx / 32, ty_n = by / 32;
  const size_t B = (size_t)bx * by;
  uint8_t *dst[6] = {y, chroma, chroma + B, y + B, chroma + 2 * B, chroma + 3 * B}; /* Y1 Co1 Cg1 Y2 Co2 Cg2 */
  uint64_t clips = 0;
  int16_t blk[6][1024];
  for (uint32_t ty = 0; ty < ty_n; ++ty) {
    for (uint32_t tx = 0; tx < tx_n; ++tx) {
      for (int i = 0; i < 1024; ++i) {
        const uint64_t b = blocks[((size_t)ty * 32 + (size_t)(i / 32)) * bx + (size_t)tx * 32 + (size_t)(i % 32)];
        int v[6];
        rgb565_to_ycocg667((uint16_t)b, &v[0], &v[1], &v[2]);
        rgb565_to_ycocg667((uint16_t)(b >> 16), &v[3], &v[4], &v[5]);
        for (int p = 0; p < 6; ++p) blk[p][i] = (int16_t)v[p];
      }
      for (int p = 0; p < 6; ++p) {
        for (int dim = 32; dim > 1; dim /= 2) forward_level(blk[p], dim);
        uint8_t *o = dst[p] + ((size_t)ty * tx_n + tx) * 1024;
        for (int i = 0; i < 1024; ++i) {
          if (blk[p][i] < -128 || blk[p][i] > 127) ++clips;
          o[i] = (uint8_t)(blk[p][i] + 128);
        }
      }
    }
  }
  return clips;
}

uint32_t gsto_run_palette(uint32_t w, uint32_t h, const uint64_t *blocks, uint8_t *palette, size_t pal_cap,
                          uint8_t *deltas) {
  const size_t B = (size_t)(w / 4) * (h / 4);
  const size_t need = (4 * B + GSTO_SYMS_PER_GROUP - 1) / GSTO_SYMS_PER_GROUP * GSTO_SYMS_PER_GROUP;
  if (pal_cap < need) return 0;
  size_t n = 0;
  for (size_t b = 0; b < B; ++b) {
    const uint32_t word = (uint32_t)(blocks[b] >> 32);
    const int fresh = b == 0 || word != (uint32_t)(blocks[b - 1] >> 32);
    if (fresh) wr32(palette + 4 * n++, word);
    deltas[b] = (uint8_t)(128 + (b > 0 && fresh ? 1 : 0));
  }
  const size_t bytes = (4 * n + GSTO_SYMS_PER_GROUP - 1) / GSTO_SYMS_PER_GROUP * GSTO_SYMS_PER_GROUP;
  memset(palette + 4 * n, 0, bytes - 4 * n);
  return (uint32_t)bytes;
}

/* ---- DXTImage::Reencode: the sequential index-palette search ---------------
 * codec/dxt_image.cpp:510-624 with its helpers (Decode565 :53-72, Pack565
 * :74-80, ToFiveBits / ToSixBits :82-130, PhysicalToLogical :144-170,
 * CompressedBlock::Error :266-285, AssignIndices + RecalculateEndpoints
 * :295-359).  Float arithmetic is the reference's as compiled for x86-64 (SSE,
 * no fused multiply-add: this file is built with -ffp-contract=off), including
 * the float -> int32 conversion of cvttss2si. */

/* cvttss2si: truncation toward zero; NaN and values outside the int32 range
 * give INT32_MIN (dxt_image.cpp:345-346 on x86-64). */
static int32_t f2i_x86(float q) {
  if (!(q >= -2147483648.0f && q < 2147483648.0f)) return INT32_MIN;
  return (int32_t)q;
}

static uint8_t absdiff8(uint8_t a, uint8_t b) { return a > b ? (uint8_t)(a - b) : (uint8_t)(b - a); }

/* ToFiveBits (bits = 5) / ToSixBits (bits = 6): the nearest value of the form
 * v | v >> bits among the channel's base, the next and the previous step. */
static uint8_t snap_channel(uint8_t x, int bits) {
  const uint8_t mask = bits == 5 ? 0xF8 : 0xFC, step = bits == 5 ? 4 : 2;
  uint8_t base = (uint8_t)(x & mask);
  uint8_t high = (uint8_t)(base + step);
  uint8_t low = base == 0 ? base : (uint8_t)(base - step);
  base = (uint8_t)(base | (base >> bits));
  high = (uint8_t)(high | (high >> bits));
  low = (uint8_t)(low | (low >> bits));
  const uint8_t db = absdiff8(x, base), dh = absdiff8(x, high), dl = absdiff8(x, low);
  if (db <= dh) return db < dl ? base : low;
  return high;
}

static uint16_t pack565(const uint8_t c[3]) {
  return (uint16_t)(((c[0] & 0xF8) << 8) | ((c[1] & 0xFC) << 3) | ((c[2] & 0xF8) >> 3));
}

static void unpack565(uint16_t v, uint8_t c[3]) {
  const uint32_t r = v >> 11, g = (v >> 5) & 0x3F, b = v & 0x1F;
  c[0] = (uint8_t)((r << 3) | (r >> 2));
  c[1] = (uint8_t)((g << 2) | (g >> 4));
  c[2] = (uint8_t)((b << 3) | (b >> 2));
}

/* Sum of squared channel differences over the 16 pixels, / 48. */
static int block_error(const uint8_t px[48], uint8_t pal[4][3], uint32_t word) {
  size_t err = 0;
  for (int i = 0; i < 16; ++i) {
    const uint8_t *p = pal[(word >> (2 * i)) & 3];
    for (int c = 0; c < 3; ++c) {
      const size_t d = absdiff8(px[3 * i + c], p[c]);
      err += d * d;
    }
  }
  return (int)(err / 48);
}

/* Error of the block as given (PhysicalToLogical's palette: three-colour
 * mode, with black, when ep1 <= ep2). */
static int given_error(const uint8_t px[48], uint64_t blk) {
  const uint16_t e1 = (uint16_t)blk, e2 = (uint16_t)(blk >> 16);
  uint8_t pal[4][3];
  unpack565(e1, pal[0]);
  unpack565(e2, pal[1]);
  for (int c = 0; c < 3; ++c) {
    if (e1 <= e2) {
      pal[2][c] = (uint8_t)((pal[0][c] + pal[1][c]) / 2);
      pal[3][c] = 0;
    } else {
      pal[2][c] = (uint8_t)((2 * pal[0][c] + pal[1][c]) / 3);
      pal[3][c] = (uint8_t)((pal[0][c] + 2 * pal[1][c]) / 3);
    }
  }
  return block_error(px, pal, (uint32_t)(blk >> 32));
}

/* The block's pixels refitted to index word `word`: least-squares endpoints,
 * snapped to 5:6:5, four-colour palette.  *ok = 0 when the refit endpoints do
 * not keep the word as is (Pack565(ep1) <= Pack565(ep2) would swap them). */
int gsto_reencode_candidate(const uint8_t px[48], uint32_t word, int *ok, uint16_t *ep1, uint16_t *ep2) {
  static const float order_of[4] = {0.0f, 3.0f, 1.0f, 2.0f};
  float asq = 0.0f, bsq = 0.0f, ab = 0.0f;
  float ax[3] = {0.0f, 0.0f, 0.0f}, bx[3] = {0.0f, 0.0f, 0.0f};
  for (int i = 0; i < 16; ++i) {
    const float o = order_of[(word >> (2 * i)) & 3];
    const float a = (3.0f - o) / 3.0f, b = o / 3.0f;
    asq += a * a;
    bsq += b * b;
    ab += a * b;
    for (int c = 0; c < 3; ++c) {
      ax[c] += (float)px[3 * i + c] * a;
      bx[c] += (float)px[3 * i + c] * b;
    }
  }
  const float f = 1.0f / (asq * bsq - ab * ab);
  uint8_t pal[4][3];
  for (int c = 0; c < 3; ++c) {
    const float p1 = f * (ax[c] * bsq - bx[c] * ab);
    const float p2 = f * (bx[c] * asq - ax[c] * ab);
    int32_t q1 = f2i_x86(p1 + 0.5f), q2 = f2i_x86(p2 + 0.5f);
    q1 = q1 < 0 ? 0 : q1 > 255 ? 255 : q1;
    q2 = q2 < 0 ? 0 : q2 > 255 ? 255 : q2;
    const int bits = c == 1 ? 6 : 5;
    pal[0][c] = snap_channel((uint8_t)q1, bits);
    pal[1][c] = snap_channel((uint8_t)q2, bits);
  }
  for (int c = 0; c < 3; ++c) {
    pal[2][c] = (uint8_t)((2 * pal[0][c] + pal[1][c]) / 3);
    pal[3][c] = (uint8_t)((pal[0][c] + 2 * pal[1][c]) / 3);
  }
  *ep1 = pack565(pal[0]);
  *ep2 = pack565(pal[1]);
  *ok = *ep1 > *ep2;
  return block_error(px, pal, word);
}

uint32_t gsto_reencode(uint32_t w, uint32_t h, const uint8_t *rgb, const uint64_t *blocks_in, uint64_t *blocks_out,
                       uint8_t *palette, size_t pal_cap, uint8_t *deltas) {
  const uint32_t bw = w / 4, bh = h / 4;
  const size_t B = (size_t)bw * bh;
  const size_t need = (4 * B + GSTO_SYMS_PER_GROUP - 1) / GSTO_SYMS_PER_GROUP * GSTO_SYMS_PER_GROUP;
  if (pal_cap < need || B == 0) return 0;
  size_t n = 0;  /* palette words so far */
  long last = 0; /* palette index of the previous block */
  for (size_t b = 0; b < B; ++b) {
    const uint32_t bx = (uint32_t)(b % bw), by = (uint32_t)(b / bw);
    uint8_t px[48];
    for (int r = 0; r < 4; ++r) memcpy(px + 12 * r, rgb + ((size_t)(4 * by + r) * w + 4 * bx) * 3, 12);
    const uint64_t blk = blocks_in[b];
    const int given = given_error(px, blk);
    int best = INT32_MAX;
    size_t best_r = 0;
    uint16_t best_e1 = 0, best_e2 = 0;
    const size_t window = n < 127 ? n : 127;
    for (size_t r = 0; r < window; ++r) { /* most recent word first */
      const uint32_t word = rd32(palette + 4 * (n - 1 - r));
      int ok;
      uint16_t e1, e2;
      const int diff = gsto_reencode_candidate(px, word, &ok, &e1, &e2) - given;
      if (!ok) continue;
      if (diff < best) {
        best = diff;
        best_r = r;
        best_e1 = e1;
        best_e2 = e2;
        if (diff <= 0) break;
      }
    }
    long idx;
    if (best < 35) {
      const uint32_t word = rd32(palette + 4 * (n - 1 - best_r));
      blocks_out[b] = (uint64_t)best_e1 | ((uint64_t)best_e2 << 16) | ((uint64_t)word << 32);
      idx = (long)(n - 1 - best_r);
    } else {
      blocks_out[b] = blk;
      wr32(palette + 4 * n, (uint32_t)(blk >> 32));
      idx = (long)n++;
    }
    deltas[b] = (uint8_t)(idx - last + 128);
    last = idx;
  }
  const size_t bytes = (4 * n + GSTO_SYMS_PER_GROUP - 1) / GSTO_SYMS_PER_GROUP * GSTO_SYMS_PER_GROUP;
  memset(palette + 4 * n, 0, bytes - 4 * n);
  return (uint32_t)bytes;
}
