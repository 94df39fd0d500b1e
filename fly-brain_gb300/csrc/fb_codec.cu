// The reference's compressed data files, decoded on the host: FLYG, the connectome CSR
// (src/codec/graph.js:70-108), and FLYN, the per-neuron table (src/codec/neurons.js:25-37), both
// written with the adaptive binary range coder and Elias-gamma integer model of src/codec/rc.js.
// The web app loads the connectome from these files (src/data.js:21-34); decoding yields arrays
// identical to graph_w{minWeight}.bin and neurons.bin. A range-coded stream is one sequential
// chain of adaptive decisions, so it is decoded by one host thread; the device is not involved.
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <utility>
#include <vector>

#include "../../include/flybrain.h"

namespace fb {
int set_error(int code, const char *msg);
}

namespace {

int cfail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return fb::set_error(code, buf);
}

constexpr uint32_t kFlygMagic = 0x47594C46u;  // "FLYG" little-endian
constexpr uint32_t kFlynMagic = 0x4E594C46u;  // "FLYN"
constexpr uint32_t kProbBits = 12, kProbOne = 1u << kProbBits, kAdapt = 5;

// Binary range decoder (rc.js:31-59): 32-bit range and code, 12-bit probabilities adapted by 1/32
// of the distance to the bound, bytes past the end read as 0.
struct RangeDecoder {
  const uint8_t *buf;
  size_t len, pos;
  uint32_t range = 0xFFFFFFFFu, code = 0;

  RangeDecoder(const uint8_t *b, size_t n) : buf(b), len(n), pos(0) {
    for (int i = 0; i < 5; i++) code = (code << 8) | next();
  }
  uint32_t next() { return pos < len ? buf[pos++] : 0u; }
  void normalize() {
    while (range < (1u << 24)) {
      range <<= 8;
      code = (code << 8) | next();
    }
  }
  uint32_t bit(uint16_t &p) {
    const uint32_t pr = p, bound = (range >> kProbBits) * pr;
    uint32_t b;
    if (code < bound) {
      range = bound;
      p = (uint16_t)(pr + ((kProbOne - pr) >> kAdapt));
      b = 0;
    } else {
      code -= bound;
      range -= bound;
      p = (uint16_t)(pr - (pr >> kAdapt));
      b = 1;
    }
    normalize();
    return b;
  }
  // nbits equiprobable bits, most significant first, at most 16 per division
  uint64_t direct(int nbits) {
    uint64_t v = 0;
    while (nbits > 0) {
      const int n = nbits < 16 ? nbits : 16;
      nbits -= n;
      range >>= n;
      const uint32_t x = code / range;
      code -= x * range;
      v = (v << n) + x;
      normalize();
    }
    return v;
  }
};

// Adaptive Elias-gamma model (rc.js:79-123): per context a 5-bit tree for the bit length k of v+1,
// two context-modelled bits below the leading one, then k-2 direct bits.
struct GammaModel {
  std::vector<uint16_t> len, top;
  explicit GammaModel(int nctx) : len((size_t)nctx * 32, kProbOne / 2), top((size_t)nctx * 32 * 4, kProbOne / 2) {}
  uint64_t dec(RangeDecoder &d, int ctx) {
    const int base = ctx * 32;
    uint32_t t = 1;
    for (int i = 0; i < 5; i++) t = (t << 1) | d.bit(len[base + t]);
    const int k = (int)t - 32;
    uint64_t r = 1;
    if (k > 0) {
      const int mb = (base + k) * 4;
      r = (r << 1) | d.bit(top[mb + 1]);
      if (k >= 2) r = (r << 1) | d.bit(top[mb + 2 + (int)(r & 1u)]);
      if (k >= 3) r = (r << (k - 2)) + d.direct(k - 2);
    }
    return r - 1;
  }
  int64_t dec_signed(RangeDecoder &d, int ctx) {  // zigzag (rc.js:119-122)
    const uint64_t z = dec(d, ctx);
    return (z & 1u) ? -(int64_t)((z + 1) / 2) : (int64_t)(z / 2);
  }
};

// Bit length of x + 1 less one (rc.js:125), the usual magnitude context.
inline int lg(uint64_t x) {
  uint64_t y = x + 1;
  int n = -1;
  while (y) {
    y >>= 1;
    n++;
  }
  return n;
}
inline int lg23(uint64_t x) { return std::min(lg(x), 23); }

bool read_u32s(const uint8_t *buf, size_t len, uint32_t *out, int n) {
  if (!buf || len < (size_t)n * 4) return false;
  std::memcpy(out, buf, (size_t)n * 4);  // the files are little-endian, as both hosts are
  return true;
}

}  // namespace

extern "C" int fb_flyg_sizes(const uint8_t *buf, size_t len, fb_flyg_header *h) {
  uint32_t w[5];
  if (!h || !read_u32s(buf, len, w, 5)) return cfail(FB_EINVAL, "fb_flyg_sizes: buffer shorter than the 20-byte header");
  if (w[0] != kFlygMagic || w[1] != 1) return cfail(FB_EINVAL, "fb_flyg_sizes: not a FLYG v1 file");
  h->N = w[2];
  h->E = w[3];
  h->min_weight = w[4];
  h->pad = 0;
  return FB_OK;
}

// graph.js:70-108. Rows are coded in the encoder's neuron order (the permutation comes first, 18
// direct bits per neuron); each row: degree, copy bits over the previous coded row's targets,
// the remaining targets as a first offset from the row's own index and then gaps, the weights in
// target order (a copied edge's context is the weight it copies). The rows are then put back in
// the original numbering with every row sorted by target.
extern "C" int fb_flyg_decode(const uint8_t *buf, size_t len, uint32_t *indptr, uint32_t *indices, uint16_t *weights) {
  fb_flyg_header h;
  int rc = fb_flyg_sizes(buf, len, &h);
  if (rc) return rc;
  const uint32_t N = h.N, E = h.E, mw = h.min_weight;
  if (!indptr || (E && (!indices || !weights))) return cfail(FB_EINVAL, "fb_flyg_decode: null output array");
  if (N > (1u << 18)) return cfail(FB_EINVAL, "fb_flyg_decode: N=%u exceeds the 18-bit permutation field", N);
  RangeDecoder d(buf + 20, len - 20);
  GammaModel mDeg(24), mFirst(24), mGap(24), mW(48);
  std::vector<uint16_t> mCopy(4 * 8 * 2, kProbOne / 2);
  std::vector<uint32_t> order(N);
  std::vector<uint8_t> seen(N, 0);
  for (uint32_t r = 0; r < N; r++) {
    order[r] = (uint32_t)d.direct(18);
    if (order[r] >= N || seen[order[r]]) return cfail(FB_EINVAL, "fb_flyg_decode: corrupt permutation at row %u", r);
    seen[order[r]] = 1;
  }
  // pass 1: rows in coded order; targets in coded numbering
  std::vector<uint32_t> rowEnd(N), tgt(E);
  std::vector<uint16_t> wt(E);
  std::vector<uint32_t> cop, res;
  uint64_t pos = 0, pa = 0, pb = 0, prevDeg = 0;
  for (uint32_t r = 0; r < N; r++) {
    const uint64_t deg = mDeg.dec(d, lg23(prevDeg));
    if (pos + deg > E) return cfail(FB_EINVAL, "fb_flyg_decode: row %u overruns the %u edges", r, E);
    const uint64_t plen = pb - pa;
    const int ratio = plen ? std::min(7, std::max(0, lg(deg) - lg(plen) + 4)) : 0;
    cop.clear();
    uint32_t b = 0;
    for (uint64_t i = 0; i < plen; i++) {
      b = d.bit(mCopy[(b * 8 + (uint32_t)ratio) * 2 + (i == 0 ? 1u : 0u)]);
      if (b) cop.push_back((uint32_t)i);
    }
    if (cop.size() > deg) return cfail(FB_EINVAL, "fb_flyg_decode: row %u copies more targets than its degree", r);
    const uint64_t nr = deg - cop.size();
    res.resize(nr);
    int64_t last = -1;
    uint64_t pg = 0;
    for (uint64_t i = 0; i < nr; i++) {
      if (i == 0) {
        last = (int64_t)r + mFirst.dec_signed(d, lg23(deg));
      } else {
        const uint64_t g = mGap.dec(d, lg23(pg));
        pg = g;
        last += (int64_t)g + 1;
      }
      if (last < 0 || last >= (int64_t)N) return cfail(FB_EINVAL, "fb_flyg_decode: row %u target out of range", r);
      res[i] = (uint32_t)last;
    }
    // merge the copied targets (ascending, from the previous row) with the residual ones
    const uint64_t start = pos;
    size_t i = 0, k = 0;
    uint64_t pw = 0;
    while (i < cop.size() || k < nr) {
      const uint32_t ct = i < cop.size() ? tgt[pa + cop[i]] : 0xFFFFFFFFu;
      const uint32_t rt = k < nr ? res[k] : 0xFFFFFFFFu;
      uint64_t w;
      if (ct < rt) {
        w = mW.dec(d, 24 + lg23((uint64_t)wt[pa + cop[i]] - mw));  // every stored weight is >= mw
        tgt[pos] = ct;
        i++;
      } else {
        w = mW.dec(d, lg23(pw));
        tgt[pos] = rt;
        k++;
      }
      if (w + mw > 0xFFFFu) return cfail(FB_EINVAL, "fb_flyg_decode: row %u weight out of range", r);
      wt[pos++] = (uint16_t)(w + mw);
      pw = w;
    }
    pa = start;
    pb = pos;
    rowEnd[r] = (uint32_t)pos;
    prevDeg = deg;
  }
  if (pos != E) return cfail(FB_EINVAL, "fb_flyg_decode: %llu edges decoded, the header says %u", (unsigned long long)pos, E);
  // pass 2: original numbering, every row ascending by target
  indptr[0] = 0;
  for (uint32_t r = 0; r < N; r++) indptr[order[r] + 1] = rowEnd[r] - (r ? rowEnd[r - 1] : 0u);
  for (uint32_t o = 0; o < N; o++) indptr[o + 1] += indptr[o];
  std::vector<std::pair<uint32_t, uint16_t>> row;
  for (uint32_t r = 0; r < N; r++) {
    const uint32_t a = r ? rowEnd[r - 1] : 0u, e = rowEnd[r];
    row.clear();
    for (uint32_t j = a; j < e; j++) row.emplace_back(order[tgt[j]], wt[j]);
    std::sort(row.begin(), row.end());
    for (size_t q = 1; q < row.size(); q++)
      if (row[q].first == row[q - 1].first) return cfail(FB_EINVAL, "fb_flyg_decode: row %u repeats a target", order[r]);
    uint32_t *ix = indices + indptr[order[r]];
    uint16_t *wx = weights + indptr[order[r]];
    for (size_t q = 0; q < row.size(); q++) {
      ix[q] = row[q].first;
      wx[q] = row[q].second;
    }
  }
  return FB_OK;
}

extern "C" int fb_flyn_count(const uint8_t *buf, size_t len, uint32_t *N) {
  uint32_t w[3];
  if (!N || !read_u32s(buf, len, w, 3)) return cfail(FB_EINVAL, "fb_flyn_count: buffer shorter than the 12-byte header");
  if (w[0] != kFlynMagic || w[1] != 1) return cfail(FB_EINVAL, "fb_flyn_count: not a FLYN v1 file");
  *N = w[2];
  return FB_OK;
}

// neurons.js:25-37: per neuron the body-id gap, the superclass, then class, transmitter and side in
// the superclass's context, a has-soma bit (context: the previous neuron's), and the soma as
// offsets from the previous soma (NaN when absent).
extern "C" int fb_flyn_decode(const uint8_t *buf, size_t len, int64_t *body_ids, float *soma, uint16_t *cls,
                              uint8_t *nt, uint8_t *superclass, uint8_t *side) {
  uint32_t N = 0;
  int rc = fb_flyn_count(buf, len, &N);
  if (rc) return rc;
  if (N && (!body_ids || !soma || !cls || !nt || !superclass || !side))
    return cfail(FB_EINVAL, "fb_flyn_decode: null output array");
  RangeDecoder d(buf + 12, len - 12);
  GammaModel mId(1), mSc(32), mCls(32), mNt(32), mSide(32), mSoma(3);
  uint16_t has[2] = {kProbOne / 2, kProbOne / 2};
  int64_t id = 0, prev[3] = {0, 0, 0};
  uint32_t ph = 1;
  for (uint32_t i = 0; i < N; i++) {
    id += (int64_t)mId.dec(d, 0);
    body_ids[i] = id;
    const uint64_t s = mSc.dec(d, 0);
    if (s >= 32) return cfail(FB_EINVAL, "fb_flyn_decode: neuron %u superclass %llu out of range", i, (unsigned long long)s);
    const uint64_t c = mCls.dec(d, (int)s), t = mNt.dec(d, (int)s), sd = mSide.dec(d, (int)s);
    if (c > 0xFFFFu || t > 0xFFu || sd > 0xFFu) return cfail(FB_EINVAL, "fb_flyn_decode: neuron %u field out of range", i);
    superclass[i] = (uint8_t)s;
    cls[i] = (uint16_t)c;
    nt[i] = (uint8_t)t;
    side[i] = (uint8_t)sd;
    const uint32_t hb = d.bit(has[ph]);
    ph = hb;
    for (int k = 0; k < 3; k++) {
      if (hb) prev[k] += mSoma.dec_signed(d, k);
      soma[(size_t)i * 3 + k] = hb ? (float)prev[k] : __builtin_nanf("");
    }
  }
  return FB_OK;
}
