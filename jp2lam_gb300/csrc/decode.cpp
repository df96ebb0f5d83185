// Host half of the device decoder: JP2 boxes, the codestream's main header
// and the packet headers of a single-tile, one-layer LRCP codestream with
// one precinct per resolution (the codestreams this encoder and the
// reference write).
//
// Follows decode_jp2 (src/decode/mod.rs:56-61): parse_jp2
// (src/decode/jp2_parse.rs), the main-header and tile-part parse
// (src/decode/codestream.rs, src/j2k/decode_markers.rs) and the packet
// headers (src/decode/t2.rs): tag-tree decoding (ISO/IEC 15444-1 B.10.2),
// Table B-4 pass counts, Lblock and segment lengths (B.10.7), with the bit
// stuffing after 0xFF (B.10.1). The per-block checks of decode/t1.rs:87-130
// (bit-plane counts from QCD, the pass-count limit) are made here, before any
// device work; the device decodes the code-blocks and reconstructs the
// image (t1dec.cu, recon.cu).
#include <algorithm>
#include <string>

#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {

namespace {

struct Bytes {
  const uint8_t* b;
  size_t n, pos;
  bool ok = true;
  uint32_t u8() {
    if (pos >= n) {
      ok = false;
      return 0;
    }
    return b[pos++];
  }
  uint32_t u16() { return u8() << 8 | u8(); }
  uint32_t u32() { return u16() << 16 | u16(); }
};

// Packet-header bits; a byte after 0xFF carries 7 (B.10.1).
struct HeaderBits {
  const uint8_t* b;
  size_t n, pos;
  uint32_t cur = 0;
  int left = 0;
  bool ok = true;
  uint32_t bit() {
    if (left == 0) {
      if (pos >= n) {
        ok = false;
        return 0;
      }
      const uint32_t prev = cur;
      cur = b[pos++];
      left = prev == 0xffu ? 7 : 8;
    }
    --left;
    return (cur >> left) & 1u;
  }
  uint32_t bits(int k) {
    uint32_t v = 0;
    for (int i = 0; i < k; ++i) v = v << 1 | bit();
    return v;
  }
  // To the next byte; a header ending in 0xFF is followed by a zero byte.
  void align() {
    if (cur == 0xffu && left == 0 && pos < n) ++pos;
    left = 0;
    cur = 0;
  }
};

// Tag tree decoder (B.10.2): node values are learnt as bits arrive.
class TagDecoder {
 public:
  TagDecoder(int w, int h) {
    std::vector<std::pair<int, int>> dims;
    for (;;) {
      dims.push_back({w, h});
      if (w * h <= 1) break;
      w = (w + 1) / 2;
      h = (h + 1) / 2;
    }
    std::vector<int> base(dims.size() + 1, 0);
    for (size_t l = 0; l < dims.size(); ++l) base[l + 1] = base[l] + dims[l].first * dims[l].second;
    parent_.assign(base.back(), -1);
    value_.assign(base.back(), 1 << 30);
    low_.assign(base.back(), 0);
    for (size_t l = 0; l + 1 < dims.size(); ++l)
      for (int j = 0; j < dims[l].second; ++j)
        for (int i = 0; i < dims[l].first; ++i)
          parent_[base[l] + j * dims[l].first + i] = base[l + 1] + (j / 2) * dims[l + 1].first + i / 2;
  }
  // Whether the leaf's value is below `threshold`, reading the bits that
  // decide it.
  bool below(HeaderBits& hb, int leaf, int threshold) {
    int path[64], depth = 0, k = leaf;
    while (parent_[k] >= 0 && depth < 63) {
      path[depth++] = k;
      k = parent_[k];
    }
    int low = 0;
    for (;;) {
      if (low > low_[k]) low_[k] = low;
      else low = low_[k];
      while (low < threshold && low < value_[k]) {
        if (hb.bit()) value_[k] = low;
        else ++low;
        if (!hb.ok) return false;
      }
      low_[k] = low;
      if (depth == 0) break;
      k = path[--depth];
    }
    return value_[leaf] < threshold;
  }

 private:
  std::vector<int> parent_, value_, low_;
};

int floor_log2(uint32_t v) { return v == 0 ? 0 : 31 - __builtin_clz(v); }

bool fail(Failure* err, int code, const char* msg) {
  *err = {code, msg};
  return false;
}

}  // namespace

bool parse_codestream(const uint8_t* bytes, size_t n, int flags, DecodeLayout* out, Failure* err) {
  const bool rct_chroma_extra_bitplane = (flags & 1) != 0, accept_empty = (flags & 2) != 0;
  // JP2 boxes: the codestream is the jp2c box (src/decode/jp2_parse.rs)
  size_t cs0 = 0, csn = n;
  if (n >= 12 && bytes[4] == 'j' && bytes[5] == 'P') {
    size_t pos = 0;
    bool found = false;
    while (pos + 8 <= n) {
      Bytes br{bytes, n, pos};
      const uint32_t len = br.u32(), type = br.u32();
      if (len < 8 || pos + len > n) return fail(err, kDecodeFailed, "bad JP2 box");
      if (type == 0x6a703263u) {  // jp2c
        cs0 = pos + 8;
        csn = len - 8;
        found = true;
        break;
      }
      pos += len;
    }
    if (!found) return fail(err, kDecodeFailed, "no jp2c box");
  }
  const uint8_t* cs = bytes + cs0;
  Bytes c{cs, csn, 0};
  if (c.u16() != 0xff4fu) return fail(err, kDecodeFailed, "missing SOC");
  DecodeLayout& L = *out;
  L = DecodeLayout{};
  std::vector<std::pair<int, int>> steps;  // (exponent, mantissa) per band
  size_t payload = 0, payload_end = 0;
  for (;;) {
    const uint32_t m = c.u16();
    if (!c.ok) return fail(err, kDecodeFailed, "truncated main header");
    if (m == 0xff90u) {  // SOT: the single tile-part
      c.u16();
      c.u16();
      const uint32_t psot = c.u32();
      c.u8();
      c.u8();
      const size_t sot = c.pos - 12;
      if (c.u16() != 0xff93u) return fail(err, kDecodeFailed, "expected SOD");
      payload = c.pos;
      payload_end = psot == 0 ? csn : sot + psot;
      if (!c.ok || payload_end > csn || payload_end < payload) return fail(err, kDecodeFailed, "bad tile-part length");
      break;
    }
    const uint32_t len = c.u16();
    if (len < 2) return fail(err, kDecodeFailed, "bad marker segment length");
    const size_t end = c.pos + len - 2;
    if (m == 0xff51u) {  // SIZ
      c.u16();
      L.width = c.u32();
      L.height = c.u32();
      for (int i = 0; i < 6; ++i) c.u32();
      L.ncomp = (int)c.u16();
      for (int i = 0; i < L.ncomp; ++i) {
        if (i == 0) L.precision = (int)(c.u8() & 0x7f) + 1;
        else c.u8();
        c.u8();
        c.u8();
      }
    } else if (m == 0xff52u) {  // COD
      c.u8();
      c.u8();
      c.u16();
      L.mct = c.u8() != 0;
      L.levels = (int)c.u8();
      L.cbw = 1 << (c.u8() + 2);
      L.cbh = 1 << (c.u8() + 2);
      c.u8();
      L.reversible = c.u8() == 1;
    } else if (m == 0xff5cu) {  // QCD
      const uint32_t sq = c.u8();
      L.guard = (int)(sq >> 5);
      if ((sq & 0x1f) == 0) {
        while (c.pos < end) steps.push_back({(int)(c.u8() >> 3), 0});
      } else {
        while (c.pos + 2 <= end) {
          const uint32_t v = c.u16();
          steps.push_back({(int)(v >> 11), (int)(v & 0x7ff)});
        }
      }
    }
    if (end > csn) return fail(err, kDecodeFailed, "marker segment past the codestream");
    c.pos = end;
  }
  if (L.width == 0 || L.height == 0 || (L.ncomp != 1 && L.ncomp != 3) || L.precision != 8)
    return fail(err, kUnsupportedFeature, "only 8-bit gray or 3-component codestreams are decoded");
  if ((uint64_t)L.width * L.height > (1ull << 30)) return fail(err, kUnsupportedFeature, "image too large to decode");
  if (L.levels > 32 || L.cbw > 64 || L.cbh > 64)
    return fail(err, kUnsupportedFeature, "unsupported coding parameters");
  // resolution ladder (index 0 = the smallest) and band rectangles
  L.ladder.assign(L.levels + 1, {0, 0});
  {
    int w = (int)L.width, h = (int)L.height;
    for (int r = L.levels; r >= 0; --r) {
      L.ladder[r] = {w, h};
      w = (w + 1) / 2;
      h = (h + 1) / 2;
    }
  }
  struct Rect {
    int res, orient, x0, y0, x1, y1;
  };
  std::vector<Rect> rects;
  rects.push_back({0, LL, 0, 0, L.ladder[0].first, L.ladder[0].second});
  for (int i = 0; i < L.levels; ++i) {
    const auto lo = L.ladder[i], full = L.ladder[i + 1];
    rects.push_back({i + 1, HL, lo.first, 0, full.first, lo.second});
    rects.push_back({i + 1, LH, 0, lo.second, lo.first, full.second});
    rects.push_back({i + 1, HH, lo.first, lo.second, full.first, full.second});
  }
  if (steps.size() < rects.size()) return fail(err, kDecodeFailed, "QCD has fewer entries than subbands");
  // packets: resolution, then component (LRCP, one layer)
  size_t pos = cs0 + payload;
  const size_t end = cs0 + payload_end;
  for (int res = 0; res <= L.levels; ++res)
    for (int comp = 0; comp < L.ncomp; ++comp) {
      HeaderBits hb{bytes, end, pos};
      if (hb.bit() == 0) {
        if (!hb.ok) return fail(err, kDecodeFailed, "packet header truncated");
        return fail(err, kUnsupportedFeature, "empty packets are not produced by this encoder");
      }
      const size_t first = L.blocks.size();
      for (size_t bi = 0; bi < rects.size(); ++bi) {
        const Rect& rc = rects[bi];
        if (rc.res != res || rc.x1 <= rc.x0 || rc.y1 <= rc.y0) continue;
        const int ncbx = (rc.x1 - rc.x0 + L.cbw - 1) / L.cbw, ncby = (rc.y1 - rc.y0 + L.cbh - 1) / L.cbh;
        TagDecoder incl(ncbx, ncby), imsb(ncbx, ncby);
        const int mb = L.guard - 1 + steps[bi].first +
                       (rct_chroma_extra_bitplane && L.reversible && L.mct && comp > 0 ? 1 : 0);
        const float step = quant_step_from_qcd(L.precision, rc.orient, steps[bi].first, steps[bi].second);
        for (int i = 0; i < ncbx * ncby; ++i) {
          DecBlock b{};
          const int bx = i % ncbx, by = i / ncbx;
          const int x0 = rc.x0 + bx * L.cbw, y0 = rc.y0 + by * L.cbh;
          b.plane_off = ((uint64_t)comp * L.height + (uint64_t)y0) * L.width + (uint64_t)x0;
          b.stride = L.width;
          b.w = (uint16_t)(std::min(x0 + L.cbw, rc.x1) - x0);
          b.h = (uint16_t)(std::min(y0 + L.cbh, rc.y1) - y0);
          b.orient = (uint8_t)rc.orient;
          b.reversible = L.reversible ? 1 : 0;
          b.mb = (uint8_t)std::max(0, std::min(mb, 255));
          b.step = step;
          if (incl.below(hb, i, 1)) {
            int z = 0;
            while (!imsb.below(hb, i, z + 1) && hb.ok && z < 255) ++z;
            b.zbp = (uint8_t)z;
            int np;  // Table B-4
            if (!hb.bit()) np = 1;
            else if (!hb.bit()) np = 2;
            else {
              const uint32_t v = hb.bits(2);
              if (v != 3) np = 3 + (int)v;
              else {
                const uint32_t v5 = hb.bits(5);
                np = v5 != 31 ? 6 + (int)v5 : 37 + (int)hb.bits(7);
              }
            }
            b.npasses = (uint16_t)np;
            int lblock = 3;
            while (hb.bit() && hb.ok && lblock < 32) ++lblock;
            const int nb = lblock + floor_log2((uint32_t)np);
            if (nb > 32) return fail(err, kDecodeFailed, "code-block length field too long");
            b.data_len = hb.bits(nb);
          }
          if (!hb.ok) return fail(err, kDecodeFailed, "packet header truncated");
          L.blocks.push_back(b);
        }
      }
      hb.align();
      size_t body = hb.pos;
      for (size_t k = first; k < L.blocks.size(); ++k) {
        DecBlock& b = L.blocks[k];
        if (b.npasses == 0) continue;
        if (body + b.data_len > end) return fail(err, kDecodeFailed, "code-block data past tile-part end");
        b.data_off = (uint32_t)body;
        body += b.data_len;
        // decode/t1.rs:87-130: bit-planes from QCD, the pass-count limit
        if (b.data_len == 0 && !accept_empty)
          return fail(err, kDecodeFailed, "non-empty code-block has no compressed bytes");
        if (b.zbp > b.mb) return fail(err, kDecodeFailed, "zero-bitplane count exceeds subband bit-plane count");
        const int mbp = b.mb - b.zbp;
        if (mbp == 0) return fail(err, kDecodeFailed, "non-empty code-block has no magnitude bit-planes");
        if (mbp > 31) return fail(err, kUnsupportedFeature, "more than 31 magnitude bit-planes");
        if (b.npasses > 1 + 3 * (mbp - 1)) return fail(err, kDecodeFailed, "code-block pass count exceeds maximum");
      }
      pos = body;
    }
  if (n > 0xffffffffull) return fail(err, kUnsupportedFeature, "input too large");
  return true;
}

}  // namespace jp2g
