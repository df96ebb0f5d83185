// Host Tier-2 and codestream assembly from the device's per-block results.
//
// Replaces build_packet_header / build_packet_sequence_for_components
// (src/encode/backend/native/t2.rs:337-473), the SIZ/COD/QCD/SOT writers
// (src/j2k/markers.rs:8-110, src/j2k/write.rs:9-77) and the JP2 box writer
// (src/jp2.rs:13-71). One layer, one precinct per resolution, LRCP order:
// packets run resolution-major, then component; the blocks of a packet are
// contiguous in the device work list, so its body is one contiguous range of
// the compacted byte buffer.
#include <algorithm>
#include <cstring>

#include "jp2g_internal.h"

namespace jp2g {

namespace {

// Packet-header bit writer with 0xFF stuffing (ISO 15444-1 B.10.1).
class BitWriter {
 public:
  explicit BitWriter(std::vector<uint8_t>* out) : out_(out) {}
  void bit(uint32_t b) {
    if (free_ == 0) next();
    --free_;
    cur_ |= (b & 1u) << free_;
  }
  void bits(uint32_t v, int n) {
    while (n-- > 0) bit((v >> n) & 1u);
  }
  void finish() {
    next();
    if (free_ == 7) next();  // a final 0xFF is followed by a zero byte
  }

 private:
  void next() {
    // Emit the pending byte; a byte after 0xFF carries only 7 bits.
    uint32_t shifted = (cur_ << 8) & 0xffffu;
    out_->push_back((uint8_t)(shifted >> 8));
    free_ = shifted == 0xff00u ? 7 : 8;
    cur_ = 0;
  }
  std::vector<uint8_t>* out_;
  uint32_t cur_ = 0;
  int free_ = 8;
};

// Tag tree (ISO 15444-1 B.10.2) with explicit levels; node (i, j) of a level
// has parent (i/2, j/2) in the next.
class TagTree {
 public:
  TagTree(int w, int h) {
    int lw = std::max(w, 1), lh = std::max(h, 1);
    for (;;) {
      lw_.push_back(lw);
      lh_.push_back(lh);
      off_.push_back(total_);
      total_ += lw * lh;
      if (lw * lh <= 1) break;
      lw = (lw + 1) / 2;
      lh = (lh + 1) / 2;
    }
    value_.assign(total_, 999);
    low_.assign(total_, 0);
    known_.assign(total_, 0);
  }
  void set(int leaf, int v) {
    int i = leaf % lw_[0], j = leaf / lw_[0];
    for (size_t l = 0; l < lw_.size(); ++l, i >>= 1, j >>= 1) {
      int& cur = value_[off_[l] + j * lw_[l] + i];
      if (cur <= v) break;
      cur = v;
    }
  }
  void encode(BitWriter& bw, int leaf, int threshold) {
    int path[32];
    int depth = 0;
    int i = leaf % lw_[0], j = leaf / lw_[0];
    for (size_t l = 0; l < lw_.size(); ++l, i >>= 1, j >>= 1) path[depth++] = off_[l] + j * lw_[l] + i;
    int low = 0;
    for (int k = depth - 1; k >= 0; --k) {  // root first
      int n = path[k];
      if (low > low_[n]) low_[n] = low;
      else low = low_[n];
      while (low < threshold) {
        if (low >= value_[n]) {
          if (!known_[n]) {
            bw.bit(1);
            known_[n] = 1;
          }
          break;
        }
        bw.bit(0);
        ++low;
      }
      low_[n] = low;
    }
  }

 private:
  std::vector<int> lw_, lh_, off_, value_, low_;
  std::vector<uint8_t> known_;
  int total_ = 0;
};

int flog2(uint32_t v) { return v == 0 ? 0 : 31 - __builtin_clz(v); }

// Number-of-passes codeword, Table B-4.
void put_passes(BitWriter& bw, uint32_t n) {
  if (n == 1) bw.bits(0, 1);
  else if (n == 2) bw.bits(2, 2);
  else if (n <= 5) bw.bits(0xcu | (n - 3), 4);
  else if (n <= 36) bw.bits(0x1e0u | (n - 6), 9);
  else bw.bits(0xff80u | (std::min(n, 164u) - 37), 16);
}

void be16(std::vector<uint8_t>& o, uint32_t v) {
  o.push_back((uint8_t)(v >> 8));
  o.push_back((uint8_t)v);
}
void be32(std::vector<uint8_t>& o, uint32_t v) {
  be16(o, v >> 16);
  be16(o, v & 0xffffu);
}

}  // namespace

// Packet header for the bands of one (resolution, component).
static void packet_header(const PagePlan& p, size_t band_begin, size_t band_end,
                          const BlockKeep* keep, std::vector<uint8_t>* out) {
  BitWriter bw(out);
  bw.bit(1);  // packet present (t2.rs:337-344)
  for (size_t bi = band_begin; bi < band_end; ++bi) {
    const BandGeom& g = p.bands[bi];
    const int n = g.ncbx * g.ncby;
    if (n == 0) continue;
    TagTree incl(g.ncbx, g.ncby), zbp(g.ncbx, g.ncby);
    for (int i = 0; i < n; ++i) {
      const BlockKeep& k = keep[g.first_block + i];
      zbp.set(i, k.zbp);
      if (k.npasses > 0) incl.set(i, 0);
    }
    for (int i = 0; i < n; ++i) {
      const BlockKeep& k = keep[g.first_block + i];
      incl.encode(bw, i, 1);
      if (k.npasses == 0) continue;
      zbp.encode(bw, i, 999);
      put_passes(bw, k.npasses);
      // One terminated segment of seg_len bytes; Lblock starts at 3
      // (B.10.7.1) and grows once, by the comma code, to fit it.
      const uint32_t lblock = 3;
      uint32_t need = k.seg_len == 0 ? 0 : (uint32_t)flog2(k.seg_len) + 1;
      uint32_t have = lblock + (uint32_t)flog2(k.npasses);
      uint32_t inc = need > have ? need - have : 0;
      for (uint32_t t = 0; t < inc; ++t) bw.bit(1);
      bw.bit(0);
      bw.bits(k.seg_len, (int)(lblock + inc + (uint32_t)flog2(k.npasses)));
    }
  }
  bw.finish();
}

bool assemble_codestream(const PagePlan& p, const BlockKeep* keep, const uint8_t* body,
                         const uint32_t* offsets, std::vector<uint8_t>* out, Failure* err) {
  std::vector<uint8_t> pay;
  pay.reserve(offsets[p.nblocks] + 64 * (size_t)(p.levels + 1) * p.ncomp + 1024);
  // bands are stored res -> comp -> orient, i.e. already in packet order
  size_t bi = 0;
  while (bi < p.bands.size()) {
    size_t be = bi;
    while (be < p.bands.size() && p.bands[be].res == p.bands[bi].res &&
           p.bands[be].comp == p.bands[bi].comp)
      ++be;
    packet_header(p, bi, be, keep, &pay);
    uint32_t b0 = p.bands[bi].first_block;
    const BandGeom& last = p.bands[be - 1];
    uint32_t b1 = last.first_block + (uint32_t)(last.ncbx * last.ncby);
    pay.insert(pay.end(), body + offsets[b0], body + offsets[b1]);
    bi = be;
  }
  std::vector<uint8_t>& o = *out;
  o.clear();
  o.reserve(pay.size() + 256);
  be16(o, 0xff4f);  // SOC
  be16(o, 0xff51);  // SIZ
  be16(o, 38 + 3 * p.ncomp);
  be16(o, 0);
  be32(o, p.width);
  be32(o, p.height);
  be32(o, 0);
  be32(o, 0);
  be32(o, p.width);
  be32(o, p.height);
  be32(o, 0);
  be32(o, 0);
  be16(o, p.ncomp);
  for (int c = 0; c < p.ncomp; ++c) {
    o.push_back((uint8_t)((p.precision - 1) & 0x7f));
    o.push_back(1);
    o.push_back(1);
  }
  be16(o, 0xff52);  // COD
  be16(o, 12);
  o.push_back(0);  // Scod
  o.push_back(0);  // LRCP
  be16(o, 1);      // one layer
  o.push_back(p.use_mct ? 1 : 0);
  o.push_back((uint8_t)p.levels);
  o.push_back((uint8_t)(__builtin_ctz((unsigned)p.cbw) - 2));
  o.push_back((uint8_t)(__builtin_ctz((unsigned)p.cbh) - 2));
  o.push_back(0);
  o.push_back(p.lossless ? 1 : 0);
  be16(o, 0xff5c);  // QCD
  if (p.lossless) {
    be16(o, 3 + (uint32_t)p.quants.size());
    o.push_back((uint8_t)(p.guard_bits << 5));
    for (const auto& q : p.quants) o.push_back((uint8_t)(q.exponent << 3));
  } else {
    be16(o, 3 + 2 * (uint32_t)p.quants.size());
    o.push_back((uint8_t)((p.guard_bits << 5) | 2));
    for (const auto& q : p.quants) be16(o, (((uint32_t)q.exponent & 0xffu) << 11 | ((uint32_t)q.mantissa & 0x7ffu)) & 0xffffu);
  }
  uint64_t psot = 12 + 2 + (uint64_t)pay.size();
  if (psot > 0xffffffffull) {
    *err = {kEncodeFailed, "tile-part length exceeds Psot range"};
    return false;
  }
  be16(o, 0xff90);  // SOT
  be16(o, 10);
  be16(o, 0);
  be32(o, (uint32_t)psot);
  o.push_back(0);
  o.push_back(1);
  be16(o, 0xff93);  // SOD
  o.insert(o.end(), pay.begin(), pay.end());
  be16(o, 0xffd9);  // EOC
  if (p.format == 1) {
    std::vector<uint8_t> j;
    uint64_t jl = (uint64_t)o.size() + 8;
    if (jl > 0xffffffffull) {
      *err = {kEncodeFailed, "JP2 box length exceeds 32-bit limit"};
      return false;
    }
    j.reserve(o.size() + 85);
    auto box = [&](uint32_t len, const char* t) {
      be32(j, len);
      j.insert(j.end(), t, t + 4);
    };
    box(12, "jP  ");
    j.insert(j.end(), {0x0d, 0x0a, 0x87, 0x0a});
    box(20, "ftyp");
    j.insert(j.end(), {'j', 'p', '2', ' '});
    be32(j, 0);
    j.insert(j.end(), {'j', 'p', '2', ' '});
    box(8 + 22 + 15, "jp2h");
    box(22, "ihdr");
    be32(j, p.height);
    be32(j, p.width);
    be16(j, p.ncomp);
    j.insert(j.end(), {7, 7, 0, 0});  // BPC, compression type 7, UnkC, IPR
    box(15, "colr");
    j.insert(j.end(), {1, 0, 0});
    be32(j, p.srgb ? 16 : 17);
    box((uint32_t)jl, "jp2c");
    j.insert(j.end(), o.begin(), o.end());
    o.swap(j);
  }
  return true;
}

}  // namespace jp2g
