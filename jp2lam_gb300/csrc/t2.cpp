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
  // The n low bits of v, most significant first (as n calls of bit()), a
  // byte's worth at a time.
  void bits(uint32_t v, int n) {
    while (n > 0) {
      if (free_ == 0) next();
      const int take = n < free_ ? n : free_;
      n -= take;
      free_ -= take;
      cur_ |= ((v >> n) & ((1u << take) - 1u)) << free_;
    }
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
// has parent (i/2, j/2) in the next. reset() keeps the storage, so one tree
// per thread serves every band.
class TagTree {
 public:
  void reset(int w, int h) {
    int lw = std::max(w, 1), lh = std::max(h, 1);
    levels_ = 0;
    total_ = 0;
    for (;;) {
      lw_[levels_] = lw;
      off_[levels_] = total_;
      ++levels_;
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
    for (int l = 0; l < levels_; ++l, i >>= 1, j >>= 1) {
      int& cur = value_[off_[l] + j * lw_[l] + i];
      if (cur <= v) break;
      cur = v;
    }
  }
  void encode(BitWriter& bw, int leaf, int threshold) {
    int path[32];
    int i = leaf % lw_[0], j = leaf / lw_[0];
    for (int l = 0; l < levels_; ++l, i >>= 1, j >>= 1) path[l] = off_[l] + j * lw_[l] + i;
    int low = 0;
    for (int k = levels_ - 1; k >= 0; --k) {  // root first
      const int n = path[k];
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
  int lw_[32], off_[32];
  int levels_ = 0, total_ = 0;
  std::vector<int> value_, low_;
  std::vector<uint8_t> known_;
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
    thread_local TagTree incl, zbp;
    incl.reset(g.ncbx, g.ncby);
    zbp.reset(g.ncbx, g.ncby);
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

// The bytes of a page's codestream ahead of its packets: the JP2 boxes (for
// JP2 output, src/jp2.rs:13-71), SOC, SIZ, COD, QCD, the SOT segment and SOD
// (src/j2k/markers.rs:8-110, src/j2k/write.rs:9-77), for a packet payload of
// `payload` bytes. *psot_pos is the offset of the Psot field and *jp2c_pos
// that of the jp2c box header (~0 for J2K), so a writer that learns the
// payload later can fill them in. False (with *err) when a length overflows.
bool codestream_prefix(const PagePlan& p, uint64_t payload, std::vector<uint8_t>* out, uint32_t* psot_pos,
                       uint32_t* jp2c_pos, Failure* err) {
  std::vector<uint8_t> mh;
  mh.reserve(256);
  be16(mh, 0xff4f);  // SOC
  be16(mh, 0xff51);  // SIZ
  be16(mh, 38 + 3 * p.ncomp);
  be16(mh, 0);
  be32(mh, p.width);
  be32(mh, p.height);
  be32(mh, 0);
  be32(mh, 0);
  be32(mh, p.width);
  be32(mh, p.height);
  be32(mh, 0);
  be32(mh, 0);
  be16(mh, p.ncomp);
  for (int c = 0; c < p.ncomp; ++c) {
    mh.push_back((uint8_t)((p.precision - 1) & 0x7f));
    mh.push_back(1);
    mh.push_back(1);
  }
  be16(mh, 0xff52);  // COD
  be16(mh, 12);
  mh.push_back(0);  // Scod
  mh.push_back(0);  // LRCP
  be16(mh, 1);      // one layer
  mh.push_back(p.use_mct ? 1 : 0);
  mh.push_back((uint8_t)p.levels);
  mh.push_back((uint8_t)(__builtin_ctz((unsigned)p.cbw) - 2));
  mh.push_back((uint8_t)(__builtin_ctz((unsigned)p.cbh) - 2));
  mh.push_back(0);
  mh.push_back(p.lossless ? 1 : 0);
  be16(mh, 0xff5c);  // QCD
  if (p.lossless) {
    be16(mh, 3 + (uint32_t)p.quants.size());
    mh.push_back((uint8_t)(p.guard_bits << 5));
    for (const auto& q : p.quants) mh.push_back((uint8_t)(q.exponent << 3));
  } else {
    be16(mh, 3 + 2 * (uint32_t)p.quants.size());
    mh.push_back((uint8_t)((p.guard_bits << 5) | 2));
    for (const auto& q : p.quants) be16(mh, (((uint32_t)q.exponent & 0xffu) << 11 | ((uint32_t)q.mantissa & 0x7ffu)) & 0xffffu);
  }
  const uint64_t psot = 12 + 2 + payload;
  if (psot > 0xffffffffull) {
    *err = {kEncodeFailed, "tile-part length exceeds Psot range"};
    return false;
  }
  be16(mh, 0xff90);  // SOT
  be16(mh, 10);
  be16(mh, 0);
  const size_t psot_at = mh.size();
  be32(mh, (uint32_t)psot);
  mh.push_back(0);
  mh.push_back(1);
  be16(mh, 0xff93);  // SOD
  const uint64_t cs_len = mh.size() + payload + 2;  // + EOC

  std::vector<uint8_t>& o = *out;
  o.clear();
  *jp2c_pos = ~0u;
  if (p.format == 1) {
    const uint64_t jl = cs_len + 8;
    if (jl > 0xffffffffull) {
      *err = {kEncodeFailed, "JP2 box length exceeds 32-bit limit"};
      return false;
    }
    auto box = [&](uint32_t len, const char* t) {
      be32(o, len);
      o.insert(o.end(), t, t + 4);
    };
    box(12, "jP  ");
    o.insert(o.end(), {0x0d, 0x0a, 0x87, 0x0a});
    box(20, "ftyp");
    o.insert(o.end(), {'j', 'p', '2', ' '});
    be32(o, 0);
    o.insert(o.end(), {'j', 'p', '2', ' '});
    box(8 + 22 + 15, "jp2h");
    box(22, "ihdr");
    be32(o, p.height);
    be32(o, p.width);
    be16(o, p.ncomp);
    o.insert(o.end(), {7, 7, 0, 0});  // BPC, compression type 7, UnkC, IPR
    box(15, "colr");
    o.insert(o.end(), {1, 0, 0});
    be32(o, p.srgb ? 16 : 17);
    *jp2c_pos = (uint32_t)o.size();
    box((uint32_t)jl, "jp2c");
  }
  *psot_pos = (uint32_t)(o.size() + psot_at);
  o.insert(o.end(), mh.begin(), mh.end());
  return true;
}

bool assemble_codestream(const PagePlan& p, const BlockKeep* keep, const uint8_t* body,
                         const uint32_t* offsets, std::vector<uint8_t>* out, Failure* err) {
  // Packet headers first (small), so every length is known before the
  // output is laid out; then each byte of the output is written once.
  std::vector<uint8_t> hdr;
  hdr.reserve(64 * (size_t)(p.levels + 1) * p.ncomp + 1024);
  struct Packet {
    size_t hdr_end;       // end of the packet's header in hdr
    uint32_t body0, body1;  // its body bytes in `body`
  };
  std::vector<Packet> packets;
  uint64_t pay = 0;
  // bands are stored res -> comp -> orient, i.e. already in packet order
  size_t bi = 0;
  while (bi < p.bands.size()) {
    size_t be = bi;
    while (be < p.bands.size() && p.bands[be].res == p.bands[bi].res &&
           p.bands[be].comp == p.bands[bi].comp)
      ++be;
    packet_header(p, bi, be, keep, &hdr);
    const uint32_t b0 = p.bands[bi].first_block;
    const BandGeom& last = p.bands[be - 1];
    const uint32_t b1 = last.first_block + (uint32_t)(last.ncbx * last.ncby);
    packets.push_back({hdr.size(), offsets[b0], offsets[b1]});
    pay += offsets[b1] - offsets[b0];
    bi = be;
  }
  pay += hdr.size();
  std::vector<uint8_t> pre;
  uint32_t psot_pos, jp2c_pos;
  if (!codestream_prefix(p, pay, &pre, &psot_pos, &jp2c_pos, err)) return false;
  std::vector<uint8_t>& o = *out;
  o.resize(pre.size() + pay + 2);
  uint8_t* w = o.data();
  auto put = [&](const uint8_t* src, size_t n) {
    if (n) std::memcpy(w, src, n);
    w += n;
  };
  put(pre.data(), pre.size());
  size_t h0 = 0;
  for (const Packet& k : packets) {
    put(hdr.data() + h0, k.hdr_end - h0);
    put(body + k.body0, k.body1 - k.body0);
    h0 = k.hdr_end;
  }
  const uint8_t eoc[2] = {0xff, 0xd9};
  put(eoc, 2);
  return true;
}

}  // namespace jp2g
