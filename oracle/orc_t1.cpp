// Oracle (test infrastructure): MQ coder and EBCOT Tier-1 with the
// single-termination policy. Restates src/mq/mod.rs, src/tier1/*.rs and
// src/encode/backend/native/t1.rs. Context tables are generated here from the
// rules of ISO/IEC 15444-1 Annex D (Tables D.1 and D.3) and the probability
// table from Annex C (Table C.2); tests check them against the reference's
// tables.
#include <cstring>

#include "orc.h"

namespace orc {

// Context numbers (src/mq/mod.rs:5-10).
static const int kCtxZC = 0, kCtxSC = 9, kCtxMAG = 14, kCtxAGG = 17, kCtxUNI = 18;
static const int kNumCtx = 19;

// ---------------------------------------------------------------- tables ---
// Annex C Table C.2: Qe, NMPS, NLPS, SWITCH for the 47 probability states.
struct QeRow { uint16_t qe; uint8_t nmps, nlps, sw; };
static const QeRow kQeTable[47] = {
    {0x5601, 1, 1, 1},   {0x3401, 2, 6, 0},   {0x1801, 3, 9, 0},
    {0x0AC1, 4, 12, 0},  {0x0521, 5, 29, 0},  {0x0221, 38, 33, 0},
    {0x5601, 7, 6, 1},   {0x5401, 8, 14, 0},  {0x4801, 9, 14, 0},
    {0x3801, 10, 14, 0}, {0x3001, 11, 17, 0}, {0x2401, 12, 18, 0},
    {0x1C01, 13, 20, 0}, {0x1601, 29, 21, 0}, {0x5601, 15, 14, 1},
    {0x5401, 16, 14, 0}, {0x5101, 17, 15, 0}, {0x4801, 18, 16, 0},
    {0x3801, 19, 17, 0}, {0x3401, 20, 18, 0}, {0x3001, 21, 19, 0},
    {0x2801, 22, 19, 0}, {0x2401, 23, 20, 0}, {0x2201, 24, 21, 0},
    {0x1C01, 25, 22, 0}, {0x1801, 26, 23, 0}, {0x1601, 27, 24, 0},
    {0x1401, 28, 25, 0}, {0x1201, 29, 26, 0}, {0x1101, 30, 27, 0},
    {0x0AC1, 31, 28, 0}, {0x09C1, 32, 29, 0}, {0x08A1, 33, 30, 0},
    {0x0521, 34, 31, 0}, {0x0441, 35, 32, 0}, {0x02A1, 36, 33, 0},
    {0x0221, 37, 34, 0}, {0x0141, 38, 35, 0}, {0x0111, 39, 36, 0},
    {0x0085, 40, 37, 0}, {0x0049, 41, 38, 0}, {0x0025, 42, 39, 0},
    {0x0015, 43, 40, 0}, {0x0009, 44, 41, 0}, {0x0005, 45, 42, 0},
    {0x0001, 45, 43, 0}, {0x5601, 46, 46, 0},
};

// Expanded (state, mps) table, index = 2*state + mps, like the reference's
// 94-entry MQ_STATES (src/mq/mod.rs:434-530).
const MqState* mq_states() {
  static MqState t[94];
  static bool init = false;
  if (!init) {
    for (int s = 0; s < 47; ++s)
      for (int m = 0; m < 2; ++m) {
        MqState& e = t[2 * s + m];
        e.qe = kQeTable[s].qe;
        e.mps = (uint8_t)m;
        e.nmps = (uint8_t)(2 * kQeTable[s].nmps + m);
        e.nlps = (uint8_t)(2 * kQeTable[s].nlps + (m ^ kQeTable[s].sw));
      }
    init = true;
  }
  return t;
}

// Zero-coding context (Table D.1). Neighbour mask bits: NW=0 N=1 NE=2 W=3
// (centre=4, ignored) E=5 SW=6 S=7 SE=8 (src/tier1/consts.rs:1-25).
static int zc_rule(int f, int orient) {
  int h = ((f >> 3) & 1) + ((f >> 5) & 1);
  int v = ((f >> 1) & 1) + ((f >> 7) & 1);
  int d = (f & 1) + ((f >> 2) & 1) + ((f >> 6) & 1) + ((f >> 8) & 1);
  if (orient == HL) std::swap(h, v);
  if (orient != HH) {
    if (h == 2) return 8;
    if (h == 1) return v >= 1 ? 7 : (d >= 1 ? 6 : 5);
    if (v == 2) return 4;
    if (v == 1) return 3;
    return d >= 2 ? 2 : d;
  }
  int hv = h + v;
  if (d >= 3) return 8;
  if (d == 2) return hv >= 1 ? 7 : 6;
  if (d == 1) return hv >= 2 ? 5 : (hv == 1 ? 4 : 3);
  return hv >= 2 ? 2 : hv;
}

// Sign-coding context and sign-prediction bit (Table D.3). Index bits
// (src/tier1/consts.rs:32-39): SGN_W=0 SIG_N=1 SGN_E=2 SIG_W=3 SGN_N=4
// SIG_E=5 SGN_S=6 SIG_S=7. A neighbour contributes +1 if significant and
// positive, -1 if significant and negative; each direction is clamped.
static void sc_rule(int f, int* ctx, int* spb) {
  auto contrib = [&](int sig_bit, int sgn_bit) {
    if (!((f >> sig_bit) & 1)) return std::make_pair(0, 0);
    return ((f >> sgn_bit) & 1) ? std::make_pair(0, 1) : std::make_pair(1, 0);
  };
  auto w = contrib(3, 0), e = contrib(5, 2), n = contrib(1, 4), s = contrib(7, 6);
  int hp = w.first + e.first, hn = w.second + e.second;
  int vp = n.first + s.first, vn = n.second + s.second;
  int H = std::min(hp, 1) - std::min(hn, 1);
  int V = std::min(vp, 1) - std::min(vn, 1);
  // (H, V) -> (context, xor bit)
  int c = 9, x = 0;
  if (H == 1) { c = V == 1 ? 13 : V == 0 ? 12 : 11; x = 0; }
  else if (H == 0) { c = V == 0 ? 9 : 10; x = V == -1 ? 1 : 0; }
  else { c = V == 1 ? 11 : V == 0 ? 12 : 13; x = 1; }
  *ctx = c;
  *spb = x;
}

static uint8_t g_zc[4][512], g_sc[256], g_spb[256];
static bool g_tables = false;
static void init_tables() {
  if (g_tables) return;
  for (int o = 0; o < 4; ++o)
    for (int f = 0; f < 512; ++f) g_zc[o][f] = (uint8_t)zc_rule(f, o);
  for (int f = 0; f < 256; ++f) {
    int c, x;
    sc_rule(f, &c, &x);
    g_sc[f] = (uint8_t)c;
    g_spb[f] = (uint8_t)x;
  }
  g_tables = true;
}
const uint8_t* zc_lut() { init_tables(); return &g_zc[0][0]; }
const uint8_t* sc_lut() { init_tables(); return g_sc; }
const uint8_t* spb_lut() { init_tables(); return g_spb; }

// ------------------------------------------------------------ MQ encoder ---
// src/mq/mod.rs:163-432. out[0] is the pre-byte; `pos` indexes the last
// written byte, numbytes() == pos.
struct Mq {
  uint32_t a = 0x8000, c = 0, ct = 12;
  std::vector<uint8_t> out{0};
  size_t pos = 0;
  uint8_t ctx[kNumCtx];
  Mq() { reset_ctx(); }
  void reset_ctx() {  // src/mq/mod.rs:195-200
    std::memset(ctx, 0, sizeof ctx);
    ctx[kCtxUNI] = 0 + (46 << 1);
    ctx[kCtxAGG] = 0 + (3 << 1);
    ctx[kCtxZC] = 0 + (4 << 1);
  }
  void write_next(uint8_t b) {
    ++pos;
    if (pos == out.size()) out.push_back(b); else out[pos] = b;
  }
  void byteout() {  // src/mq/mod.rs:382-404
    if (out[pos] == 0xff) {
      write_next((uint8_t)(c >> 20));
      c &= 0xfffff;
      ct = 7;
    } else if ((c & 0x8000000) == 0) {
      write_next((uint8_t)(c >> 19));
      c &= 0x7ffff;
      ct = 8;
    } else {
      out[pos] = (uint8_t)(out[pos] + 1);
      if (out[pos] == 0xff) {
        c &= 0x7ffffff;
        write_next((uint8_t)(c >> 20));
        c &= 0xfffff;
        ct = 7;
      } else {
        write_next((uint8_t)(c >> 19));
        c &= 0x7ffff;
        ct = 8;
      }
    }
  }
  void renorme() {
    while ((a & 0x8000) == 0) {
      a <<= 1;
      c <<= 1;
      if (--ct == 0) byteout();
    }
  }
  void encode(int cx, int bit) {  // src/mq/mod.rs:213-242
    const MqState& s = mq_states()[ctx[cx]];
    if (bit == s.mps) {
      a -= s.qe;
      if ((a & 0x8000) == 0) {
        if (a < s.qe) a = s.qe; else c += s.qe;
        ctx[cx] = s.nmps;
        renorme();
      } else {
        c += s.qe;
      }
    } else {
      a -= s.qe;
      if (a < s.qe) c += s.qe; else a = s.qe;
      ctx[cx] = s.nlps;
      renorme();
    }
  }
  void setbits() {
    uint32_t t = c + a;
    c |= 0xffff;
    if (c >= t) c -= 0x8000;
  }
  void flush() {  // src/mq/mod.rs:244-250
    setbits();
    c <<= ct;
    byteout();
    c <<= ct;
    byteout();
  }
  std::vector<uint8_t> take_bytes() const {  // src/mq/mod.rs:416-423
    size_t end = out[pos] == 0xff ? pos : pos + 1;
    return std::vector<uint8_t>(out.begin() + 1, out.begin() + end);
  }
  std::vector<uint8_t> erterm() {  // src/mq/mod.rs:274-286
    int k = 11 - (int)ct + 1;
    while (k > 0) {
      c <<= ct;
      ct = 0;
      byteout();
      k -= (int)ct;
    }
    if (out[pos] != 0xff) byteout();
    return std::vector<uint8_t>(out.begin() + 1, out.begin() + pos);
  }
  size_t numbytes() const { return pos; }
};

std::vector<uint8_t> mq_encode(const uint8_t* syms, size_t n) {
  Mq m;
  for (size_t i = 0; i < n; ++i) m.encode(syms[i] >> 1, syms[i] & 1);
  m.flush();
  return m.take_bytes();
}

std::vector<uint8_t> mq_erterm(const uint8_t* syms, size_t n) {
  Mq m;
  for (size_t i = 0; i < n; ++i) m.encode(syms[i] >> 1, syms[i] & 1);
  return m.erterm();
}

// Second, independently structured encoder in the manner of the C model the
// reference cross-checks against (src/mq/mod.rs:533-719): explicit code-MPS /
// code-LPS procedures, a fixed output array with a byte pointer, and the
// trailing-0xFF rule applied inside flush.
std::vector<uint8_t> mq_encode_alt(const uint8_t* syms, size_t n) {
  std::vector<uint8_t> buf(16 + 4 * n + 16, 0);
  size_t bp = 0;
  uint32_t A = 0x8000, C = 0, CT = 12;
  int st[kNumCtx] = {0};
  st[kCtxUNI] = 92;
  st[kCtxAGG] = 6;
  st[kCtxZC] = 8;
  const MqState* T = mq_states();
  auto byteout = [&]() {
    if (buf[bp] == 0xff) {
      buf[++bp] = (uint8_t)(C >> 20); C &= 0xfffff; CT = 7;
    } else if (!(C & 0x8000000)) {
      buf[++bp] = (uint8_t)(C >> 19); C &= 0x7ffff; CT = 8;
    } else {
      buf[bp]++;
      if (buf[bp] == 0xff) {
        C &= 0x7ffffff; buf[++bp] = (uint8_t)(C >> 20); C &= 0xfffff; CT = 7;
      } else {
        buf[++bp] = (uint8_t)(C >> 19); C &= 0x7ffff; CT = 8;
      }
    }
  };
  auto renorm = [&]() {
    do {
      A <<= 1; C <<= 1;
      if (--CT == 0) byteout();
    } while (!(A & 0x8000));
  };
  for (size_t i = 0; i < n; ++i) {
    int cx = syms[i] >> 1, d = syms[i] & 1;
    const MqState& s = T[st[cx]];
    if (s.mps == d) {
      A -= s.qe;
      if (!(A & 0x8000)) {
        if (A < s.qe) A = s.qe; else C += s.qe;
        st[cx] = s.nmps;
        renorm();
      } else {
        C += s.qe;
      }
    } else {
      A -= s.qe;
      if (A < s.qe) C += s.qe; else A = s.qe;
      st[cx] = s.nlps;
      renorm();
    }
  }
  uint32_t t = C + A;
  C |= 0xffff;
  if (C >= t) C -= 0x8000;
  C <<= CT; byteout();
  C <<= CT; byteout();
  if (buf[bp] != 0xff) ++bp;
  return std::vector<uint8_t>(buf.begin() + 1, buf.begin() + bp);
}

// ------------------------------------------------------------ MQ decoder ---
// src/mq/mod.rs:38-160 (INITDEC / DECODE / RENORMD / BYTEIN).
struct MqDec {
  const uint8_t* b;
  size_t n, bp = 0;
  uint32_t a = 0x8000, c, ct = 0;
  uint8_t ctx[kNumCtx];
  uint8_t at(size_t i) const { return i < n ? b[i] : 0xff; }
  MqDec(const uint8_t* bytes, size_t len) : b(bytes), n(len) {
    c = n == 0 ? (0xffu << 16) : ((uint32_t)b[0] << 16);
    std::memset(ctx, 0, sizeof ctx);
    ctx[kCtxUNI] = 92; ctx[kCtxAGG] = 6; ctx[kCtxZC] = 8;
    bytein();
    c <<= 7;
    ct = ct >= 7 ? ct - 7 : 0;
  }
  void bytein() {
    uint8_t next = at(bp + 1);
    if (at(bp) == 0xff) {
      if (next > 0x8f) { c += 0xff00; ct = 8; }
      else { ++bp; c += (uint32_t)next << 9; ct = 7; }
    } else {
      ++bp; c += (uint32_t)next << 8; ct = 8;
    }
  }
  int decode(int cx) {
    const MqState& s = mq_states()[ctx[cx]];
    a -= s.qe;
    int bit;
    if ((c >> 16) < s.qe) {
      uint32_t post = a;
      a = s.qe;
      if (post < s.qe) { ctx[cx] = s.nmps; bit = s.mps; }
      else { ctx[cx] = s.nlps; bit = 1 ^ s.mps; }
    } else {
      c -= (uint32_t)s.qe << 16;
      if ((a & 0x8000) == 0) {
        if (a < s.qe) { ctx[cx] = s.nlps; bit = 1 ^ s.mps; }
        else { ctx[cx] = s.nmps; bit = s.mps; }
      } else {
        bit = s.mps;
      }
    }
    while (a < 0x8000) {
      if (ct == 0) bytein();
      a <<= 1; c <<= 1; --ct;
    }
    return bit;
  }
};

void mq_decode(const uint8_t* bytes, size_t nbytes, const uint8_t* ctxs,
               size_t n, uint8_t* bits_out) {
  MqDec d(bytes, nbytes);
  for (size_t i = 0; i < n; ++i) bits_out[i] = (uint8_t)d.decode(ctxs[i]);
}

// ------------------------------------------------------------- flag grid ---
// src/tier1/flags.rs:33-296: per-sample significance / visited / refined /
// sign bits plus the 8 neighbour-significance bits.
namespace {
enum : uint16_t {
  F_SIG = 1, F_VIS = 2, F_REF = 4, F_SGN = 8,
  N_W = 1 << 4, N_E = 1 << 5, N_N = 1 << 6, N_S = 1 << 7,
  N_NW = 1 << 8, N_NE = 1 << 9, N_SW = 1 << 10, N_SE = 1 << 11,
};
const uint16_t N_ANY = N_W | N_E | N_N | N_S | N_NW | N_NE | N_SW | N_SE;

struct Grid {
  int w, h;
  std::vector<uint16_t> f;
  Grid(int w_, int h_) : w(w_), h(h_), f((size_t)w_ * h_, 0) {}
  uint16_t& at(int x, int y) { return f[(size_t)y * w + x]; }
  bool sig(int x, int y) { return at(x, y) & F_SIG; }
  bool vis(int x, int y) { return at(x, y) & F_VIS; }
  bool ref(int x, int y) { return at(x, y) & F_REF; }
  void mark_sig(int x, int y, int sign) {
    uint16_t& c = at(x, y);
    c |= F_SIG;
    if (sign) c |= F_SGN; else c &= (uint16_t)~F_SGN;
    if (x > 0) at(x - 1, y) |= N_E;
    if (x + 1 < w) at(x + 1, y) |= N_W;
    if (y > 0) at(x, y - 1) |= N_S;
    if (y + 1 < h) at(x, y + 1) |= N_N;
    if (x > 0 && y > 0) at(x - 1, y - 1) |= N_SE;
    if (x + 1 < w && y > 0) at(x + 1, y - 1) |= N_SW;
    if (x > 0 && y + 1 < h) at(x - 1, y + 1) |= N_NE;
    if (x + 1 < w && y + 1 < h) at(x + 1, y + 1) |= N_NW;
  }
  int nmask(int x, int y) {  // T1_SIGMA layout
    uint16_t v = at(x, y);
    int m = 0;
    if (v & N_NW) m |= 1 << 0;
    if (v & N_N) m |= 1 << 1;
    if (v & N_NE) m |= 1 << 2;
    if (v & N_W) m |= 1 << 3;
    if (v & N_E) m |= 1 << 5;
    if (v & N_SW) m |= 1 << 6;
    if (v & N_S) m |= 1 << 7;
    if (v & N_SE) m |= 1 << 8;
    return m;
  }
  int sign_index(int x, int y) {  // src/tier1/flags.rs:237-296
    auto nb = [&](int nx, int ny, bool* s, int* sg) {
      if (nx < 0 || ny < 0 || nx >= w || ny >= h) { *s = false; *sg = 0; return; }
      uint16_t v = at(nx, ny);
      *s = v & F_SIG;
      *sg = (v & F_SGN) ? 1 : 0;
    };
    bool ws, ns, es, ss;
    int wg, ng, eg, sgg;
    nb(x - 1, y, &ws, &wg);
    nb(x, y - 1, &ns, &ng);
    nb(x + 1, y, &es, &eg);
    nb(x, y + 1, &ss, &sgg);
    int lu = 0;  // src/tier1/helpers.rs:52-88
    if (ws) { lu |= 1 << 3; if (wg) lu |= 1 << 0; }
    if (ns) { lu |= 1 << 1; if (ng) lu |= 1 << 4; }
    if (es) { lu |= 1 << 5; if (eg) lu |= 1 << 2; }
    if (ss) { lu |= 1 << 7; if (sgg) lu |= 1 << 6; }
    return lu;
  }
  bool stripe_clean(int x, int k) {
    for (int ci = 0; ci < 4; ++ci) {
      int y = k + ci;
      if (y >= h) break;
      if (at(x, y) & (F_SIG | F_VIS | N_ANY)) return false;
    }
    return true;
  }
  void clear_vis_all() {
    for (auto& v : f) v &= (uint16_t)~F_VIS;
  }
};

static inline int mag_ctx(bool nb, bool refined) {  // src/tier1/helpers.rs:36-50
  if (refined) return kCtxMAG + 2;
  return nb ? kCtxMAG + 1 : kCtxMAG;
}
}  // namespace

// Single-termination code-block encoder (src/encode/backend/native/t1.rs:508-658).
EncBlock encode_block(const int32_t* coefs, int w, int h, Band band, int mb) {
  init_tables();
  EncBlock out{};
  out.band = band;
  uint32_t maxm = 0;
  size_t nnz = 0, count = (size_t)w * h;
  for (size_t i = 0; i < count; ++i) {  // analyze_codeblock (t1.rs:215-258)
    uint32_t m = coefs[i] < 0 ? (uint32_t)(-(int64_t)coefs[i]) : (uint32_t)coefs[i];
    if (m > maxm) maxm = m;
    if (coefs[i] != 0) ++nnz;
  }
  out.max_mag = maxm;
  out.mbp = maxm == 0 ? 0 : 32 - __builtin_clz(maxm);
  out.zbp = mb > out.mbp ? mb - out.mbp : 0;
  float frac = count == 0 ? 0.0f : (float)nnz / (float)count;
  // classify_from_nonzero_fraction (src/profile.rs:122-130)
  out.cls = frac <= 0.05f ? 0 : (frac <= 0.30f ? 1 : 2);
  if (out.mbp == 0) {
    out.cls = 0;  // empty blocks report BlockClass::Flat (t1.rs:330-342)
    return out;
  }
  const uint8_t* zc = &g_zc[band][0];
  Grid g(w, h);
  Mq mq;
  auto magv = [&](int x, int y) {
    int32_t v = coefs[(size_t)y * w + x];
    return v < 0 ? (uint32_t)(-(int64_t)v) : (uint32_t)v;
  };
  struct Meta { int kind, bp; uint32_t ns; size_t snap; uint32_t sb; };
  std::vector<Meta> metas;
  uint32_t sig_so_far = 0;
  const int full = h / 4 * 4, rem = h % 4;

  // Regular (non-AGG) cleanup step (t1.rs:1150-1197).
  auto cl_regular = [&](int x, int y, uint32_t one, uint32_t& ns) {
    if (g.sig(x, y) || g.vis(x, y)) {
      g.at(x, y) &= (uint16_t)~F_VIS;
      return;
    }
    int nm = g.nmask(x, y);
    int cx = nm ? zc[nm] : kCtxZC;
    int bit = (magv(x, y) & one) ? 1 : 0;
    mq.encode(cx, bit);
    g.at(x, y) &= (uint16_t)~F_VIS;
    if (bit) {
      int sb = coefs[(size_t)y * w + x] < 0;
      int lu = g.sign_index(x, y);
      mq.encode(g_sc[lu], sb ^ g_spb[lu]);
      g.mark_sig(x, y, sb);
      ++ns;
    }
  };
  // Cleanup pass (t1.rs:977-1148).
  auto cleanup = [&](int bp) {
    uint32_t one = 1u << bp, ns = 0;
    for (int k = 0; k < full; k += 4)
      for (int x = 0; x < w; ++x) {
        if (g.stripe_clean(x, k)) {
          int rl = -1;
          for (int ci = 0; ci < 4; ++ci)
            if (magv(x, k + ci) & one) { rl = ci; break; }
          if (rl >= 0) {
            mq.encode(kCtxAGG, 1);
            mq.encode(kCtxUNI, (rl >> 1) & 1);
            mq.encode(kCtxUNI, rl & 1);
            int y = k + rl;
            int sb = coefs[(size_t)y * w + x] < 0;
            int lu = g.sign_index(x, y);
            mq.encode(g_sc[lu], sb ^ g_spb[lu]);
            g.mark_sig(x, y, sb);
            ++ns;
            g.at(x, y) &= (uint16_t)~F_VIS;
            for (int ci = rl + 1; ci < 4; ++ci) cl_regular(x, k + ci, one, ns);
          } else {
            mq.encode(kCtxAGG, 0);
            for (int ci = 0; ci < 4; ++ci) g.at(x, k + ci) &= (uint16_t)~F_VIS;
          }
        } else {
          for (int ci = 0; ci < 4; ++ci) cl_regular(x, k + ci, one, ns);
        }
      }
    if (rem > 0)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < rem; ++ci) cl_regular(x, full + ci, one, ns);
    return ns;
  };
  // Significance propagation (t1.rs:805-905).
  auto sigpass = [&](int bp) {
    uint32_t one = 1u << bp, ns = 0;
    auto step = [&](int x, int y) {
      if (g.sig(x, y)) return;
      int nm = g.nmask(x, y);
      if (nm == 0) return;
      int bit = (magv(x, y) & one) ? 1 : 0;
      mq.encode(zc[nm], bit);
      g.at(x, y) |= F_VIS;
      if (bit) {
        int sb = coefs[(size_t)y * w + x] < 0;
        int lu = g.sign_index(x, y);
        mq.encode(g_sc[lu], sb ^ g_spb[lu]);
        g.mark_sig(x, y, sb);
        ++ns;
      }
    };
    for (int k = 0; k < full; k += 4)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < 4; ++ci) step(x, k + ci);
    if (rem > 0)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < rem; ++ci) step(x, full + ci);
    return ns;
  };
  // Magnitude refinement (t1.rs:914-965).
  auto refpass = [&](int bp) {
    uint32_t one = 1u << bp;
    auto step = [&](int x, int y) {
      if (!g.sig(x, y) || g.vis(x, y)) return;
      int cx = mag_ctx(g.nmask(x, y) != 0, g.ref(x, y));
      mq.encode(cx, (magv(x, y) & one) ? 1 : 0);
      g.at(x, y) |= F_REF;
    };
    for (int k = 0; k < full; k += 4)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < 4; ++ci) step(x, k + ci);
    if (rem > 0)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < rem; ++ci) step(x, full + ci);
  };

  int top = out.mbp - 1;
  uint32_t ns = cleanup(top);
  metas.push_back({kCL, top, ns, mq.numbytes(), 0});
  sig_so_far += ns;
  g.clear_vis_all();
  for (int bp = top - 1; bp >= 0; --bp) {
    uint32_t before = sig_so_far;
    uint32_t sp = sigpass(bp);
    metas.push_back({kSP, bp, sp, mq.numbytes(), before});
    sig_so_far += sp;
    refpass(bp);
    metas.push_back({kMR, bp, 0, mq.numbytes(), before});
    uint32_t cl = cleanup(bp);
    metas.push_back({kCL, bp, cl, mq.numbytes(), sig_so_far});
    sig_so_far += cl;
    g.clear_vis_all();
  }
  // Single termination (t1.rs:580-607).
  mq.flush();
  std::vector<uint8_t> term = mq.take_bytes();
  size_t total = term.size(), prev = 0, sum = 0, cum = 0;
  for (size_t i = 0; i < metas.size(); ++i) {
    size_t len = metas[i].snap >= prev ? metas[i].snap - prev : 0;
    prev = metas[i].snap;
    bool last = i + 1 == metas.size();
    if (last) len = total >= sum ? total - sum : 0;
    sum += len;
    cum += len;
    Pass p;
    p.kind = metas[i].kind;
    p.bitplane = metas[i].bp;
    p.ns = metas[i].ns;
    p.sig_before = metas[i].sb;
    p.length = (uint32_t)len;
    p.cumulative = (uint32_t)cum;
    p.terminated = last;
    out.passes.push_back(p);
  }
  out.payload = std::move(term);
  return out;
}

// ------------------------------------------------------- Tier-1 decoding ---
// Code-block decoder used for round trips (src/decode/t1.rs:87-400).
std::vector<int32_t> decode_block(const uint8_t* data, size_t n, int w, int h,
                                  Band band, int mb, int zbp, int npasses, bool allow_empty = false);

// allow_empty: a segment of zero bytes is decoded (every byte read as 0xFF,
// ISO/IEC 15444-1 C.3.4) instead of rejected as decode/t1.rs:109-111 does.
std::vector<int32_t> decode_block(const uint8_t* data, size_t n, int w, int h,
                                  Band band, int mb, int zbp, int npasses, bool allow_empty) {
  init_tables();
  std::vector<int32_t> outc((size_t)w * h, 0);
  if (npasses == 0) return outc;
  if (n == 0 && !allow_empty) throw Error(kDecodeFailed, "non-empty code-block has no compressed bytes");
  if (zbp > mb) throw Error(kDecodeFailed, "zero-bitplane count exceeds subband bit-plane count");
  int mbp = mb - zbp;
  if (mbp == 0) throw Error(kDecodeFailed, "non-empty code-block has no magnitude bit-planes");
  int maxp = 1 + 3 * (mbp - 1);
  if (npasses > maxp) throw Error(kDecodeFailed, "code-block pass count exceeds maximum");
  std::vector<uint32_t> mag((size_t)w * h, 0);
  std::vector<uint8_t> sgn((size_t)w * h, 0);
  const uint8_t* zc = &g_zc[band][0];
  Grid g(w, h);
  MqDec d(data, n);
  const int full = h / 4 * 4, rem = h % 4;
  auto idx = [&](int x, int y) { return (size_t)y * w + x; };
  auto sign_dec = [&](int x, int y) {
    int lu = g.sign_index(x, y);
    int s = d.decode(g_sc[lu]) ^ g_spb[lu];
    sgn[idx(x, y)] = (uint8_t)s;
    g.mark_sig(x, y, s);
  };
  auto cl_regular = [&](int x, int y, uint32_t one) {
    if (g.sig(x, y) || g.vis(x, y)) { g.at(x, y) &= (uint16_t)~F_VIS; return; }
    int nm = g.nmask(x, y);
    int bit = d.decode(nm ? zc[nm] : kCtxZC);
    g.at(x, y) &= (uint16_t)~F_VIS;
    if (bit) { mag[idx(x, y)] |= one; sign_dec(x, y); }
  };
  auto cleanup = [&](int bp) {
    uint32_t one = 1u << bp;
    for (int k = 0; k < full; k += 4)
      for (int x = 0; x < w; ++x) {
        if (g.stripe_clean(x, k)) {
          if (d.decode(kCtxAGG) == 0) {
            for (int ci = 0; ci < 4; ++ci) g.at(x, k + ci) &= (uint16_t)~F_VIS;
            continue;
          }
          int rl = d.decode(kCtxUNI) << 1;
          rl |= d.decode(kCtxUNI);
          int y = k + rl;
          mag[idx(x, y)] |= one;
          sign_dec(x, y);
          g.at(x, y) &= (uint16_t)~F_VIS;
          for (int ci = rl + 1; ci < 4; ++ci) cl_regular(x, k + ci, one);
        } else {
          for (int ci = 0; ci < 4; ++ci) cl_regular(x, k + ci, one);
        }
      }
    if (rem > 0)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < rem; ++ci) cl_regular(x, full + ci, one);
  };
  auto sigpass = [&](int bp) {
    uint32_t one = 1u << bp;
    auto step = [&](int x, int y) {
      if (g.sig(x, y)) return;
      int nm = g.nmask(x, y);
      if (nm == 0) return;
      int bit = d.decode(zc[nm]);
      g.at(x, y) |= F_VIS;
      if (bit) { mag[idx(x, y)] |= one; sign_dec(x, y); }
    };
    for (int k = 0; k < full; k += 4)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < 4; ++ci) step(x, k + ci);
    if (rem > 0)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < rem; ++ci) step(x, full + ci);
  };
  auto refpass = [&](int bp) {
    uint32_t one = 1u << bp;
    auto step = [&](int x, int y) {
      if (!g.sig(x, y) || g.vis(x, y)) return;
      int bit = d.decode(mag_ctx(g.nmask(x, y) != 0, g.ref(x, y)));
      if (bit) mag[idx(x, y)] |= one;
      g.at(x, y) |= F_REF;
    };
    for (int k = 0; k < full; k += 4)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < 4; ++ci) step(x, k + ci);
    if (rem > 0)
      for (int x = 0; x < w; ++x)
        for (int ci = 0; ci < rem; ++ci) step(x, full + ci);
  };
  int remaining = npasses;
  int top = mbp - 1;
  cleanup(top);
  --remaining;
  g.clear_vis_all();
  for (int bp = top - 1; bp >= 0 && remaining > 0; --bp) {
    sigpass(bp);
    if (--remaining == 0) break;
    refpass(bp);
    if (--remaining == 0) break;
    cleanup(bp);
    --remaining;
    g.clear_vis_all();
  }
  for (size_t i = 0; i < outc.size(); ++i)
    outc[i] = sgn[i] ? -(int32_t)mag[i] : (int32_t)mag[i];
  return outc;
}

}  // namespace orc
