// Tier-1 context tables and the MQ probability-state table, derived on the
// host from ISO/IEC 15444-1 and uploaded to constant memory.
//
// Zero-coding contexts follow Table D.1 (HL swaps the horizontal and
// vertical neighbour counts; HH keys on diagonals), sign contexts and the
// sign-prediction bit follow Table D.3, and the 47-state probability table
// follows Table C.2. The neighbour-mask and sign-index bit layouts are the
// ones jp2lam indexes its tables with (src/tier1/consts.rs:1-39); the
// expanded state table is indexed by 2*state + MPS like src/mq/mod.rs:434-530.
#include <algorithm>
#include <cstdint>

namespace jp2g {

bool upload_t1_tables(const uint8_t* zc, const uint8_t* sc, const uint8_t* spb,
                      const uint32_t* mq);
bool upload_decode_tables(const uint8_t* zc, const uint8_t* sc, const uint8_t* spb, const uint32_t* mq);

namespace {

struct QeEntry {
  uint16_t qe;
  uint8_t next_mps, next_lps, switch_mps;
};

// Table C.2.
const QeEntry kQe[47] = {
    {0x5601, 1, 1, 1},   {0x3401, 2, 6, 0},   {0x1801, 3, 9, 0},   {0x0AC1, 4, 12, 0},
    {0x0521, 5, 29, 0},  {0x0221, 38, 33, 0}, {0x5601, 7, 6, 1},   {0x5401, 8, 14, 0},
    {0x4801, 9, 14, 0},  {0x3801, 10, 14, 0}, {0x3001, 11, 17, 0}, {0x2401, 12, 18, 0},
    {0x1C01, 13, 20, 0}, {0x1601, 29, 21, 0}, {0x5601, 15, 14, 1}, {0x5401, 16, 14, 0},
    {0x5101, 17, 15, 0}, {0x4801, 18, 16, 0}, {0x3801, 19, 17, 0}, {0x3401, 20, 18, 0},
    {0x3001, 21, 19, 0}, {0x2801, 22, 19, 0}, {0x2401, 23, 20, 0}, {0x2201, 24, 21, 0},
    {0x1C01, 25, 22, 0}, {0x1801, 26, 23, 0}, {0x1601, 27, 24, 0}, {0x1401, 28, 25, 0},
    {0x1201, 29, 26, 0}, {0x1101, 30, 27, 0}, {0x0AC1, 31, 28, 0}, {0x09C1, 32, 29, 0},
    {0x08A1, 33, 30, 0}, {0x0521, 34, 31, 0}, {0x0441, 35, 32, 0}, {0x02A1, 36, 33, 0},
    {0x0221, 37, 34, 0}, {0x0141, 38, 35, 0}, {0x0111, 39, 36, 0}, {0x0085, 40, 37, 0},
    {0x0049, 41, 38, 0}, {0x0025, 42, 39, 0}, {0x0015, 43, 40, 0}, {0x0009, 44, 41, 0},
    {0x0005, 45, 42, 0}, {0x0001, 45, 43, 0}, {0x5601, 46, 46, 0},
};

int zero_coding(int mask, int orient) {
  int h = ((mask >> 3) & 1) + ((mask >> 5) & 1);  // W, E
  int v = ((mask >> 1) & 1) + ((mask >> 7) & 1);  // N, S
  int d = (mask & 1) + ((mask >> 2) & 1) + ((mask >> 6) & 1) + ((mask >> 8) & 1);
  if (orient == 3) {  // HH
    int hv = h + v;
    if (d >= 3) return 8;
    if (d == 2) return hv ? 7 : 6;
    if (d == 1) return hv >= 2 ? 5 : (hv == 1 ? 4 : 3);
    return std::min(hv, 2);
  }
  if (orient == 1) std::swap(h, v);  // HL
  if (h == 2) return 8;
  if (h == 1) return v ? 7 : (d ? 6 : 5);
  if (v == 2) return 4;
  if (v == 1) return 3;
  return std::min(d, 2);
}

// Horizontal/vertical sign contributions clamped to [-1, 1] -> (ctx, xor).
void sign_coding(int lu, uint8_t* ctx, uint8_t* xr) {
  auto side = [&](int sig_bit, int neg_bit, int* pos, int* neg) {
    if ((lu >> sig_bit) & 1) {
      if ((lu >> neg_bit) & 1) ++*neg;
      else ++*pos;
    }
  };
  int hp = 0, hn = 0, vp = 0, vn = 0;
  side(3, 0, &hp, &hn);  // W
  side(5, 2, &hp, &hn);  // E
  side(1, 4, &vp, &vn);  // N
  side(7, 6, &vp, &vn);  // S
  int H = std::min(hp, 1) - std::min(hn, 1);
  int V = std::min(vp, 1) - std::min(vn, 1);
  int c, x;
  if (H == 0) {
    c = V == 0 ? 9 : 10;
    x = V < 0;
  } else {
    int hv = H * V;  // same sign -> 13, opposite -> 11, V == 0 -> 12
    c = hv > 0 ? 13 : (hv < 0 ? 11 : 12);
    x = H < 0;
  }
  *ctx = (uint8_t)c;
  *xr = (uint8_t)x;
}

}  // namespace

void build_t1_tables(uint8_t* zc, uint8_t* sc, uint8_t* spb, uint32_t* mq) {
  for (int o = 0; o < 4; ++o)
    for (int f = 0; f < 512; ++f) zc[o * 512 + f] = (uint8_t)zero_coding(f, o);
  for (int f = 0; f < 256; ++f) sign_coding(f, &sc[f], &spb[f]);
  for (int s = 0; s < 47; ++s)
    for (int mps = 0; mps < 2; ++mps) {
      uint32_t nm = 2u * kQe[s].next_mps + (uint32_t)mps;
      uint32_t nl = 2u * kQe[s].next_lps + (uint32_t)(mps ^ kQe[s].switch_mps);
      mq[2 * s + mps] = kQe[s].qe | (nm << 16) | (nl << 24);
    }
}

bool init_t1_tables() {
  uint8_t zc[2048], sc[256], spb[256];
  uint32_t mq[94];
  build_t1_tables(zc, sc, spb, mq);
  return upload_t1_tables(zc, sc, spb, mq) && upload_decode_tables(zc, sc, spb, mq);
}

}  // namespace jp2g
