// Seeded synthetic document pages: the input generator for the benchmarks
// and parity tests (no public dataset is involved).
//
// Background: uniform integer 242..248 per pixel. Text lines every 24 px
// (line k spans rows 24k+3 .. 24k+20); dark glyph rectangles 6..14 wide and
// 10..18 tall sit on the line's baseline, value 20 +/- 10, placed left to
// right with gaps of 2..8 px. In sRGB pages each text line gets its own dark
// colour (each channel 10..60). An optional "photo" rectangle holds white
// noise blurred with a sigma = 8 kernel and rescaled to +/-60 around 128
// (independent noise per channel in sRGB).
//
// Everything is integer arithmetic or IEEE add/mul/div in a fixed order, so
// x86 and Arm builds produce identical pages; the blur kernel is the
// binomial B(256, k), whose standard deviation is exactly 8, truncated to
// radius 24 and normalised (no exp()).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  int range(int lo, int hi) { return lo + (int)(next() % (uint64_t)(hi - lo + 1)); }
  double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

void blur_kernel(double* k, int radius) {
  // C(256, 128 + d) / C(256, 128) as a running product.
  k[radius] = 1.0;
  double v = 1.0;
  for (int d = 1; d <= radius; ++d) {
    v = v * (double)(128 - d + 1) / (double)(128 + d);
    k[radius + d] = v;
    k[radius - d] = v;
  }
  double sum = 0.0;
  for (int i = 0; i <= 2 * radius; ++i) sum += k[i];
  for (int i = 0; i <= 2 * radius; ++i) k[i] = k[i] / sum;
}

void photo(uint8_t* out, uint32_t W, int ncomp, int x0, int y0, int pw, int ph, SplitMix64& rng) {
  const int R = 24;
  double k[2 * R + 1];
  blur_kernel(k, R);
  std::vector<double> noise((size_t)pw * ph), tmp((size_t)pw * ph);
  for (int c = 0; c < ncomp; ++c) {
    for (auto& v : noise) v = rng.unit() * 2.0 - 1.0;
    for (int y = 0; y < ph; ++y)  // horizontal, edge-replicated
      for (int x = 0; x < pw; ++x) {
        double s = 0.0;
        for (int t = -R; t <= R; ++t) {
          int xx = std::min(std::max(x + t, 0), pw - 1);
          s = s + k[t + R] * noise[(size_t)y * pw + xx];
        }
        tmp[(size_t)y * pw + x] = s;
      }
    double mx = 0.0;
    for (int y = 0; y < ph; ++y)  // vertical
      for (int x = 0; x < pw; ++x) {
        double s = 0.0;
        for (int t = -R; t <= R; ++t) {
          int yy = std::min(std::max(y + t, 0), ph - 1);
          s = s + k[t + R] * tmp[(size_t)yy * pw + x];
        }
        noise[(size_t)y * pw + x] = s;
        mx = std::max(mx, std::fabs(s));
      }
    double scale = mx > 0.0 ? 60.0 / mx : 0.0;
    for (int y = 0; y < ph; ++y)
      for (int x = 0; x < pw; ++x) {
        double v = std::round(noise[(size_t)y * pw + x] * scale + 128.0);
        v = std::min(std::max(v, 0.0), 255.0);
        int chan = ncomp == 1 ? 0 : c;
        out[((size_t)(y0 + y) * W + (x0 + x)) * ncomp + chan] = (uint8_t)v;
      }
  }
}

}  // namespace

extern "C" {

// Fills `out` (w * h * ncomp bytes, interleaved) with a synthetic page.
// glyphs < 0 selects round(400 * w * h / 512^2). A photo region is drawn
// when photo_w and photo_h are positive, or when photo_frac > 0 (a 4:3
// rectangle of that fraction of the page area). Returns the glyph count.
int jp2g_synth_page(uint8_t* out, uint32_t w, uint32_t h, int ncomp, uint64_t seed, int glyphs,
                    int photo_w, int photo_h, double photo_frac) {
  if (!out || w == 0 || h == 0 || (ncomp != 1 && ncomp != 3)) return -1;
  SplitMix64 rng{seed};
  const size_t n = (size_t)w * h;
  for (size_t i = 0; i < n; ++i) {
    uint8_t v = (uint8_t)rng.range(242, 248);
    for (int c = 0; c < ncomp; ++c) out[i * ncomp + c] = v;
  }
  if (glyphs < 0) glyphs = (int)std::llround(400.0 * (double)w * (double)h / (512.0 * 512.0));
  int placed = 0;
  for (uint32_t line = 0; placed < glyphs; ++line) {
    const int top = 24 * (int)line + 3, bottom = 24 * (int)line + 21;  // exclusive
    if (top >= (int)h) break;
    int col[3];
    for (int c = 0; c < 3; ++c) col[c] = rng.range(10, 60);
    int x = rng.range(2, 8);
    while (placed < glyphs) {
      int gw = rng.range(6, 14), gh = rng.range(10, 18);
      int val = 20 + rng.range(-10, 10);
      if (x + gw > (int)w) break;
      int y1 = std::min(bottom, (int)h), y0 = std::max(bottom - gh, top);
      for (int y = y0; y < y1; ++y)
        for (int xx = x; xx < x + gw; ++xx) {
          uint8_t* p = out + ((size_t)y * w + xx) * ncomp;
          if (ncomp == 1) p[0] = (uint8_t)val;
          else
            for (int c = 0; c < 3; ++c) p[c] = (uint8_t)std::min(std::max(col[c] + (val - 20), 0), 255);
        }
      ++placed;
      x += gw + rng.range(2, 8);
    }
  }
  int pw = photo_w, ph = photo_h;
  if ((pw <= 0 || ph <= 0) && photo_frac > 0.0) {
    double area = photo_frac * (double)w * (double)h;
    pw = (int)std::sqrt(area * 4.0 / 3.0);
    ph = pw * 3 / 4;
  }
  if (pw > 0 && ph > 0) {
    pw = std::min(pw, (int)w);
    ph = std::min(ph, (int)h);
    int x0 = rng.range(0, (int)w - pw), y0 = rng.range(0, (int)h - ph);
    photo(out, w, ncomp, x0, y0, pw, ph, rng);
  }
  return placed;
}

}  // extern "C"
