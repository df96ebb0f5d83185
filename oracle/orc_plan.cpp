// Oracle (test infrastructure): encoding plan, step sizes and quantiser
// parameters. Restates src/plan/{mod,derive,validate}.rs and src/dwt/norms.rs.
#include <cmath>

#include "orc.h"

namespace orc {

// 9/7 synthesis norms per orientation and decomposition level
// (src/dwt/norms.rs:21-34). A data table that the step sizes and PCRD
// weights are defined by; kept value-for-value.
static const double kNorms97[4][10] = {
    {1.000, 1.965, 4.177, 8.403, 16.90, 33.84, 67.69, 135.3, 270.6, 540.9},
    {2.022, 3.989, 8.355, 17.04, 34.27, 68.63, 137.3, 274.6, 549.0, 0.0},
    {2.022, 3.989, 8.355, 17.04, 34.27, 68.63, 137.3, 274.6, 549.0, 0.0},
    {2.080, 3.865, 8.307, 17.18, 34.71, 69.59, 139.3, 278.6, 557.2, 0.0},
};

double get_norm_97(int level, Band band) {  // src/dwt/norms.rs:47-55
  int o = static_cast<int>(band);
  int cap = (o == 0) ? 9 : 8;
  int l = level < cap ? level : cap;
  return kNorms97[o][l];
}

int band_gain(Band b) {  // src/dwt/norms.rs:57-63
  switch (b) {
    case LL: return 0;
    case HL: case LH: return 1;
    default: return 2;
  }
}

static int floor_log2_i(int v) {  // src/dwt/norms.rs:94-96
  if (v < 1) v = 1;
  return 31 - __builtin_clz(static_cast<unsigned>(v));
}

void encode_stepsize(int stepsize, int numbps, int* exponent, int* mantissa) {
  // src/dwt/norms.rs:85-92
  int p = floor_log2_i(stepsize) - 13;
  int n = 11 - floor_log2_i(stepsize);
  int m = (n < 0 ? (stepsize >> -n) : (stepsize << n)) & 0x7ff;
  int e = numbps - p;
  if (e < 0) e = 0;
  *exponent = e & 0xff;
  *mantissa = m;
}

void irreversible_expounded_quant(int precision, int nres, int res, Band band,
                                  int* exponent, int* mantissa) {
  // src/dwt/norms.rs:70-83
  int gain = band_gain(band);
  int level = nres - 1;
  if (level < 0) level = 0;
  level -= res;
  if (level < 0) level = 0;
  double norm = get_norm_97(level, band);
  double stepsize = static_cast<double>(1u << gain) / norm;
  encode_stepsize(static_cast<int>(std::floor(stepsize * 8192.0)),
                  precision + gain, exponent, mantissa);
}

double quality_step_scaler(int q) {  // src/plan/derive.rs:74-86
  if (q == 0) return 8.0;
  if (q <= 50) return std::pow(2.0, (50.0 - static_cast<double>(q)) / 20.0);
  if (q <= 90) return std::pow(2.0, -((static_cast<double>(q) - 50.0) / 20.0));
  double t = (static_cast<double>(q) - 90.0) / 9.0;
  return 0.25 * std::pow(2.0, -3.0 * t);
}

static SubbandQuant scale_one_quant(const SubbandQuant& sq, double scale) {
  // src/plan/derive.rs:94-107
  double base = 1.0 + static_cast<double>(sq.mantissa) / 2048.0;
  double scaled = base * scale;
  if (scaled < 1.0 / 8192.0) scaled = 1.0 / 8192.0;
  int k = static_cast<int>(std::floor(std::log2(scaled)));
  double base_new = scaled / std::ldexp(1.0, k);
  int e = sq.exponent - k;
  if (e < 0) e = 0;
  double m = std::round((base_new - 1.0) * 2048.0);
  if (m < 0.0) m = 0.0;
  if (m > 2047.0) m = 2047.0;
  SubbandQuant out = sq;
  out.exponent = e & 0xff;
  out.mantissa = static_cast<int>(m);
  return out;
}

int max_decompositions(uint32_t w, uint32_t h) {  // src/plan/derive.rs:128-139
  uint32_t m = w < h ? w : h;
  if (m <= 1) return 0;
  if (m < 32) return 31 - __builtin_clz(m);
  uint32_t ratio = m / 32;
  int l = 1 + (31 - __builtin_clz(ratio));
  return l < 6 ? l : 6;
}

float quant_step_f32(int precision, Band band, int exponent, int mantissa) {
  // src/encode/backend/native/backend.rs:602-620
  int numbps = precision + band_gain(band);
  float base = 1.0f + static_cast<float>(mantissa) / 2048.0f;
  float s = base * std::ldexp(1.0f, numbps - exponent);
  return s > 1e-6f ? s : 1e-6f;
}

double quant_step_f64(int precision, Band band, int exponent, int mantissa) {
  // src/encode/backend/native/rate.rs:316-320
  int numbps = precision + band_gain(band);
  double frac = static_cast<double>(mantissa) / 2048.0;
  return (1.0 + frac) * std::ldexp(1.0, numbps - exponent);
}

Plan build_plan(uint32_t w, uint32_t h, int ncomp, int quality, int format) {
  // src/plan/mod.rs:116-177, validation src/plan/validate.rs:4-62
  if (w == 0 || h == 0)
    throw Error(kInvalidInput, "image dimensions must be non-zero");
  if (ncomp != 1 && ncomp != 3)
    throw Error(kInvalidInput, "images must have 1 or 3 components");
  Plan p;
  p.width = w;
  p.height = h;
  p.ncomp = ncomp;
  p.srgb = (ncomp == 3);
  p.quality = quality;
  p.format = format;
  p.lossless = quality >= 100;
  int cap = p.srgb ? 6 : 5;  // src/plan/derive.rs:109-115
  int lv = max_decompositions(w, h);
  p.levels = lv < cap ? lv : cap;
  p.nres = p.levels + 1;
  p.use_mct = p.srgb;  // src/plan/derive.rs:117-119
  p.guard_bits = 2;
  p.precision = 8;
  // src/plan/derive.rs:159-165
  p.cbw = p.cbh = (quality < 30) ? 32 : 64;
  // src/plan/derive.rs:23-55
  auto push = [&](int res, Band b) {
    SubbandQuant sq{res, b, 0, 0};
    if (p.lossless) {
      sq.exponent = p.precision + band_gain(b);
      sq.mantissa = 0;
    } else {
      irreversible_expounded_quant(p.precision, p.nres, res, b, &sq.exponent,
                                   &sq.mantissa);
    }
    p.quants.push_back(sq);
  };
  push(0, LL);
  for (int r = 1; r <= p.levels; ++r) {
    push(r, HL);
    push(r, LH);
    push(r, HH);
  }
  if (!p.lossless) {  // src/plan/derive.rs:62-71
    double scale = quality_step_scaler(quality);
    for (auto& q : p.quants) q = scale_one_quant(q, scale);
  }
  return p;
}

}  // namespace orc
