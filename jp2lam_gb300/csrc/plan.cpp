// Host-side encoding plan: decomposition levels, code-block size, quantiser
// step sizes, subband geometry and the flat code-block work list order.
// Follows src/plan/{mod,derive,validate}.rs and src/dwt/norms.rs.
#include <algorithm>
#include <cmath>

#include "jp2g_internal.h"

namespace jp2g {

// 9/7 synthesis norms (src/dwt/norms.rs:21-34): the step sizes and PCRD
// weights are defined by this table, so it is kept value-for-value.
static const double kNorm97[4][10] = {
    {1.000, 1.965, 4.177, 8.403, 16.90, 33.84, 67.69, 135.3, 270.6, 540.9},
    {2.022, 3.989, 8.355, 17.04, 34.27, 68.63, 137.3, 274.6, 549.0, 0.0},
    {2.022, 3.989, 8.355, 17.04, 34.27, 68.63, 137.3, 274.6, 549.0, 0.0},
    {2.080, 3.865, 8.307, 17.18, 34.71, 69.59, 139.3, 278.6, 557.2, 0.0},
};

double norm97(int level, int orient) {
  int cap = orient == LL ? 9 : 8;
  return kNorm97[orient][std::min(level, cap)];
}

int band_gain(int orient) { return orient == LL ? 0 : (orient == HH ? 2 : 1); }

// The f32 quantiser step of a band from its QCD exponent and mantissa,
// floored at 1e-6 (backend.rs:602-620).
float quant_step_from_qcd(int precision, int orient, int exponent, int mantissa) {
  const int numbps = precision + band_gain(orient);
  const float base = 1.0f + (float)mantissa / 2048.0f;
  const float s = base * std::ldexp(1.0f, numbps - exponent);
  return s > 1e-6f ? s : 1e-6f;
}

static int ilog2(int v) { return 31 - __builtin_clz((unsigned)std::max(v, 1)); }

// Step packing: exponent/mantissa of an 8192-scaled step (norms.rs:85-92).
static void pack_step(int step, int numbps, int* e, int* m) {
  int p = ilog2(step) - 13, n = 11 - ilog2(step);
  *m = (n < 0 ? step >> -n : step << n) & 0x7ff;
  *e = std::max(numbps - p, 0) & 0xff;
}

// Quality step multiplier (derive.rs:74-86).
static double step_scaler(int q) {
  if (q == 0) return 8.0;
  if (q <= 50) return std::pow(2.0, (50.0 - q) / 20.0);
  if (q <= 90) return std::pow(2.0, -((q - 50.0) / 20.0));
  return 0.25 * std::pow(2.0, -3.0 * ((q - 90.0) / 9.0));
}

// Multiply one step by `scale`, re-packing exponent and mantissa
// (derive.rs:94-107).
static void rescale(double scale, int* e, int* m) {
  double scaled = std::max((1.0 + *m / 2048.0) * scale, 1.0 / 8192.0);
  int k = (int)std::floor(std::log2(scaled));
  double b = scaled / std::ldexp(1.0, k);
  *e = std::max(*e - k, 0) & 0xff;
  *m = (int)std::min(std::max(std::round((b - 1.0) * 2048.0), 0.0), 2047.0);
}

static int decompositions(uint32_t w, uint32_t h) {  // derive.rs:128-139
  uint32_t m = std::min(w, h);
  if (m <= 1) return 0;
  if (m < 32) return 31 - __builtin_clz(m);
  return std::min(1 + (31 - __builtin_clz(m / 32)), 6);
}

double quality_to_lambda(int q, uint32_t pixels) {  // pcrd.rs:1425-1456
  if (q >= 100) return 0.0;
  if (q == 0) return 1.7976931348623157e308;
  double t = (q - 1.0) / 98.0;
  double base = std::max(std::pow(10.0, 5.68 - 2.618 * std::pow(t, 0.85)), 1e-3);
  double tail = 1.0;
  if (q >= 90) {
    double tt = (99.0 - std::min(q, 99)) / 9.0;
    tail = tt * tt;
  }
  return base * std::pow(pixels / 12000000.0, 0.35) * tail;
}

bool build_plan(uint32_t w, uint32_t h, int ncomp, int quality, int format,
                PagePlan* p, Failure* err) {
  // validate_image (src/plan/validate.rs:4-62) for the 8-bit byte inputs
  // this API accepts.
  if (w == 0 || h == 0) {
    *err = {kInvalidInput, "image dimensions must be non-zero"};
    return false;
  }
  if (ncomp != 1 && ncomp != 3) {
    *err = {kInvalidInput, "images must have exactly 1 (gray) or 3 (sRGB) component(s)"};
    return false;
  }
  if (quality < 0 || quality > 255) {
    *err = {kInvalidInput, "quality must fit in a u8"};
    return false;
  }
  if (format != 0 && format != 1) {
    *err = {kInvalidInput, "format must be 0 (J2K) or 1 (JP2)"};
    return false;
  }
  *p = PagePlan();
  p->width = w;
  p->height = h;
  p->ncomp = ncomp;
  p->srgb = ncomp == 3;
  p->quality = quality;
  p->format = format;
  p->lossless = quality >= 100;
  p->use_mct = p->srgb;
  p->levels = std::min(decompositions(w, h), p->srgb ? 6 : 5);
  p->cbw = p->cbh = quality < 30 ? 32 : 64;
  const int nres = p->levels + 1;
  // Subband quantisation (derive.rs:23-55 + 62-71).
  auto add_quant = [&](int res, int o) {
    BandQuant q{res, o, 0, 0, 0.f, 0.0};
    if (p->lossless) {
      q.exponent = p->precision + band_gain(o);
    } else {
      int level = std::max(std::max(nres - 1, 0) - res, 0);
      double step = (double)(1u << band_gain(o)) / norm97(level, o);
      pack_step((int)std::floor(step * 8192.0), p->precision + band_gain(o), &q.exponent,
                &q.mantissa);
    }
    p->quants.push_back(q);
  };
  add_quant(0, LL);
  for (int r = 1; r <= p->levels; ++r) {
    add_quant(r, HL);
    add_quant(r, LH);
    add_quant(r, HH);
  }
  if (!p->lossless) {
    double s = step_scaler(quality);
    for (auto& q : p->quants) rescale(s, &q.exponent, &q.mantissa);
  }
  for (auto& q : p->quants) {
    int numbps = p->precision + band_gain(q.orient);
    q.step_f32 = quant_step_from_qcd(p->precision, q.orient, q.exponent, q.mantissa);
    q.step_f64 = (1.0 + q.mantissa / 2048.0) * std::ldexp(1.0, numbps - q.exponent);
  }
  // Resolution ladder and subband rectangles (layout.rs:37-173).
  int cw = (int)w, ch = (int)h;
  p->ladder.push_back({cw, ch});
  for (int i = 0; i < p->levels; ++i) {
    cw = (cw + 1) / 2;
    ch = (ch + 1) / 2;
    p->ladder.push_back({cw, ch});
  }
  std::reverse(p->ladder.begin(), p->ladder.end());
  uint32_t next = 0;
  for (int r = 0; r <= p->levels; ++r)
    for (int c = 0; c < ncomp; ++c) {
      auto add_band = [&](int o, int qi, int x0, int y0, int x1, int y1) {
        BandGeom g{};
        g.comp = c;
        g.res = r;
        g.orient = o;
        g.x0 = x0; g.y0 = y0; g.x1 = x1; g.y1 = y1;
        g.ncbx = x1 > x0 ? (x1 - x0 + p->cbw - 1) / p->cbw : 0;
        g.ncby = y1 > y0 ? (y1 - y0 + p->cbh - 1) / p->cbh : 0;
        g.first_block = next;
        next += (uint32_t)(g.ncbx * g.ncby);
        g.quant = qi;
        // Maximum bit-planes (backend.rs:161-204, t1.rs:19-22): lossless
        // uses precision (+1 for RCT chroma) + gain; lossy uses the QCD
        // exponent.
        if (p->lossless)
          g.mb = p->guard_bits - 1 + p->precision + ((p->use_mct && c > 0) ? 1 : 0) + band_gain(o);
        else
          g.mb = p->guard_bits - 1 + p->quants[qi].exponent;
        p->max_mb = std::max(p->max_mb, g.mb);
        p->bands.push_back(g);
      };
      if (r == 0) {
        add_band(LL, 0, 0, 0, p->ladder[0].first, p->ladder[0].second);
      } else {
        auto lo = p->ladder[r - 1], full = p->ladder[r];
        int qb = 1 + 3 * (r - 1);
        add_band(HL, qb + 0, lo.first, 0, full.first, lo.second);
        add_band(LH, qb + 1, 0, lo.second, lo.first, full.second);
        add_band(HH, qb + 2, lo.first, lo.second, full.first, full.second);
      }
    }
  p->nblocks = next;
  // PCRD constants (pcrd.rs:1465-1514, backend.rs:696-718).
  uint32_t pixels = w * h;
  p->lambda_raw = quality_to_lambda(quality, pixels);
  p->lambda_floor = quality_to_lambda(1, pixels);
  for (int c = 0; c < 3; ++c) {
    p->comp_weight[c] = 1.0;
    if (p->use_mct && p->srgb && c > 0) {
      double q = std::min(quality, 99);
      p->comp_weight[c] = 1.20 + 1.80 * std::pow(1.0 - q / 99.0, 0.70);
    }
  }
  return true;
}

}  // namespace jp2g

namespace jp2g {

// Allocation-free subset of build_plan for the DWT stage: decomposition
// levels, the reversible flag, the f32 quantiser step of every band (LL, then
// HL/LH/HH per resolution) and the resolution ladder (rw/rh: size of
// resolution r; lo_w/lo_h: size of resolution r-1, i.e. of the LL band that
// resolution r's level produces). Arrays hold up to 1 + 3*6 steps and 7
// resolutions.
bool plan_dwt_steps(uint32_t w, uint32_t h, int ncomp, int quality, int* levels, int* lossless,
                    float* steps, int* lo_w, int* lo_h, int* rw, int* rh) {
  if (w == 0 || h == 0 || (ncomp != 1 && ncomp != 3) || quality < 0 || quality > 255) return false;
  const bool rev = quality >= 100;
  const int L = std::min(decompositions(w, h), ncomp == 3 ? 6 : 5);
  const int nres = L + 1;
  const int precision = 8;
  const double scale = rev ? 1.0 : step_scaler(quality);
  int k = 0;
  for (int r = 0; r <= L; ++r)
    for (int oi = 0; oi < (r == 0 ? 1 : 3); ++oi) {
      const int o = r == 0 ? LL : oi + 1;
      int e, m = 0;
      if (rev) {
        e = precision + band_gain(o);
      } else {
        int level = std::max(std::max(nres - 1, 0) - r, 0);
        double st = (double)(1u << band_gain(o)) / norm97(level, o);
        pack_step((int)std::floor(st * 8192.0), precision + band_gain(o), &e, &m);
        rescale(scale, &e, &m);
      }
      float base = 1.0f + (float)m / 2048.0f;
      float s = base * std::ldexp(1.0f, precision + band_gain(o) - e);
      steps[k++] = s > 1e-6f ? s : 1e-6f;
    }
  int cw[8], chh[8];
  cw[L] = (int)w;
  chh[L] = (int)h;
  for (int r = L - 1; r >= 0; --r) {
    cw[r] = (cw[r + 1] + 1) / 2;
    chh[r] = (chh[r + 1] + 1) / 2;
  }
  for (int r = 0; r <= L; ++r) {
    rw[r] = cw[r];
    rh[r] = chh[r];
    lo_w[r] = r > 0 ? cw[r - 1] : 0;
    lo_h[r] = r > 0 ? chh[r - 1] : 0;
  }
  *levels = L;
  *lossless = rev ? 1 : 0;
  return true;
}

}  // namespace jp2g
