// Oracle (test infrastructure): level shift, RCT/ICT, 5/3 and 9/7 lifting,
// deadzone quantisation. Restates src/simd/scalar.rs, src/dwt/rev53.rs,
// src/dwt/irrev97.rs and the quantiser in src/encode/backend/native/backend.rs.
// Compiled with -ffp-contract=off so f32 expressions round exactly as the
// reference's (Rust does not contract a*b+c into FMA).
#include <algorithm>
#include <cmath>
#include <atomic>
#include <thread>

#include "orc.h"

namespace orc {

// src/dwt/irrev97.rs:10-15 (ISO 15444-1 Annex F.4.8.2 lifting constants).
static const float kAlpha = -1.586134342059924f;
static const float kBeta = -0.052980118572961f;
static const float kGamma = 0.882911075530934f;
static const float kDelta = 0.443506852043971f;
static const float kK = 1.230174104914001f;
static const float kInvK = 1.0f / 1.230174104914001f;
// src/dwt/irrev97.rs:16
static const size_t kParallelRowThreshold = 2u * 1024u * 1024u;

template <class F>
static void parallel_for(int n, int threads, F&& f) {
  if (threads <= 1 || n <= 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int> next{0};
  int t = std::min(threads, n);
  std::vector<std::thread> pool;
  for (int k = 0; k < t; ++k)
    pool.emplace_back([&] {
      for (int i = next++; i < n; i = next++) f(i);
    });
  for (auto& th : pool) th.join();
}

static std::vector<std::pair<int, int>> resolutions(int w, int h, int levels) {
  // encode_resolutions (src/dwt/rev53.rs:911-923): index 0 is the smallest.
  std::vector<std::pair<int, int>> r;
  r.push_back({w, h});
  for (int i = 0; i < levels; ++i) {
    w = (w + 1) / 2;
    h = (h + 1) / 2;
    r.push_back({w, h});
  }
  std::reverse(r.begin(), r.end());
  return r;
}

// ---------------------------------------------------------------- 5/3 ------
// Forward 1-D, even origin (src/dwt/rev53.rs:143-203): split, predict
// d[i] -= (s[i] + s[min(i+1,sn-1)]) >> 1, update
// s[i] += (d[clamp(i-1)] + d[min(i,dn-1)] + 2) >> 2.
static void fwd53_1d(int32_t* x, int n, size_t stride, int32_t* tmp) {
  if (n <= 1) return;
  int sn = (n + 1) / 2, dn = n - sn;
  int32_t* s = tmp;
  int32_t* d = tmp + sn;
  for (int i = 0; i < sn; ++i) s[i] = x[(size_t)(2 * i) * stride];
  for (int i = 0; i < dn; ++i) d[i] = x[(size_t)(2 * i + 1) * stride];
  for (int i = 0; i < dn; ++i) {
    int r = std::min(i + 1, sn - 1);
    d[i] -= (s[i] + s[r]) >> 1;
  }
  for (int i = 0; i < sn; ++i) {
    int l = std::min(std::max(i - 1, 0), dn - 1);
    int r = std::min(i, dn - 1);
    s[i] += (d[l] + d[r] + 2) >> 2;
  }
  for (int i = 0; i < n; ++i) x[(size_t)i * stride] = tmp[i];
}

// Inverse 1-D (src/dwt/rev53.rs:234-268).
static void inv53_1d(int32_t* x, int n, size_t stride, int32_t* tmp) {
  if (n <= 1) return;
  int sn = (n + 1) / 2, dn = n - sn;
  std::vector<int32_t> s(sn), d(dn), out(n);
  for (int i = 0; i < sn; ++i) s[i] = x[(size_t)i * stride];
  for (int i = 0; i < dn; ++i) d[i] = x[(size_t)(sn + i) * stride];
  (void)tmp;
  std::vector<int32_t> e(sn);
  for (int i = 0; i < sn; ++i) {
    int l = std::min(std::max(i - 1, 0), dn - 1);
    int r = std::min(i, dn - 1);
    e[i] = s[i] - ((d[l] + d[r] + 2) >> 2);
  }
  for (int i = 0; i < sn; ++i) out[2 * i] = e[i];
  for (int i = 0; i < dn; ++i)
    out[2 * i + 1] = (i + 1 < sn) ? d[i] + ((e[i] + e[i + 1]) >> 1) : d[i] + e[i];
  for (int i = 0; i < n; ++i) x[(size_t)i * stride] = out[i];
}

void fwd53_2d(int32_t* data, int w, int h, int levels) {
  // src/dwt/rev53.rs:34-75: per level, vertical first, then rows.
  if (w == 0 || h == 0 || levels == 0) return;
  auto res = resolutions(w, h, levels);
  std::vector<int32_t> tmp(std::max(w, h));
  for (int li = levels; li >= 1; --li) {
    int rw = res[li].first, rh = res[li].second;
    for (int x = 0; x < rw; ++x) fwd53_1d(data + x, rh, (size_t)w, tmp.data());
    for (int y = 0; y < rh; ++y) fwd53_1d(data + (size_t)y * w, rw, 1, tmp.data());
  }
}

void inv53_2d(int32_t* data, int w, int h, int levels) {
  // src/dwt/rev53.rs:96-129: per level, rows first, then vertical.
  if (w == 0 || h == 0 || levels == 0) return;
  auto res = resolutions(w, h, levels);
  std::vector<int32_t> tmp(std::max(w, h));
  for (int li = 1; li <= levels; ++li) {
    int rw = res[li].first, rh = res[li].second;
    for (int y = 0; y < rh; ++y) inv53_1d(data + (size_t)y * w, rw, 1, tmp.data());
    for (int x = 0; x < rw; ++x) inv53_1d(data + x, rh, (size_t)w, tmp.data());
  }
}

// ---------------------------------------------------------------- 9/7 ------
// Whole-sample symmetric extension index (src/dwt/irrev97.rs:523-536).
static inline int sym_index(int n, int i) {
  if (n <= 1) return 0;
  if (i >= 0 && i < n) return i;
  int period = 2 * (n - 1);
  int k = i % period;
  if (k < 0) k += period;
  return k >= n ? period - k : k;
}

// One lifting step over positions of `parity` (src/dwt/irrev97.rs:159-172):
// x[j] = x[j] + c * (x[j-1] + x[j+1]).
static void lift(float* x, int n, size_t stride, int parity, float c) {
  for (int j = parity; j < n; j += 2) {
    float l = x[(size_t)sym_index(n, j - 1) * stride];
    float r = x[(size_t)sym_index(n, j + 1) * stride];
    x[(size_t)j * stride] = x[(size_t)j * stride] + c * (l + r);
  }
}

// Forward 1-D (src/dwt/irrev97.rs:92-129), deinterleaved output.
static void fwd97_1d(float* x, int n, size_t stride, float* tmp) {
  if (n < 2) {
    if (n == 1) x[0] = x[0] * kInvK;
    return;
  }
  lift(x, n, stride, 1, kAlpha);
  lift(x, n, stride, 0, kBeta);
  lift(x, n, stride, 1, kGamma);
  lift(x, n, stride, 0, kDelta);
  for (int i = 0; i < n; i += 2) x[(size_t)i * stride] = x[(size_t)i * stride] * kInvK;
  for (int i = 1; i < n; i += 2) x[(size_t)i * stride] = x[(size_t)i * stride] * kK;
  int sn = (n + 1) / 2, dn = n - sn;
  for (int i = 0; i < sn; ++i) tmp[i] = x[(size_t)(2 * i) * stride];
  for (int i = 0; i < dn; ++i) tmp[sn + i] = x[(size_t)(2 * i + 1) * stride];
  for (int i = 0; i < n; ++i) x[(size_t)i * stride] = tmp[i];
}

// Inverse 1-D (src/dwt/irrev97.rs:634-667).
static void inv97_1d(float* x, int n, size_t stride, float* tmp) {
  if (n < 2) {
    if (n == 1) x[0] = x[0] * kK;
    return;
  }
  int sn = (n + 1) / 2, dn = n - sn;
  for (int i = 0; i < sn; ++i) tmp[2 * i] = x[(size_t)i * stride];
  for (int i = 0; i < dn; ++i) tmp[2 * i + 1] = x[(size_t)(sn + i) * stride];
  for (int i = 0; i < n; i += 2) tmp[i] = tmp[i] * kK;
  for (int i = 1; i < n; i += 2) tmp[i] = tmp[i] * kInvK;
  lift(tmp, n, 1, 0, -kDelta);
  lift(tmp, n, 1, 1, -kGamma);
  lift(tmp, n, 1, 0, -kBeta);
  lift(tmp, n, 1, 1, -kAlpha);
  for (int i = 0; i < n; ++i) x[(size_t)i * stride] = tmp[i];
}

// Vertical forward pass over the active rectangle (src/dwt/irrev97.rs:261-336):
// the column-wise lifting equals the reference's whole-row lifting, because
// every column is independent and sees the same operations in the same order.
static void fwd97_vertical(float* data, int stride, int rw, int rh) {
  if (rw == 0 || rh == 0) return;
  if (rh < 2) {
    for (int x = 0; x < rw; ++x) data[x] = data[x] * kInvK;
    return;
  }
  std::vector<float> tmp(rh);
  for (int x = 0; x < rw; ++x) {
    float* col = data + x;
    lift(col, rh, stride, 1, kAlpha);
    lift(col, rh, stride, 0, kBeta);
    lift(col, rh, stride, 1, kGamma);
    lift(col, rh, stride, 0, kDelta);
    for (int y = 0; y < rh; y += 2) col[(size_t)y * stride] = col[(size_t)y * stride] * kInvK;
    for (int y = 1; y < rh; y += 2) col[(size_t)y * stride] = col[(size_t)y * stride] * kK;
    int sn = (rh + 1) / 2, dn = rh - sn;
    for (int i = 0; i < sn; ++i) tmp[i] = col[(size_t)(2 * i) * stride];
    for (int i = 0; i < dn; ++i) tmp[sn + i] = col[(size_t)(2 * i + 1) * stride];
    for (int y = 0; y < rh; ++y) col[(size_t)y * stride] = tmp[y];
  }
}

static void inv97_vertical(float* data, int stride, int rw, int rh) {
  // src/dwt/irrev97.rs:723-796
  if (rw == 0 || rh == 0) return;
  if (rh < 2) {
    for (int x = 0; x < rw; ++x) data[x] = data[x] * kK;
    return;
  }
  std::vector<float> tmp(rh);
  for (int x = 0; x < rw; ++x) inv97_1d(data + x, rh, stride, tmp.data());
}

void fwd97_2d(float* data, int w, int h, int levels, int threads) {
  // src/dwt/irrev97.rs:51-82
  if (w == 0 || h == 0 || levels == 0) return;
  auto res = resolutions(w, h, levels);
  for (int li = levels; li >= 1; --li) {
    int rw = res[li].first, rh = res[li].second;
    fwd97_vertical(data, w, rw, rh);
    // Rows go parallel above 2 Mi active samples (src/dwt/irrev97.rs:139-145).
    int t = ((size_t)rw * rh >= kParallelRowThreshold) ? threads : 1;
    parallel_for(rh, t, [&](int y) {
      std::vector<float> tmp(rw);
      fwd97_1d(data + (size_t)y * w, rw, 1, tmp.data());
    });
  }
}

void inv97_2d(float* data, int w, int h, int levels) {
  // src/dwt/irrev97.rs:601-615
  if (w == 0 || h == 0 || levels == 0) return;
  auto res = resolutions(w, h, levels);
  std::vector<float> tmp(std::max(w, h));
  for (int li = 1; li <= levels; ++li) {
    int rw = res[li].first, rh = res[li].second;
    for (int y = 0; y < rh; ++y) inv97_1d(data + (size_t)y * w, rw, 1, tmp.data());
    inv97_vertical(data, w, rw, rh);
  }
}

// ------------------------------------------------------- colour + quant ----
// src/simd/scalar.rs:100-106
static inline int32_t quantize(float v, float step) {
  if (step <= 0.0f || !std::isfinite(v)) return 0;
  float q = std::trunc(v / step);
  if (q <= -2147483648.0f) return INT32_MIN;
  if (q >= 2147483647.0f) return INT32_MAX;
  return static_cast<int32_t>(q);
}

std::vector<int32_t> component_coefficients(const Plan& p, const Planes& px,
                                            int comp, int threads) {
  const int w = p.width, h = p.height;
  const size_t n = (size_t)w * h;
  if (p.lossless) {
    // reversible_input_component (src/encode/backend/native/backend.rs:478-517)
    std::vector<int32_t> d(n);
    if (!p.use_mct) {
      for (size_t i = 0; i < n; ++i) d[i] = px[comp][i] - 128;
    } else {
      const auto &r = px[0], &g = px[1], &b = px[2];
      for (size_t i = 0; i < n; ++i) {  // src/simd/scalar.rs:173-195
        int32_t rv = r[i] - 128, gv = g[i] - 128, bv = b[i] - 128;
        d[i] = comp == 0 ? (rv + 2 * gv + bv) >> 2 : comp == 1 ? bv - gv : rv - gv;
      }
    }
    fwd53_2d(d.data(), w, h, p.levels);
    return d;
  }
  std::vector<float> f = component_unquantized_f32(p, px, comp, threads);
  // quantize_97_coefficients (backend.rs:519-587)
  std::vector<int32_t> out(n, 0);
  auto res = resolutions(w, h, p.levels);
  auto step_of = [&](int r, Band b) {
    for (const auto& q : p.quants)
      if (q.resolution == r && q.band == b)
        return quant_step_f32(p.precision, b, q.exponent, q.mantissa);
    throw Error(kEncodeFailed, "missing quantization parameters");
  };
  auto rect = [&](int x0, int y0, int x1, int y1, float step) {
    for (int y = y0; y < y1; ++y)
      for (int x = x0; x < x1; ++x)
        out[(size_t)y * w + x] = quantize(f[(size_t)y * w + x], step);
  };
  rect(0, 0, res[0].first, res[0].second, step_of(0, LL));
  for (int i = 0; i < p.levels; ++i) {
    auto lo = res[i], full = res[i + 1];
    int r = i + 1;
    rect(lo.first, 0, full.first, lo.second, step_of(r, HL));
    rect(0, lo.second, lo.first, full.second, step_of(r, LH));
    rect(lo.first, lo.second, full.first, full.second, step_of(r, HH));
  }
  return out;
}

// The irreversible path before quantisation: level shift, ICT and the f32
// 9/7 transform of one component.
std::vector<float> component_unquantized_f32(const Plan& p, const Planes& px, int comp, int threads) {
  const int w = p.width, h = p.height;
  const size_t n = (size_t)w * h;
  // irreversible_input_component (backend.rs:436-476)
  std::vector<float> f(n);
  if (!p.use_mct) {
    for (size_t i = 0; i < n; ++i) f[i] = static_cast<float>(px[comp][i] - 128);
  } else {
    const auto &r = px[0], &g = px[1], &b = px[2];
    for (size_t i = 0; i < n; ++i) {  // src/simd/scalar.rs:149-171
      float rf = static_cast<float>(r[i] - 128);
      float gf = static_cast<float>(g[i] - 128);
      float bf = static_cast<float>(b[i] - 128);
      if (comp == 0)
        f[i] = 0.299f * rf + 0.587f * gf + 0.114f * bf;
      else if (comp == 1)
        f[i] = -0.16875f * rf + -0.33126f * gf + 0.5f * bf;
      else
        f[i] = 0.5f * rf - 0.41869f * gf - 0.08131f * bf;
    }
  }
  fwd97_2d(f.data(), w, h, p.levels, threads);
  return f;
}

// ------------------------------------------------------ FP64 lifting ------
// The irreversible path of component_coefficients in double precision: the
// level shift and ICT (src/simd/scalar.rs:135-171) and every 9/7 lifting step
// and scaling (src/dwt/irrev97.rs:10-15, 92-129, 261-336) in the same order,
// with the constants' decimal values as doubles. It measures how far the
// reference's f32 pipeline is from exact lifting; quantised with the same
// steps it gives the indices an f64 pipeline would code.
static const double kAlpha64 = -1.586134342059924, kBeta64 = -0.052980118572961;
static const double kGamma64 = 0.882911075530934, kDelta64 = 0.443506852043971;
static const double kK64 = 1.230174104914001, kInvK64 = 1.0 / 1.230174104914001;

static void lift64(double* x, int n, size_t stride, int parity, double c) {
  for (int j = parity; j < n; j += 2) {
    double l = x[(size_t)sym_index(n, j - 1) * stride];
    double r = x[(size_t)sym_index(n, j + 1) * stride];
    x[(size_t)j * stride] = x[(size_t)j * stride] + c * (l + r);
  }
}

static void fwd97_1d_f64(double* x, int n, size_t stride, double* tmp) {
  if (n < 2) {
    if (n == 1) x[0] = x[0] * kInvK64;
    return;
  }
  lift64(x, n, stride, 1, kAlpha64);
  lift64(x, n, stride, 0, kBeta64);
  lift64(x, n, stride, 1, kGamma64);
  lift64(x, n, stride, 0, kDelta64);
  for (int i = 0; i < n; i += 2) x[(size_t)i * stride] = x[(size_t)i * stride] * kInvK64;
  for (int i = 1; i < n; i += 2) x[(size_t)i * stride] = x[(size_t)i * stride] * kK64;
  int sn = (n + 1) / 2, dn = n - sn;
  for (int i = 0; i < sn; ++i) tmp[i] = x[(size_t)(2 * i) * stride];
  for (int i = 0; i < dn; ++i) tmp[sn + i] = x[(size_t)(2 * i + 1) * stride];
  for (int i = 0; i < n; ++i) x[(size_t)i * stride] = tmp[i];
}

std::vector<double> component_coefficients_f64(const Plan& p, const Planes& px, int comp) {
  const int w = p.width, h = p.height;
  const size_t n = (size_t)w * h;
  std::vector<double> f(n);
  for (size_t i = 0; i < n; ++i) {
    if (!p.use_mct) {
      f[i] = (double)(px[comp][i] - 128);
    } else {
      const double r = px[0][i] - 128, g = px[1][i] - 128, b = px[2][i] - 128;
      f[i] = comp == 0 ? 0.299 * r + 0.587 * g + 0.114 * b
                       : comp == 1 ? -0.16875 * r + -0.33126 * g + 0.5 * b : 0.5 * r - 0.41869 * g - 0.08131 * b;
    }
  }
  auto res = resolutions(w, h, p.levels);
  std::vector<double> tmp(std::max(w, h));
  for (int li = p.levels; li >= 1; --li) {
    const int rw = res[li].first, rh = res[li].second;
    for (int x = 0; x < rw; ++x) fwd97_1d_f64(f.data() + x, rh, w, tmp.data());
    for (int y = 0; y < rh; ++y) fwd97_1d_f64(f.data() + (size_t)y * w, rw, 1, tmp.data());
  }
  return f;
}

// Quantiser step of every coefficient position of a plane (Mallat layout).
std::vector<float> coefficient_steps(const Plan& p) {
  const int w = p.width, h = p.height;
  std::vector<float> st((size_t)w * h, 1.0f);
  auto res = resolutions(w, h, p.levels);
  auto step_of = [&](int r, Band b) {
    for (const auto& q : p.quants)
      if (q.resolution == r && q.band == b) return quant_step_f32(p.precision, b, q.exponent, q.mantissa);
    throw Error(kEncodeFailed, "missing quantization parameters");
  };
  auto rect = [&](int x0, int y0, int x1, int y1, float step) {
    for (int y = y0; y < y1; ++y)
      for (int x = x0; x < x1; ++x) st[(size_t)y * w + x] = step;
  };
  rect(0, 0, res[0].first, res[0].second, step_of(0, LL));
  for (int i = 0; i < p.levels; ++i) {
    auto lo = res[i], full = res[i + 1];
    rect(lo.first, 0, full.first, lo.second, step_of(i + 1, HL));
    rect(0, lo.second, lo.first, full.second, step_of(i + 1, LH));
    rect(lo.first, lo.second, full.first, full.second, step_of(i + 1, HH));
  }
  return st;
}

Planes planes_from_bytes(const uint8_t* px, uint32_t w, uint32_t h, int ncomp) {
  // Image::from_gray_bytes / from_rgb_bytes (src/model.rs:87-140)
  size_t n = (size_t)w * h;
  Planes p(ncomp, std::vector<int32_t>(n));
  for (size_t i = 0; i < n; ++i)
    for (int c = 0; c < ncomp; ++c) p[c][i] = px[i * ncomp + c];
  return p;
}

}  // namespace orc
