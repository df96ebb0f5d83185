// Oracle (test infrastructure): code-block layout, PCRD rate control, Tier-2
// packets, codestream markers, JP2 boxes, the top-level encode, and a decoder
// for round trips. Restates src/encode/backend/native/{backend,layout,rate,
// t2}.rs, src/dwt/pcrd.rs, src/profile.rs:122-154, src/j2k/{markers,write}.rs,
// src/jp2.rs and the decoder in src/decode/*.rs.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>

#include "orc.h"

namespace orc {

std::vector<int32_t> decode_block(const uint8_t* data, size_t n, int w, int h,
                                  Band band, int mb, int zbp, int npasses, bool allow_empty = false);

template <class F>
static void par_for(int n, int threads, F&& f) {
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

static std::vector<std::pair<int, int>> ladder(int w, int h, int levels) {
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

struct BandRect { int res; Band band; int x0, y0, x1, y1; };

// build_component_layout (src/encode/backend/native/layout.rs:37-97): LL,
// then HL/LH/HH per resolution.
static std::vector<BandRect> band_rects(int w, int h, int levels) {
  auto r = ladder(w, h, levels);
  std::vector<BandRect> out;
  out.push_back({0, LL, 0, 0, r[0].first, r[0].second});
  for (int i = 0; i < levels; ++i) {
    auto lo = r[i], full = r[i + 1];
    out.push_back({i + 1, HL, lo.first, 0, full.first, lo.second});
    out.push_back({i + 1, LH, 0, lo.second, lo.first, full.second});
    out.push_back({i + 1, HH, lo.first, lo.second, full.first, full.second});
  }
  return out;
}

// Maximum bit-planes Mb per band (backend.rs:161-204, t1.rs:19-22).
static int band_mb(const Plan& p, int comp, int res, Band b) {
  if (p.lossless) {
    int eff = p.precision + ((p.use_mct && comp > 0) ? 1 : 0);
    return p.guard_bits - 1 + eff + band_gain(b);
  }
  for (const auto& q : p.quants)
    if (q.resolution == res && q.band == b) return p.guard_bits - 1 + q.exponent;
  return p.guard_bits - 1 + p.precision + band_gain(b);
}

// ------------------------------------------------------------------ PCRD ---
struct Pt { int passes; uint32_t bytes; double dist; double slope; };

double rd_slope(const Pt& a, const Pt& b) {  // src/dwt/pcrd.rs:539-554
  if (b.bytes < a.bytes) throw Error(kEncodeFailed, "PCRD point had negative byte delta");
  double db = (double)(b.bytes - a.bytes);
  double dd = b.dist - a.dist;
  if (db == 0.0) return dd > 0.0 ? std::numeric_limits<double>::infinity() : 0.0;
  return dd / db;
}

void fill_slopes(std::vector<Pt>& pts) {  // src/dwt/pcrd.rs:526-537
  if (pts.empty()) return;
  pts[0].slope = std::numeric_limits<double>::infinity();
  for (size_t i = 1; i < pts.size(); ++i) pts[i].slope = rd_slope(pts[i - 1], pts[i]);
}

double band_distortion_bias(Band b, int quality) {  // src/dwt/pcrd.rs:728-748
  if (quality < 50) {
    double t = (double)quality / 50.0;
    if (b == LL) return 3.0 - 1.8 * t;
    if (b == HH) return 0.20 + 0.62 * t;
    return 1.0;
  }
  if (b == LL) return 1.20;
  if (b == HH) return 0.82;
  return 1.00;
}

static double class_weight(int cls, bool is_ll) {  // src/profile.rs:141-154
  double base = cls == 0 ? 2.5 : cls == 1 ? 1.5 : 1.0;
  return is_ll ? base * 1.1 : base;
}

// estimate_pass_distortion_delta_pass_kind_aware (src/dwt/pcrd.rs:669-696)
// with visibility weight 1.0 (src/encode/backend/native/rate.rs:128-180).
static double pass_delta(const Pass& ps, double quant_step, double sw, Band b,
                         int quality, int cls) {
  int bp = ps.bitplane < 30 ? ps.bitplane : 30;
  double plane_weight = (double)(1ull << bp) * quant_step;
  double energy = plane_weight * plane_weight;
  double contrib;
  if (ps.kind == kSP) contrib = (double)ps.ns * energy;
  else if (ps.kind == kMR) contrib = (double)ps.sig_before * energy * 0.25;
  else contrib = (double)ps.ns * energy * 0.85;
  double bias = band_distortion_bias(b, quality);
  double bw = class_weight(cls, b == LL);
  double raw = sw * bias * bw * contrib;
  // apply_contrast_masking_to_delta (pcrd.rs:764-802), visibility 1.0.
  if (raw <= 0.0) return 0.0;
  double q = (double)quality / 100.0;
  double lrs = std::min(std::max(1.0 - q, 0.0), 1.0);
  double cs = cls == 0 ? 0.10 : cls == 1 ? 0.20 : 1.00;
  double eff = lrs * cs;
  double blended = 1.0 + eff * (1.0 - 1.0);
  blended = std::min(std::max(blended, 0.20), 1.0);
  return raw * blended;
}

double quality_to_lambda(int quality, uint32_t pixels) {  // pcrd.rs:1425-1456
  if (quality >= 100) return 0.0;
  if (quality == 0) return std::numeric_limits<double>::max();
  double t = ((double)quality - 1.0) / 98.0;
  double log_lambda = 5.68 - 2.618 * std::pow(t, 0.85);
  double base = std::pow(10.0, log_lambda);
  if (base < 1e-3) base = 1e-3;
  double tail = 1.0;
  if (quality >= 90) {
    double tt = (99.0 - (double)std::min(quality, 99)) / 9.0;
    tail = tt * tt;
  }
  double rf = std::pow((double)pixels / 12000000.0, 0.35);
  return base * rf * tail;
}

static double component_weight(const Plan& p, int comp) {  // backend.rs:696-718
  if (!p.use_mct || !p.srgb) return 1.0;
  if (comp == 0) return 1.0;
  double q = (double)std::min(p.quality, 99);
  return 1.20 + 1.80 * std::pow(1.0 - q / 99.0, 0.70);
}

// apply_pcrd_selection for one component (backend.rs:641-694).
static void pcrd_component(const Plan& p, int comp, Layout& layout) {
  const uint32_t pixels = p.width * p.height;
  double cw = component_weight(p, comp);
  std::vector<std::vector<Pt>> hulls;
  for (auto& band : layout) {
    int level = band.band == LL ? std::max(p.nres - 1, 0)
                                : std::max(std::max(p.nres - 1, 0) - band.res, 0);
    double norm = get_norm_97(level, band.band);
    double sw = norm * norm;  // rate.rs:304-313
    double qs = 1.0;
    for (const auto& q : p.quants)
      if (q.resolution == band.res && q.band == band.band) {
        qs = quant_step_f64(p.precision, band.band, q.exponent, q.mantissa);
        break;
      }
    for (auto& blk : band.blocks) {
      // raw_records_for_block (rate.rs:128-180) + build_raw_curve (pcrd.rs:151-202)
      std::vector<Pt> pts;
      pts.push_back({0, 0, 0.0, std::numeric_limits<double>::infinity()});
      double cum_d = 0.0;
      uint32_t prev = 0;
      for (size_t i = 0; i < blk.passes.size(); ++i) {
        const Pass& ps = blk.passes[i];
        double dd = pass_delta(ps, qs, sw, band.band, p.quality, blk.cls) * cw;
        uint32_t cum = ps.cumulative + 2u;  // HEADER_OVERHEAD_BYTES
        if (cum < prev) throw Error(kEncodeFailed, "non-monotone cumulative bytes");
        prev = cum;
        if (!std::isfinite(dd) || dd < 0.0) throw Error(kEncodeFailed, "invalid distortion delta");
        cum_d += dd;
        pts.push_back({(int)i + 1, cum, cum_d, 0.0});
      }
      fill_slopes(pts);
      // prune_to_convex_hull (pcrd.rs:209-243)
      std::vector<Pt> hull;
      for (const Pt& pt : pts) {
        hull.push_back(pt);
        while (hull.size() >= 3) {
          const Pt& c = hull[hull.size() - 1];
          const Pt& b = hull[hull.size() - 2];
          const Pt& a = hull[hull.size() - 3];
          double sab = rd_slope(a, b), sbc = rd_slope(b, c);
          if (sbc >= sab) hull.erase(hull.end() - 2);
          else break;
        }
      }
      fill_slopes(hull);
      hulls.push_back(std::move(hull));
    }
  }
  if (hulls.empty()) return;
  // select_for_quality + calibrate_lambda (pcrd.rs:1465-1514)
  double raw = quality_to_lambda(p.quality, pixels);
  double lambda = raw;
  if (p.quality < 100) {
    double maxs = 0.0;
    for (auto& h : hulls)
      for (size_t i = 1; i < h.size(); ++i)
        if (std::isfinite(h[i].slope) && h[i].slope > 0.0) maxs = std::max(maxs, h[i].slope);
    if (maxs > 0.0) {
      double floor_l = quality_to_lambda(1, pixels);
      double target = maxs * 1.2;
      if (!(target >= floor_l)) lambda = raw * (target / floor_l);
    }
  }
  // choose_block_point (pcrd.rs:406-424), then truncate_layout_passes
  // (backend.rs:834-897).
  size_t hi = 0;
  for (auto& band : layout)
    for (auto& blk : band.blocks) {
      const auto& h = hulls[hi++];
      int keep = 0;
      for (size_t i = 1; i < h.size(); ++i) {
        if (h[i].slope >= lambda) keep = h[i].passes;
        else break;
      }
      int retain = std::min<int>(keep, (int)blk.passes.size());
      if (retain == 0) {
        blk.passes.clear();
        blk.payload.clear();
        continue;
      }
      blk.passes.resize(retain);
      uint32_t cum = 0;
      for (int i = 0; i < retain; ++i) {
        cum += blk.passes[i].length;
        blk.passes[i].cumulative = cum;
        blk.passes[i].terminated = (i + 1 == retain);
      }
      size_t plen = std::min<size_t>(cum, blk.payload.size());
      blk.payload.resize(plen);
    }
}

// ----------------------------------------------------------- Tier-1 glue ---
std::vector<Layout> tier1_layouts(const Plan& p, const Planes& px,
                                  const EncodeOptions& opt, bool apply_pcrd) {
  std::vector<Layout> layouts(p.ncomp);
  // Components in parallel (backend.rs:219-245); code-blocks in parallel
  // inside (t1.rs:191-196, 287-290).
  int outer = std::min(opt.threads, p.ncomp);
  int inner = std::max(1, opt.threads / std::max(1, outer));
  par_for(p.ncomp, outer, [&](int c) {
    std::vector<int32_t> coef = component_coefficients(p, px, c, inner);
    auto rects = band_rects(p.width, p.height, p.levels);
    Layout lay;
    struct Job { size_t band; int x0, y0, x1, y1; };
    std::vector<Job> jobs;
    for (size_t bi = 0; bi < rects.size(); ++bi) {
      const auto& r = rects[bi];
      lay.push_back({r.res, r.band, {}});
      // split_codeblocks (layout.rs:120-159)
      for (int by = r.y0; by < r.y1; by = std::min(by + p.cbh, r.y1))
        for (int bx = r.x0; bx < r.x1; bx = std::min(bx + p.cbw, r.x1))
          jobs.push_back({bi, bx, by, std::min(bx + p.cbw, r.x1), std::min(by + p.cbh, r.y1)});
    }
    std::vector<EncBlock> enc(jobs.size());
    par_for((int)jobs.size(), inner, [&](int j) {
      const Job& jb = jobs[j];
      int bw = jb.x1 - jb.x0, bh = jb.y1 - jb.y0;
      std::vector<int32_t> blk((size_t)bw * bh);
      for (int y = 0; y < bh; ++y)
        std::memcpy(&blk[(size_t)y * bw], &coef[(size_t)(jb.y0 + y) * p.width + jb.x0],
                    sizeof(int32_t) * bw);
      const auto& r = rects[jb.band];
      EncBlock e = encode_block(blk.data(), bw, bh, r.band, band_mb(p, c, r.res, r.band));
      e.res = r.res;
      e.x0 = jb.x0; e.y0 = jb.y0; e.x1 = jb.x1; e.y1 = jb.y1;
      enc[j] = std::move(e);
    });
    for (size_t j = 0; j < jobs.size(); ++j) lay[jobs[j].band].blocks.push_back(std::move(enc[j]));
    layouts[c] = std::move(lay);
  });
  if (apply_pcrd && p.quality < 100) {
    if (opt.contrast_mask) contrast_mask_work(p, px);
    for (int c = 0; c < p.ncomp; ++c) pcrd_component(p, c, layouts[c]);
  }
  return layouts;
}

std::vector<Layout> layouts_from_blocks(const Plan& p, const uint16_t* npasses, const uint8_t* zbp,
                                        const uint32_t* seg_len, const uint8_t* body, uint32_t nblocks) {
  std::vector<Layout> layouts(p.ncomp);
  auto rects = band_rects(p.width, p.height, p.levels);
  for (int c = 0; c < p.ncomp; ++c)
    for (const auto& r : rects) {
      EncBand b{r.res, r.band, {}};
      // split_codeblocks (layout.rs:120-159)
      for (int by = r.y0; by < r.y1; by = std::min(by + p.cbh, r.y1))
        for (int bx = r.x0; bx < r.x1; bx = std::min(bx + p.cbw, r.x1)) {
          EncBlock e{};
          e.res = r.res;
          e.band = r.band;
          e.x0 = bx; e.y0 = by; e.x1 = std::min(bx + p.cbw, r.x1); e.y1 = std::min(by + p.cbh, r.y1);
          b.blocks.push_back(std::move(e));
        }
      layouts[c].push_back(std::move(b));
    }
  // codestream order: resolution, then component, then the component's
  // bands of that resolution, then raster order within a band
  int maxr = 0;
  for (const auto& r : rects) maxr = std::max(maxr, r.res);
  uint32_t k = 0;
  size_t at = 0;
  for (int res = 0; res <= maxr; ++res)
    for (int c = 0; c < p.ncomp; ++c)
      for (auto& band : layouts[c]) {
        if (band.res != res) continue;
        for (auto& e : band.blocks) {
          if (k >= nblocks) throw Error(kInvalidInput, "fewer block records than code-blocks");
          e.zbp = zbp[k];
          for (uint32_t i = 0; i < npasses[k]; ++i) {
            Pass ps{};
            ps.terminated = i + 1 == npasses[k];
            ps.length = ps.terminated ? seg_len[k] : 0;
            e.passes.push_back(ps);
          }
          if (npasses[k] > 0) e.payload.assign(body + at, body + at + seg_len[k]);
          at += npasses[k] > 0 ? seg_len[k] : 0;
          ++k;
        }
      }
  if (k != nblocks) throw Error(kInvalidInput, "more block records than code-blocks");
  return layouts;
}

// ------------------------------------------------------------------ T2 -----
struct Bio {  // src/encode/backend/native/t2.rs:25-67
  std::vector<uint8_t> buf;
  uint32_t reg = 0, ct = 8;
  void byteout() {
    reg = (reg << 8) & 0xffff;
    ct = reg == 0xff00 ? 7 : 8;
    buf.push_back((uint8_t)(reg >> 8));
  }
  void put(uint32_t b) {
    if (ct == 0) byteout();
    --ct;
    reg |= b << ct;
  }
  void bits(uint32_t v, int n) {
    for (int i = n - 1; i >= 0; --i) put((v >> i) & 1);
  }
  std::vector<uint8_t> flush() {
    byteout();
    if (ct == 7) byteout();
    return buf;
  }
};

// Tag tree (ISO 15444-1 B.10.2): level 0 holds the leaves in raster order,
// node (i, j) of level l has parent (i/2, j/2) in level l+1.
struct TagTree {
  struct Node { int parent, value, low; bool known; };
  std::vector<Node> nodes;
  TagTree(int nw, int nh) {
    std::vector<std::pair<int, int>> dims;
    int w = nw, h = nh;
    for (;;) {
      dims.push_back({w, h});
      if (w * h <= 1) break;
      w = (w + 1) / 2;
      h = (h + 1) / 2;
    }
    std::vector<int> base(dims.size() + 1, 0);
    for (size_t l = 0; l < dims.size(); ++l) base[l + 1] = base[l] + dims[l].first * dims[l].second;
    nodes.assign(base.back(), Node{-1, 999, 0, false});
    for (size_t l = 0; l + 1 < dims.size(); ++l)
      for (int j = 0; j < dims[l].second; ++j)
        for (int i = 0; i < dims[l].first; ++i)
          nodes[base[l] + j * dims[l].first + i].parent =
              base[l + 1] + (j / 2) * dims[l + 1].first + (i / 2);
  }
  void set(int leaf, int v) {
    for (int n = leaf; n >= 0 && nodes[n].value > v; n = nodes[n].parent) nodes[n].value = v;
  }
  void encode(Bio& bio, int leaf, int threshold) {
    int stk[64], depth = 0, n = leaf;
    while (nodes[n].parent >= 0) { stk[depth++] = n; n = nodes[n].parent; }
    int low = 0;
    for (;;) {
      Node& nd = nodes[n];
      if (low > nd.low) nd.low = low; else low = nd.low;
      while (low < threshold) {
        if (low >= nd.value) {
          if (!nd.known) { bio.put(1); nd.known = true; }
          break;
        }
        bio.put(0);
        ++low;
      }
      nd.low = low;
      if (depth == 0) break;
      n = stk[--depth];
    }
  }
};

int floor_log2_u(uint32_t v) { return v == 0 ? 0 : 31 - __builtin_clz(v); }

void put_numpasses(Bio& bio, uint32_t n) {  // Table B-4 (t2.rs:243-259)
  if (n == 1) bio.bits(0, 1);
  else if (n == 2) bio.bits(0x2, 2);
  else if (n <= 5) bio.bits(0xc | (n - 3), 4);
  else if (n <= 36) bio.bits(0x1e0 | (n - 6), 9);
  else if (n <= 164) bio.bits(0xff80 | (n - 37), 16);
  else bio.bits(0xff80 | (164 - 37), 16);
}

// One packet header (t2.rs:337-396).
static std::vector<uint8_t> packet_header(const std::vector<const EncBand*>& bands,
                                          int cbw, int cbh) {
  (void)cbw; (void)cbh;
  Bio bio;
  bio.put(1);
  for (const EncBand* band : bands) {
    size_t n = band->blocks.size();
    if (n == 0) continue;
    // band_cb_dims (t2.rs:312-330)
    int x0 = INT32_MAX, y0 = INT32_MAX, x1 = 0, y1 = 0;
    for (const auto& b : band->blocks) {
      x0 = std::min(x0, b.x0); y0 = std::min(y0, b.y0);
      x1 = std::max(x1, b.x1); y1 = std::max(y1, b.y1);
    }
    int bw = band->blocks[0].x1 - band->blocks[0].x0;
    int bh = band->blocks[0].y1 - band->blocks[0].y0;
    int cx, cy;
    if (bw == 0 || bh == 0) { cx = 1; cy = (int)n; }
    else { cx = (x1 - x0 + bw - 1) / bw; cy = (y1 - y0 + bh - 1) / bh; }
    TagTree incl(std::max(cx, 1), std::max(cy, 1)), imsb(std::max(cx, 1), std::max(cy, 1));
    for (size_t i = 0; i < n; ++i) {
      imsb.set((int)i, band->blocks[i].zbp);
      if (!band->blocks[i].passes.empty()) incl.set((int)i, 0);
    }
    for (size_t i = 0; i < n; ++i) {
      const EncBlock& b = band->blocks[i];
      incl.encode(bio, (int)i, 1);
      if (b.passes.empty()) continue;
      imsb.encode(bio, (int)i, 999);
      put_numpasses(bio, (uint32_t)b.passes.size());
      // codeblock_segments + length_increment (t2.rs:273-306)
      std::vector<std::pair<uint32_t, uint32_t>> segs;
      uint32_t sl = 0, sn = 0;
      for (size_t k = 0; k < b.passes.size(); ++k) {
        ++sn;
        sl += b.passes[k].length;
        if (b.passes[k].terminated || k + 1 == b.passes.size()) {
          segs.push_back({sl, sn});
          sl = sn = 0;
        }
      }
      uint32_t lblock = 3, inc = 0;
      for (auto& s : segs) {
        if (s.first == 0) continue;
        uint32_t need = floor_log2_u(s.first) + 1;
        uint32_t have = lblock + floor_log2_u(s.second);
        inc = std::max(inc, need > have ? need - have : 0u);
      }
      for (uint32_t k = 0; k < inc; ++k) bio.put(1);
      bio.put(0);
      lblock += inc;
      for (auto& s : segs) bio.bits(s.first, (int)(lblock + floor_log2_u(s.second)));
    }
  }
  return bio.flush();
}

std::vector<uint8_t> build_payload(const std::vector<Layout>& layouts) {
  // build_packet_sequence_for_components (t2.rs:422-473): LRCP with one layer
  // and one precinct -> for each resolution, for each component.
  int maxr = 0;
  for (const auto& l : layouts)
    for (const auto& b : l) maxr = std::max(maxr, b.res);
  std::vector<uint8_t> out;
  for (int r = 0; r <= maxr; ++r)
    for (const auto& l : layouts) {
      std::vector<const EncBand*> bands;
      for (const auto& b : l)
        if (b.res == r) bands.push_back(&b);
      if (bands.empty()) continue;
      auto hdr = packet_header(bands, 0, 0);
      out.insert(out.end(), hdr.begin(), hdr.end());
      for (const EncBand* b : bands)
        for (const auto& blk : b->blocks) out.insert(out.end(), blk.payload.begin(), blk.payload.end());
    }
  return out;
}

static void be16(std::vector<uint8_t>& o, uint32_t v) { o.push_back((uint8_t)(v >> 8)); o.push_back((uint8_t)v); }
static void be32(std::vector<uint8_t>& o, uint32_t v) { be16(o, v >> 16); be16(o, v & 0xffff); }

// SIZ, COD and QCD marker segments of a plan (src/j2k/markers.rs:8-110).
static std::vector<uint8_t> siz_segment(const Plan& p) {
  std::vector<uint8_t> o;
  be16(o, 0xff51);
  be16(o, 38 + 3 * p.ncomp);
  be16(o, 0);
  be32(o, p.width); be32(o, p.height);
  be32(o, 0); be32(o, 0);
  be32(o, p.width); be32(o, p.height);
  be32(o, 0); be32(o, 0);
  be16(o, p.ncomp);
  for (int c = 0; c < p.ncomp; ++c) {
    o.push_back((uint8_t)((p.precision - 1) & 0x7f));
    o.push_back(1);
    o.push_back(1);
  }
  return o;
}

static std::vector<uint8_t> cod_segment(const Plan& p) {
  std::vector<uint8_t> o;
  be16(o, 0xff52);
  be16(o, 12);
  o.push_back(0);
  o.push_back(0);  // LRCP
  be16(o, 1);
  o.push_back(p.use_mct ? 1 : 0);
  o.push_back((uint8_t)p.levels);
  o.push_back((uint8_t)(__builtin_ctz(p.cbw) - 2));
  o.push_back((uint8_t)(__builtin_ctz(p.cbh) - 2));
  o.push_back(0);
  o.push_back(p.lossless ? 1 : 0);
  return o;
}

static std::vector<uint8_t> qcd_segment(const Plan& p) {
  std::vector<uint8_t> o;
  be16(o, 0xff5c);
  if (p.lossless) {
    be16(o, 3 + (uint32_t)p.quants.size());
    o.push_back((uint8_t)(p.guard_bits << 5));
    for (const auto& q : p.quants) o.push_back((uint8_t)(q.exponent << 3));
  } else {
    be16(o, 3 + 2 * (uint32_t)p.quants.size());
    o.push_back((uint8_t)((p.guard_bits << 5) | 2));
    for (const auto& q : p.quants) be16(o, ((uint32_t)(q.exponent & 0xff) << 11 | (q.mantissa & 0x7ff)) & 0xffff);
  }
  return o;
}

// A main-header segment as the writer emits it: SIZ and COD are re-encoded
// from the plan when the plan's segment has the same length, QCD only for a
// reversible plan, anything else passes through (src/j2k/write.rs:80-113).
static void put_main_segment(std::vector<uint8_t>& o, const std::vector<uint8_t>& seg, const Plan& p) {
  const uint32_t m = seg.size() >= 2 ? ((uint32_t)seg[0] << 8 | seg[1]) : 0u;
  std::vector<uint8_t> local;
  if (m == 0xff51) local = siz_segment(p);
  else if (m == 0xff52) local = cod_segment(p);
  else if (m == 0xff5c && p.lossless) local = qcd_segment(p);
  const std::vector<uint8_t>& use = !local.empty() && local.size() == seg.size() ? local : seg;
  for (uint8_t b : use) o.push_back(b);
}

// Codestream framing (CodestreamParts::encode, src/j2k/write.rs:9-77): SOC,
// the main-header segments, then per tile-part an SOT segment (Lsot 10,
// Isot, Psot = 12 + header segments + 2 + payload, TPsot, TNsot), its header
// segments, SOD and its payload; EOC.
std::vector<uint8_t> frame_codestream(const Plan& p, const std::vector<std::vector<uint8_t>>& main_segments,
                                      const std::vector<TilePartBytes>& parts) {
  if (p.ncomp == 0) throw Error(kEncodeFailed, "cannot emit codestream with zero components");
  std::vector<uint8_t> o;
  be16(o, 0xff4f);
  for (const auto& seg : main_segments) put_main_segment(o, seg, p);
  for (const auto& tp : parts) {
    uint64_t psot = 12 + 2 + (uint64_t)tp.payload.size();
    for (const auto& h : tp.header_segments) psot += h.size();
    if (psot > 0xffffffffull) throw Error(kEncodeFailed, "tile-part length exceeds Psot range");
    be16(o, 0xff90);
    be16(o, 10);
    be16(o, tp.tile_index);
    be32(o, (uint32_t)psot);
    o.push_back(tp.part_index);
    o.push_back(tp.total_parts);
    for (const auto& h : tp.header_segments) o.insert(o.end(), h.begin(), h.end());
    be16(o, 0xff93);
    o.insert(o.end(), tp.payload.begin(), tp.payload.end());
  }
  be16(o, 0xffd9);
  return o;
}

// Splits a single-tile codestream into its main-header segments and one
// tile-part (CodestreamParts::parse_single_tile, src/j2k/parse.rs): marker
// segments are delimited by their length fields; the payload runs from SOD
// to the EOC that ends the stream.
bool parse_single_tile(const uint8_t* b, size_t n, std::vector<std::vector<uint8_t>>* main_segments,
                       TilePartBytes* tp) {
  auto u16 = [&](size_t i) { return (uint32_t)b[i] << 8 | b[i + 1]; };
  if (n < 4 || u16(0) != 0xff4f || u16(n - 2) != 0xffd9) return false;
  size_t i = 2;
  while (i + 4 <= n && u16(i) != 0xff90) {
    const size_t len = 2 + u16(i + 2);
    if (i + len > n) return false;
    main_segments->emplace_back(b + i, b + i + len);
    i += len;
  }
  if (i + 12 > n || u16(i) != 0xff90 || u16(i + 2) != 10) return false;
  tp->tile_index = (uint16_t)u16(i + 4);
  tp->part_index = b[i + 10];
  tp->total_parts = b[i + 11];
  i += 12;
  while (i + 2 <= n && u16(i) != 0xff93) {
    if (i + 4 > n) return false;
    const size_t len = 2 + u16(i + 2);
    if (i + len > n) return false;
    tp->header_segments.emplace_back(b + i, b + i + len);
    i += len;
  }
  if (i + 2 > n - 2) return false;
  tp->payload.assign(b + i + 2, b + n - 2);
  return true;
}

std::vector<uint8_t> build_codestream(const Plan& p, const std::vector<uint8_t>& payload) {
  // the encoder's one tile-part: tile 0, part 0 of 1 (backend.rs:275-290)
  TilePartBytes tp;
  tp.tile_index = 0;
  tp.part_index = 0;
  tp.total_parts = 1;
  tp.payload = payload;
  return frame_codestream(p, {siz_segment(p), cod_segment(p), qcd_segment(p)}, {tp});
}

std::vector<uint8_t> wrap_jp2(const Plan& p, const std::vector<uint8_t>& cs) {
  // src/jp2.rs:13-71
  std::vector<uint8_t> o;
  auto hdr = [&](uint32_t len, const char* t) { be32(o, len); o.insert(o.end(), t, t + 4); };
  hdr(12, "jP  ");
  o.insert(o.end(), {0x0d, 0x0a, 0x87, 0x0a});
  hdr(20, "ftyp");
  o.insert(o.end(), {'j', 'p', '2', ' '});
  be32(o, 0);
  o.insert(o.end(), {'j', 'p', '2', ' '});
  hdr(8 + 22 + 15, "jp2h");
  hdr(22, "ihdr");
  be32(o, p.height); be32(o, p.width);
  be16(o, p.ncomp);
  o.push_back(7); o.push_back(7); o.push_back(0); o.push_back(0);
  hdr(15, "colr");
  o.push_back(1); o.push_back(0); o.push_back(0);
  be32(o, p.srgb ? 16 : 17);
  uint64_t bl = (uint64_t)cs.size() + 8;
  if (bl > 0xffffffffull) throw Error(kEncodeFailed, "JP2 box length exceeds 32-bit limit");
  hdr((uint32_t)bl, "jp2c");
  o.insert(o.end(), cs.begin(), cs.end());
  return o;
}

std::vector<uint8_t> encode(const Plan& p, const Planes& px, const EncodeOptions& opt) {
  // encode (src/encode/mod.rs:84-101)
  auto layouts = tier1_layouts(p, px, opt, true);
  auto payload = build_payload(layouts);
  auto cs = build_codestream(p, payload);
  if (p.format == 0) return cs;
  return wrap_jp2(p, cs);
}

// -------------------------------------------------------------- decoder ----
// Narrow decoder for this encoder's own output (src/decode/*.rs): JP2 boxes,
// SIZ/COD/QCD, one tile-part, LRCP packets with one layer and one precinct,
// Tier-1 decode with Mb taken from QCD (src/decode/t1.rs:56), midpoint
// dequantisation, inverse DWT and inverse MCT.
namespace {
struct Reader {
  const uint8_t* b; size_t n, pos = 0;
  uint32_t u8() { if (pos >= n) throw Error(kDecodeFailed, "truncated"); return b[pos++]; }
  uint32_t u16() { uint32_t v = u8() << 8; return v | u8(); }
  uint32_t u32() { uint32_t v = u16() << 16; return v | u16(); }
};
struct BitReader {  // packet header bit reader with 0xFF stuffing
  const uint8_t* b; size_t n, pos; uint32_t buf = 0, ct = 0;
  uint32_t bit() {
    if (ct == 0) {
      if (pos >= n) throw Error(kDecodeFailed, "packet header truncated");
      uint32_t prev = buf;
      buf = b[pos++];
      ct = (prev == 0xff) ? 7 : 8;
    }
    --ct;
    return (buf >> ct) & 1;
  }
  uint32_t bits(int k) { uint32_t v = 0; for (int i = 0; i < k; ++i) v = (v << 1) | bit(); return v; }
  void align() { if (buf == 0xff && ct == 0) { if (pos < n) ++pos; } ct = 0; buf = 0; }
};
struct DTagTree {
  struct Node { int parent, value, low; };
  std::vector<Node> nodes;
  DTagTree(int nw, int nh) {
    std::vector<std::pair<int, int>> dims;
    int w = nw, h = nh;
    for (;;) { dims.push_back({w, h}); if (w * h <= 1) break; w = (w + 1) / 2; h = (h + 1) / 2; }
    std::vector<int> base(dims.size() + 1, 0);
    for (size_t l = 0; l < dims.size(); ++l) base[l + 1] = base[l] + dims[l].first * dims[l].second;
    nodes.assign(base.back(), Node{-1, 999, 0});
    for (size_t l = 0; l + 1 < dims.size(); ++l)
      for (int j = 0; j < dims[l].second; ++j)
        for (int i = 0; i < dims[l].first; ++i)
          nodes[base[l] + j * dims[l].first + i].parent = base[l + 1] + (j / 2) * dims[l + 1].first + (i / 2);
  }
  // Returns true when value(leaf) < threshold (decoding the standard way).
  bool decode(BitReader& br, int leaf, int threshold) {
    int stk[64], depth = 0, n = leaf;
    while (nodes[n].parent >= 0) { stk[depth++] = n; n = nodes[n].parent; }
    int low = 0;
    for (;;) {
      Node& nd = nodes[n];
      if (low > nd.low) nd.low = low; else low = nd.low;
      while (low < threshold && low < nd.value) {
        if (br.bit()) nd.value = low; else ++low;
      }
      nd.low = low;
      if (depth == 0) break;
      n = stk[--depth];
    }
    return nodes[leaf].value < threshold;
  }
};
}  // namespace

Decoded decode(const uint8_t* bytes, size_t n, bool rct_chroma_extra_bitplane, bool accept_empty_segments) {

  const uint8_t* cs = bytes;
  size_t csn = n;
  int colr = -1;
  if (n >= 12 && bytes[4] == 'j' && bytes[5] == 'P') {
    // JP2 boxes (src/decode/jp2_parse.rs)
    size_t pos = 0;
    bool found = false;
    while (pos + 8 <= n) {
      Reader br{bytes, n, pos};
      uint32_t len = br.u32();
      uint32_t t = br.u32();
      if (len < 8 || pos + len > n) throw Error(kDecodeFailed, "bad JP2 box");
      if (t == 0x6a703268) {  // jp2h: look for colr
        size_t q = pos + 8;
        while (q + 8 <= pos + len) {
          Reader sb{bytes, n, q};
          uint32_t sl = sb.u32(), st = sb.u32();
          if (st == 0x636f6c72) { sb.u8(); sb.u8(); sb.u8(); colr = (int)sb.u32(); }
          if (sl < 8) break;
          q += sl;
        }
      }
      if (t == 0x6a703263) { cs = bytes + pos + 8; csn = len - 8; found = true; break; }
      pos += len;
    }
    if (!found) throw Error(kDecodeFailed, "no jp2c box");
  }
  Reader c{cs, csn};
  if (c.u16() != 0xff4f) throw Error(kDecodeFailed, "missing SOC");
  uint32_t W = 0, H = 0; int C = 0, levels = 0, cbw = 64, cbh = 64, guard = 2;
  bool rev = true, mct = false;
  std::vector<std::pair<int, int>> steps;  // (exponent, mantissa)
  size_t payload_start = 0, payload_end = 0;
  for (;;) {
    uint32_t m = c.u16();
    if (m == 0xff90) {
      uint32_t len = c.u16(); (void)len;
      c.u16();
      uint32_t psot = c.u32();
      c.u8(); c.u8();
      size_t sot_start = c.pos - 12;
      uint32_t sod = c.u16();
      if (sod != 0xff93) throw Error(kDecodeFailed, "expected SOD");
      payload_start = c.pos;
      payload_end = sot_start + psot;
      break;
    }
    uint32_t len = c.u16();
    size_t end = c.pos + len - 2;
    if (m == 0xff51) {
      c.u16(); W = c.u32(); H = c.u32(); c.u32(); c.u32(); c.u32(); c.u32(); c.u32(); c.u32();
      C = (int)c.u16();
      for (int i = 0; i < C; ++i) { c.u8(); c.u8(); c.u8(); }
    } else if (m == 0xff52) {
      c.u8(); c.u8(); c.u16(); mct = c.u8() != 0; levels = (int)c.u8();
      cbw = 1 << (c.u8() + 2); cbh = 1 << (c.u8() + 2); c.u8(); rev = c.u8() == 1;
    } else if (m == 0xff5c) {
      uint32_t sq = c.u8();
      guard = (int)(sq >> 5);
      if ((sq & 0x1f) == 0) {
        for (size_t i = c.pos; i < end; ++i) steps.push_back({(int)(c.u8() >> 3), 0});
      } else {
        while (c.pos + 1 < end + 1 && c.pos < end) {
          uint32_t v = c.u16();
          steps.push_back({(int)(v >> 11), (int)(v & 0x7ff)});
        }
      }
    }
    c.pos = end;
  }
  (void)colr;
  Decoded out{W, H, C, Planes(C, std::vector<int32_t>((size_t)W * H, 0))};
  auto rects = band_rects(W, H, levels);
  // Coefficient planes per component.
  std::vector<std::vector<int32_t>> coef(C, std::vector<int32_t>((size_t)W * H, 0));
  BitReader br{cs, payload_end, payload_start};
  size_t pos = payload_start;
  for (int res = 0; res <= levels; ++res)
    for (int comp = 0; comp < C; ++comp) {
      struct Blk { int bi, x0, y0, x1, y1; bool inc = false; int zbp = 0, np = 0; uint32_t len = 0; };
      std::vector<Blk> blks;
      br.pos = pos; br.ct = 0; br.buf = 0;
      if (br.bit() == 0) throw Error(kUnsupportedFeature, "empty packets are not produced by this encoder");
      for (size_t bi = 0; bi < rects.size(); ++bi) {
        const auto& rc = rects[bi];
        if (rc.res != res) continue;
        std::vector<Blk> bb;
        for (int by = rc.y0; by < rc.y1; by = std::min(by + cbh, rc.y1))
          for (int bx = rc.x0; bx < rc.x1; bx = std::min(bx + cbw, rc.x1))
            bb.push_back({(int)bi, bx, by, std::min(bx + cbw, rc.x1), std::min(by + cbh, rc.y1)});
        if (bb.empty()) continue;
        int fw = bb[0].x1 - bb[0].x0, fh = bb[0].y1 - bb[0].y0;
        int cx = (rc.x1 - rc.x0 + fw - 1) / fw, cy = (rc.y1 - rc.y0 + fh - 1) / fh;
        DTagTree incl(cx, cy), imsb(cx, cy);
        for (size_t i = 0; i < bb.size(); ++i) {
          Blk& b = bb[i];
          b.inc = incl.decode(br, (int)i, 1);
          if (!b.inc) continue;
          int z = 0;
          while (!imsb.decode(br, (int)i, z + 1)) ++z;
          b.zbp = z;
          // Table B-4
          int np;
          if (!br.bit()) np = 1;
          else if (!br.bit()) np = 2;
          else {
            uint32_t v = br.bits(2);
            if (v != 3) np = 3 + (int)v;
            else {
              v = br.bits(5);
              if (v != 31) np = 6 + (int)v;
              else np = 37 + (int)br.bits(7);
            }
          }
          b.np = np;
          int lblock = 3;
          while (br.bit()) ++lblock;
          b.len = br.bits(lblock + floor_log2_u((uint32_t)np));
        }
        blks.insert(blks.end(), bb.begin(), bb.end());
      }
      br.align();
      size_t body = br.pos;
      for (auto& b : blks) {
        if (!b.inc) continue;
        const auto& rc = rects[b.bi];
        if (body + b.len > payload_end) throw Error(kDecodeFailed, "code-block data past tile-part end");
        size_t si = b.bi % steps.size();
        // Mb from QCD as the reference's decoder takes it (decode/t1.rs:56);
        // optionally with the extra bit-plane the encoder gives RCT chroma
        // at q >= 100 (backend.rs:179-189), which QCD does not signal
        int mb = guard - 1 + steps[si].first + (rct_chroma_extra_bitplane && rev && mct && comp > 0 ? 1 : 0);
        int bw = b.x1 - b.x0, bh = b.y1 - b.y0;
        auto dv = decode_block(cs + body, b.len, bw, bh, rc.band, mb, b.zbp, b.np, accept_empty_segments);
        for (int y = 0; y < bh; ++y)
          for (int x = 0; x < bw; ++x) coef[comp][(size_t)(b.y0 + y) * W + b.x0 + x] = dv[(size_t)y * bw + x];
        body += b.len;
      }
      pos = body;
    }
  // Reconstruction (src/decode/reconstruct.rs).
  if (rev) {
    for (int comp = 0; comp < C; ++comp) inv53_2d(coef[comp].data(), W, H, levels);
    for (size_t i = 0; i < (size_t)W * H; ++i) {
      if (mct && C == 3) {  // inverse RCT (src/simd/scalar.rs:216-228)
        int32_t yy = coef[0][i], db = coef[1][i], dr = coef[2][i];
        int32_t g = yy - ((db + dr) >> 2);
        coef[0][i] = dr + g; coef[1][i] = g; coef[2][i] = db + g;
      }
      for (int comp = 0; comp < C; ++comp)
        out.comps[comp][i] = std::min(std::max(coef[comp][i] + 128, 0), 255);
    }
  } else {
    std::vector<std::vector<float>> f(C, std::vector<float>((size_t)W * H, 0.0f));
    for (int comp = 0; comp < C; ++comp) {
      for (size_t bi = 0; bi < rects.size(); ++bi) {
        const auto& rc = rects[bi];
        float step = quant_step_f32(8, rc.band, steps[bi].first, steps[bi].second);
        for (int y = rc.y0; y < rc.y1; ++y)
          for (int x = rc.x0; x < rc.x1; ++x) {
            int32_t q = coef[comp][(size_t)y * W + x];
            float v = 0.0f;  // src/simd/scalar.rs:122-129
            if (q != 0) {
              float sign = q >= 0 ? 1.0f : -1.0f;
              uint32_t a = q < 0 ? (uint32_t)(-(int64_t)q) : (uint32_t)q;
              v = sign * ((float)a + 0.5f) * step;
            }
            f[comp][(size_t)y * W + x] = v;
          }
      }
      inv97_2d(f[comp].data(), W, H, levels);
    }
    for (size_t i = 0; i < (size_t)W * H; ++i) {
      if (mct && C == 3) {  // inverse ICT (src/simd/scalar.rs:201-214)
        float yy = f[0][i], cb = f[1][i], cr = f[2][i];
        f[0][i] = yy + 1.402f * cr;
        f[1][i] = yy - 0.34413f * cb - 0.71414f * cr;
        f[2][i] = yy + 1.772f * cb;
      }
      for (int comp = 0; comp < C; ++comp) {  // finalize_f32 (scalar.rs:237-242)
        float v = std::round(f[comp][i] + 128.0f);
        v = std::min(std::max(v, 0.0f), 255.0f);
        out.comps[comp][i] = (int32_t)v;
      }
    }
  }
  return out;
}

// ------------------------------------------------------- quality metrics ---
static double mssim_8x8(const std::vector<float>& a, const std::vector<float>& b, int w, int h) {
  // backend.rs:911-959
  const double C1 = 6.5025, C2 = 58.5225;
  int br = h / 8, bc = w / 8;
  if (br == 0 || bc == 0) return 1.0;
  double sum = 0.0, n = 64.0;
  for (int y0 = 0; y0 < br; ++y0)
    for (int x0 = 0; x0 < bc; ++x0) {
      double sx = 0, sy = 0, sxx = 0, syy = 0, sxy = 0;
      for (int dy = 0; dy < 8; ++dy)
        for (int dx = 0; dx < 8; ++dx) {
          size_t i = (size_t)(y0 * 8 + dy) * w + x0 * 8 + dx;
          double x = a[i], y = b[i];
          sx += x; sy += y; sxx += x * x; syy += y * y; sxy += x * y;
        }
      double ux = sx / n, uy = sy / n;
      double vx = std::max(sxx / n - ux * ux, 0.0), vy = std::max(syy / n - uy * uy, 0.0);
      double cxy = sxy / n - ux * uy;
      sum += ((2 * ux * uy + C1) * (2 * cxy + C2)) / ((ux * ux + uy * uy + C1) * (vx + vy + C2));
    }
  return sum / (double)(br * bc);
}

void quality_metrics(const Plan& p, const Planes& px, const EncodeOptions& opt,
                     double* psnr, double* ssim) {
  // compute_quality_metrics (backend.rs:305-433)
  if (p.quality >= 100) { *psnr = std::numeric_limits<double>::infinity(); *ssim = 1.0; return; }
  auto layouts = tier1_layouts(p, px, opt, true);
  int W = p.width, H = p.height;
  size_t N = (size_t)W * H;
  std::vector<std::vector<float>> rec;
  for (int c = 0; c < p.ncomp; ++c) {
    auto q = component_coefficients(p, px, c, opt.threads);
    std::vector<float> d(N, 0.0f);
    for (const auto& band : layouts[c]) {
      float step = 1.0f;
      for (const auto& sq : p.quants)
        if (sq.resolution == band.res && sq.band == band.band)
          step = quant_step_f32(p.precision, band.band, sq.exponent, sq.mantissa);
      for (const auto& blk : band.blocks) {
        bool has = !blk.passes.empty();
        int lb = has ? blk.passes.back().bitplane : 0;
        for (int y = blk.y0; y < blk.y1; ++y)
          for (int x = blk.x0; x < blk.x1; ++x) {
            int32_t v = q[(size_t)y * W + x];
            float out = 0.0f;
            if (has) {  // dequantize_truncated_coeff (backend.rs:628-639)
              uint32_t a = v < 0 ? (uint32_t)(-(int64_t)v) : (uint32_t)v;
              uint32_t t = (a >> lb) << lb;
              if (t != 0) out = (v >= 0 ? 1.0f : -1.0f) * ((float)t + 0.5f) * step;
            }
            d[(size_t)y * W + x] = out;
          }
      }
    }
    inv97_2d(d.data(), W, H, p.levels);
    rec.push_back(std::move(d));
  }
  std::vector<float> dl(N), ol(N);
  double sse = 0.0;
  size_t ns;
  if (p.ncomp == 1) {
    ns = N;
    for (size_t i = 0; i < N; ++i) {
      float dec = std::min(std::max(rec[0][i] + 128.0f, 0.0f), 255.0f);
      float diff = dec - (float)px[0][i];
      sse += (double)(diff * diff);
      dl[i] = dec;
      ol[i] = (float)px[0][i];
    }
  } else {
    ns = N * 3;
    for (size_t i = 0; i < N; ++i) {
      float yc = rec[0][i], cb = rec[1][i], cr = rec[2][i];
      float r = std::min(std::max(yc + 1.402f * cr + 128.0f, 0.0f), 255.0f);
      float g = std::min(std::max(yc - 0.34413f * cb - 0.71414f * cr + 128.0f, 0.0f), 255.0f);
      float b = std::min(std::max(yc + 1.772f * cb + 128.0f, 0.0f), 255.0f);
      float dr = r - (float)px[0][i], dg = g - (float)px[1][i], db = b - (float)px[2][i];
      sse += (double)(dr * dr + dg * dg + db * db);
      dl[i] = 0.299f * r + 0.587f * g + 0.114f * b;
      ol[i] = 0.299f * (float)px[0][i] + 0.587f * (float)px[1][i] + 0.114f * (float)px[2][i];
    }
  }
  double mse = sse / (double)ns;
  *psnr = mse < 1e-10 ? 100.0 : 20.0 * std::log10(255.0 / std::sqrt(mse));
  *ssim = mssim_8x8(ol, dl, W, H);
}

// ------------------------------------------------------ contrast mask ------
// build_luma_contrast_mask (backend.rs:724-769) -> contrast_mask.rs:225-291.
// Its result is discarded by the reference (rate.rs:56-60); it is restated
// only so that the "as shipped" CPU baseline does the same work.
double contrast_mask_work(const Plan& p, const Planes& px) {
  int W = p.width, H = p.height;
  std::vector<uint8_t> luma((size_t)W * H);
  for (size_t i = 0; i < luma.size(); ++i) {
    if (p.ncomp == 1) luma[i] = (uint8_t)std::min(std::max(px[0][i], 0), 255);
    else {
      double y = 0.299 * px[0][i] + 0.587 * px[1][i] + 0.114 * px[2][i];
      y = std::min(std::max(y, 0.0), 255.0);
      luma[i] = (uint8_t)y;
    }
  }
  static const double csf[8][8] = {
      {0.0000, 0.8264, 1.0000, 0.3906, 0.1736, 0.0625, 0.0384, 0.0269},
      {0.6944, 0.6944, 0.5102, 0.2770, 0.1479, 0.0297, 0.0278, 0.0331},
      {0.5102, 0.5917, 0.3906, 0.1736, 0.0625, 0.0308, 0.0210, 0.0319},
      {0.5102, 0.3460, 0.2066, 0.1189, 0.0384, 0.0132, 0.0156, 0.0260},
      {0.3086, 0.2066, 0.0730, 0.0319, 0.0216, 0.0084, 0.0094, 0.0169},
      {0.1736, 0.0816, 0.0331, 0.0244, 0.0152, 0.0092, 0.0078, 0.0118},
      {0.0416, 0.0244, 0.0164, 0.0132, 0.0094, 0.0068, 0.0069, 0.0098},
      {0.0193, 0.0118, 0.0111, 0.0104, 0.0080, 0.0100, 0.0094, 0.0102}};
  int bx = (W + 7) / 8, by = (H + 7) / 8;
  std::vector<double> energies;
  energies.reserve((size_t)bx * by);
  double acc = 0.0;
  for (int yb = 0; yb < by; ++yb)
    for (int xb = 0; xb < bx; ++xb) {
      double blk[64];
      for (int y = 0; y < 8; ++y)
        for (int x = 0; x < 8; ++x) {
          int sx = std::min(xb * 8 + x, W - 1), sy = std::min(yb * 8 + y, H - 1);
          blk[y * 8 + x] = luma[(size_t)sy * W + sx];
        }
      double ew = 0.0;
      for (int u = 0; u < 8; ++u)
        for (int v = 0; v < 8; ++v) {  // naive DCT with cos in the inner loop
          double au = u == 0 ? 1.0 / std::sqrt(2.0) : 1.0, av = v == 0 ? 1.0 / std::sqrt(2.0) : 1.0;
          double s = 0.0;
          for (int y = 0; y < 8; ++y)
            for (int x = 0; x < 8; ++x)
              s += blk[y * 8 + x] * std::cos(((2 * x + 1) * (double)u * M_PI) / 16.0) *
                   std::cos(((2 * y + 1) * (double)v * M_PI) / 16.0);
          double cf = 0.25 * au * av * s;
          ew += cf * cf * csf[u][v];
        }
      double mean = 0.0;
      for (double v : blk) mean += v;
      mean /= 64.0;
      double var = 0.0;
      for (double v : blk) var += (v - mean) * (v - mean);
      var /= 64.0;
      energies.push_back(ew * (var > 1e-9 ? 1.0 : 0.0) / 16.0);
      acc += ew;
    }
  if (!energies.empty()) {
    size_t k = (size_t)(0.75 * (double)(energies.size() - 1));
    std::nth_element(energies.begin(), energies.begin() + k, energies.end());
    acc += energies[k];
  }
  return acc;
}

}  // namespace orc

// ------------------------------------------------ known-answer helpers -----
// Small entry points for the ported unit tests (t2.rs:594-649, pcrd.rs:1022-1100).
extern "C" {

// Table B-4 codeword of `n` passes, returned as its bit string in `bits`.
int orc_t2_numpasses_bits(uint32_t n, uint32_t* code, int* width) {
  orc::Bio bio;
  orc::put_numpasses(bio, n);
  uint32_t v = 0;
  int k = 0;
  // Re-read the bits from the register/buffer: the writer stores MSB first.
  std::vector<uint8_t> bytes = bio.buf;
  uint32_t reg = bio.reg, ct = bio.ct;
  // A byte after 0xFF carries only 7 bits (its MSB is the stuffed 0).
  int top = 7;
  for (uint8_t b : bytes) {
    for (int i = top; i >= 0; --i) { v = (v << 1) | ((b >> i) & 1); ++k; }
    top = (b == 0xff) ? 6 : 7;
  }
  for (int i = top; i >= (int)ct; --i) { v = (v << 1) | ((reg >> i) & 1); ++k; }
  *code = v;
  *width = k;
  return 0;
}

// Segments of a pass sequence and the Lblock increment from Lblock=3.
int orc_t2_segments(const uint32_t* lengths, const int* terminated, int n,
                    uint32_t* seg_len, uint32_t* seg_np, int* nseg, uint32_t* increment) {
  std::vector<std::pair<uint32_t, uint32_t>> segs;
  uint32_t sl = 0, sn = 0;
  for (int k = 0; k < n; ++k) {
    ++sn;
    sl += lengths[k];
    if (terminated[k] || k + 1 == n) { segs.push_back({sl, sn}); sl = sn = 0; }
  }
  uint32_t inc = 0;
  for (auto& s : segs) {
    if (s.first == 0) continue;
    uint32_t need = orc::floor_log2_u(s.first) + 1;
    uint32_t have = 3 + orc::floor_log2_u(s.second);
    inc = std::max(inc, need > have ? need - have : 0u);
  }
  for (size_t i = 0; i < segs.size(); ++i) { seg_len[i] = segs[i].first; seg_np[i] = segs[i].second; }
  *nseg = (int)segs.size();
  *increment = inc;
  return 0;
}

// Build the hull of one raw curve (cumulative bytes, incremental distortion)
// and return the pass count chosen at `lambda`; the hull is written to
// hull_passes / hull_slopes.
int orc_pcrd_select(const uint32_t* cum_bytes, const double* dist, int n, double lambda,
                    int* hull_passes, double* hull_slopes, int* nhull) {
  try {
    std::vector<orc::Pt> pts;
    pts.push_back({0, 0, 0.0, std::numeric_limits<double>::infinity()});
    double cd = 0.0;
    for (int i = 0; i < n; ++i) { cd += dist[i]; pts.push_back({i + 1, cum_bytes[i], cd, 0.0}); }
    orc::fill_slopes(pts);
    std::vector<orc::Pt> hull;
    for (const auto& pt : pts) {
      hull.push_back(pt);
      while (hull.size() >= 3) {
        double sab = orc::rd_slope(hull[hull.size() - 3], hull[hull.size() - 2]);
        double sbc = orc::rd_slope(hull[hull.size() - 2], hull[hull.size() - 1]);
        if (sbc >= sab) hull.erase(hull.end() - 2); else break;
      }
    }
    orc::fill_slopes(hull);
    int keep = 0;
    for (size_t i = 1; i < hull.size(); ++i) {
      if (hull[i].slope >= lambda) keep = hull[i].passes; else break;
    }
    for (size_t i = 0; i < hull.size(); ++i) { hull_passes[i] = hull[i].passes; hull_slopes[i] = hull[i].slope; }
    *nhull = (int)hull.size();
    return keep;
  } catch (const orc::Error&) {
    return -1;
  }
}

// Tier-1 decode of one code-block (src/decode/t1.rs:87-210).
int orc_t1_decode(const uint8_t* data, size_t n, int w, int h, int band, int mb, int zbp,
                  int npasses, int32_t* out) {
  try {
    auto v = orc::decode_block(data, n, w, h, (orc::Band)band, mb, zbp, npasses);
    std::memcpy(out, v.data(), v.size() * sizeof(int32_t));
    return 0;
  } catch (const orc::Error& e) {
    return e.code;
  }
}

}  // extern "C"
