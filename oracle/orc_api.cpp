// Oracle (test infrastructure): C ABI used by tests/ through ctypes, by
// __graft_entry__.smoke() as the checker, and by bench.py's cpu_baseline leg.
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <string>

#include "orc.h"

namespace {
thread_local std::string g_err;

int fail(const orc::Error& e) {
  g_err = e.what();
  return e.code;
}

uint8_t* dup(const std::vector<uint8_t>& v, size_t* len) {
  uint8_t* p = static_cast<uint8_t*>(std::malloc(v.empty() ? 1 : v.size()));
  if (!v.empty()) std::memcpy(p, v.data(), v.size());
  *len = v.size();
  return p;
}

int check_input(uint32_t w, uint32_t h, int ncomp) {
  if (w == 0 || h == 0) {
    g_err = "image dimensions must be non-zero";
    return orc::kInvalidInput;
  }
  if (ncomp != 1 && ncomp != 3) {
    g_err = "images must have 1 or 3 components";
    return orc::kInvalidInput;
  }
  return 0;
}
}  // namespace

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }
void orc_free(void* p) { std::free(p); }

// Full encode of interleaved 8-bit pixels (gray or RGB) -> J2K/JP2 bytes.
int orc_encode(const uint8_t* px, uint32_t w, uint32_t h, int ncomp, int quality,
               int format, int threads, int contrast_mask, uint8_t** out,
               size_t* out_len) {
  if (int rc = check_input(w, h, ncomp)) return rc;
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, format);
    orc::Planes planes = orc::planes_from_bytes(px, w, h, ncomp);
    orc::EncodeOptions opt;
    opt.threads = threads < 1 ? 1 : threads;
    opt.contrast_mask = contrast_mask != 0;
    *out = dup(orc::encode(p, planes, opt), out_len);
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

// Tier-2, markers and JP2 boxes of a page from per-block retained data in
// codestream order (see layouts_from_blocks); the bodies are consecutive in
// `body`.
int orc_assemble(uint32_t w, uint32_t h, int ncomp, int quality, int format, const uint16_t* npasses,
                 const uint8_t* zbp, const uint32_t* seg_len, const uint8_t* body, uint32_t nblocks,
                 uint8_t** out, size_t* out_len) {
  if (int rc = check_input(w, h, ncomp)) return rc;
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, format);
    auto layouts = orc::layouts_from_blocks(p, npasses, zbp, seg_len, body, nblocks);
    auto cs = orc::build_codestream(p, orc::build_payload(layouts));
    *out = dup(format == 1 ? orc::wrap_jp2(p, cs) : cs, out_len);
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

// Codestream framing alone (src/j2k/write.rs:9-113) under the plan of a
// w x h x ncomp page at `quality`: SOC, the main-header segments in `main`
// (marker segments back to back, split by their length fields), one
// tile-part (tile, part, parts) with the header segments in `tile_hdr` and
// the payload bytes, EOC.
int orc_frame(uint32_t w, uint32_t h, int ncomp, int quality, const uint8_t* main, size_t main_n,
              const uint8_t* tile_hdr, size_t tile_hdr_n, int tile, int part, int parts,
              const uint8_t* payload, size_t payload_n, uint8_t** out, size_t* out_len) {
  if (int rc = check_input(w, h, ncomp)) return rc;
  auto split = [](const uint8_t* b, size_t n, std::vector<std::vector<uint8_t>>* segs) {
    size_t i = 0;
    while (i + 4 <= n) {
      const size_t len = 2 + ((size_t)b[i + 2] << 8 | b[i + 3]);
      if (i + len > n) return false;
      segs->emplace_back(b + i, b + i + len);
      i += len;
    }
    return i == n;
  };
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, 0);
    std::vector<std::vector<uint8_t>> segs;
    orc::TilePartBytes tp;
    if (!split(main, main_n, &segs) || !split(tile_hdr, tile_hdr_n, &tp.header_segments)) {
      g_err = "malformed marker segments";
      return orc::kInvalidInput;
    }
    tp.tile_index = (uint16_t)tile;
    tp.part_index = (uint8_t)part;
    tp.total_parts = (uint8_t)parts;
    tp.payload.assign(payload, payload + payload_n);
    *out = dup(orc::frame_codestream(p, segs, {tp}), out_len);
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

// Parses a single-tile codestream into its parts and frames it again under
// the plan of a w x h x ncomp page at `quality`
// (CodestreamParts::parse_single_tile + encode, src/j2k/parse.rs,
// src/j2k/write.rs).
int orc_reframe(const uint8_t* cs, size_t n, uint32_t w, uint32_t h, int ncomp, int quality, uint8_t** out,
                size_t* out_len) {
  if (int rc = check_input(w, h, ncomp)) return rc;
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, 0);
    std::vector<std::vector<uint8_t>> segs;
    orc::TilePartBytes tp;
    if (!orc::parse_single_tile(cs, n, &segs, &tp)) {
      g_err = "not a single-tile codestream";
      return orc::kDecodeFailed;
    }
    *out = dup(orc::frame_codestream(p, segs, {tp}), out_len);
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

// FP64 9/7 coefficients of one component (irreversible path, unquantised,
// Mallat layout, W*H double), the quantiser step of each position (W*H
// float) and, when f32_out is not null, the restatement's own f32
// coefficients before quantisation, for measuring the f32 pipeline against
// exact lifting.
int orc_coefficients_f64(const uint8_t* px, uint32_t w, uint32_t h, int ncomp, int quality, int comp,
                         double* out, float* steps, float* f32_out) {
  if (int rc = check_input(w, h, ncomp)) return rc;
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, 0);
    if (p.lossless) {
      g_err = "the FP64 9/7 path is for lossy qualities";
      return orc::kInvalidInput;
    }
    orc::Planes planes = orc::planes_from_bytes(px, w, h, ncomp);
    auto c = orc::component_coefficients_f64(p, planes, comp);
    if (f32_out) {
      auto f = orc::component_unquantized_f32(p, planes, comp, 1);
      std::memcpy(f32_out, f.data(), f.size() * sizeof(float));
    }
    auto st = orc::coefficient_steps(p);
    std::memcpy(out, c.data(), c.size() * sizeof(double));
    std::memcpy(steps, st.data(), st.size() * sizeof(float));
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

// Quantised coefficient plane of one component (Mallat layout, W*H int32).
int orc_coefficients(const uint8_t* px, uint32_t w, uint32_t h, int ncomp,
                     int quality, int comp, int32_t* out) {
  if (int rc = check_input(w, h, ncomp)) return rc;
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, 0);
    orc::Planes planes = orc::planes_from_bytes(px, w, h, ncomp);
    auto c = orc::component_coefficients(p, planes, comp, 1);
    std::memcpy(out, c.data(), c.size() * sizeof(int32_t));
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

// Plan summary: levels, cbw, quants as (res, band, exponent, mantissa).
int orc_plan(uint32_t w, uint32_t h, int ncomp, int quality, int* levels,
             int* cbw, int* nquant, int* quants /* 4 * 32 */) {
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, 0);
    *levels = p.levels;
    *cbw = p.cbw;
    *nquant = (int)p.quants.size();
    for (size_t i = 0; i < p.quants.size() && i < 32; ++i) {
      quants[4 * i + 0] = p.quants[i].resolution;
      quants[4 * i + 1] = p.quants[i].band;
      quants[4 * i + 2] = p.quants[i].exponent;
      quants[4 * i + 3] = p.quants[i].mantissa;
    }
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

void orc_encode_stepsize(int stepsize, int numbps, int* e, int* m) {
  orc::encode_stepsize(stepsize, numbps, e, m);
}
void orc_irreversible_quant(int precision, int nres, int res, int band, int* e, int* m) {
  orc::irreversible_expounded_quant(precision, nres, res, (orc::Band)band, e, m);
}
double orc_quality_to_lambda(int q, uint32_t pixels);
double orc_norm97(int level, int band) { return orc::get_norm_97(level, (orc::Band)band); }

int orc_fwd53(int32_t* d, int w, int h, int levels) { orc::fwd53_2d(d, w, h, levels); return 0; }
int orc_inv53(int32_t* d, int w, int h, int levels) { orc::inv53_2d(d, w, h, levels); return 0; }
int orc_fwd97(float* d, int w, int h, int levels) { orc::fwd97_2d(d, w, h, levels, 1); return 0; }
int orc_inv97(float* d, int w, int h, int levels) { orc::inv97_2d(d, w, h, levels); return 0; }

// Tables for comparison with the reference's literal tables.
void orc_tables(uint8_t* zc /*2048*/, uint8_t* sc /*256*/, uint8_t* spb /*256*/,
                uint16_t* mq /*94*4*/) {
  std::memcpy(zc, orc::zc_lut(), 2048);
  std::memcpy(sc, orc::sc_lut(), 256);
  std::memcpy(spb, orc::spb_lut(), 256);
  const orc::MqState* s = orc::mq_states();
  for (int i = 0; i < 94; ++i) {
    mq[4 * i + 0] = s[i].qe;
    mq[4 * i + 1] = s[i].mps;
    mq[4 * i + 2] = s[i].nmps;
    mq[4 * i + 3] = s[i].nlps;
  }
}

// MQ helpers: symbols are (ctx << 1) | bit.
uint8_t* orc_mq_encode(const uint8_t* syms, size_t n, int variant, size_t* len) {
  if (variant == 0) return dup(orc::mq_encode(syms, n), len);
  if (variant == 1) return dup(orc::mq_encode_alt(syms, n), len);
  return dup(orc::mq_erterm(syms, n), len);
}
void orc_mq_decode(const uint8_t* bytes, size_t nbytes, const uint8_t* ctxs, size_t n,
                   uint8_t* bits) {
  orc::mq_decode(bytes, nbytes, ctxs, n, bits);
}

// One code-block through Tier-1. Pass records: 6 ints per pass
// (kind, bitplane, ns, sig_before, length, cumulative).
int orc_t1_block(const int32_t* coefs, int w, int h, int band, int mb, int* mbp,
                 int* zbp, int* cls, int* npasses, int* passes /* 6 * cap */,
                 int cap, uint8_t** payload, size_t* plen) {
  try {
    orc::EncBlock b = orc::encode_block(coefs, w, h, (orc::Band)band, mb);
    *mbp = b.mbp;
    *zbp = b.zbp;
    *cls = b.cls;
    *npasses = (int)b.passes.size();
    for (size_t i = 0; i < b.passes.size() && (int)i < cap; ++i) {
      int* r = passes + 6 * i;
      r[0] = b.passes[i].kind;
      r[1] = b.passes[i].bitplane;
      r[2] = (int)b.passes[i].ns;
      r[3] = (int)b.passes[i].sig_before;
      r[4] = (int)b.passes[i].length;
      r[5] = (int)b.passes[i].cumulative;
    }
    *payload = dup(b.payload, plen);
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

// Per-block summary of the (PCRD-truncated) Tier-1 layout of every
// component, in codestream order: 8 ints per block
// (comp, res, band, x0, y0, mbp, zbp, npasses) plus the payload length.
int orc_block_summary(const uint8_t* px, uint32_t w, uint32_t h, int ncomp,
                      int quality, int pcrd, int* rows, int cap, int* nblocks) {
  if (int rc = check_input(w, h, ncomp)) return rc;
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, 0);
    orc::Planes planes = orc::planes_from_bytes(px, w, h, ncomp);
    orc::EncodeOptions opt;
    auto layouts = orc::tier1_layouts(p, planes, opt, pcrd != 0);
    int n = 0;
    for (int r = 0; r <= p.levels; ++r)
      for (int c = 0; c < p.ncomp; ++c)
        for (const auto& band : layouts[c]) {
          if (band.res != r) continue;
          for (const auto& b : band.blocks) {
            if (n < cap) {
              int* o = rows + 9 * n;
              o[0] = c; o[1] = b.res; o[2] = b.band; o[3] = b.x0; o[4] = b.y0;
              o[5] = b.mbp; o[6] = b.zbp; o[7] = (int)b.passes.size();
              o[8] = (int)b.payload.size();
            }
            ++n;
          }
        }
    *nblocks = n;
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

// Decode J2K/JP2 bytes -> interleaved 8-bit pixels (caller buffer W*H*C).
// The same, optionally reading RCT chroma code-blocks with the extra
// bit-plane their encoder used (the reference's decoder does not).
// flags: bit 0 = the extra RCT chroma bit-plane, bit 1 = accept code-blocks
// whose segment has zero bytes.
int orc_decode_ex(const uint8_t* bytes, size_t n, int flags, uint32_t* w, uint32_t* h,
                  int* ncomp, uint8_t* px, size_t cap) {
  try {
    orc::Decoded d = orc::decode(bytes, n, (flags & 1) != 0, (flags & 2) != 0);
    *w = d.width;
    *h = d.height;
    *ncomp = d.ncomp;
    size_t N = (size_t)d.width * d.height;
    if (px && cap >= N * d.ncomp)
      for (size_t i = 0; i < N; ++i)
        for (int c = 0; c < d.ncomp; ++c) px[i * d.ncomp + c] = (uint8_t)d.comps[c][i];
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

int orc_decode(const uint8_t* bytes, size_t n, uint32_t* w, uint32_t* h, int* ncomp,
               uint8_t* px, size_t cap) {
  return orc_decode_ex(bytes, n, 0, w, h, ncomp, px, cap);
}

int orc_quality_metrics(const uint8_t* px, uint32_t w, uint32_t h, int ncomp,
                        int quality, double* psnr, double* ssim) {
  if (int rc = check_input(w, h, ncomp)) return rc;
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, 0);
    orc::Planes planes = orc::planes_from_bytes(px, w, h, ncomp);
    orc::EncodeOptions opt;
    orc::quality_metrics(p, planes, opt, psnr, ssim);
    return 0;
  } catch (const orc::Error& e) {
    return fail(e);
  }
}

// Wall-clock timing of `iters` encodes after one warm-up, mirroring
// examples/benchmark.rs:177-238. Returns mean seconds per encode.
double orc_time_encode(const uint8_t* px, uint32_t w, uint32_t h, int ncomp,
                       int quality, int format, int threads, int contrast_mask,
                       int iters) {
  try {
    orc::Plan p = orc::build_plan(w, h, ncomp, quality, format);
    orc::Planes planes = orc::planes_from_bytes(px, w, h, ncomp);
    orc::EncodeOptions opt;
    opt.threads = threads < 1 ? 1 : threads;
    opt.contrast_mask = contrast_mask != 0;
    orc::encode(p, planes, opt);
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < iters; ++i) orc::encode(p, planes, opt);
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count() / (iters > 0 ? iters : 1);
  } catch (const orc::Error& e) {
    g_err = e.what();
    return -1.0;
  }
}

}  // extern "C"

namespace orc {
double quality_to_lambda(int quality, uint32_t pixels);
}
extern "C" double orc_quality_to_lambda(int q, uint32_t pixels) {
  return orc::quality_to_lambda(q, pixels);
}
