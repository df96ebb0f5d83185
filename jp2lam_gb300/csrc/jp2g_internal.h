// Internal structures shared by the host pipeline and the CUDA kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace jp2g {

// Status codes map 1:1 to Jp2LamError variants (src/error.rs:7-13).
enum Status : int {
  kOk = 0,
  kInvalidInput = 1,
  kEncodeFailed = 2,
  kDecodeFailed = 3,
  kUnsupportedFeature = 4,
  kIo = 5,
};

struct Failure {
  int code;
  std::string msg;
};

// Band orientation index (LL=0, HL=1, LH=2, HH=3), also the row of the
// zero-coding context table.
enum Orient : int { LL = 0, HL = 1, LH = 2, HH = 3 };

// ----------------------------------------------------------------- plan ----
struct BandQuant {
  int res;
  int orient;
  int exponent;
  int mantissa;
  float step_f32;    // quantiser step (backend.rs:602-620)
  double step_f64;   // PCRD step (rate.rs:316-320)
};

// One subband of one component, with its code-block grid.
struct BandGeom {
  int comp;
  int res;
  int orient;
  int x0, y0, x1, y1;  // Mallat-layout rectangle
  int ncbx, ncby;      // code-block grid
  uint32_t first_block;  // index of its first block in the page work list
  int mb;              // maximum bit-planes for zero bit-plane counting
  int quant;           // index into PagePlan::quants
};

struct PagePlan {
  uint32_t width = 0, height = 0;
  int ncomp = 1;
  bool srgb = false;
  int quality = 85;
  int format = 1;
  bool lossless = false;
  bool use_mct = false;
  int levels = 0;
  int cbw = 64, cbh = 64;
  int guard_bits = 2;
  int precision = 8;
  std::vector<BandQuant> quants;     // LL, then (HL, LH, HH) per resolution
  std::vector<BandGeom> bands;       // codestream order: res -> comp -> band
  uint32_t nblocks = 0;
  int max_mb = 0;
  // Resolution ladder, index 0 = smallest (LL), index levels = full size.
  std::vector<std::pair<int, int>> ladder;
  // PCRD parameters computed on the host with the platform libm, like the
  // reference (quality_to_lambda at q and at q=1; chroma weight).
  double lambda_raw = 0.0, lambda_floor = 0.0;
  double comp_weight[3] = {1.0, 1.0, 1.0};
};

bool build_plan(uint32_t w, uint32_t h, int ncomp, int quality, int format,
                PagePlan* plan, Failure* err);
float quant_step_from_qcd(int precision, int orient, int exponent, int mantissa);

// -------------------------------------------------------- device layout ----
// Per-block descriptor in the flat work list.
struct BlockDesc {
  uint32_t coef_slot;   // coefficient slot index (slot = cbw*cbh int32)
  uint16_t w, h;        // block size
  uint8_t orient;
  uint8_t mb;           // maximum bit-planes of the band
  uint16_t band_param;  // index into the PCRD band table
  uint32_t comp_key;    // (page, component) key for the PCRD lambda
  uint32_t out_off;     // byte offset of the block's payload slot
  uint32_t out_cap;     // capacity of the payload slot
  uint32_t pass_off;    // index of the block's first pass record
};

// Tier-1 per-pass record (t1.rs:508-607): numbytes() snapshot after the pass,
// newly-significant count and significant-before count.
struct PassRec {
  uint32_t snap;
  uint32_t ns;
  uint32_t sig_before;
  uint8_t kind;      // 0 SP, 1 MR, 2 CL
  uint8_t bitplane;
  uint16_t pad;
};

// Tier-1 modelling result of one (code-block, bit-plane) item: symbol counts
// of its passes (SP, MR, cleanup), newly significant counts, and the number
// of samples significant before the bit-plane.
struct ItemRec {
  uint32_t n_sp, n_mr, n_cl;
  uint32_t ns_sp, ns_cl;
  uint32_t sig_before;
  uint32_t bitplane;
  uint32_t pad;
};

// Tier-1 per-block result.
struct BlockOut {
  uint32_t payload_len;  // terminated byte count (take_bytes)
  uint16_t npasses;
  uint8_t mbp;
  uint8_t zbp;
  uint8_t cls;       // BlockClass 0 Flat, 1 Gradient, 2 TexturePhoto
  uint8_t status;    // 0 ok, 1 payload slot overflow
  uint16_t pad;
  uint32_t pad2;
};

// Retained (PCRD-selected) result per block, read back by the host.
struct BlockKeep {
  uint32_t seg_len;   // signalled segment length (sum of retained lengths)
  uint32_t body_len;  // bytes copied into the packet body
  uint16_t npasses;   // retained passes
  uint8_t zbp;
  uint8_t status;
};

// PCRD constants per band (rate.rs:43-85).
struct BandParam {
  double quant_step;
  double subband_weight;  // norm97^2
  double band_bias;
  uint32_t is_ll;
  uint32_t pad;
};

// PCRD constants per (page, component).
struct CompParam {
  double lambda_raw;
  double lambda_floor;
  double comp_weight;
  uint32_t lossless;  // PCRD skipped when quality >= 100
  int32_t quality;
};

}  // namespace jp2g
