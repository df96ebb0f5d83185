// Oracle: CPU restatement of jp2lam's JPEG 2000 encode path.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product library links, loads or
// calls this code; it is the checker that the CUDA path is compared against
// (tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg only).
//
// Every function cites the reference file:line it restates. Parity of this
// restatement is pinned by the reference's own known-answer tests (ported in
// tests/test_oracle_kat.py) and by cross-implementation checks that mirror the
// reference's test strategy (two MQ coders, encode->decode round trips).
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

// Jp2LamError variants (src/error.rs:7-13) as integer codes.
enum ErrorCode : int {
  kOk = 0,
  kInvalidInput = 1,
  kEncodeFailed = 2,
  kDecodeFailed = 3,
  kUnsupportedFeature = 4,
  kIo = 5,
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// BandOrientation (src/plan/mod.rs:33-39); the integer value is the
// orientation index used by the context tables (src/tier1/helpers.rs:12-19).
enum Band : int { LL = 0, HL = 1, LH = 2, HH = 3 };

struct SubbandQuant {  // src/plan/mod.rs:73-79
  int resolution;
  Band band;
  int exponent;
  int mantissa;
};

// EncodingPlan (src/plan/mod.rs:93-114), reduced to the fields the encode
// path reads.
struct Plan {
  uint32_t width = 0, height = 0;
  int ncomp = 1;
  bool srgb = false;
  int quality = 85;
  int format = 1;  // 0 = J2K, 1 = JP2
  bool lossless = false;  // Reversible53 when true, Irreversible97 otherwise
  bool use_mct = false;
  int levels = 0;
  int nres = 1;
  int cbw = 64, cbh = 64;
  int guard_bits = 2;
  int precision = 8;
  std::vector<SubbandQuant> quants;
};

Plan build_plan(uint32_t w, uint32_t h, int ncomp, int quality, int format);

// --- plan helpers exposed for known-answer tests ---------------------------
int max_decompositions(uint32_t w, uint32_t h);
void encode_stepsize(int stepsize, int numbps, int* exponent, int* mantissa);
void irreversible_expounded_quant(int precision, int nres, int res, Band band,
                                  int* exponent, int* mantissa);
double quality_step_scaler(int quality);
double get_norm_97(int level, Band band);
int band_gain(Band b);
float quant_step_f32(int precision, Band band, int exponent, int mantissa);
double quant_step_f64(int precision, Band band, int exponent, int mantissa);

// --- colour + DWT + quantisation -------------------------------------------
// Planar component samples as the reference Image stores them (i32, 0..255).
using Planes = std::vector<std::vector<int32_t>>;

void fwd53_2d(int32_t* data, int w, int h, int levels);
void inv53_2d(int32_t* data, int w, int h, int levels);
void fwd97_2d(float* data, int w, int h, int levels, int threads);
void inv97_2d(float* data, int w, int h, int levels);

// Quantised (9/7) or raw (5/3) coefficient plane of one component in the
// reference's deinterleaved Mallat layout.
// FP64 forward 9/7 of one component (unquantised, Mallat layout) and the
// quantiser step of every coefficient position.
std::vector<float> component_unquantized_f32(const Plan& p, const Planes& px, int comp, int threads);
std::vector<double> component_coefficients_f64(const Plan& p, const Planes& px, int comp);
std::vector<float> coefficient_steps(const Plan& p);
std::vector<int32_t> component_coefficients(const Plan& p, const Planes& px,
                                            int comp, int threads);

// --- Tier-1 ------------------------------------------------------------------
enum PassKind : int { kSP = 0, kMR = 1, kCL = 2 };

struct Pass {
  int kind;
  int bitplane;
  uint32_t ns;           // newly significant
  uint32_t sig_before;   // significant_before as recorded by the reference
  uint32_t length;
  uint32_t cumulative;
  bool terminated;
};

struct EncBlock {
  int res;
  Band band;
  int x0, y0, x1, y1;
  int mbp;          // magnitude bit-planes
  int zbp;          // zero bit-planes
  int cls;          // BlockClass: 0 Flat, 1 Gradient, 2 TexturePhoto
  uint32_t max_mag;
  std::vector<Pass> passes;
  std::vector<uint8_t> payload;  // bytes carried by the last retained pass
};

struct EncBand {
  int res;
  Band band;
  std::vector<EncBlock> blocks;
};

using Layout = std::vector<EncBand>;

// Encode one code-block with the single-termination policy.
EncBlock encode_block(const int32_t* coefs, int w, int h, Band band, int mb);

// Tables built from the standard's rules (Annex C/D).
const uint8_t* zc_lut();   // [4][512]
const uint8_t* sc_lut();   // [256]
const uint8_t* spb_lut();  // [256]
struct MqState { uint16_t qe; uint8_t mps, nmps, nlps; };
const MqState* mq_states();  // [94]

// MQ helpers for tests: symbols are (ctx << 1) | bit.
std::vector<uint8_t> mq_encode(const uint8_t* syms, size_t n);
std::vector<uint8_t> mq_encode_alt(const uint8_t* syms, size_t n);
std::vector<uint8_t> mq_erterm(const uint8_t* syms, size_t n);
void mq_decode(const uint8_t* bytes, size_t nbytes, const uint8_t* ctxs,
               size_t n, uint8_t* bits_out);

// --- full pipeline -------------------------------------------------------
struct EncodeOptions {
  int threads = 1;
  bool contrast_mask = false;  // compute the (output-neutral) contrast mask
};

std::vector<uint8_t> encode(const Plan& p, const Planes& px,
                            const EncodeOptions& opt);
std::vector<Layout> tier1_layouts(const Plan& p, const Planes& px,
                                  const EncodeOptions& opt, bool apply_pcrd);

// Tier-2 / codestream / JP2 (host side in the reference).
std::vector<uint8_t> build_payload(const std::vector<Layout>& layouts);
// One tile-part of a codestream as the writer frames it.
struct TilePartBytes {
  uint16_t tile_index = 0;
  uint8_t part_index = 0, total_parts = 0;
  std::vector<std::vector<uint8_t>> header_segments;
  std::vector<uint8_t> payload;
};
std::vector<uint8_t> frame_codestream(const Plan& p, const std::vector<std::vector<uint8_t>>& main_segments,
                                      const std::vector<TilePartBytes>& parts);
bool parse_single_tile(const uint8_t* b, size_t n, std::vector<std::vector<uint8_t>>* main_segments,
                       TilePartBytes* tp);
std::vector<uint8_t> build_codestream(const Plan& p,
                                      const std::vector<uint8_t>& payload);
std::vector<uint8_t> wrap_jp2(const Plan& p, const std::vector<uint8_t>& cs);
// Layouts of a page whose code-blocks, taken in codestream order (resolution,
// component, band, raster), retain npasses[i] passes in one terminated
// segment of seg_len[i] bytes from `body`, above zbp[i] zero bit-planes:
// the geometry of tier1_layouts without running Tier-1.
std::vector<Layout> layouts_from_blocks(const Plan& p, const uint16_t* npasses, const uint8_t* zbp,
                                        const uint32_t* seg_len, const uint8_t* body, uint32_t nblocks);

// --- decoder (parity checker for round trips) --------------------------------
struct Decoded {
  uint32_t width, height;
  int ncomp;
  Planes comps;
};
Decoded decode(const uint8_t* bytes, size_t n, bool rct_chroma_extra_bitplane = false,
               bool accept_empty_segments = false);

// Quality metrics as encode_with_psnr defines them.
void quality_metrics(const Plan& p, const Planes& px, const EncodeOptions& opt,
                     double* psnr, double* ssim);

// Contrast mask (output-neutral work the reference does on every lossy encode).
double contrast_mask_work(const Plan& p, const Planes& px);

// Synthetic inputs are generated by the product's generator; the oracle only
// consumes planes.
Planes planes_from_bytes(const uint8_t* px, uint32_t w, uint32_t h, int ncomp);

}  // namespace orc
