// Kernel launch interfaces (device side of the pipeline).
#pragma once

#include <cuda_runtime.h>

#include <utility>
#include <vector>

#include "jp2g_internal.h"

namespace jp2g {

// Where one subband of one component lands in code-block storage.
struct DwtBandOut {
  uint32_t first_block;
  int ncbx;
  float step;  // quantiser step (irreversible path)
};

struct DwtLevelArgs {
  // Input: the page's pixels (first level) or the previous level's LL plane.
  int from_pixels;
  const uint8_t* px;
  size_t px_pitch;  // bytes per pixel row
  int mct;          // apply RCT/ICT (three interleaved components)
  const void* src;  // previous LL plane (int32 or float), component-major
  size_t src_pitch, src_comp;
  int ncomp;
  int rw, rh;        // region size at this level
  int no_transform;  // zero decomposition levels: copy (and quantise) only
  // Output: next LL plane, or nullptr to send LL to code-block storage.
  void* ll;
  size_t ll_pitch, ll_comp;
  int32_t* coef;
  int cbw, cbh;
  DwtBandOut band[3][4];
};

// One level of one page with the shared-memory lifting kernel: used for
// pages with no decomposition level and regions under 2 samples wide or high.
void launch_dwt_level(const DwtLevelArgs& a, bool reversible, cudaStream_t st);

// One level of many pages in one launch: d_args[i] describes page i's level
// (region at least 2x2), d_tile_base[i] its first tile in the flat tile
// list (npages + 1 entries, d_tile_base[npages] = the tile count).
void launch_dwt_batch(const DwtLevelArgs* d_args, const uint32_t* d_tile_base, uint32_t npages,
                      uint32_t ntiles, bool reversible, cudaStream_t st);
// Tiles of one page's level in the flat tile list.
uint32_t dwt_tiles(int rw, int rh, int ncomp);

struct T1Args {
  const BlockDesc* blocks;
  uint32_t nblocks;
  const int32_t* coef;
  int cbw, cbh;
  uint8_t* out;
  PassRec* passes;
  uint32_t pass_cap;  // pass records available per block
  BlockOut* res;
  // (block, bit-plane) modelling items
  uint32_t* nplanes;     // per block: magnitude bit-planes to model
  uint32_t* plane_base;  // per block: first item (exclusive prefix of nplanes)
  uint32_t* items;       // per item: its block
  uint32_t nitems;
  uint32_t* planes;      // per item: column masks of its plane (t1_planes_kernel), 1 KiB
  uint32_t* signs;       // per block: sign column masks, 512 B
  ItemRec* item_rec;
  uint8_t* sym;          // per item: a slot of sym_slot symbol bytes
  uint32_t sym_slot;
  unsigned long long* sym_count;  // total MQ symbols coded (statistics)
  const uint32_t* mq_order;       // MQ processing order of the blocks, or null (work-list order)
};

void launch_t1_analyze(const T1Args& a, cudaStream_t st);
// Items list and per-item bit-plane column masks (after the plane-count scan).
void launch_t1_planes(const T1Args& a, cudaStream_t st);
void launch_t1_model(const T1Args& a, int num_sms, cudaStream_t st);
// bpw: code-blocks per warp, 1..32, or 0 for automatic.
void launch_t1_mq(const T1Args& a, int num_sms, int bpw, cudaStream_t st);
// One block per warp, blocks taken in a.mq_order from an atomic counter
// (*next, zeroed here) by warps_per_sm warps on each SM.
void launch_t1_mq_pull(const T1Args& a, int num_sms, int warps_per_sm, uint32_t* next, cudaStream_t st);
// Producer/consumer warp pairs (interval chain | code register chain)
// coding `chains` blocks at once each (1: all lanes of a warp on one chain;
// 2: one chain per half-warp), pulling the `heavy` first blocks of
// a.mq_order (0 = all) from *next (zeroed here), pipes_per_sm pairs on each
// SM; the remaining blocks are coded 32 to a warp in the same launch.
void launch_t1_mq_pipe(const T1Args& a, int num_sms, int pipes_per_sm, int chains, uint32_t heavy,
                       uint32_t* next, cudaStream_t st);
// Code-blocks per warp that launch_t1_mq uses for `bpw` (0 = automatic).
int mq_blocks_per_warp(const T1Args& a, int num_sms, int bpw);
// Orders the blocks by their MQ symbol count, largest first (counting sort
// on 1024 buckets), into order[nblocks]. scratch: nblocks + 2048 words.
void launch_mq_order(const T1Args& a, uint32_t* order, uint32_t* scratch, cudaStream_t st);

// Exclusive prefix sum of n uint32 values read with a stride of `stride`
// words: out[i] = sum of in[0..i), out[n] = total. `scratch` holds
// ceil(n/1024)+1 words.
void launch_scan_u32(const uint32_t* in, uint32_t stride, uint32_t n, uint32_t* out,
                     uint32_t* scratch, cudaStream_t st);

struct PcrdArgs {
  const BlockDesc* blocks;
  uint32_t nblocks;
  const BlockOut* res;
  const PassRec* passes;
  const BandParam* bands;
  const CompParam* comps;
  unsigned long long* comp_max_slope;  // f64 bit patterns (non-negative)
  uint32_t ncomp_keys;
  uint16_t* hull_passes;  // per pass slot
  double* hull_slope;
  uint8_t* hull_n;        // hull points per block
  BlockKeep* keep;
};

void launch_pcrd(const PcrdArgs& a, cudaStream_t st);

// ------------------------------------------------------ device Tier-2 --
struct T2Node {  // tag-tree node: minimum zero bit-planes, first included leaf (or ~0)
  uint32_t zmin;
  uint32_t first_inc;
};
struct T2Band {
  uint32_t first_block;  // in the wave's work list
  uint32_t tree_off;     // its tag-tree nodes in T2Args::tree
  uint16_t ncbx, ncby;
};
struct T2Packet {  // the bands of one (resolution, component) of a page
  uint32_t band0, nbands;
  uint32_t raw_off;  // its unstuffed header bits (words of T2Args::raw)
  uint32_t hdr_off;  // its header bytes (T2Args::hdr)
  uint32_t b0, b1;   // its code-blocks [b0, b1) in the wave's work list
  uint32_t page;
  uint32_t pad;
};
struct T2Page {
  uint32_t packet0, npackets;
  uint32_t tmpl_off, tmpl_len;  // the marker prefix (JP2 boxes, SOC..SOD) in T2Args::tmpl
  uint32_t psot_pos, jp2c_pos;  // fields filled in once the payload is known (jp2c: ~0 for J2K)
};
struct T2Args {
  const T2Packet* packets;
  uint32_t npackets;
  const T2Band* bands;
  const T2Page* pages;
  uint32_t npages;
  const BlockKeep* keep;
  const uint32_t* offsets;  // retained bytes of each block in `body` (nblocks + 1)
  const uint8_t* body;
  const uint8_t* tmpl;
  T2Node* tree;
  uint32_t* raw;  // zeroed before the launch
  uint8_t* hdr;
  uint32_t* hdr_len;   // per packet
  uint32_t* pkt_off;   // per packet: its offset in its page
  uint32_t* page_len;  // per page
  uint32_t* page_off;  // per page (npages + 1): its offset in `out`
  uint32_t* nchunks;     // per packet: copy jobs
  uint32_t* chunk_base;  // per packet (npackets + 1): first copy job
  uint8_t* out;
};
// Packet headers, page layout (page_off[npages] = total bytes) and the
// finished codestreams in `out`. scan_scratch: ceil(max(npages,
// npackets)/1024)+1 words.
void launch_t2(const T2Args& a, uint32_t* scan_scratch, int num_sms, cudaStream_t st);

// ------------------------------------------------------------- decoding --
// One code-block of a codestream being decoded.
struct DecBlock {
  uint64_t plane_off;           // its first sample in the planes buffer (elements)
  uint32_t data_off, data_len;  // its segment in the input bytes
  uint32_t stride;              // its plane's row pitch (the image width)
  uint16_t w, h;
  uint8_t orient, mb, zbp;  // mb: bit-planes from QCD (decode/t1.rs:56)
  uint8_t reversible;       // 1: signed integers out, 0: dequantised f32 bits
  uint16_t npasses;
  uint16_t pad;
  float step;  // quantiser step (irreversible codestreams)
};

// What the host parse learns from a codestream (decode.cpp). Block
// plane_off and data_off are relative to the page's planes (component c at
// c * width * height) and to the start of its bytes.
struct DecodeLayout {
  uint32_t width = 0, height = 0;
  int ncomp = 0, precision = 0, levels = 0, cbw = 64, cbh = 64, guard = 2;
  bool reversible = true, mct = false;
  std::vector<std::pair<int, int>> ladder;  // resolution sizes, index 0 = the smallest
  std::vector<DecBlock> blocks;
};
// flags: bit 0 one more magnitude bit-plane for RCT chroma, bit 1 accept
// code-blocks whose segment has zero bytes (the JP2G_DECODE_* flags).
bool parse_codestream(const uint8_t* bytes, size_t n, int flags, DecodeLayout* out, Failure* err);

// One component of one page at one inverse-DWT level: its planes hold
// int32 (5/3) or f32 (9/7) samples, rows `stride` apart; the level's
// rw x rh region is transformed rows first (plane -> tmp), then columns
// (tmp -> plane). row_base / tile_base: the job's first global row and
// first 32-column tile in the level's launch.
struct IdwtJob {
  void* plane;
  void* tmp;
  uint32_t stride, rw, rh, reversible;
  uint32_t row_base, tile_base;
};
// One page's final samples: inverse RCT/ICT (when mct and 3 components),
// level shift and clamp into interleaved 8-bit samples.
struct PixJob {
  const int32_t* planes;  // ncomp planes of npx samples (int32 or f32 bits)
  uint8_t* px;
  uint64_t npx, pix_base;  // pix_base: the page's first global sample index
  uint32_t ncomp, mct, reversible, pad;
};
// Tier-1 decoding of every code-block (t1dec.cu) into zeroed planes, one
// or two (per_warp) decoders per warp.
void launch_t1_decode(const DecBlock* blocks, uint32_t nblocks, const uint8_t* data, int32_t* planes, int per_warp,
                      cudaStream_t st);
// One inverse-DWT level for njobs jobs (recon.cu).
void launch_idwt_level(const IdwtJob* jobs, uint32_t njobs, uint32_t total_rows, uint32_t total_tiles,
                       cudaStream_t st);
constexpr int kIdwtTileRows = 64;  // rows per column tile of launch_idwt_level
void launch_dec_pixels(const PixJob* jobs, uint32_t njobs, uint64_t total_px, cudaStream_t st);
bool upload_decode_tables(const uint8_t* zc, const uint8_t* sc, const uint8_t* spb, const uint32_t* mq);

// Where a code-block's samples sit in its component's plane (Mallat
// layout), and its quantiser step.
struct ReconBlock {
  uint32_t x0, y0;
  uint32_t comp;
  float step;
};

// Reconstruction of one encoded page for its quality metrics (recon.cu).
struct ReconArgs {
  const BlockDesc* blocks;
  const ReconBlock* rblocks;
  const BlockKeep* keep;
  const PassRec* passes;
  const int32_t* coef;
  int cbw, cbh;
  uint32_t nblocks;
  uint32_t width, height;
  int ncomp;
  const uint8_t* px;  // the page's interleaved pixels on the device
  float* plane;       // ncomp planes of width * height
  float* tmp;         // ncomp planes of scratch
  IdwtJob* jobs;      // device room for ncomp * levels inverse-DWT jobs
  float* luma_orig;
  float* luma_dec;
  double* stats;      // [0] sum of squared errors, [1] sum of 8x8 block SSIMs
};

// Dequantisation of the retained bit-planes, inverse 9/7 per component
// (ladder[0..levels], index 0 the smallest resolution), colour and the two
// sums of the metrics.
void launch_recon(const ReconArgs& r, const std::pair<int, int>* ladder, int levels, cudaStream_t st);

// Packs the retained payload bytes of every block, in work-list order, into
// `dst`; offsets[b] receives the byte offset of block b and offsets[n] the
// total. `scratch` holds ceil(n/1024)+1 uint32.
void launch_compact(const BlockDesc* blocks, const BlockKeep* keep, uint32_t nblocks,
                    const uint8_t* src, uint8_t* dst, uint32_t* offsets, uint32_t* scratch,
                    cudaStream_t st);

}  // namespace jp2g
