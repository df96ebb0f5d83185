// C ABI and the per-page device pipeline.
//
// jp2g_encode follows jp2lam::encode (src/encode/mod.rs:84-101): plan on the
// host, then on the device colour+DWT+quantisation (one launch per level),
// Tier-1 (one warp per code-block over the flat work list), PCRD (hull +
// lambda selection) and compaction of the retained bytes; the per-block
// retained table and the packed bytes come back to the host, which writes
// the packet headers, markers and JP2 boxes.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/jp2g.h"
#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {
bool init_t1_tables();
void build_t1_tables(uint8_t* zc, uint8_t* sc, uint8_t* spb, uint32_t* mq);
bool assemble_codestream(const PagePlan& p, const BlockKeep* keep, const uint8_t* body,
                         const uint32_t* offsets, std::vector<uint8_t>* out, Failure* err);
double norm97(int level, int orient);
}  // namespace jp2g

using namespace jp2g;

namespace {

thread_local std::string g_create_error;

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

struct HostBuf {
  void* p = nullptr;
  size_t cap = 0;
};

enum Stage { kH2D = 0, kDWT, kT1, kPCRD, kCompact, kD2H, kHost, kTotal, kNumStages };
enum SubEvent { kEvAnalyzeEnd = kNumStages + 1, kEvModelEnd, kNumEvents };

}  // namespace

struct jp2g_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0;
  uint64_t allocated = 0;
  std::string err;
  std::mutex mu;
  // device pools
  DevBuf px, ll0, ll1, coef, payload, passes, res, keep, blocks, bands, comps, maxslope, hullp,
      hulls, hulln, offsets, scratch, body, nplanes, planebase, items, itemrec, sym;
  // pinned host staging
  HostBuf hpx, hkeep, hoffsets, hbody, hres, hcount;
  bool timing = false;
  cudaEvent_t ev[kNumEvents] = {};
  float stage_ms[kNumStages + 3] = {};
  uint64_t counters[8] = {};
};

namespace {

int set_err(jp2g_ctx* c, int code, const std::string& m) {
  c->err = m;
  return code;
}

bool cuda_ok(jp2g_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  c->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

bool reserve(jp2g_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes <= b.cap) return true;
  size_t want = std::max(bytes, b.cap + b.cap / 2);
  want = (want + 255) & ~size_t(255);
  if (c->budget && c->allocated - b.cap + want > c->budget) {
    c->err = "device memory budget exhausted (" + std::to_string(c->budget) + " bytes)";
    return false;
  }
  if (b.p) cudaFree(b.p);
  c->allocated -= b.cap;
  b.p = nullptr;
  b.cap = 0;
  if (!cuda_ok(c, cudaMalloc(&b.p, want), "cudaMalloc")) return false;
  b.cap = want;
  c->allocated += want;
  return true;
}

bool reserve_host(jp2g_ctx* c, HostBuf& b, size_t bytes) {
  if (bytes <= b.cap) return true;
  size_t want = std::max(bytes, b.cap + b.cap / 2);
  if (b.p) cudaFreeHost(b.p);
  b.p = nullptr;
  b.cap = 0;
  if (!cuda_ok(c, cudaMallocHost(&b.p, want), "cudaMallocHost")) return false;
  b.cap = want;
  return true;
}

template <class T>
T* dptr(DevBuf& b) {
  return reinterpret_cast<T*>(b.p);
}

void record(jp2g_ctx* c, int i) {
  if (c->timing) cudaEventRecord(c->ev[i], c->stream);
}

// Per-block payload capacity and pass-record capacity for a plan.
uint32_t slot_cap(const PagePlan& p) { return (uint32_t)(p.cbw * p.cbh * 4 + 1024); }
uint32_t pass_cap(const PagePlan& p) {
  int maxbp = std::min(std::max(p.max_mb + 4, 20), 42);  // <= 124 passes
  return (uint32_t)(1 + 3 * (maxbp - 1));
}

// Host-side work list, band and component tables for one page.
void build_tables(const PagePlan& p, std::vector<BlockDesc>* blocks, std::vector<BandParam>* bands,
                  std::vector<CompParam>* comps) {
  const uint32_t cap = slot_cap(p), pcap = pass_cap(p);
  blocks->resize(p.nblocks);
  for (const BandGeom& g : p.bands) {
    for (int by = 0; by < g.ncby; ++by)
      for (int bx = 0; bx < g.ncbx; ++bx) {
        uint32_t idx = g.first_block + (uint32_t)(by * g.ncbx + bx);
        BlockDesc& d = (*blocks)[idx];
        int x0 = g.x0 + bx * p.cbw, y0 = g.y0 + by * p.cbh;
        d.coef_slot = idx;
        d.w = (uint16_t)(std::min(x0 + p.cbw, g.x1) - x0);
        d.h = (uint16_t)(std::min(y0 + p.cbh, g.y1) - y0);
        d.orient = (uint8_t)g.orient;
        d.mb = (uint8_t)std::min(g.mb, 255);
        d.band_param = (uint16_t)g.quant;
        d.comp_key = (uint32_t)g.comp;
        d.out_off = idx * cap;
        d.out_cap = cap;
        d.pass_off = idx * pcap;
      }
  }
  // PCRD band constants (rate.rs:43-85, pcrd.rs:728-748), one per quant entry.
  const int nres = p.levels + 1;
  bands->clear();
  for (const BandQuant& q : p.quants) {
    BandParam bp{};
    int level = q.orient == LL ? std::max(nres - 1, 0) : std::max(std::max(nres - 1, 0) - q.res, 0);
    double n = norm97(level, q.orient);
    bp.subband_weight = n * n;
    bp.quant_step = q.step_f64;
    if (p.quality < 50) {
      double t = (double)p.quality / 50.0;
      bp.band_bias = q.orient == LL ? 3.0 - 1.8 * t : (q.orient == HH ? 0.20 + 0.62 * t : 1.0);
    } else {
      bp.band_bias = q.orient == LL ? 1.20 : (q.orient == HH ? 0.82 : 1.00);
    }
    bp.is_ll = q.orient == LL;
    bands->push_back(bp);
  }
  comps->clear();
  for (int c = 0; c < p.ncomp; ++c) {
    CompParam cp{};
    cp.lambda_raw = p.lambda_raw;
    cp.lambda_floor = p.lambda_floor;
    cp.comp_weight = p.comp_weight[c];
    cp.lossless = p.quality >= 100;
    cp.quality = p.quality;
    comps->push_back(cp);
  }
}

// Runs colour+DWT+quantisation for the page whose interleaved pixels are at
// `d_px` on the device, filling code-block storage.
int run_dwt(jp2g_ctx* c, const PagePlan& p, const uint8_t* d_px) {
  const int L = p.levels;
  size_t llw = (p.width + 1) / 2, llh = (p.height + 1) / 2;
  size_t ll_elems = llw * llh * p.ncomp;
  if (L >= 2) {
    if (!reserve(c, c->ll0, ll_elems * 4) || !reserve(c, c->ll1, ll_elems * 4)) return kEncodeFailed;
  }
  auto band_out = [&](DwtLevelArgs& a, int res) {
    for (const BandGeom& g : p.bands) {
      if (g.res != res) continue;
      DwtBandOut& o = a.band[g.comp][g.orient];
      o.first_block = g.first_block;
      o.ncbx = std::max(g.ncbx, 1);
      o.step = p.quants[g.quant].step_f32;
    }
  };
  const void* src = nullptr;
  size_t src_pitch = 0, src_comp = 0;
  int launches = 0;
  if (L == 0) {
    DwtLevelArgs a{};
    a.from_pixels = 1;
    a.px = d_px;
    a.px_pitch = (size_t)p.width * p.ncomp;
    a.mct = p.use_mct;
    a.ncomp = p.ncomp;
    a.rw = p.width;
    a.rh = p.height;
    a.no_transform = 1;
    a.ll = nullptr;
    a.coef = dptr<int32_t>(c->coef);
    a.cbw = p.cbw;
    a.cbh = p.cbh;
    band_out(a, 0);
    launch_dwt_level(a, p.lossless, c->stream);
    ++launches;
  }
  for (int l = 1; l <= L; ++l) {
    DwtLevelArgs a{};
    const int res = L - l + 1;  // resolution whose detail bands this level makes
    a.rw = p.ladder[res].first;
    a.rh = p.ladder[res].second;
    a.ncomp = p.ncomp;
    a.mct = p.use_mct;
    if (l == 1) {
      a.from_pixels = 1;
      a.px = d_px;
      a.px_pitch = (size_t)p.width * p.ncomp;
    } else {
      a.from_pixels = 0;
      a.src = src;
      a.src_pitch = src_pitch;
      a.src_comp = src_comp;
    }
    a.coef = dptr<int32_t>(c->coef);
    a.cbw = p.cbw;
    a.cbh = p.cbh;
    band_out(a, res);
    if (l == L) {
      a.ll = nullptr;
      band_out(a, 0);
    } else {
      DevBuf& dst = (l % 2) ? c->ll0 : c->ll1;
      a.ll = dst.p;
      a.ll_pitch = (size_t)p.ladder[res - 1].first;
      a.ll_comp = a.ll_pitch * (size_t)p.ladder[res - 1].second;
      src = a.ll;
      src_pitch = a.ll_pitch;
      src_comp = a.ll_comp;
    }
    launch_dwt_level(a, p.lossless, c->stream);
    ++launches;
  }
  c->counters[5] += (uint64_t)launches;
  return kOk;
}

int encode_impl(jp2g_ctx* c, const uint8_t* host_px, const uint8_t* dev_px, uint32_t w,
                uint32_t h, uint32_t ncomp, int interleaved, int quality, int format,
                std::vector<uint8_t>* out, PagePlan* plan_out, std::vector<BlockKeep>* keep_out,
                std::vector<BlockOut>* res_out, bool stop_after_dwt) {
  PagePlan p;
  Failure f{};
  if (!build_plan(w, h, (int)ncomp, quality, format, &p, &f)) return set_err(c, f.code, f.msg);
  if (host_px == nullptr && dev_px == nullptr) return set_err(c, kInvalidInput, "pixel pointer is null");
  if (ncomp == 3 && host_px && !interleaved) {
    // planar input: interleave on the host (Image::from_rgb_bytes takes RGBRGB)
  }
  std::memset(c->counters, 0, sizeof c->counters);
  const size_t npx = (size_t)w * h * ncomp;
  std::vector<BlockDesc> blocks;
  std::vector<BandParam> bands;
  std::vector<CompParam> comps;
  build_tables(p, &blocks, &bands, &comps);
  const uint32_t nb = p.nblocks;
  const size_t slot = (size_t)p.cbw * p.cbh;
  const uint32_t pcap = pass_cap(p);
  if (!reserve(c, c->coef, std::max<size_t>(nb, 1) * slot * 4) ||
      !reserve(c, c->payload, std::max<size_t>(nb, 1) * slot_cap(p)) ||
      !reserve(c, c->passes, std::max<size_t>(nb, 1) * pcap * sizeof(PassRec)) ||
      !reserve(c, c->res, std::max<size_t>(nb, 1) * sizeof(BlockOut)) ||
      !reserve(c, c->keep, std::max<size_t>(nb, 1) * sizeof(BlockKeep)) ||
      !reserve(c, c->blocks, std::max<size_t>(nb, 1) * sizeof(BlockDesc)) ||
      !reserve(c, c->bands, bands.size() * sizeof(BandParam)) ||
      !reserve(c, c->comps, comps.size() * sizeof(CompParam)) ||
      !reserve(c, c->maxslope, 8 * sizeof(unsigned long long)) ||
      !reserve(c, c->hullp, std::max<size_t>(nb, 1) * pcap * sizeof(uint16_t)) ||
      !reserve(c, c->hulls, std::max<size_t>(nb, 1) * pcap * sizeof(double)) ||
      !reserve(c, c->hulln, std::max<size_t>(nb, 1)) ||
      !reserve(c, c->offsets, (size_t)(nb + 1) * 4) ||
      !reserve(c, c->scratch, ((size_t)nb / 1024 + 2) * 4) ||
      !reserve(c, c->nplanes, std::max<size_t>(nb, 1) * 4) ||
      !reserve(c, c->planebase, (size_t)(nb + 1) * 4) ||
      !reserve(c, c->body, std::max<size_t>(nb, 1) * slot_cap(p)))
    return kEncodeFailed;

  auto t_host0 = std::chrono::steady_clock::now();
  record(c, 0);
  // ---- inputs ----
  const uint8_t* d_px = dev_px;
  if (host_px) {
    if (!reserve(c, c->px, npx) || !reserve_host(c, c->hpx, npx)) return kEncodeFailed;
    uint8_t* staging = reinterpret_cast<uint8_t*>(c->hpx.p);
    if (ncomp == 3 && !interleaved) {
      const size_t n = (size_t)w * h;
      for (size_t i = 0; i < n; ++i) {
        staging[3 * i + 0] = host_px[i];
        staging[3 * i + 1] = host_px[n + i];
        staging[3 * i + 2] = host_px[2 * n + i];
      }
    } else {
      std::memcpy(staging, host_px, npx);
    }
    if (!cuda_ok(c, cudaMemcpyAsync(c->px.p, staging, npx, cudaMemcpyHostToDevice, c->stream), "H2D"))
      return kEncodeFailed;
    d_px = reinterpret_cast<const uint8_t*>(c->px.p);
  }
  if (!cuda_ok(c, cudaMemcpyAsync(c->blocks.p, blocks.data(), nb * sizeof(BlockDesc),
                                  cudaMemcpyHostToDevice, c->stream), "H2D blocks") ||
      !cuda_ok(c, cudaMemcpyAsync(c->bands.p, bands.data(), bands.size() * sizeof(BandParam),
                                  cudaMemcpyHostToDevice, c->stream), "H2D bands") ||
      !cuda_ok(c, cudaMemcpyAsync(c->comps.p, comps.data(), comps.size() * sizeof(CompParam),
                                  cudaMemcpyHostToDevice, c->stream), "H2D comps"))
    return kEncodeFailed;
  record(c, 1);
  // ---- colour + DWT + quantisation ----
  if (int rc = run_dwt(c, p, d_px)) return rc;
  record(c, 2);
  if (stop_after_dwt) {
    if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "DWT")) return kEncodeFailed;
    *plan_out = p;
    return kOk;
  }
  // ---- Tier-1 ----
  T1Args ta{};
  ta.blocks = dptr<BlockDesc>(c->blocks);
  ta.nblocks = nb;
  ta.coef = dptr<int32_t>(c->coef);
  ta.cbw = p.cbw;
  ta.cbh = p.cbh;
  ta.out = dptr<uint8_t>(c->payload);
  ta.passes = dptr<PassRec>(c->passes);
  ta.pass_cap = pcap;
  ta.res = dptr<BlockOut>(c->res);
  ta.nplanes = dptr<uint32_t>(c->nplanes);
  ta.plane_base = dptr<uint32_t>(c->planebase);
  ta.sym_slot = (uint32_t)(((size_t)p.cbw * p.cbh * 5 / 2 + 15) & ~size_t(15));
  launch_t1_analyze(ta, c->stream);
  launch_scan_u32(ta.nplanes, 1, nb, ta.plane_base, dptr<uint32_t>(c->scratch), c->stream);
  // the number of (block, bit-plane) items sizes the symbol buffer
  if (!reserve_host(c, c->hcount, 16) ||
      !cuda_ok(c, cudaMemcpyAsync(c->hcount.p, ta.plane_base + nb, 4, cudaMemcpyDeviceToHost, c->stream),
               "D2H item count") ||
      !cuda_ok(c, cudaStreamSynchronize(c->stream), "tier-1 analysis"))
    return kEncodeFailed;
  ta.nitems = *reinterpret_cast<uint32_t*>(c->hcount.p);
  if (!reserve(c, c->items, std::max<size_t>(ta.nitems, 1) * 4) ||
      !reserve(c, c->itemrec, std::max<size_t>(ta.nitems, 1) * sizeof(ItemRec)) ||
      !reserve(c, c->sym, std::max<size_t>(ta.nitems, 1) * ta.sym_slot + 64))  // the MQ reader runs 48 B ahead
    return kEncodeFailed;
  ta.items = dptr<uint32_t>(c->items);
  ta.item_rec = dptr<ItemRec>(c->itemrec);
  ta.sym = dptr<uint8_t>(c->sym);
  launch_t1_items(ta, c->stream);
  record(c, kEvAnalyzeEnd);
  launch_t1_model(ta, c->num_sms, c->stream);
  record(c, kEvModelEnd);
  launch_t1_mq(ta, c->num_sms, c->stream);
  c->counters[5] += 5 + (nb > 1024 ? 1 : 0);
  record(c, 3);
  // ---- PCRD ----
  PcrdArgs pa{};
  pa.blocks = ta.blocks;
  pa.nblocks = nb;
  pa.res = ta.res;
  pa.passes = ta.passes;
  pa.bands = dptr<BandParam>(c->bands);
  pa.comps = dptr<CompParam>(c->comps);
  pa.comp_max_slope = dptr<unsigned long long>(c->maxslope);
  pa.ncomp_keys = (uint32_t)comps.size();
  pa.hull_passes = dptr<uint16_t>(c->hullp);
  pa.hull_slope = dptr<double>(c->hulls);
  pa.hull_n = dptr<uint8_t>(c->hulln);
  pa.keep = dptr<BlockKeep>(c->keep);
  launch_pcrd(pa, c->stream);
  record(c, 4);
  // ---- compaction ----
  launch_compact(ta.blocks, pa.keep, nb, ta.out, dptr<uint8_t>(c->body), dptr<uint32_t>(c->offsets),
                 dptr<uint32_t>(c->scratch), c->stream);
  c->counters[5] += 3 + (nb > 1024 ? 1 : 0);  // 2 PCRD, scan + copy kernels
  record(c, 5);
  // ---- read back ----
  if (!reserve_host(c, c->hkeep, std::max<size_t>(nb, 1) * sizeof(BlockKeep)) ||
      !reserve_host(c, c->hres, std::max<size_t>(nb, 1) * sizeof(BlockOut)) ||
      !reserve_host(c, c->hoffsets, (size_t)(nb + 1) * 4))
    return kEncodeFailed;
  if (!cuda_ok(c, cudaMemcpyAsync(c->hkeep.p, c->keep.p, nb * sizeof(BlockKeep),
                                  cudaMemcpyDeviceToHost, c->stream), "D2H keep") ||
      !cuda_ok(c, cudaMemcpyAsync(c->hoffsets.p, c->offsets.p, (size_t)(nb + 1) * 4,
                                  cudaMemcpyDeviceToHost, c->stream), "D2H offsets") ||
      !cuda_ok(c, cudaMemcpyAsync(c->hres.p, c->res.p, nb * sizeof(BlockOut),
                                  cudaMemcpyDeviceToHost, c->stream), "D2H results") ||
      !cuda_ok(c, cudaStreamSynchronize(c->stream), "encode kernels"))
    return kEncodeFailed;
  const BlockKeep* hk = reinterpret_cast<const BlockKeep*>(c->hkeep.p);
  const uint32_t* hoff = reinterpret_cast<const uint32_t*>(c->hoffsets.p);
  for (uint32_t i = 0; i < nb; ++i) {
    if (hk[i].status == 1)
      return set_err(c, kEncodeFailed, "code-block payload exceeded its device slot");
    if (hk[i].status >= 2)
      return set_err(c, kEncodeFailed, "code-block bit-plane count exceeds the supported maximum");
  }
  const uint32_t total = hoff[nb];
  if (!reserve_host(c, c->hbody, std::max<size_t>(total, 1))) return kEncodeFailed;
  if (total > 0 &&
      !cuda_ok(c, cudaMemcpyAsync(c->hbody.p, c->body.p, total, cudaMemcpyDeviceToHost, c->stream),
               "D2H body"))
    return kEncodeFailed;
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "D2H")) return kEncodeFailed;
  record(c, 6);
  // ---- host Tier-2 + codestream ----
  if (!assemble_codestream(p, hk, reinterpret_cast<const uint8_t*>(c->hbody.p), hoff, out, &f))
    return set_err(c, f.code, f.msg);
  record(c, 7);
  record(c, 8);
  if (c->timing) {
    cudaEventSynchronize(c->ev[8]);
    for (int s = 0; s < kTotal; ++s) cudaEventElapsedTime(&c->stage_ms[s], c->ev[s], c->ev[s + 1]);
    cudaEventElapsedTime(&c->stage_ms[kTotal], c->ev[0], c->ev[8]);
    // tier-1 split: analysis (+item list), modelling, MQ coding
    cudaEventElapsedTime(&c->stage_ms[kNumStages + 0], c->ev[2], c->ev[kEvAnalyzeEnd]);
    cudaEventElapsedTime(&c->stage_ms[kNumStages + 1], c->ev[kEvAnalyzeEnd], c->ev[kEvModelEnd]);
    cudaEventElapsedTime(&c->stage_ms[kNumStages + 2], c->ev[kEvModelEnd], c->ev[3]);
    (void)t_host0;
  }
  const BlockOut* hr = reinterpret_cast<const BlockOut*>(c->hres.p);
  c->counters[0] = nb;
  for (uint32_t i = 0; i < nb; ++i) {
    c->counters[1] += hr[i].mbp > 0;
    c->counters[2] += hr[i].npasses;
    c->counters[3] += hr[i].payload_len;
    c->counters[6] += (uint64_t)hr[i].mbp * blocks[i].w * blocks[i].h;
  }
  c->counters[4] = total;
  if (keep_out) keep_out->assign(hk, hk + nb);
  if (res_out) res_out->assign(hr, hr + nb);
  if (plan_out) *plan_out = p;
  return kOk;
}

}  // namespace

namespace jp2g {
// Records a message for jp2g_last_error(NULL) on the calling thread.
void set_thread_error(const char* msg) { g_create_error = msg ? msg : ""; }
}  // namespace jp2g

extern "C" {

int jp2g_create(jp2g_ctx** out, int device, uint64_t hbm_budget_bytes) {
  if (!out) {
    g_create_error = "ctx pointer is null";
    return JP2G_INVALID_INPUT;
  }
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    g_create_error = std::string("no CUDA device available: ") + cudaGetErrorString(e);
    return JP2G_ENCODE_FAILED;
  }
  if (device < 0 || device >= count) {
    g_create_error = "device index out of range";
    return JP2G_INVALID_INPUT;
  }
  jp2g_ctx* c = new jp2g_ctx();
  c->device = device;
  c->budget = hbm_budget_bytes;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess || !init_t1_tables()) {
    g_create_error = "CUDA initialisation failed";
    delete c;
    return JP2G_ENCODE_FAILED;
  }
  for (auto& ev : c->ev) cudaEventCreate(&ev);
  *out = c;
  return JP2G_OK;
}

void jp2g_destroy(jp2g_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  DevBuf* bufs[] = {&c->px, &c->ll0, &c->ll1, &c->coef, &c->payload, &c->passes, &c->res, &c->keep,
                    &c->blocks, &c->bands, &c->comps, &c->maxslope, &c->hullp, &c->hulls, &c->hulln,
                    &c->offsets, &c->scratch, &c->body, &c->nplanes, &c->planebase, &c->items,
                    &c->itemrec, &c->sym};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  HostBuf* hb[] = {&c->hpx, &c->hkeep, &c->hoffsets, &c->hbody, &c->hres, &c->hcount};
  for (HostBuf* b : hb)
    if (b->p) cudaFreeHost(b->p);
  for (auto& ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  cudaStreamDestroy(c->stream);
  delete c;
}

static int finish_output(jp2g_ctx* c, int rc, std::vector<uint8_t>& bytes, uint8_t** out,
                         size_t* out_len) {
  if (rc != JP2G_OK) return rc;
  uint8_t* p = static_cast<uint8_t*>(std::malloc(std::max<size_t>(bytes.size(), 1)));
  if (!p) return set_err(c, JP2G_ENCODE_FAILED, "out of host memory");
  std::memcpy(p, bytes.data(), bytes.size());
  *out = p;
  *out_len = bytes.size();
  return JP2G_OK;
}

int jp2g_encode(jp2g_ctx* c, const uint8_t* px, uint32_t w, uint32_t h, uint32_t ncomp,
                int interleaved, uint8_t quality, int format, uint8_t** out, size_t* out_len) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!out || !out_len) return set_err(c, JP2G_INVALID_INPUT, "output pointer is null");
  if (!px) return set_err(c, JP2G_INVALID_INPUT, "pixel pointer is null");
  cudaSetDevice(c->device);
  std::vector<uint8_t> bytes;
  int rc = encode_impl(c, px, nullptr, w, h, ncomp, interleaved, quality, format, &bytes, nullptr,
                       nullptr, nullptr, false);
  return finish_output(c, rc, bytes, out, out_len);
}

int jp2g_encode_device(jp2g_ctx* c, const uint8_t* d_px, uint32_t w, uint32_t h, uint32_t ncomp,
                       uint8_t quality, int format, uint8_t** out, size_t* out_len) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!out || !out_len) return set_err(c, JP2G_INVALID_INPUT, "output pointer is null");
  if (!d_px) return set_err(c, JP2G_INVALID_INPUT, "pixel pointer is null");
  cudaSetDevice(c->device);
  std::vector<uint8_t> bytes;
  int rc = encode_impl(c, nullptr, d_px, w, h, ncomp, 1, quality, format, &bytes, nullptr, nullptr,
                       nullptr, false);
  return finish_output(c, rc, bytes, out, out_len);
}

void jp2g_free(uint8_t* p) { std::free(p); }

const char* jp2g_last_error(jp2g_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

void* jp2g_stream(jp2g_ctx* c) { return c ? (void*)c->stream : nullptr; }

int jp2g_set_timing(jp2g_ctx* c, int enabled) {
  if (!c) return JP2G_INVALID_INPUT;
  c->timing = enabled != 0;
  return JP2G_OK;
}

int jp2g_stage_times(jp2g_ctx* c, float* ms, int n) {
  if (!c || !ms) return 0;
  int k = std::min(n, (int)kNumStages + 3);
  for (int i = 0; i < k; ++i) ms[i] = c->stage_ms[i];
  return k;
}

int jp2g_counters(jp2g_ctx* c, uint64_t* out, int n) {
  if (!c || !out) return 0;
  int k = std::min(n, 8);
  for (int i = 0; i < k; ++i) out[i] = c->counters[i];
  return k;
}

int jp2g_debug_coefficients(jp2g_ctx* c, const uint8_t* px, uint32_t w, uint32_t h,
                            uint32_t ncomp, uint8_t quality, uint32_t comp, int32_t* plane) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!px || !plane) return set_err(c, JP2G_INVALID_INPUT, "null pointer");
  if (comp >= ncomp) return set_err(c, JP2G_INVALID_INPUT, "component index out of range");
  cudaSetDevice(c->device);
  PagePlan p;
  int rc = encode_impl(c, px, nullptr, w, h, ncomp, 1, quality, 0, nullptr, &p, nullptr, nullptr, true);
  if (rc) return rc;
  const size_t slot = (size_t)p.cbw * p.cbh;
  std::vector<int32_t> coef((size_t)p.nblocks * slot);
  if (!cuda_ok(c, cudaMemcpy(coef.data(), c->coef.p, coef.size() * 4, cudaMemcpyDeviceToHost), "D2H"))
    return JP2G_ENCODE_FAILED;
  for (const BandGeom& g : p.bands) {
    if ((uint32_t)g.comp != comp) continue;
    for (int y = g.y0; y < g.y1; ++y)
      for (int x = g.x0; x < g.x1; ++x) {
        int u = x - g.x0, v = y - g.y0;
        size_t blk = g.first_block + (size_t)(v / p.cbh) * g.ncbx + (size_t)(u / p.cbw);
        plane[(size_t)y * w + x] = coef[blk * slot + (size_t)(v % p.cbh) * p.cbw + (u % p.cbw)];
      }
  }
  return JP2G_OK;
}

int jp2g_debug_blocks(jp2g_ctx* c, const uint8_t* px, uint32_t w, uint32_t h, uint32_t ncomp,
                      uint8_t quality, int32_t* rows, uint32_t cap, uint32_t* nblocks) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!px || !nblocks) return set_err(c, JP2G_INVALID_INPUT, "null pointer");
  cudaSetDevice(c->device);
  PagePlan p;
  std::vector<BlockKeep> keep;
  std::vector<BlockOut> res;
  std::vector<uint8_t> bytes;
  int rc = encode_impl(c, px, nullptr, w, h, ncomp, 1, quality, 0, &bytes, &p, &keep, &res, false);
  if (rc) return rc;
  *nblocks = p.nblocks;
  for (uint32_t i = 0; i < p.nblocks && i < cap && rows; ++i) {
    int32_t* r = rows + 8 * i;
    r[0] = res[i].mbp;
    r[1] = res[i].zbp;
    r[2] = res[i].npasses;
    r[3] = (int32_t)res[i].payload_len;
    r[4] = res[i].cls;
    r[5] = res[i].status;
    r[6] = keep[i].npasses;
    r[7] = (int32_t)keep[i].body_len;
  }
  return JP2G_OK;
}

// Host-only: the Tier-1 tables the device uses, for checking against the
// reference's literal tables without a GPU.
void jp2g_tables(uint8_t* zc, uint8_t* sc, uint8_t* spb, uint32_t* mq) {
  build_t1_tables(zc, sc, spb, mq);
}

}  // extern "C"
