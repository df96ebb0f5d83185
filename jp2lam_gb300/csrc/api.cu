// C ABI and the per-page device pipeline.
//
// jp2g_encode follows jp2lam::encode (src/encode/mod.rs:84-101): plan on the
// host, then on the device colour+DWT+quantisation (one launch per level),
// Tier-1 (bit-plane masks, modelling, MQ over the flat work list), PCRD
// (hull + lambda selection), compaction of the retained bytes and Tier-2
// (packet headers, markers, JP2 boxes and the codestream itself); only the
// finished codestreams come back to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <cmath>
#include <limits>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/jp2g.h"
#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {
bool init_t1_tables();
void build_t1_tables(uint8_t* zc, uint8_t* sc, uint8_t* spb, uint32_t* mq);
bool assemble_codestream(const PagePlan& p, const BlockKeep* keep, const uint8_t* body,
                         const uint32_t* offsets, std::vector<uint8_t>* out, Failure* err);
bool codestream_prefix(const PagePlan& p, uint64_t payload, std::vector<uint8_t>* out, uint32_t* psot_pos,
                       uint32_t* jp2c_pos, Failure* err);
double norm97(int level, int orient);
void context_labels_from_logic(uint8_t* zc, uint8_t* sc, uint8_t* spb);
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
enum SubEvent { kEvAnalyzeEnd = kNumStages + 1, kEvModelEnd, kEvT2End, kNumEvents };

// One page of a wave: its request, its plan and, after the device phase,
// the page-local retained blocks and bytes that Tier-2 needs.
struct PageJob {
  const uint8_t* host_px = nullptr;
  const uint8_t* dev_px = nullptr;
  uint32_t w = 0, h = 0, ncomp = 0;
  int interleaved = 1, quality = 0, format = 0;
  int status = 0;
  std::string err;
  PagePlan plan;            // band first_block relative to the page
  uint32_t block_base = 0;  // the page's first code-block in the wave
  size_t px_off = 0;        // the page's pixels in the wave's staging buffer
  bool staged = false;      // copied to the device from pinned staging
  bool laid_out = false;    // has a place (px_off) in the wave's pixel buffer
  uint8_t* cs = nullptr;  // the finished codestream (J2K or JP2), malloc'd
  size_t cs_len = 0;
  PageJob() = default;
  PageJob(const PageJob&) = delete;
  PageJob& operator=(const PageJob&) = delete;
  ~PageJob() { std::free(cs); }
  void drop_output() {
    std::free(cs);
    cs = nullptr;
    cs_len = 0;
  }
};

// A submitted request and, once done, its result.
struct Ticket {
  uint64_t id = 0;
  PageJob job;
  bool done = false;
  std::atomic<bool> cancelled{false};  // jp2g_cancel was called: the result is dropped
};

}  // namespace

struct jp2g_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0;
  std::atomic<uint64_t> allocated{0};  // device pool bytes (also grown by the serving stager)
  bool budget_hit = false;         // the last pool growth was refused by the budget
  uint64_t budget_wave_blocks = 0;  // most code-blocks per wave that fit the budget (0: no cap learnt)
  std::string err;  // guarded by errmu
  std::mutex errmu;
  std::mutex mu;    // device pools and stream: one wave (or encode) at a time
  // device pools
  DevBuf px, px2, ll0, coef, payload, passes, res, keep, blocks, bands, comps, maxslope, hullp,
      hulls, hulln, offsets, scratch, body, nplanes, planebase, items, itemrec, planes, signs, sym, stats,
      dwtargs, dwtbases, mqorder, mqscratch, recon, reconblk, t2pk, t2bd, t2pg, t2tmpl, t2tree, t2raw, t2hdr,
      t2hdrlen, t2pktoff, t2pagelen, t2pageoff, t2nchunks, t2chunkbase, t2out;
  // pinned host staging
  HostBuf hpx, hpx2, hkeep, hres, hcount, hpageoff, hout;
  bool timing = false;
  cudaEvent_t ev[kNumEvents] = {};
  // batches: a wave's pixels go up on copy_stream (the next wave's while the
  // current one computes), alternating between px and px2; its DWT waits
  // on ev_up
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_up[2] = {};
  uint8_t* wave_px = nullptr;  // the current wave's device pixels
  float stage_ms[kNumStages + 4] = {};
  uint64_t counters[8] = {};
  // default wave: 240,000 code-blocks (the autotuner's choice on sRGB and
  // uneven batches: fewer waves, fewer MQ tails); 160,000 under a budget
  int64_t opt[JP2G_NUM_OPTS] = {240000, 0, 0, 0, 0, 0, 0};
  // submit/poll: a worker thread forms waves from the queue and runs them;
  // a finisher thread marks the finished waves' tickets done. Without a
  // memory budget a stager thread forms the waves instead: it gathers each
  // wave's pixels into pinned memory and uploads them on its own stream
  // while the worker runs the previous wave, through two pinned and two
  // device pixel buffers of its own (the wave in buffer k holds it until the
  // worker is done with it).
  std::mutex qmu;
  std::condition_variable qcv, fcv, dcv, rcv;
  std::deque<std::shared_ptr<Ticket>> pending;
  std::deque<std::vector<std::shared_ptr<Ticket>>> finishing;
  std::unordered_map<uint64_t, std::shared_ptr<Ticket>> tickets;
  uint64_t next_ticket = 1;
  int inflight = 0;  // waves taken off `pending` and not yet handed to the finisher
  bool stop = false;
  std::thread worker, finisher, stager;
  struct StagedWave {
    std::vector<std::shared_ptr<Ticket>> tickets;
    size_t total = 0;       // stage_pixels' layout bytes
    int buf = 0;            // serving pixel buffer pair
    bool uploaded = false;  // the pixels are on their way (serve_ev[buf])
  };
  std::deque<StagedWave> staged;  // formed and gathered, not yet taken by the worker (at most one)
  bool serve_buf_busy[2] = {false, false};
  uint64_t serve_waves = 0;  // waves the stager has formed
  HostBuf serve_hpx[2];
  DevBuf serve_px[2];
  cudaStream_t serve_stream = nullptr;
  cudaEvent_t serve_ev[2] = {};
};

namespace {

void set_msg(jp2g_ctx* c, const std::string& m) {
  std::lock_guard<std::mutex> lk(c->errmu);
  c->err = m;
}

std::string get_msg(jp2g_ctx* c) {
  std::lock_guard<std::mutex> lk(c->errmu);
  return c->err;
}

int set_err(jp2g_ctx* c, int code, const std::string& m) {
  set_msg(c, m);
  return code;
}

bool cuda_ok(jp2g_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  set_msg(c, std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

bool reserve(jp2g_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes <= b.cap) return true;
  size_t want = std::max(bytes, b.cap + b.cap / 2);
  want = (want + 255) & ~size_t(255);
  // under a budget, growth beyond the request is dropped before giving up
  if (c->budget && c->allocated - b.cap + want > c->budget) want = (bytes + 255) & ~size_t(255);
  if (c->budget && c->allocated - b.cap + want > c->budget) {
    c->budget_hit = true;
    set_msg(c, "device memory budget exhausted (" + std::to_string(c->budget) + " bytes)");
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

// Appends one page's code-blocks, PCRD band constants and component keys to
// the wave's tables; the page's blocks start at `block_base`, its band
// constants at `band_base` and its component keys at `key_base`.
void build_tables(const PagePlan& p, uint32_t block_base, uint32_t band_base, uint32_t key_base,
                  uint32_t cap, uint32_t pcap, std::vector<BlockDesc>* blocks,
                  std::vector<BandParam>* bands, std::vector<CompParam>* comps) {
  blocks->resize((size_t)block_base + p.nblocks);
  for (const BandGeom& g : p.bands) {
    for (int by = 0; by < g.ncby; ++by)
      for (int bx = 0; bx < g.ncbx; ++bx) {
        uint32_t idx = block_base + g.first_block + (uint32_t)(by * g.ncbx + bx);
        BlockDesc& d = (*blocks)[idx];
        int x0 = g.x0 + bx * p.cbw, y0 = g.y0 + by * p.cbh;
        d.coef_slot = idx;
        d.w = (uint16_t)(std::min(x0 + p.cbw, g.x1) - x0);
        d.h = (uint16_t)(std::min(y0 + p.cbh, g.y1) - y0);
        d.orient = (uint8_t)g.orient;
        d.mb = (uint8_t)std::min(g.mb, 255);
        d.band_param = (uint16_t)(band_base + (uint32_t)g.quant);
        d.comp_key = key_base + (uint32_t)g.comp;
        d.out_off = idx * cap;
        d.out_cap = cap;
        d.pass_off = idx * pcap;
      }
  }
  // PCRD band constants (rate.rs:43-85, pcrd.rs:728-748), one per quant entry.
  const int nres = p.levels + 1;
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

// Arguments of decomposition level l (1 = first) of a page whose pixels are
// at d_px; llA/llB are the page's two LL planes (level l writes its LL to
// llA when l is odd, to llB when even, and reads the other).
// Samples per row of an intermediate LL plane: a multiple of 16, so the tile
// kernel stores each 16-sample run as aligned 16-byte vectors within the row.
size_t ll_pitch(int width) { return ((size_t)width + 15) & ~size_t(15); }

// Samples of each of a page's two LL planes (the first level's LL is the
// largest), rounded to 64 so both planes stay 256-byte aligned.
size_t ll_plane_elems(const PagePlan& p) {
  return (ll_pitch((p.width + 1) / 2) * (size_t)((p.height + 1) / 2) * p.ncomp + 63) & ~size_t(63);
}

DwtLevelArgs level_args(const PagePlan& p, int l, const uint8_t* d_px, uint32_t block_base,
                        int32_t* coef, void* llA, void* llB) {
  DwtLevelArgs a{};
  const int L = p.levels;
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
    a.src = (l - 1) % 2 ? llA : llB;
    a.src_pitch = ll_pitch(p.ladder[res].first);
    a.src_comp = a.src_pitch * (size_t)p.ladder[res].second;
  }
  a.coef = coef;
  a.cbw = p.cbw;
  a.cbh = p.cbh;
  auto band_out = [&](int r) {
    for (const BandGeom& g : p.bands) {
      if (g.res != r) continue;
      DwtBandOut& o = a.band[g.comp][g.orient];
      o.first_block = block_base + g.first_block;
      o.ncbx = std::max(g.ncbx, 1);
      o.step = p.quants[g.quant].step_f32;
    }
  };
  band_out(res);
  if (l == L) {
    a.ll = nullptr;
    band_out(0);
  } else {
    a.ll = l % 2 ? llA : llB;
    a.ll_pitch = ll_pitch(p.ladder[res - 1].first);
    a.ll_comp = a.ll_pitch * (size_t)p.ladder[res - 1].second;
  }
  return a;
}

// Colour + DWT + quantisation of every page of a wave. Each level is one
// launch over the tiles of all pages that have it (one per transform kind);
// a page whose region at some level is under 2 samples wide or high, or that
// has no decomposition level, takes the per-page kernel there.
int run_dwt_wave(jp2g_ctx* c, const std::vector<PageJob*>& live, bool raw) {
  const size_t n = live.size();
  std::vector<size_t> ll_off(n, 0);
  size_t ll_total = 0;
  int maxL = 0;
  for (size_t i = 0; i < n; ++i) {
    const PagePlan& p = live[i]->plan;
    maxL = std::max(maxL, p.levels);
    if (p.levels >= 2) {
      ll_off[i] = ll_total;
      ll_total += 2 * ll_plane_elems(p);
    }
  }
  if (ll_total > 0 && !reserve(c, c->ll0, ll_total * 4)) return kEncodeFailed;
  int32_t* coef = dptr<int32_t>(c->coef);
  auto page_px = [&](size_t i) {
    return live[i]->dev_px ? live[i]->dev_px : c->wave_px + live[i]->px_off;
  };
  int launches = 0;
  // pages with no decomposition level: copy (and quantise) into blocks
  for (size_t i = 0; i < n; ++i) {
    const PagePlan& p = live[i]->plan;
    if (p.levels != 0) continue;
    DwtLevelArgs a{};
    a.from_pixels = 1;
    a.px = page_px(i);
    a.px_pitch = (size_t)p.width * p.ncomp;
    a.mct = p.use_mct;
    a.ncomp = p.ncomp;
    a.rw = p.width;
    a.rh = p.height;
    a.no_transform = 1;
    a.coef = coef;
    a.cbw = p.cbw;
    a.cbh = p.cbh;
    for (const BandGeom& g : p.bands) {
      DwtBandOut& o = a.band[g.comp][g.orient];
      o.first_block = live[i]->block_base + g.first_block;
      o.ncbx = std::max(g.ncbx, 1);
      o.step = raw ? 0.0f : p.quants[g.quant].step_f32;
    }
    launch_dwt_level(a, p.lossless, c->stream);
    ++launches;
  }
  struct Group {
    size_t arg0, base0;
    uint32_t npages, ntiles;
    bool rev;
  };
  std::vector<DwtLevelArgs> args;
  std::vector<uint32_t> bases;
  std::vector<std::vector<Group>> groups(maxL + 1);
  std::vector<std::vector<std::pair<DwtLevelArgs, bool>>> singles(maxL + 1);
  for (int l = 1; l <= maxL; ++l)
    for (int kind = 0; kind < 2; ++kind) {
      const bool rev = kind == 0;
      Group g{args.size(), bases.size(), 0, 0, rev};
      for (size_t i = 0; i < n; ++i) {
        const PagePlan& p = live[i]->plan;
        if (p.levels < l || p.lossless != rev) continue;
        int32_t* ll = dptr<int32_t>(c->ll0) + ll_off[i];
        const size_t half = p.levels >= 2 ? ll_plane_elems(p) : 0;
        DwtLevelArgs a = level_args(p, l, page_px(i), live[i]->block_base, coef, ll, ll + half);
        if (raw)
          for (auto& bc : a.band)
            for (auto& bo : bc) bo.step = 0.0f;
        if (a.rw >= 2 && a.rh >= 2) {
          args.push_back(a);
          bases.push_back(g.ntiles);
          g.ntiles += dwt_tiles(a.rw, a.rh, a.ncomp);
          ++g.npages;
        } else {
          singles[l].push_back({a, rev});
        }
      }
      bases.push_back(g.ntiles);
      if (g.npages > 0) groups[l].push_back(g);
    }
  if (!args.empty()) {
    if (!reserve(c, c->dwtargs, args.size() * sizeof(DwtLevelArgs)) ||
        !reserve(c, c->dwtbases, bases.size() * sizeof(uint32_t)) ||
        !cuda_ok(c, cudaMemcpyAsync(c->dwtargs.p, args.data(), args.size() * sizeof(DwtLevelArgs),
                                    cudaMemcpyHostToDevice, c->stream), "H2D level arguments") ||
        !cuda_ok(c, cudaMemcpyAsync(c->dwtbases.p, bases.data(), bases.size() * sizeof(uint32_t),
                                    cudaMemcpyHostToDevice, c->stream), "H2D tile bases"))
      return kEncodeFailed;
  }
  const DwtLevelArgs* d_args = dptr<DwtLevelArgs>(c->dwtargs);
  const uint32_t* d_bases = dptr<uint32_t>(c->dwtbases);
  for (int l = 1; l <= maxL; ++l) {
    for (const Group& g : groups[l]) {
      launch_dwt_batch(d_args + g.arg0, d_bases + g.base0, g.npages, g.ntiles, g.rev, c->stream);
      ++launches;
    }
    for (const auto& sa : singles[l]) {
      launch_dwt_level(sa.first, sa.second, c->stream);
      ++launches;
    }
  }
  c->counters[5] += (uint64_t)launches;
  return kOk;
}

// Code-blocks each MQ producer/consumer pair codes at once. Automatic: one
// (all lanes on the chain) up to 8 blocks per SM, where the heaviest
// block's chain sets the time; two (one per half-warp) up to 24, where
// instruction issue does; four (one per quarter-warp, on 4 pairs per SM)
// above (measured on gray pages of 1275x1650 to 3400x4400 and 2550x3300
// sRGB pages: 4.5 against 5.6 ms of MQ for the sRGB page).
int mq_chains_per_pair(const jp2g_ctx* c, uint32_t nb) {
  const int64_t v = c->opt[JP2G_OPT_MQ_CHAINS_PER_PAIR];
  if (v == 1 || v == 2 || v == 4) return (int)v;
  return nb <= (uint32_t)c->num_sms * 8u ? 1 : (nb <= (uint32_t)c->num_sms * 24u ? 2 : 4);
}

// Runs f(0..n-1) on up to `threads` host threads.
template <class F>
void parallel_for(size_t n, int threads, F f) {
  const size_t t = std::min<size_t>(n, (size_t)std::max(threads, 1));
  if (t <= 1) {
    for (size_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  pool.reserve(t);
  for (size_t k = 0; k < t; ++k)
    pool.emplace_back([&] {
      for (size_t i; (i = next.fetch_add(1)) < n;) f(i);
    });
  for (auto& th : pool) th.join();
}

// Host threads for staging and Tier-2. By default two hardware threads stay
// free for the thread that launches the next wave and waits on the stream,
// so overlapped Tier-2 never delays the device.
int host_threads(jp2g_ctx* c) {
  if (c->opt[JP2G_OPT_HOST_THREADS] > 0) return (int)c->opt[JP2G_OPT_HOST_THREADS];
  return std::max(1, (int)std::thread::hardware_concurrency() - 2);
}

// Debug captures of a single-page wave.
struct WaveDebug {
  bool stop_after_dwt = false;
  bool raw_coefficients = false;  // lossy: f32 coefficient bits instead of quantised indices
  std::vector<BlockOut>* res = nullptr;
  std::vector<BlockKeep>* keep = nullptr;  // the retained-pass table
};

// Pixels of a wave's host-memory pages, staged in pinned memory.
struct Prestaged {
  HostBuf* buf;
  size_t total;
  DevBuf* dev = nullptr;              // the wave's device pixel buffer (default: px)
  cudaEvent_t uploaded = nullptr;     // set: the pixels are already on their way (wait on it)
};
constexpr size_t kStageFailed = ~size_t(0);

// Lays out the host pixels of the valid pages among jobs in the wave's
// device pixel buffer (sets each page's px_off; returns the bytes, or
// kStageFailed). Small pages already in the device layout (gray,
// interleaved RGB) are later copied straight from the caller's memory; the
// others are copied into `buf` (pinned, at the same offsets), planar RGB
// interleaved on the way (Image::from_rgb_bytes takes RGBRGB), in 2 MiB
// tasks over the host threads.
// Host pixels reach the device one copy per page. A wave holding at most
// kDirectCopyMax bytes of host pixels copies pages in the device layout
// (gray, interleaved RGB) straight from the caller's memory; a larger wave
// (a big page, or many pages) is first gathered into pinned staging by the
// host threads: a pageable copy runs near the pinned rate only for memory
// the driver has already seen (a first copy of fresh pages is several
// times slower), and for every wave after a batch's first the gathering
// overlaps the previous wave's device work. Planar RGB is always staged: it
// is interleaved on the way.
constexpr size_t kDirectCopyMax = 32u << 20;
bool needs_staging(const PageJob* j, size_t wave_host_bytes) {
  return (j->ncomp == 3 && !j->interleaved) || wave_host_bytes > kDirectCopyMax;
}

// on_staged (optional) is called, on the host thread that finished it, for
// each page once its pixels are in `buf`, so its upload can start while the
// other pages are still being gathered.
size_t stage_pixels(jp2g_ctx* c, PageJob* const* jobs, size_t n, HostBuf& buf,
                    const std::function<void(const PageJob*)>& on_staged = nullptr) {
  size_t total = 0, host_bytes = 0;
  std::vector<PageJob*> paged;
  for (size_t i = 0; i < n; ++i) {
    PageJob* j = jobs[i];
    PagePlan p;
    Failure f{};
    j->staged = false;
    j->laid_out = false;
    if (!j->host_px || !build_plan(j->w, j->h, (int)j->ncomp, j->quality, j->format, &p, &f)) continue;
    j->laid_out = true;
    j->px_off = total;
    total += ((size_t)j->w * j->h * j->ncomp + 255) & ~size_t(255);
    host_bytes += (size_t)j->w * j->h * j->ncomp;
    paged.push_back(j);
  }
  std::vector<PageJob*> staged;
  for (PageJob* j : paged)
    if (needs_staging(j, host_bytes)) {
      j->staged = true;
      staged.push_back(j);
    }
  if (staged.empty()) return total;
  if (!reserve_host(c, buf, total)) return kStageFailed;
  uint8_t* staging = reinterpret_cast<uint8_t*>(buf.p);
  struct CopyTask {
    const PageJob* j;
    size_t p0, p1;  // pixel range
    size_t page;    // index in `staged`
  };
  std::vector<CopyTask> tasks;
  std::unique_ptr<std::atomic<int>[]> left(new std::atomic<int>[staged.size()]);
  for (size_t i = 0; i < staged.size(); ++i) {
    const PageJob* j = staged[i];
    const size_t np = (size_t)j->w * j->h, step = std::max<size_t>((2u << 20) / j->ncomp, 1);
    int count = 0;
    for (size_t p0 = 0; p0 < np; p0 += step, ++count) tasks.push_back({j, p0, std::min(np, p0 + step), i});
    left[i].store(count);
  }
  parallel_for(tasks.size(), tasks.size() > 2 ? host_threads(c) : 1, [&](size_t k) {
    const CopyTask& t = tasks[k];
    struct Done {  // the last task of a page hands it on
      const CopyTask& t;
      std::atomic<int>* left;
      const std::function<void(const PageJob*)>& cb;
      ~Done() {
        if (cb && left[t.page].fetch_sub(1) == 1) cb(t.j);
      }
    } done{t, left.get(), on_staged};
    const PageJob* j = t.j;
    uint8_t* dst = staging + j->px_off;
    const size_t np = (size_t)j->w * j->h;
    if (j->ncomp == 3 && !j->interleaved) {
      for (size_t i = t.p0; i < t.p1; ++i) {
        dst[3 * i + 0] = j->host_px[i];
        dst[3 * i + 1] = j->host_px[np + i];
        dst[3 * i + 2] = j->host_px[2 * np + i];
      }
    } else {
      std::memcpy(dst + t.p0 * j->ncomp, j->host_px + t.p0 * j->ncomp, (t.p1 - t.p0) * j->ncomp);
    }
  });

  return total;
}

// Nodes of a tag tree over w x h leaves (ISO/IEC 15444-1 B.10.2): every
// level down to a single root.
uint64_t tag_tree_nodes(int w, int h) {
  if (w <= 0 || h <= 0) return 0;
  uint64_t total = 0;
  for (;;) {
    total += (uint64_t)w * h;
    if (w * h <= 1) return total;
    w = (w + 1) / 2;
    h = (h + 1) / 2;
  }
}

// Tier-2 of the wave's pages on the device (t2dev.cu): the packet, band and
// page tables and each page's marker prefix are made on the host from the
// plans; the header and assembly kernels write the finished codestreams into
// one device buffer; only those bytes come back, into pinned memory, and from
// there into each page's own malloc'd buffer. Pages already failed are
// skipped.
int run_tier2(jp2g_ctx* c, const std::vector<PageJob*>& live, const BlockKeep* d_keep,
              const uint32_t* d_offsets, const uint8_t* d_body, uint32_t body_total) {
  std::vector<T2Packet> pks;
  std::vector<T2Band> bds;
  std::vector<T2Page> pgs;
  std::vector<uint8_t> tmpl;
  std::vector<PageJob*> pages;
  uint64_t tree_nodes = 0, raw_words = 0, hdr_bytes = 0;
  for (PageJob* j : live) {
    if (j->status != kOk) continue;
    const PagePlan& p = j->plan;
    T2Page pg{};
    pg.packet0 = (uint32_t)pks.size();
    pg.tmpl_off = (uint32_t)tmpl.size();
    std::vector<uint8_t> pre;
    Failure f{};
    if (!codestream_prefix(p, 0, &pre, &pg.psot_pos, &pg.jp2c_pos, &f)) {
      j->status = f.code;
      j->err = f.msg;
      continue;
    }
    tmpl.insert(tmpl.end(), pre.begin(), pre.end());
    pg.tmpl_len = (uint32_t)pre.size();
    // bands are stored res -> comp -> orient: a packet is a run of one
    // (resolution, component)
    size_t bi = 0;
    while (bi < p.bands.size()) {
      size_t be = bi;
      while (be < p.bands.size() && p.bands[be].res == p.bands[bi].res && p.bands[be].comp == p.bands[bi].comp)
        ++be;
      T2Packet pk{};
      pk.band0 = (uint32_t)bds.size();
      pk.nbands = (uint32_t)(be - bi);
      pk.page = (uint32_t)pgs.size();
      uint64_t nblk = 0;
      for (size_t k = bi; k < be; ++k) {
        const BandGeom& g = p.bands[k];
        T2Band b{};
        b.first_block = j->block_base + g.first_block;
        b.tree_off = (uint32_t)tree_nodes;
        b.ncbx = (uint16_t)g.ncbx;
        b.ncby = (uint16_t)g.ncby;
        bds.push_back(b);
        tree_nodes += tag_tree_nodes(g.ncbx, g.ncby);
        nblk += (uint64_t)g.ncbx * g.ncby;
      }
      const BandGeom& last = p.bands[be - 1];
      pk.b0 = j->block_base + p.bands[bi].first_block;
      pk.b1 = j->block_base + last.first_block + (uint32_t)(last.ncbx * last.ncby);
      // header bounds per code-block: 400 unstuffed bits (inclusion and
      // zero bit-plane tree bits, Table B-4 code, Lblock comma and length),
      // 60 stuffed bytes
      pk.raw_off = (uint32_t)raw_words;
      raw_words += (1 + 400 * nblk) / 32 + 2;
      pk.hdr_off = (uint32_t)hdr_bytes;
      hdr_bytes += 60 * nblk + 16;
      pks.push_back(pk);
      bi = be;
    }
    pg.npackets = (uint32_t)pks.size() - pg.packet0;
    pgs.push_back(pg);
    pages.push_back(j);
  }
  if (pgs.empty()) return kOk;
  const uint64_t out_bound = tmpl.size() + hdr_bytes + body_total + 2 * pgs.size();
  if (out_bound > 0xffffffffull || raw_words > 0xffffffffull)
    return set_err(c, kUnsupportedFeature, "codestreams of one device wave exceed 4 GiB");
  const uint32_t npk = (uint32_t)pks.size(), npg = (uint32_t)pgs.size();
  if (!reserve(c, c->t2pk, npk * sizeof(T2Packet)) || !reserve(c, c->t2bd, bds.size() * sizeof(T2Band)) ||
      !reserve(c, c->t2pg, npg * sizeof(T2Page)) || !reserve(c, c->t2tmpl, tmpl.size()) ||
      !reserve(c, c->t2tree, std::max<uint64_t>(tree_nodes, 1) * sizeof(T2Node)) ||
      !reserve(c, c->t2raw, (raw_words + 2) * 4) || !reserve(c, c->t2hdr, hdr_bytes) ||
      !reserve(c, c->t2hdrlen, npk * 4) || !reserve(c, c->t2pktoff, npk * 4) || !reserve(c, c->t2pagelen, npg * 4) ||
      !reserve(c, c->t2pageoff, (npg + 1) * 4) || !reserve(c, c->t2nchunks, npk * 4) ||
      !reserve(c, c->t2chunkbase, (npk + 1) * 4) || !reserve(c, c->t2out, out_bound) ||
      !reserve(c, c->scratch, ((size_t)std::max(npg, npk) / 1024 + 2) * 4) ||
      !reserve_host(c, c->hpageoff, (npg + 1) * 4))
    return kEncodeFailed;
  if (!cuda_ok(c, cudaMemcpyAsync(c->t2pk.p, pks.data(), npk * sizeof(T2Packet), cudaMemcpyHostToDevice, c->stream),
               "H2D packets") ||
      !cuda_ok(c, cudaMemcpyAsync(c->t2bd.p, bds.data(), bds.size() * sizeof(T2Band), cudaMemcpyHostToDevice,
                                  c->stream), "H2D bands") ||
      !cuda_ok(c, cudaMemcpyAsync(c->t2pg.p, pgs.data(), npg * sizeof(T2Page), cudaMemcpyHostToDevice, c->stream),
               "H2D pages") ||
      !cuda_ok(c, cudaMemcpyAsync(c->t2tmpl.p, tmpl.data(), tmpl.size(), cudaMemcpyHostToDevice, c->stream),
               "H2D marker prefixes") ||
      !cuda_ok(c, cudaMemsetAsync(c->t2raw.p, 0, (raw_words + 2) * 4, c->stream), "memset"))
    return kEncodeFailed;
  T2Args a{};
  a.packets = dptr<T2Packet>(c->t2pk);
  a.npackets = npk;
  a.bands = dptr<T2Band>(c->t2bd);
  a.pages = dptr<T2Page>(c->t2pg);
  a.npages = npg;
  a.keep = d_keep;
  a.offsets = d_offsets;
  a.body = d_body;
  a.tmpl = dptr<uint8_t>(c->t2tmpl);
  a.tree = dptr<T2Node>(c->t2tree);
  a.raw = dptr<uint32_t>(c->t2raw);
  a.hdr = dptr<uint8_t>(c->t2hdr);
  a.hdr_len = dptr<uint32_t>(c->t2hdrlen);
  a.pkt_off = dptr<uint32_t>(c->t2pktoff);
  a.page_len = dptr<uint32_t>(c->t2pagelen);
  a.page_off = dptr<uint32_t>(c->t2pageoff);
  a.nchunks = dptr<uint32_t>(c->t2nchunks);
  a.chunk_base = dptr<uint32_t>(c->t2chunkbase);
  a.out = dptr<uint8_t>(c->t2out);
  launch_t2(a, dptr<uint32_t>(c->scratch), c->num_sms, c->stream);
  c->counters[5] += 6 + (npg > 1024 ? 1 : 0) + (npk > 1024 ? 1 : 0);
  record(c, kEvT2End);
  const uint32_t* hoff = reinterpret_cast<const uint32_t*>(c->hpageoff.p);
  if (!cuda_ok(c, cudaMemcpyAsync(c->hpageoff.p, a.page_off, (npg + 1) * 4, cudaMemcpyDeviceToHost, c->stream),
               "D2H page offsets") ||
      !cuda_ok(c, cudaStreamSynchronize(c->stream), "tier-2 kernels"))
    return kEncodeFailed;
  const uint32_t total = hoff[npg];
  if (!reserve_host(c, c->hout, std::max<size_t>(total, 1)) ||
      !cuda_ok(c, cudaMemcpyAsync(c->hout.p, a.out, total, cudaMemcpyDeviceToHost, c->stream), "D2H codestreams") ||
      !cuda_ok(c, cudaStreamSynchronize(c->stream), "D2H codestreams"))
    return kEncodeFailed;
  const uint8_t* hout = reinterpret_cast<const uint8_t*>(c->hout.p);
  std::atomic<bool> oom{false};
  auto take = [&](size_t i) {
    PageJob* j = pages[i];
    const size_t len = hoff[i + 1] - hoff[i];
    j->drop_output();
    j->cs = static_cast<uint8_t*>(std::malloc(std::max<size_t>(len, 1)));
    if (!j->cs) {
      oom = true;
      j->status = kEncodeFailed;
      j->err = "out of host memory";
      return;
    }
    std::memcpy(j->cs, hout + hoff[i], len);
    j->cs_len = len;
  };
  parallel_for(pages.size(), pages.size() >= 8 && total >= (8u << 20) ? host_threads(c) : 1, take);
  (void)oom;
  return kOk;
}

// Device phase of a wave of pages: plans and validation, inputs,
// colour+DWT+quantisation per page, then Tier-1, PCRD and compaction over
// the wave's flat code-block list (all pages' blocks, page after page), and
// the read-back of each page's retained blocks and bytes into its job. A page
// that fails validation or overflows a block slot is marked and the rest
// carry on; a CUDA failure fails the wave (return code). `pre`: the wave's
// host pixels already staged by stage_pixels (else they are staged here).
int run_wave(jp2g_ctx* c, PageJob* const* jobs, size_t njobs, WaveDebug* dbg,
             const Prestaged* pre = nullptr) {
  std::memset(c->counters, 0, sizeof c->counters);
  std::vector<PageJob*> live;
  int cbw = 0;
  uint32_t pcap = 0;
  for (size_t i = 0; i < njobs; ++i) {
    PageJob* j = jobs[i];
    Failure f{};
    j->status = kOk;
    if (!build_plan(j->w, j->h, (int)j->ncomp, j->quality, j->format, &j->plan, &f)) {
      j->status = f.code;
      j->err = f.msg;
      continue;
    }
    if (!j->host_px && !j->dev_px) {
      j->status = kInvalidInput;
      j->err = "pixel pointer is null";
      continue;
    }
    if (cbw == 0) cbw = j->plan.cbw;
    if (j->plan.cbw != cbw) {  // waves are formed per code-block size
      j->status = kEncodeFailed;
      j->err = "pages of one wave must share the code-block size";
      continue;
    }
    pcap = std::max(pcap, pass_cap(j->plan));
    live.push_back(j);
  }
  if (live.empty()) return kOk;
  const PagePlan& p0 = live[0]->plan;
  const uint32_t cap = slot_cap(p0);
  const size_t slot = (size_t)p0.cbw * p0.cbh;
  std::vector<BlockDesc> blocks;
  std::vector<BandParam> bands;
  std::vector<CompParam> comps;
  uint64_t nb64 = 0;
  for (PageJob* j : live) {
    j->block_base = (uint32_t)nb64;
    build_tables(j->plan, j->block_base, (uint32_t)bands.size(), (uint32_t)comps.size(), cap, pcap,
                 &blocks, &bands, &comps);
    nb64 += j->plan.nblocks;
  }
  if (nb64 * cap > 0xffffffffull)
    return set_err(c, kUnsupportedFeature,
                   "too many code-blocks in one device wave (" + std::to_string(nb64) + ")");
  if (bands.size() > 0xffff)
    return set_err(c, kUnsupportedFeature, "too many pages in one device wave");
  const uint32_t nb = (uint32_t)nb64;
  if (!reserve(c, c->coef, std::max<size_t>(nb, 1) * slot * 4) ||
      !reserve(c, c->payload, std::max<size_t>(nb, 1) * cap) ||
      !reserve(c, c->passes, std::max<size_t>(nb, 1) * pcap * sizeof(PassRec)) ||
      !reserve(c, c->res, std::max<size_t>(nb, 1) * sizeof(BlockOut)) ||
      !reserve(c, c->keep, std::max<size_t>(nb, 1) * sizeof(BlockKeep)) ||
      !reserve(c, c->blocks, std::max<size_t>(nb, 1) * sizeof(BlockDesc)) ||
      !reserve(c, c->bands, bands.size() * sizeof(BandParam)) ||
      !reserve(c, c->comps, comps.size() * sizeof(CompParam)) ||
      !reserve(c, c->maxslope, std::max<size_t>(comps.size(), 8) * sizeof(unsigned long long)) ||
      !reserve(c, c->hullp, std::max<size_t>(nb, 1) * pcap * sizeof(uint16_t)) ||
      !reserve(c, c->hulls, std::max<size_t>(nb, 1) * pcap * sizeof(double)) ||
      !reserve(c, c->hulln, std::max<size_t>(nb, 1)) ||
      !reserve(c, c->offsets, (size_t)(nb + 1) * 4) ||
      !reserve(c, c->scratch, ((size_t)nb / 1024 + 2) * 4) ||
      !reserve(c, c->nplanes, std::max<size_t>(nb, 1) * 4) ||
      !reserve(c, c->planebase, (size_t)(nb + 1) * 4) ||
      !reserve(c, c->body, std::max<size_t>(nb, 1) * cap) ||
      !reserve(c, c->stats, 64) || !reserve_host(c, c->hcount, 64))
    return kEncodeFailed;

  record(c, 0);
  // ---- inputs ----
  size_t hpx_total = 0;
  const uint8_t* staging = nullptr;
  if (pre) {
    hpx_total = pre->total;
    staging = reinterpret_cast<const uint8_t*>(pre->buf->p);
  } else {
    hpx_total = stage_pixels(c, live.data(), live.size(), c->hpx);
    if (hpx_total == kStageFailed) return kEncodeFailed;
    staging = reinterpret_cast<const uint8_t*>(c->hpx.p);
  }
  DevBuf& pxbuf = pre && pre->dev ? *pre->dev : c->px;
  if (pre && pre->uploaded) {
    // uploaded on the copy stream while the previous wave computed
    if (!cuda_ok(c, cudaStreamWaitEvent(c->stream, pre->uploaded, 0), "wait for pixels")) return kEncodeFailed;
  } else if (hpx_total > 0) {
    if (!reserve(c, pxbuf, hpx_total)) return kEncodeFailed;
    // one copy per page: from pinned staging, or straight from the caller's
    // memory for small pages in the device layout
    for (PageJob* j : live) {
      if (!j->host_px) continue;
      const uint8_t* from = j->staged ? staging + j->px_off : j->host_px;
      if (!cuda_ok(c, cudaMemcpyAsync(dptr<uint8_t>(pxbuf) + j->px_off, from, (size_t)j->w * j->h * j->ncomp,
                                      cudaMemcpyHostToDevice, c->stream), "H2D"))
        return kEncodeFailed;
    }
  }
  c->wave_px = dptr<uint8_t>(pxbuf);
  if (!cuda_ok(c, cudaMemcpyAsync(c->blocks.p, blocks.data(), nb * sizeof(BlockDesc),
                                  cudaMemcpyHostToDevice, c->stream), "H2D blocks") ||
      !cuda_ok(c, cudaMemcpyAsync(c->bands.p, bands.data(), bands.size() * sizeof(BandParam),
                                  cudaMemcpyHostToDevice, c->stream), "H2D bands") ||
      !cuda_ok(c, cudaMemcpyAsync(c->comps.p, comps.data(), comps.size() * sizeof(CompParam),
                                  cudaMemcpyHostToDevice, c->stream), "H2D comps"))
    return kEncodeFailed;
  record(c, 1);
  // ---- colour + DWT + quantisation, one launch per level for the wave ----
  if (int rc = run_dwt_wave(c, live, dbg && dbg->raw_coefficients)) return rc;
  record(c, 2);
  if (dbg && dbg->stop_after_dwt) {
    if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "DWT")) return kEncodeFailed;
    return kOk;
  }
  // ---- Tier-1 over the wave's code-blocks ----
  T1Args ta{};
  ta.blocks = dptr<BlockDesc>(c->blocks);
  ta.nblocks = nb;
  ta.coef = dptr<int32_t>(c->coef);
  ta.cbw = p0.cbw;
  ta.cbh = p0.cbh;
  ta.out = dptr<uint8_t>(c->payload);
  ta.passes = dptr<PassRec>(c->passes);
  ta.pass_cap = pcap;
  ta.res = dptr<BlockOut>(c->res);
  ta.nplanes = dptr<uint32_t>(c->nplanes);
  ta.plane_base = dptr<uint32_t>(c->planebase);
  ta.sym_slot = (uint32_t)((slot * 5 / 2 + 15) & ~size_t(15));
  ta.sym_count = dptr<unsigned long long>(c->stats);
  if (!cuda_ok(c, cudaMemsetAsync(c->stats.p, 0, 8, c->stream), "memset")) return kEncodeFailed;
  launch_t1_analyze(ta, c->stream);
  launch_scan_u32(ta.nplanes, 1, nb, ta.plane_base, dptr<uint32_t>(c->scratch), c->stream);
  // the number of (block, bit-plane) items sizes the symbol buffer
  if (!cuda_ok(c, cudaMemcpyAsync(c->hcount.p, ta.plane_base + nb, 4, cudaMemcpyDeviceToHost, c->stream),
               "D2H item count") ||
      !cuda_ok(c, cudaStreamSynchronize(c->stream), "tier-1 analysis"))
    return kEncodeFailed;
  ta.nitems = *reinterpret_cast<uint32_t*>(c->hcount.p);
  if (!reserve(c, c->items, std::max<size_t>(ta.nitems, 1) * 4) ||
      !reserve(c, c->itemrec, std::max<size_t>(ta.nitems, 1) * sizeof(ItemRec)) ||
      !reserve(c, c->planes, std::max<size_t>(ta.nitems, 1) * 1024) ||
      !reserve(c, c->signs, std::max<size_t>(nb, 1) * 512) ||
      !reserve(c, c->sym, std::max<size_t>(ta.nitems, 1) * ta.sym_slot + 64))  // the MQ reader runs 48 B ahead
    return kEncodeFailed;
  ta.items = dptr<uint32_t>(c->items);
  ta.item_rec = dptr<ItemRec>(c->itemrec);
  ta.planes = dptr<uint32_t>(c->planes);
  ta.signs = dptr<uint32_t>(c->signs);
  ta.sym = dptr<uint8_t>(c->sym);
  launch_t1_planes(ta, c->stream);
  record(c, kEvAnalyzeEnd);
  launch_t1_model(ta, c->num_sms, c->stream);
  record(c, kEvModelEnd);
  // Blocks are coded heaviest first: with several blocks per warp so that a
  // warp's lanes carry similar symbol counts; with one block per warp by a
  // fixed number of warps per SM that pull blocks in that order, so the
  // longest chains start first and share their schedulers with few others.
  // Automatic choice (measured on 1275x1650 to 5100x6600 pages): up to 48
  // blocks per SM, producer/consumer pipelines pulling blocks; beyond that,
  // 2..32 blocks packed per warp.
  const int64_t bpw_opt = c->opt[JP2G_OPT_MQ_BLOCKS_PER_WARP];
  const int64_t wps_opt = c->opt[JP2G_OPT_MQ_WARPS_PER_SM];
  const uint32_t sms = (uint32_t)c->num_sms;
  const int bpw = mq_blocks_per_warp(ta, c->num_sms, (int)bpw_opt);
  const bool use_pull = bpw == 1 && wps_opt >= 0;
  const int pull = wps_opt > 0 ? (int)wps_opt : (nb <= sms * 16u ? 8 : 12);
  int order_launches = 0;
  if (bpw > 1 || use_pull) {
    if (!reserve(c, c->mqorder, (size_t)nb * 4) || !reserve(c, c->mqscratch, ((size_t)nb + 2048) * 4))
      return kEncodeFailed;
    launch_mq_order(ta, dptr<uint32_t>(c->mqorder), dptr<uint32_t>(c->mqscratch), c->stream);
    ta.mq_order = dptr<uint32_t>(c->mqorder);
    order_launches = 3;
  }
  // Producer/consumer pairs shorten each block's chain (8 pairs per SM, one
  // or two chains each); up to 48 blocks per SM they beat single-warp
  // pulling and packed warps.
  const int64_t pipes_opt = c->opt[JP2G_OPT_MQ_PIPES_PER_SM];
  const bool use_pipe = use_pull && (pipes_opt > 0 || (pipes_opt == 0 && nb <= sms * 48u));
  if (use_pipe) {
    // four chains per pair run on 4 pairs per SM (16 chains per SM, as 8
    // pairs of two): measured best for an sRGB 2550x3300 page
    const int chains = mq_chains_per_pair(c, nb);
    launch_t1_mq_pipe(ta, c->num_sms, pipes_opt > 0 ? (int)pipes_opt : (chains == 4 ? 4 : 8), chains,
                      (uint32_t)c->opt[JP2G_OPT_MQ_HEAVY], dptr<uint32_t>(c->stats) + 2, c->stream);
  }
  else if (use_pull)
    launch_t1_mq_pull(ta, c->num_sms, pull, dptr<uint32_t>(c->stats) + 2, c->stream);
  else
    launch_t1_mq(ta, c->num_sms, bpw, c->stream);
  c->counters[5] += 5 + (nb > 1024 ? 1 : 0) + order_launches;
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
  // ---- read back the per-block results ----
  if (!reserve_host(c, c->hkeep, std::max<size_t>(nb, 1) * sizeof(BlockKeep)) ||
      !reserve_host(c, c->hres, std::max<size_t>(nb, 1) * sizeof(BlockOut)))
    return kEncodeFailed;
  uint32_t* hcount = reinterpret_cast<uint32_t*>(c->hcount.p);
  if (!cuda_ok(c, cudaMemcpyAsync(c->hkeep.p, c->keep.p, nb * sizeof(BlockKeep),
                                  cudaMemcpyDeviceToHost, c->stream), "D2H keep") ||
      !cuda_ok(c, cudaMemcpyAsync(c->hres.p, c->res.p, nb * sizeof(BlockOut),
                                  cudaMemcpyDeviceToHost, c->stream), "D2H results") ||
      !cuda_ok(c, cudaMemcpyAsync(hcount + 2, c->stats.p, 8, cudaMemcpyDeviceToHost, c->stream),
               "D2H statistics") ||
      !cuda_ok(c, cudaMemcpyAsync(hcount + 4, dptr<uint32_t>(c->offsets) + nb, 4, cudaMemcpyDeviceToHost,
                                  c->stream), "D2H retained bytes") ||
      !cuda_ok(c, cudaStreamSynchronize(c->stream), "encode kernels"))
    return kEncodeFailed;
  const BlockKeep* hk = reinterpret_cast<const BlockKeep*>(c->hkeep.p);
  const uint32_t total = hcount[4];
  for (PageJob* j : live) {
    const uint32_t b0 = j->block_base, n = j->plan.nblocks;
    for (uint32_t i = 0; i < n; ++i) {
      if (hk[b0 + i].status == 1) {
        j->status = kEncodeFailed;
        j->err = "code-block payload exceeded its device slot";
        break;
      }
      if (hk[b0 + i].status >= 2) {
        j->status = kEncodeFailed;
        j->err = "code-block bit-plane count exceeds the supported maximum";
        break;
      }
    }
  }
  // ---- Tier-2 and codestream assembly on the device ----
  if (int rc = run_tier2(c, live, pa.keep, dptr<uint32_t>(c->offsets), dptr<uint8_t>(c->body), total)) return rc;
  record(c, 6);
  const BlockOut* hr = reinterpret_cast<const BlockOut*>(c->hres.p);
  c->counters[0] = nb;
  for (uint32_t i = 0; i < nb; ++i) {
    c->counters[1] += hr[i].mbp > 0;
    c->counters[2] += hr[i].npasses;
    c->counters[3] += hr[i].payload_len;
    c->counters[6] += (uint64_t)hr[i].mbp * blocks[i].w * blocks[i].h;
  }
  c->counters[4] = total;
  c->counters[7] = *reinterpret_cast<const uint64_t*>(hcount + 2);
  if (dbg && dbg->res) dbg->res->assign(hr, hr + nb);
  if (dbg && dbg->keep) dbg->keep->assign(hk, hk + nb);
  return kOk;
}

// Frees every device pool (after the stream has drained), so the next wave
// allocates exactly what it needs under the budget.
void release_pools(jp2g_ctx* c) {
  cudaStreamSynchronize(c->stream);
  DevBuf* bufs[] = {&c->px, &c->px2, &c->ll0, &c->coef, &c->payload, &c->passes, &c->res, &c->keep,
                    &c->blocks, &c->bands, &c->comps, &c->maxslope, &c->hullp, &c->hulls, &c->hulln,
                    &c->offsets, &c->scratch, &c->body, &c->nplanes, &c->planebase, &c->items,
                    &c->itemrec, &c->planes, &c->signs, &c->sym, &c->stats, &c->dwtargs, &c->dwtbases,
                    &c->mqorder, &c->mqscratch, &c->recon, &c->reconblk, &c->t2pk, &c->t2bd, &c->t2pg,
                    &c->t2tmpl, &c->t2tree, &c->t2raw, &c->t2hdr, &c->t2hdrlen, &c->t2pktoff, &c->t2pagelen,
                    &c->t2pageoff, &c->t2nchunks, &c->t2chunkbase, &c->t2out};
  for (DevBuf* b : bufs) {
    if (b->p) cudaFree(b->p);
    b->p = nullptr;
    b->cap = 0;
  }
  c->allocated.store(0);
}

// Admission by the device memory budget: runs a wave, and when a pool could
// not grow within the budget, releases the pools and runs the two halves of
// the wave one after the other (recursively), instead of failing its pages.
// The largest wave that fitted caps later waves (budget_wave_blocks). A single
// page that does not fit on its own fails alone, with the budget message;
// the other pages carry on. Counters cover all the parts.
int run_wave_within_budget(jp2g_ctx* c, PageJob* const* jobs, size_t n, const Prestaged* pre) {
  c->budget_hit = false;
  int rc = run_wave(c, jobs, n, nullptr, pre);
  if (rc == kOk || !c->budget_hit) return rc;
  // pools sized by earlier waves may crowd out the one this wave needs: try
  // again from empty pools before splitting
  release_pools(c);
  c->budget_hit = false;
  rc = run_wave(c, jobs, n, nullptr, pre);
  if (rc == kOk || !c->budget_hit) return rc;
  const std::string msg = get_msg(c);
  release_pools(c);
  uint64_t blocks = 0;
  for (size_t i = 0; i < n; ++i) blocks += jobs[i]->plan.nblocks;
  if (n == 1) {
    jobs[0]->status = kEncodeFailed;
    jobs[0]->err = msg + ": the page does not fit on its own";
    return kOk;
  }
  c->budget_wave_blocks = std::max<uint64_t>(1, blocks / 2);
  const size_t h = n / 2;
  uint64_t counters[8];
  if ((rc = run_wave_within_budget(c, jobs, h, pre))) return rc;
  std::memcpy(counters, c->counters, sizeof counters);
  if ((rc = run_wave_within_budget(c, jobs + h, n - h, pre))) return rc;
  for (int k = 0; k < 8; ++k) c->counters[k] += counters[k];
  return kOk;
}

// Device Tier-2 (compaction end -> kEvT2End) is reported on its own; the
// read-back stage then runs from kEvT2End to event 6.
float stage_span(jp2g_ctx* c, int s) {
  float ms = 0;
  if (s == kD2H) cudaEventElapsedTime(&ms, c->ev[kEvT2End], c->ev[6]);
  else cudaEventElapsedTime(&ms, c->ev[s], c->ev[s + 1]);
  return ms;
}

// Adds the device stages of the wave just run (events 0..6) to stage_ms.
void add_wave_stage_times(jp2g_ctx* c) {
  if (!c->timing) return;
  cudaEventSynchronize(c->ev[6]);
  float ms = 0;
  for (int s = 0; s < kHost; ++s) c->stage_ms[s] += stage_span(c, s);
  cudaEventElapsedTime(&ms, c->ev[kCompact + 1], c->ev[kEvT2End]);
  c->stage_ms[kNumStages + 3] += ms;
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[6]);
  c->stage_ms[kTotal] += ms;
  const int sub[3][2] = {{2, kEvAnalyzeEnd}, {kEvAnalyzeEnd, kEvModelEnd}, {kEvModelEnd, 3}};
  for (int k = 0; k < 3; ++k) {
    cudaEventElapsedTime(&ms, c->ev[sub[k][0]], c->ev[sub[k][1]]);
    c->stage_ms[kNumStages + k] += ms;
  }
}

// Reads the stage events of the last wave into stage_ms.
void read_stage_times(jp2g_ctx* c) {
  if (!c->timing) return;
  cudaEventSynchronize(c->ev[8]);
  for (int s = 0; s < kTotal; ++s) c->stage_ms[s] = stage_span(c, s);
  cudaEventElapsedTime(&c->stage_ms[kTotal], c->ev[0], c->ev[8]);
  cudaEventElapsedTime(&c->stage_ms[kNumStages + 3], c->ev[kCompact + 1], c->ev[kEvT2End]);
  // tier-1 split: analysis (+item list), modelling, MQ coding
  cudaEventElapsedTime(&c->stage_ms[kNumStages + 0], c->ev[2], c->ev[kEvAnalyzeEnd]);
  cudaEventElapsedTime(&c->stage_ms[kNumStages + 1], c->ev[kEvAnalyzeEnd], c->ev[kEvModelEnd]);
  cudaEventElapsedTime(&c->stage_ms[kNumStages + 2], c->ev[kEvModelEnd], c->ev[3]);
}

// One page through the whole pipeline (jp2g_encode and the debug entry
// points).
int encode_one(jp2g_ctx* c, PageJob* j, WaveDebug* dbg) {
  PageJob* jobs[1] = {j};
  c->budget_hit = false;
  int rc = run_wave(c, jobs, 1, dbg, nullptr);
  if (rc != kOk && c->budget_hit) {  // pools of earlier waves crowd the budget: retry from empty pools
    release_pools(c);
    c->budget_hit = false;
    rc = run_wave(c, jobs, 1, dbg, nullptr);
  }
  if (rc) return rc;
  if (j->status != kOk) return set_err(c, j->status, j->err);
  if (dbg && dbg->stop_after_dwt) return kOk;
  record(c, 7);
  record(c, 8);
  read_stage_times(c);
  if (j->status != kOk) return set_err(c, j->status, j->err);
  return kOk;
}

// Splits jobs into waves: consecutive runs of pages with the same
// code-block size, at most `wave_blocks` code-blocks (a larger page forms a
// wave of its own) and at most kMaxWavePages pages (band constants are
// indexed by 16 bits, 19 per page at most).
constexpr size_t kMaxWavePages = 3000;
// Code-blocks one wave may hold: the wave-size option, capped so that the
// wave's payload slots stay addressable with 32-bit byte offsets.
uint64_t wave_block_limit(const jp2g_ctx* c, int cbw) {
  const uint64_t cap = (uint64_t)cbw * (uint64_t)cbw * 4u + 1024u;  // slot_cap of a cbw x cbw block
  uint64_t lim = std::min<uint64_t>((uint64_t)c->opt[JP2G_OPT_WAVE_BLOCKS], 0xffffffffull / cap);
  if (c->budget_wave_blocks) lim = std::min(lim, c->budget_wave_blocks);
  return lim;
}

std::vector<std::vector<PageJob*>> form_waves(jp2g_ctx* c, const std::vector<PageJob*>& jobs) {
  std::vector<std::vector<PageJob*>> waves;
  std::vector<PageJob*> cur;
  uint64_t cur_blocks = 0;
  int cur_cbw = 0;
  for (PageJob* j : jobs) {
    PagePlan p;
    Failure f{};
    uint64_t nb = 0;
    int cbw = cur_cbw;
    if (build_plan(j->w, j->h, (int)j->ncomp, j->quality, j->format, &p, &f)) {
      nb = p.nblocks;
      cbw = p.cbw;
    }
    if (!cur.empty() &&
        (cbw != cur_cbw || cur_blocks + nb > wave_block_limit(c, cbw) || cur.size() >= kMaxWavePages)) {
      waves.push_back(std::move(cur));
      cur.clear();
      cur_blocks = 0;
    }
    if (cur.empty()) cur_cbw = cbw;
    cur.push_back(j);
    cur_blocks += nb;
  }
  if (!cur.empty()) waves.push_back(std::move(cur));
  return waves;
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
  // under a budget, waves start at 160,000 code-blocks (about 24 GB of
  // pools for 64x64 blocks) so that the first waves need no split
  if (hbm_budget_bytes) c->opt[JP2G_OPT_WAVE_BLOCKS] = 160000;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess || !init_t1_tables()) {
    g_create_error = "CUDA initialisation failed";
    delete c;
    return JP2G_ENCODE_FAILED;
  }
  for (auto& ev : c->ev) cudaEventCreate(&ev);
  cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
  cudaStreamCreateWithFlags(&c->serve_stream, cudaStreamNonBlocking);
  for (int k = 0; k < 2; ++k) {
    cudaEventCreateWithFlags(&c->ev_up[k], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->serve_ev[k], cudaEventDisableTiming);
  }
  *out = c;
  return JP2G_OK;
}

void jp2g_destroy(jp2g_ctx* c) {
  if (!c) return;
  {
    std::lock_guard<std::mutex> lk(c->qmu);
    c->stop = true;
  }
  c->qcv.notify_all();
  c->fcv.notify_all();
  c->rcv.notify_all();
  if (c->stager.joinable()) c->stager.join();
  if (c->worker.joinable()) c->worker.join();
  if (c->finisher.joinable()) c->finisher.join();
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  DevBuf* bufs[] = {&c->px, &c->px2, &c->ll0, &c->coef, &c->payload, &c->passes, &c->res, &c->keep,
                    &c->blocks, &c->bands, &c->comps, &c->maxslope, &c->hullp, &c->hulls, &c->hulln,
                    &c->offsets, &c->scratch, &c->body, &c->nplanes, &c->planebase, &c->items,
                    &c->itemrec, &c->planes, &c->signs, &c->sym, &c->stats, &c->dwtargs, &c->dwtbases,
                    &c->mqorder, &c->mqscratch, &c->recon, &c->reconblk, &c->t2pk, &c->t2bd, &c->t2pg,
                    &c->t2tmpl, &c->t2tree, &c->t2raw, &c->t2hdr, &c->t2hdrlen, &c->t2pktoff, &c->t2pagelen,
                    &c->t2pageoff, &c->t2nchunks, &c->t2chunkbase, &c->t2out};
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  if (c->serve_stream) {
    cudaStreamSynchronize(c->serve_stream);
    cudaStreamDestroy(c->serve_stream);
  }
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  for (DevBuf& b : c->serve_px)
    if (b.p) cudaFree(b.p);
  HostBuf* hb[] = {&c->hpx, &c->hpx2, &c->hkeep, &c->hres, &c->hcount, &c->hpageoff, &c->hout,
                   &c->serve_hpx[0], &c->serve_hpx[1]};
  for (HostBuf* b : hb)
    if (b->p) cudaFreeHost(b->p);
  for (auto& ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  for (int k = 0; k < 2; ++k) {
    if (c->ev_up[k]) cudaEventDestroy(c->ev_up[k]);
    if (c->serve_ev[k]) cudaEventDestroy(c->serve_ev[k]);
  }
  cudaStreamDestroy(c->stream);
  delete c;
}

// Hands the page's codestream (already in its own malloc'd buffer) to the
// caller.
static int finish_output(jp2g_ctx* c, int rc, PageJob& j, uint8_t** out, size_t* out_len) {
  if (rc != JP2G_OK) return rc;
  if (!j.cs) return set_err(c, JP2G_ENCODE_FAILED, "no codestream was produced");
  *out = j.cs;
  *out_len = j.cs_len;
  j.cs = nullptr;
  j.cs_len = 0;
  return JP2G_OK;
}

int jp2g_encode(jp2g_ctx* c, const uint8_t* px, uint32_t w, uint32_t h, uint32_t ncomp,
                int interleaved, uint8_t quality, int format, uint8_t** out, size_t* out_len) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!out || !out_len) return set_err(c, JP2G_INVALID_INPUT, "output pointer is null");
  if (!px) return set_err(c, JP2G_INVALID_INPUT, "pixel pointer is null");
  cudaSetDevice(c->device);
  PageJob j;
  j.host_px = px;
  j.w = w;
  j.h = h;
  j.ncomp = ncomp;
  j.interleaved = interleaved;
  j.quality = quality;
  j.format = format;
  int rc = encode_one(c, &j, nullptr);
  return finish_output(c, rc, j, out, out_len);
}

int jp2g_encode_device(jp2g_ctx* c, const uint8_t* d_px, uint32_t w, uint32_t h, uint32_t ncomp,
                       uint8_t quality, int format, uint8_t** out, size_t* out_len) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!out || !out_len) return set_err(c, JP2G_INVALID_INPUT, "output pointer is null");
  if (!d_px) return set_err(c, JP2G_INVALID_INPUT, "pixel pointer is null");
  cudaSetDevice(c->device);
  PageJob j;
  j.dev_px = d_px;
  j.w = w;
  j.h = h;
  j.ncomp = ncomp;
  j.quality = quality;
  j.format = format;
  int rc = encode_one(c, &j, nullptr);
  return finish_output(c, rc, j, out, out_len);
}

// Quality metrics of the page the last wave encoded (a single-page wave
// whose device buffers are still in place): compute_quality_metrics
// (backend.rs:305-433) on the device. Lossless pages give +inf and 1.0.
static int page_metrics(jp2g_ctx* c, const PageJob& j, double* psnr, double* ssim) {
  const PagePlan& p = j.plan;
  if (p.quality >= 100) {
    *psnr = std::numeric_limits<double>::infinity();
    *ssim = 1.0;
    return kOk;
  }
  if (p.ncomp == 3 && !p.use_mct)
    return set_err(c, kEncodeFailed, "quality metrics not implemented for this colorspace configuration");
  std::vector<ReconBlock> rb(p.nblocks);
  for (const BandGeom& g : p.bands)
    for (int by = 0; by < g.ncby; ++by)
      for (int bx = 0; bx < g.ncbx; ++bx) {
        ReconBlock& r = rb[g.first_block + (uint32_t)(by * g.ncbx + bx)];
        r.x0 = (uint32_t)(g.x0 + bx * p.cbw);
        r.y0 = (uint32_t)(g.y0 + by * p.cbh);
        r.comp = (uint32_t)g.comp;
        r.step = p.quants[g.quant].step_f32;
      }
  const size_t n = (size_t)p.width * p.height;
  const size_t rb_bytes = (std::max<size_t>(rb.size(), 1) * sizeof(ReconBlock) + 255) & ~size_t(255);
  if (!reserve(c, c->recon, (n * (2 * p.ncomp + 2) + 64) * sizeof(float) + 16) ||
      !reserve(c, c->reconblk, rb_bytes + (size_t)(p.ncomp * p.levels + 1) * sizeof(IdwtJob)) ||
      !cuda_ok(c, cudaMemcpyAsync(c->reconblk.p, rb.data(), rb.size() * sizeof(ReconBlock), cudaMemcpyHostToDevice,
                                  c->stream), "H2D metrics blocks"))
    return kEncodeFailed;
  ReconArgs r{};
  r.blocks = dptr<BlockDesc>(c->blocks);
  r.rblocks = dptr<ReconBlock>(c->reconblk);
  r.keep = dptr<BlockKeep>(c->keep);
  r.passes = dptr<PassRec>(c->passes);
  r.coef = dptr<int32_t>(c->coef);
  r.cbw = p.cbw;
  r.cbh = p.cbh;
  r.nblocks = p.nblocks;
  r.width = p.width;
  r.height = p.height;
  r.ncomp = p.ncomp;
  r.px = j.dev_px ? j.dev_px : c->wave_px + j.px_off;
  float* f = dptr<float>(c->recon);
  r.stats = reinterpret_cast<double*>(f);  // 16 bytes at the start
  r.plane = f + 4;
  r.tmp = r.plane + n * p.ncomp;
  r.jobs = reinterpret_cast<IdwtJob*>(static_cast<uint8_t*>(c->reconblk.p) + rb_bytes);
  r.luma_orig = r.tmp + n * p.ncomp;
  r.luma_dec = r.luma_orig + n;
  launch_recon(r, p.ladder.data(), p.levels, c->stream);
  double sums[2] = {0, 0};
  if (!cuda_ok(c, cudaMemcpyAsync(sums, r.stats, sizeof sums, cudaMemcpyDeviceToHost, c->stream), "D2H metrics") ||
      !cuda_ok(c, cudaStreamSynchronize(c->stream), "metrics kernels"))
    return kEncodeFailed;
  const double mse = sums[0] / (double)(n * (size_t)p.ncomp);
  const double max_val = (double)((1u << p.precision) - 1);
  *psnr = mse < 1e-10 ? 100.0 : 20.0 * std::log10(max_val / std::sqrt(mse));
  const uint32_t nb8 = (p.width / 8) * (p.height / 8);
  *ssim = nb8 == 0 ? 1.0 : sums[1] / (double)nb8;
  return kOk;
}

int jp2g_encode_with_psnr(jp2g_ctx* c, const uint8_t* px, uint32_t w, uint32_t h, uint32_t ncomp, int interleaved,
                          uint8_t quality, int format, uint8_t** out, size_t* out_len, double* psnr_db,
                          double* ssim) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!out || !out_len || !psnr_db || !ssim) return set_err(c, JP2G_INVALID_INPUT, "output pointer is null");
  if (!px) return set_err(c, JP2G_INVALID_INPUT, "pixel pointer is null");
  cudaSetDevice(c->device);
  PageJob j;
  j.host_px = px;
  j.w = w;
  j.h = h;
  j.ncomp = ncomp;
  j.interleaved = interleaved;
  j.quality = quality;
  j.format = format;
  int rc = encode_one(c, &j, nullptr);
  if (rc == JP2G_OK) rc = page_metrics(c, j, psnr_db, ssim);
  return finish_output(c, rc, j, out, out_len);
}

// ------------------------------------------------------------- decoding --
// decode_jp2 (src/decode/mod.rs:56-61) on the device, for many files at
// once: the host parses each file's boxes, headers and packet headers
// (decode.cpp, on host threads); a round of files then shares one Tier-1
// decoding launch over all their code-blocks, one inverse-DWT launch pair
// per level over all their components, and one launch for the samples
// (t1dec.cu, recon.cu). Rounds are sized by device memory (the context's
// budget, else 24 GiB); a round whose pools cannot grow is split.
namespace {

struct DecodePage {
  DecodeLayout L;
  int status = JP2G_OK;
  std::string msg;
  uint64_t npx = 0;
  uint64_t data_base = 0, plane_base = 0, px_base = 0;
};

uint64_t decode_device_bytes(const DecodePage& p, size_t nbytes) {
  // bytes, planes, tmp planes, samples, code-blocks, jobs
  return nbytes + p.npx * p.L.ncomp * 9 + p.L.blocks.size() * sizeof(DecBlock) +
         (uint64_t)(p.L.levels * p.L.ncomp + 1) * sizeof(IdwtJob) + sizeof(PixJob) + 1024;
}

// Decodes the pages `ids` in one device round; fills outs / out_lens.
int decode_round(jp2g_ctx* c, std::vector<DecodePage>& pg, const std::vector<size_t>& ids,
                 const uint8_t* const* bytes, const size_t* lens, uint8_t** outs, size_t* out_lens) {
  uint64_t nbytes = 0, nplane = 0, npxb = 0, nblk = 0;
  int maxl = 0;
  for (size_t i : ids) {
    DecodePage& p = pg[i];
    p.data_base = nbytes;
    p.plane_base = nplane;
    p.px_base = npxb;
    nbytes += (lens[i] + 15) & ~size_t(15);
    nplane += p.npx * p.L.ncomp;
    npxb += p.npx * p.L.ncomp;
    nblk += p.L.blocks.size();
    maxl = std::max(maxl, p.L.levels);
  }
  if (nbytes > 0xffffffffull) return set_err(c, JP2G_INVALID_INPUT, "decode round exceeds 4 GiB of input");
  // device job tables: blocks, then per-level inverse-DWT jobs, then pixel jobs
  std::vector<DecBlock> blk;
  blk.reserve(nblk);
  for (size_t i : ids)
    for (DecBlock b : pg[i].L.blocks) {
      b.plane_off += pg[i].plane_base;
      b.data_off += (uint32_t)pg[i].data_base;
      blk.push_back(b);
    }
  const size_t planes_bytes = (size_t)nplane * 4;
  if (!reserve(c, c->t2out, std::max<uint64_t>(nbytes, 16)) ||
      !reserve(c, c->recon, planes_bytes * 2 + (size_t)npxb + 256))
    return JP2G_DECODE_FAILED;
  int32_t* planes = dptr<int32_t>(c->recon);
  int32_t* tmp = planes + nplane;
  uint8_t* dpx = reinterpret_cast<uint8_t*>(tmp + nplane);
  std::vector<IdwtJob> jobs;
  std::vector<uint32_t> first(maxl + 2, 0), rows(maxl + 2, 0), tiles(maxl + 2, 0);
  for (int l = 1; l <= maxl; ++l) {
    first[l] = (uint32_t)jobs.size();
    for (size_t i : ids) {
      const DecodePage& p = pg[i];
      if (p.L.levels < l) continue;
      const uint32_t rw = (uint32_t)p.L.ladder[l].first, rh = (uint32_t)p.L.ladder[l].second;
      for (int comp = 0; comp < p.L.ncomp; ++comp) {
        IdwtJob j{};
        j.plane = planes + p.plane_base + (uint64_t)comp * p.npx;
        j.tmp = tmp + p.plane_base + (uint64_t)comp * p.npx;
        j.stride = p.L.width;
        j.rw = rw;
        j.rh = rh;
        j.reversible = p.L.reversible ? 1u : 0u;
        j.row_base = rows[l];
        j.tile_base = tiles[l];
        rows[l] += rh;
        tiles[l] += ((rw + 31) / 32) * ((rh + kIdwtTileRows - 1) / kIdwtTileRows);
        jobs.push_back(j);
      }
    }
  }
  first[maxl + 1] = (uint32_t)jobs.size();
  std::vector<PixJob> pix;
  uint64_t total_px = 0;
  for (size_t i : ids) {
    const DecodePage& p = pg[i];
    PixJob j{};
    j.planes = planes + p.plane_base;
    j.px = dpx + p.px_base;
    j.npx = p.npx;
    j.pix_base = total_px;
    j.ncomp = (uint32_t)p.L.ncomp;
    j.mct = p.L.mct ? 1u : 0u;
    j.reversible = p.L.reversible ? 1u : 0u;
    total_px += p.npx;
    pix.push_back(j);
  }
  const size_t blk_bytes = (blk.size() * sizeof(DecBlock) + 255) & ~size_t(255);
  const size_t job_bytes = (jobs.size() * sizeof(IdwtJob) + 255) & ~size_t(255);
  if (!reserve(c, c->reconblk, blk_bytes + job_bytes + pix.size() * sizeof(PixJob) + 256) ||
      !reserve_host(c, c->hpx, std::max<uint64_t>(nbytes, 16)))
    return JP2G_DECODE_FAILED;
  uint8_t* meta = static_cast<uint8_t*>(c->reconblk.p);
  DecBlock* dblk = reinterpret_cast<DecBlock*>(meta);
  IdwtJob* djobs = reinterpret_cast<IdwtJob*>(meta + blk_bytes);
  PixJob* dpix = reinterpret_cast<PixJob*>(meta + blk_bytes + job_bytes);
  parallel_for(ids.size(), ids.size() >= 8 ? host_threads(c) : 1,
               [&](size_t k) { std::memcpy(static_cast<uint8_t*>(c->hpx.p) + pg[ids[k]].data_base, bytes[ids[k]], lens[ids[k]]); });
  if (!cuda_ok(c, cudaMemcpyAsync(c->t2out.p, c->hpx.p, nbytes, cudaMemcpyHostToDevice, c->stream), "H2D files") ||
      (!blk.empty() && !cuda_ok(c, cudaMemcpyAsync(dblk, blk.data(), blk.size() * sizeof(DecBlock),
                                                   cudaMemcpyHostToDevice, c->stream), "H2D code-blocks")) ||
      (!jobs.empty() && !cuda_ok(c, cudaMemcpyAsync(djobs, jobs.data(), jobs.size() * sizeof(IdwtJob),
                                                    cudaMemcpyHostToDevice, c->stream), "H2D jobs")) ||
      !cuda_ok(c, cudaMemcpyAsync(dpix, pix.data(), pix.size() * sizeof(PixJob), cudaMemcpyHostToDevice, c->stream),
               "H2D pages") ||
      !cuda_ok(c, cudaMemsetAsync(planes, 0, planes_bytes, c->stream), "memset planes"))
    return JP2G_DECODE_FAILED;
  // two decoders per warp once the blocks fill the warps the SMs hold at
  // once (16 per SM) four times over: more chains in flight for batches
  // (64 sRGB 2550x3300 files: 290 -> 251 ms end to end); one otherwise, so
  // a file's heaviest chains run alone (one sRGB file: 10.0 against 13.4 ms)
  const int per_warp = blk.size() > (size_t)c->num_sms * 64u ? 2 : 1;
  launch_t1_decode(dblk, (uint32_t)blk.size(), dptr<uint8_t>(c->t2out), planes, per_warp, c->stream);
  for (int l = 1; l <= maxl; ++l) launch_idwt_level(djobs + first[l], first[l + 1] - first[l], rows[l], tiles[l], c->stream);
  launch_dec_pixels(dpix, (uint32_t)pix.size(), total_px, c->stream);
  if (!cuda_ok(c, cudaGetLastError(), "decode kernels")) return JP2G_DECODE_FAILED;
  if (ids.size() >= 8) {
    // many files: one read-back into pinned memory, then the host threads
    // copy each file's samples into its own buffer
    if (!reserve_host(c, c->hout, std::max<uint64_t>(npxb, 16)) ||
        !cuda_ok(c, cudaMemcpyAsync(c->hout.p, dpx, npxb, cudaMemcpyDeviceToHost, c->stream), "D2H samples") ||
        !cuda_ok(c, cudaStreamSynchronize(c->stream), "decode"))
      return JP2G_DECODE_FAILED;
    std::atomic<bool> oom{false};
    parallel_for(ids.size(), host_threads(c), [&](size_t k) {
      const DecodePage& p = pg[ids[k]];
      const size_t len = (size_t)p.npx * p.L.ncomp;
      uint8_t* o = static_cast<uint8_t*>(std::malloc(std::max<size_t>(len, 1)));
      if (!o) {
        oom = true;
        return;
      }
      std::memcpy(o, static_cast<const uint8_t*>(c->hout.p) + p.px_base, len);
      outs[ids[k]] = o;
      out_lens[ids[k]] = len;
    });
    if (!oom) return JP2G_OK;
    for (size_t i : ids) {
      std::free(outs[i]);
      outs[i] = nullptr;
      out_lens[i] = 0;
    }
    return set_err(c, JP2G_DECODE_FAILED, "out of host memory");
  }
  // a few files: each file's samples go straight into its own buffer
  // (pageable copies run near the pinned rate over this GPU's host link)
  auto drop = [&]() {  // a failed round hands out no buffer
    for (size_t i : ids) {
      std::free(outs[i]);
      outs[i] = nullptr;
      out_lens[i] = 0;
    }
    return JP2G_DECODE_FAILED;
  };
  for (size_t k = 0; k < ids.size(); ++k) {
    const DecodePage& p = pg[ids[k]];
    const size_t len = (size_t)p.npx * p.L.ncomp;
    uint8_t* o = static_cast<uint8_t*>(std::malloc(std::max<size_t>(len, 1)));
    if (!o) {
      set_msg(c, "out of host memory");
      return drop();
    }
    outs[ids[k]] = o;
    out_lens[ids[k]] = len;
    if (!cuda_ok(c, cudaMemcpyAsync(o, dpx + p.px_base, len, cudaMemcpyDeviceToHost, c->stream), "D2H samples"))
      return drop();
  }
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "decode")) return drop();
  return JP2G_OK;
}

// Splits `ids` into rounds that fit, halving a round whose pools could not
// grow within the budget.
int decode_rounds(jp2g_ctx* c, std::vector<DecodePage>& pg, std::vector<size_t> ids, const uint8_t* const* bytes,
                  const size_t* lens, uint8_t** outs, size_t* out_lens) {
  const uint64_t cap = c->budget ? c->budget : (uint64_t)24 << 30;
  size_t k = 0;
  while (k < ids.size()) {
    std::vector<size_t> round;
    uint64_t used = 0;
    while (k < ids.size()) {
      const uint64_t b = decode_device_bytes(pg[ids[k]], lens[ids[k]]);
      if (!round.empty() && used + b > cap) break;
      used += b;
      round.push_back(ids[k++]);
    }
    c->budget_hit = false;
    int rc = decode_round(c, pg, round, bytes, lens, outs, out_lens);
    if (rc != JP2G_OK && c->budget_hit && round.size() > 1) {
      release_pools(c);
      const size_t half = round.size() / 2;
      std::vector<size_t> a(round.begin(), round.begin() + half), b(round.begin() + half, round.end());
      rc = decode_rounds(c, pg, a, bytes, lens, outs, out_lens);
      if (rc == JP2G_OK) rc = decode_rounds(c, pg, b, bytes, lens, outs, out_lens);
    }
    if (rc != JP2G_OK) {
      const std::string m = get_msg(c);
      for (size_t i : round)
        if (!outs[i] && pg[i].status == JP2G_OK) {
          pg[i].status = rc;
          pg[i].msg = m;
        }
    }
  }
  return JP2G_OK;
}

}  // namespace

int jp2g_decode_batch(jp2g_ctx* c, const uint8_t* const* bytes, const size_t* lens, uint32_t n, int flags,
                      uint8_t** outs, size_t* out_lens, uint32_t* ws, uint32_t* hs, uint32_t* ncomps, int* status) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (n == 0) return JP2G_OK;
  if (!bytes || !lens || !outs || !out_lens || !ws || !hs || !ncomps || !status)
    return set_err(c, JP2G_INVALID_INPUT, "array pointer is null");
  cudaSetDevice(c->device);
  std::vector<DecodePage> pg(n);
  for (uint32_t i = 0; i < n; ++i) {
    outs[i] = nullptr;
    out_lens[i] = 0;
    ws[i] = hs[i] = ncomps[i] = 0;
  }
  parallel_for(n, n >= 4 ? host_threads(c) : 1, [&](size_t i) {
    DecodePage& p = pg[i];
    Failure f{};
    if (!bytes[i] && lens[i]) {
      p.status = JP2G_INVALID_INPUT;
      p.msg = "input pointer is null";
    } else if (!parse_codestream(bytes[i], lens[i], flags, &p.L, &f)) {
      p.status = f.code;
      p.msg = f.msg;
    } else {
      p.npx = (uint64_t)p.L.width * p.L.height;
    }
  });
  std::vector<size_t> ok;
  for (uint32_t i = 0; i < n; ++i)
    if (pg[i].status == JP2G_OK) ok.push_back(i);
  decode_rounds(c, pg, ok, bytes, lens, outs, out_lens);
  int first = JP2G_OK;
  for (uint32_t i = 0; i < n; ++i) {
    status[i] = pg[i].status;
    if (pg[i].status == JP2G_OK) {
      ws[i] = pg[i].L.width;
      hs[i] = pg[i].L.height;
      ncomps[i] = (uint32_t)pg[i].L.ncomp;
    } else if (first == JP2G_OK) {
      first = pg[i].status;
      set_msg(c, pg[i].msg);
    }
  }
  return first;
}

int jp2g_decode(jp2g_ctx* c, const uint8_t* bytes, size_t n, int flags, uint8_t** px, size_t* px_len, uint32_t* w,
                uint32_t* h, uint32_t* ncomp) {
  if (!c) return JP2G_INVALID_INPUT;
  if (!px || !px_len || !w || !h || !ncomp) return set_err(c, JP2G_INVALID_INPUT, "output pointer is null");
  int st = JP2G_OK;
  return jp2g_decode_batch(c, &bytes, &n, 1, flags, px, px_len, w, h, ncomp, &st);
}

static void job_from_request(const jp2g_request& r, PageJob* j) {
  (r.on_device ? j->dev_px : j->host_px) = r.px;
  j->w = r.width;
  j->h = r.height;
  j->ncomp = r.ncomp;
  j->interleaved = r.on_device ? 1 : r.interleaved;
  j->quality = r.quality;
  j->format = r.format;
}

int jp2g_encode_batch(jp2g_ctx* c, const jp2g_request* reqs, uint32_t n, uint8_t** outs,
                      size_t* out_lens, int* status) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (n > 0 && (!reqs || !outs || !out_lens || !status))
    return set_err(c, JP2G_INVALID_INPUT, "null request or result array");
  cudaSetDevice(c->device);
  std::vector<PageJob> jobs(n);
  std::vector<PageJob*> ptrs(n);
  for (uint32_t i = 0; i < n; ++i) {
    job_from_request(reqs[i], &jobs[i]);
    ptrs[i] = &jobs[i];
    outs[i] = nullptr;
    out_lens[i] = 0;
  }
  int rc = JP2G_OK;
  uint64_t counters[8] = {};
  std::memset(c->stage_ms, 0, sizeof c->stage_ms);
  const auto t0 = std::chrono::steady_clock::now();
  // Host pixels of wave k+1 are staged (on a helper thread, into the other
  // pinned buffer) while wave k is on the device.
  auto waves = form_waves(c, ptrs);
  HostBuf* bufs[2] = {&c->hpx, &c->hpx2};
  DevBuf* devs[2] = {&c->px, &c->px2};
  // Without a budget, each wave's pixels go to the device on a copy stream
  // as they are gathered (page by page, while the host threads gather the
  // rest), into one of two device pixel buffers; from the second wave on,
  // on a helper thread while the previous wave computes. The wave's DWT
  // waits on the copy's event.
  const bool overlap = c->budget == 0;
  // room for wave k's pixels (an upper bound of what it stages); main thread
  auto room_for = [&](size_t k) {
    size_t bound = 0;
    for (PageJob* j : waves[k])
      if (j->host_px) bound += ((size_t)j->w * j->h * j->ncomp + 255) & ~size_t(255);
    return bound == 0 || reserve(c, *devs[k & 1], bound);
  };
  // gathers wave k into bufs[k & 1] and copies it into devs[k & 1] on the
  // copy stream; *sent tells whether every copy was issued
  auto upload = [&](size_t k, bool* sent) {
    HostBuf& hb = *bufs[k & 1];
    DevBuf& dev = *devs[k & 1];
    std::atomic<bool> ok{true};
    const size_t total = stage_pixels(c, waves[k].data(), waves[k].size(), hb, [&](const PageJob* j) {
      const size_t bytes = (size_t)j->w * j->h * j->ncomp;
      if (j->px_off + bytes > dev.cap ||
          cudaMemcpyAsync(dptr<uint8_t>(dev) + j->px_off, static_cast<const uint8_t*>(hb.p) + j->px_off, bytes,
                          cudaMemcpyHostToDevice, c->copy_stream) != cudaSuccess)
        ok = false;
    });
    if (total == kStageFailed) return total;
    for (PageJob* j : waves[k]) {  // pages copied straight from the caller's memory
      if (!j->laid_out || j->staged) continue;
      const size_t bytes = (size_t)j->w * j->h * j->ncomp;
      if (j->px_off + bytes > dev.cap ||
          cudaMemcpyAsync(dptr<uint8_t>(dev) + j->px_off, j->host_px, bytes, cudaMemcpyHostToDevice,
                          c->copy_stream) != cudaSuccess)
        ok = false;
    }
    *sent = ok && cudaEventRecord(c->ev_up[k & 1], c->copy_stream) == cudaSuccess;
    return total;
  };
  bool uploaded = false;  // wave w's pixels are on their way (ev_up)
  size_t staged = 0;
  if (!waves.empty()) {
    if (overlap && room_for(0)) staged = upload(0, &uploaded);
    else staged = stage_pixels(c, waves[0].data(), waves[0].size(), *bufs[0]);
  }
  for (size_t w = 0; w < waves.size(); ++w) {
    auto& wave = waves[w];
    if (staged == kStageFailed) {
      rc = JP2G_ENCODE_FAILED;
      break;
    }
    size_t next_staged = 0;
    bool next_uploaded = false;
    const bool next_room = overlap && w + 1 < waves.size() && room_for(w + 1);
    std::thread stager;
    if (w + 1 < waves.size()) {
      stager = std::thread([&, w, next_room] {
        cudaSetDevice(c->device);
        if (next_room) next_staged = upload(w + 1, &next_uploaded);
        else next_staged = stage_pixels(c, waves[w + 1].data(), waves[w + 1].size(), *bufs[(w + 1) & 1]);
      });
    }
    Prestaged pre{bufs[w & 1], staged};
    pre.dev = devs[w & 1];
    pre.uploaded = uploaded ? c->ev_up[w & 1] : nullptr;
    rc = run_wave_within_budget(c, wave.data(), wave.size(), &pre);
    if (stager.joinable()) stager.join();
    staged = next_staged;
    uploaded = next_uploaded;
    for (int k = 0; k < 8; ++k) counters[k] += c->counters[k];
    if (rc != JP2G_OK) break;
    add_wave_stage_times(c);
  }
  cudaStreamSynchronize(c->copy_stream);  // an upload for a wave that did not run
  std::memcpy(c->counters, counters, sizeof counters);
  if (c->timing) {
    // batch: device stages summed over waves; host = wall time not covered
    // by them (staging, waiting for the last wave's Tier-2); total = wall.
    const float wall = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    c->stage_ms[kHost] = std::max(0.f, wall - c->stage_ms[kTotal]);
    c->stage_ms[kTotal] = wall;
  }
  if (rc != JP2G_OK) {
    for (uint32_t i = 0; i < n; ++i) status[i] = rc;
    return rc;
  }
  int first_fail = JP2G_OK;
  for (uint32_t i = 0; i < n; ++i) {
    status[i] = jobs[i].status;
    if (jobs[i].status == JP2G_OK && jobs[i].cs) {
      outs[i] = jobs[i].cs;
      out_lens[i] = jobs[i].cs_len;
      jobs[i].cs = nullptr;
      jobs[i].cs_len = 0;
    } else if (jobs[i].status == JP2G_OK) {
      status[i] = JP2G_ENCODE_FAILED;
    } else if (first_fail == JP2G_OK) {
      first_fail = jobs[i].status;
      set_msg(c, "page " + std::to_string(i) + ": " + jobs[i].err);
    }
  }
  return first_fail;
}

namespace {

// Worker: forms a wave from the queue (FIFO, up to the wave limits), runs
// its device phase and hands it to the finisher.
// Takes the next wave off the queue: requests in arrival order while they
// share a code-block size and fit the wave limits. Called with qmu held and
// the queue not empty.
std::vector<std::shared_ptr<Ticket>> take_wave(jp2g_ctx* c) {
  std::vector<std::shared_ptr<Ticket>> wave;
  uint64_t blocks = 0;
  int cbw = 0;
  while (!c->pending.empty() && wave.size() < kMaxWavePages) {
    const PagePlan& p = c->pending.front()->job.plan;
    if (!wave.empty() && (p.cbw != cbw || blocks + p.nblocks > wave_block_limit(c, p.cbw))) break;
    cbw = p.cbw;
    blocks += p.nblocks;
    wave.push_back(c->pending.front());
    c->pending.pop_front();
  }
  return wave;
}

// Runs one wave's pages on the device and hands the wave to the finisher.
void run_served_wave(jp2g_ctx* c, std::vector<std::shared_ptr<Ticket>>& wave, const Prestaged* pre, int buf) {
  std::vector<PageJob*> jobs;
  for (auto& t : wave) jobs.push_back(&t->job);
  int rc;
  std::string err;
  {
    std::lock_guard<std::mutex> lk(c->mu);
    rc = run_wave_within_budget(c, jobs.data(), jobs.size(), pre);
    if (rc != JP2G_OK) err = get_msg(c);
  }
  if (rc != JP2G_OK)
    for (PageJob* j : jobs) {
      j->status = rc;
      j->err = err;
    }
  {
    std::lock_guard<std::mutex> lk(c->qmu);
    c->finishing.push_back(std::move(wave));
    --c->inflight;
    if (buf >= 0) c->serve_buf_busy[buf] = false;
  }
  c->fcv.notify_one();
  if (buf >= 0) c->qcv.notify_all();  // the stager may use the buffer again
}

// Worker under a memory budget: forms each wave itself and runs it (its
// pixels staged inside the wave, which may be split to fit the budget).
void worker_loop(jp2g_ctx* c) {
  cudaSetDevice(c->device);
  for (;;) {
    std::vector<std::shared_ptr<Ticket>> wave;
    {
      std::unique_lock<std::mutex> lk(c->qmu);
      c->qcv.wait(lk, [&] { return c->stop || !c->pending.empty(); });
      if (c->stop && c->pending.empty()) return;
      wave = take_wave(c);
      ++c->inflight;
    }
    run_served_wave(c, wave, nullptr, -1);
  }
}

// Stager (no budget): forms the next wave as soon as the worker has taken
// the previous one and a pixel buffer pair is free, gathers its pixels into
// the pair's pinned buffer and copies each page to the pair's device buffer
// on serve_stream as soon as it is gathered.
void stager_loop(jp2g_ctx* c) {
  cudaSetDevice(c->device);
  for (;;) {
    jp2g_ctx::StagedWave sw;
    {
      std::unique_lock<std::mutex> lk(c->qmu);
      c->qcv.wait(lk, [&] {
        return (c->stop && c->pending.empty()) ||
               (!c->pending.empty() && c->staged.empty() && !c->serve_buf_busy[c->serve_waves & 1]);
      });
      if (c->pending.empty()) break;  // stopping, nothing queued
      sw.buf = (int)(c->serve_waves++ & 1);
      c->serve_buf_busy[sw.buf] = true;
      sw.tickets = take_wave(c);
      ++c->inflight;
    }
    std::vector<PageJob*> jobs;
    size_t bound = 0;
    for (auto& t : sw.tickets) {
      jobs.push_back(&t->job);
      if (t->job.host_px) bound += ((size_t)t->job.w * t->job.h * t->job.ncomp + 255) & ~size_t(255);
    }
    HostBuf& hb = c->serve_hpx[sw.buf];
    DevBuf& dev = c->serve_px[sw.buf];
    std::atomic<bool> ok{true};
    auto send = [&](const PageJob* j, const uint8_t* from) {
      const size_t bytes = (size_t)j->w * j->h * j->ncomp;
      if (j->px_off + bytes > dev.cap || cudaMemcpyAsync(dptr<uint8_t>(dev) + j->px_off, from, bytes,
                                                         cudaMemcpyHostToDevice, c->serve_stream) != cudaSuccess)
        ok = false;
    };
    if (bound > 0 && reserve(c, dev, bound)) {
      sw.total = stage_pixels(c, jobs.data(), jobs.size(), hb, [&](const PageJob* j) {
        send(j, static_cast<const uint8_t*>(hb.p) + j->px_off);
      });
      if (sw.total != kStageFailed) {
        for (PageJob* j : jobs)  // pages copied straight from the caller's memory
          if (j->laid_out && !j->staged) send(j, j->host_px);
        sw.uploaded = ok && cudaEventRecord(c->serve_ev[sw.buf], c->serve_stream) == cudaSuccess;
      }
    } else {
      // nothing from host memory, or no room: the worker copies the pixels
      sw.total = stage_pixels(c, jobs.data(), jobs.size(), hb);
    }
    {
      std::lock_guard<std::mutex> lk(c->qmu);
      c->staged.push_back(std::move(sw));
    }
    c->rcv.notify_one();
  }
  c->rcv.notify_all();
  c->fcv.notify_all();
}

// Worker with a stager: runs the staged waves in order.
void runner_loop(jp2g_ctx* c) {
  cudaSetDevice(c->device);
  for (;;) {
    jp2g_ctx::StagedWave sw;
    {
      std::unique_lock<std::mutex> lk(c->qmu);
      c->rcv.wait(lk, [&] { return !c->staged.empty() || (c->stop && c->pending.empty() && c->inflight == 0); });
      if (c->staged.empty()) return;
      sw = std::move(c->staged.front());
      c->staged.pop_front();
    }
    c->qcv.notify_all();  // the stager may form the next wave
    if (sw.total == kStageFailed) {
      std::lock_guard<std::mutex> lk(c->qmu);
      for (auto& t : sw.tickets) {
        t->job.status = kEncodeFailed;
        t->job.err = "staging the wave's pixels failed";
      }
      c->finishing.push_back(std::move(sw.tickets));
      --c->inflight;
      c->serve_buf_busy[sw.buf] = false;
      c->fcv.notify_one();
      c->qcv.notify_all();
      continue;
    }
    Prestaged pre{&c->serve_hpx[sw.buf], sw.total};
    pre.dev = &c->serve_px[sw.buf];
    pre.uploaded = sw.uploaded ? c->serve_ev[sw.buf] : nullptr;
    run_served_wave(c, sw.tickets, &pre, sw.buf);
  }
}

// Finisher: marks the tickets of each finished wave done (a cancelled
// ticket's result is dropped) while the worker already runs the next wave.
// It exits once stopping, with nothing queued, no wave on the device
// (inflight) and nothing left to finish.
void finisher_loop(jp2g_ctx* c) {
  for (;;) {
    std::vector<std::shared_ptr<Ticket>> wave;
    {
      std::unique_lock<std::mutex> lk(c->qmu);
      c->fcv.wait(lk, [&] {
        return !c->finishing.empty() || (c->stop && c->pending.empty() && c->inflight == 0);
      });
      if (c->finishing.empty()) return;
      wave = std::move(c->finishing.front());
      c->finishing.pop_front();
    }
    {
      std::lock_guard<std::mutex> lk(c->qmu);
      for (auto& t : wave) {
        t->done = true;
        if (t->cancelled) {
          t->job.status = kEncodeFailed;
          t->job.err = "request cancelled";
          t->job.drop_output();
        }
      }
    }
    c->dcv.notify_all();
  }
}

}  // namespace

int jp2g_submit(jp2g_ctx* c, const jp2g_request* req, uint64_t* ticket) {
  if (!c) return JP2G_INVALID_INPUT;
  if (!req || !ticket) return set_err(c, JP2G_INVALID_INPUT, "null request or ticket pointer");
  auto t = std::make_shared<Ticket>();
  job_from_request(*req, &t->job);
  Failure f{};
  if (!build_plan(t->job.w, t->job.h, (int)t->job.ncomp, t->job.quality, t->job.format, &t->job.plan, &f) ||
      !req->px)
    return set_err(c, req->px ? f.code : JP2G_INVALID_INPUT, req->px ? f.msg : "pixel pointer is null");
  {
    std::lock_guard<std::mutex> lk(c->qmu);
    if (!c->worker.joinable()) {
      if (c->budget == 0) {
        c->stager = std::thread(stager_loop, c);
        c->worker = std::thread(runner_loop, c);
      } else {
        c->worker = std::thread(worker_loop, c);
      }
      c->finisher = std::thread(finisher_loop, c);
    }
    t->id = c->next_ticket++;
    c->tickets[t->id] = t;
    c->pending.push_back(t);
    *ticket = t->id;
  }
  c->qcv.notify_one();
  return JP2G_OK;
}

int jp2g_poll(jp2g_ctx* c, uint64_t ticket, uint8_t** out, size_t* out_len, int timeout_ms) {
  if (!c) return JP2G_INVALID_INPUT;
  if (!out || !out_len) return set_err(c, JP2G_INVALID_INPUT, "output pointer is null");
  std::shared_ptr<Ticket> t;
  {
    std::unique_lock<std::mutex> lk(c->qmu);
    auto it = c->tickets.find(ticket);
    if (it == c->tickets.end()) {
      lk.unlock();
      return set_err(c, JP2G_INVALID_INPUT, "unknown ticket " + std::to_string(ticket));
    }
    t = it->second;
    auto ready = [&] { return t->done; };
    if (timeout_ms < 0) c->dcv.wait(lk, ready);
    else if (!c->dcv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return JP2G_PENDING;
    c->tickets.erase(ticket);
  }
  // the result is the ticket's own; the engine mutex (held by the worker
  // for the whole device phase of a wave) is not needed
  if (t->job.status != JP2G_OK) return set_err(c, t->job.status, t->job.err);
  return finish_output(c, JP2G_OK, t->job, out, out_len);
}

int jp2g_cancel(jp2g_ctx* c, uint64_t ticket) {
  if (!c) return JP2G_INVALID_INPUT;
  std::shared_ptr<Ticket> t;
  {
    std::lock_guard<std::mutex> lk(c->qmu);
    auto it = c->tickets.find(ticket);
    if (it == c->tickets.end()) return set_err(c, JP2G_INVALID_INPUT, "unknown ticket " + std::to_string(ticket));
    t = it->second;
    if (t->done) {  // finished already: the result is dropped with the ticket
      c->tickets.erase(it);
      return JP2G_OK;
    }
    t->cancelled = true;
    auto q = std::find(c->pending.begin(), c->pending.end(), t);
    if (q == c->pending.end()) return JP2G_PENDING;  // on the device or in Tier-2: the finisher drops the result
    // not yet admitted to a wave: it never reaches the device
    c->pending.erase(q);
    c->tickets.erase(it);
    t->job.status = kEncodeFailed;
    t->job.err = "request cancelled";
    t->done = true;
  }
  c->dcv.notify_all();
  return JP2G_OK;
}

int jp2g_set_option(jp2g_ctx* c, int option, int64_t value) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  switch (option) {
    case JP2G_OPT_WAVE_BLOCKS:
      if (value < 1) return set_err(c, JP2G_INVALID_INPUT, "wave_blocks must be at least 1");
      break;
    case JP2G_OPT_MQ_BLOCKS_PER_WARP:
      if (value < 0 || value > 32) return set_err(c, JP2G_INVALID_INPUT, "mq_blocks_per_warp must be 0..32");
      break;
    case JP2G_OPT_HOST_THREADS:
      if (value < 0 || value > 1024) return set_err(c, JP2G_INVALID_INPUT, "host_threads must be 0..1024");
      break;
    case JP2G_OPT_MQ_WARPS_PER_SM:
      if (value < -1 || value > 64) return set_err(c, JP2G_INVALID_INPUT, "mq_warps_per_sm must be -1..64");
      break;
    case JP2G_OPT_MQ_PIPES_PER_SM:
      if (value < -1 || value > 32) return set_err(c, JP2G_INVALID_INPUT, "mq_pipes_per_sm must be -1..32");
      break;
    case JP2G_OPT_MQ_HEAVY:
      if (value < 0 || value > 0xffffffffll) return set_err(c, JP2G_INVALID_INPUT, "mq_heavy must be >= 0");
      break;
    case JP2G_OPT_MQ_CHAINS_PER_PAIR:
      if (value < 0 || value > 4 || value == 3)
        return set_err(c, JP2G_INVALID_INPUT, "mq_chains_per_pair must be 0, 1, 2 or 4");
      break;
    default:
      return set_err(c, JP2G_INVALID_INPUT, "unknown option " + std::to_string(option));
  }
  c->opt[option] = value;
  return JP2G_OK;
}

int jp2g_get_option(jp2g_ctx* c, int option, int64_t* value) {
  if (!c || !value || option < 0 || option >= JP2G_NUM_OPTS) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  *value = c->opt[option];
  return JP2G_OK;
}

// Two stages over the scheduling knobs: the MQ schedule at the context's
// wave size, then the wave size under the chosen schedule. A candidate is
// timed as the minimum wall time of `repeats` encodes of the sample after
// one untimed encode, and must reproduce the first encode's codestreams.
int jp2g_autotune(jp2g_ctx* c, const jp2g_request* reqs, uint32_t n, int repeats, int64_t* best,
                  double* best_ms) {
  if (!c) return JP2G_INVALID_INPUT;
  if (n == 0 || !reqs || repeats < 1 || repeats > 100)
    return set_err(c, JP2G_INVALID_INPUT, "autotune needs at least one sample page and 1..100 repeats");
  int64_t saved[JP2G_NUM_OPTS];
  for (int i = 0; i < JP2G_NUM_OPTS; ++i) jp2g_get_option(c, i, &saved[i]);
  auto restore = [&] {
    for (int i = 0; i < JP2G_NUM_OPTS; ++i) jp2g_set_option(c, i, saved[i]);
  };
  std::vector<uint8_t*> outs(n);
  std::vector<size_t> lens(n);
  std::vector<int> st(n), ref_st(n);
  std::vector<std::string> ref(n);
  // One encode of the sample under `o`: its wall time in ms, -1 if the call
  // failed, -2 if a codestream differs from the reference encode.
  auto encode_once = [&](const int64_t* o, bool record) -> double {
    for (int i = 0; i < JP2G_NUM_OPTS; ++i)
      if (jp2g_set_option(c, i, o[i]) != JP2G_OK) return -1.0;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = jp2g_encode_batch(c, reqs, n, outs.data(), lens.data(), st.data());
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    bool same = true;
    for (uint32_t i = 0; i < n; ++i) {
      std::string bytes = outs[i] ? std::string(reinterpret_cast<const char*>(outs[i]), lens[i]) : std::string();
      if (record) {
        ref[i] = std::move(bytes);
        ref_st[i] = st[i];
      } else if (st[i] != ref_st[i] || bytes != ref[i]) {
        same = false;
      }
      jp2g_free(outs[i]);
      outs[i] = nullptr;
    }
    if (rc != JP2G_OK) return -1.0;
    return same ? ms : -2.0;
  };
  auto time_candidate = [&](const int64_t* o) -> double {
    double t = encode_once(o, false);  // untimed: settles buffers for this setting
    if (t < 0) return t;
    double m = 1e300;
    for (int r = 0; r < repeats; ++r) {
      t = encode_once(o, false);
      if (t < 0) return t;
      m = std::min(m, t);
    }
    return m;
  };
  auto fail = [&](const int64_t* o, double why) {
    restore();
    if (why == -2.0)
      return set_err(c, JP2G_ENCODE_FAILED,
                     "autotune: a scheduling setting changed the codestream (mq_blocks_per_warp=" +
                         std::to_string(o[JP2G_OPT_MQ_BLOCKS_PER_WARP]) + ", mq_warps_per_sm=" +
                         std::to_string(o[JP2G_OPT_MQ_WARPS_PER_SM]) + ", mq_pipes_per_sm=" +
                         std::to_string(o[JP2G_OPT_MQ_PIPES_PER_SM]) + ", mq_chains_per_pair=" +
                         std::to_string(o[JP2G_OPT_MQ_CHAINS_PER_PAIR]) + ", wave_blocks=" +
                         std::to_string(o[JP2G_OPT_WAVE_BLOCKS]) + ")");
    return set_err(c, JP2G_ENCODE_FAILED, "autotune: the sample failed to encode: " + get_msg(c));
  };
  if (encode_once(saved, true) < 0) return fail(saved, -1.0);

  // stage 1: MQ schedule (automatic; producer/consumer pipelines; single-warp
  // pulling; blocks packed per warp)
  struct Mq { int64_t bpw, wps, pipes, chains; };
  const Mq mq[] = {{0, 0, 0, 0},   {1, 0, 4, 1},   {1, 0, 8, 1},   {1, 0, 16, 1}, {1, 0, 4, 2},
                   {1, 0, 8, 2},   {1, 0, 16, 2},  {1, 0, 4, 4},   {1, 0, 8, 4},  {1, 8, -1, 0},
                   {1, 12, -1, 0}, {1, 16, -1, 0}, {2, 0, 0, 0},   {4, 0, 0, 0},  {8, 0, 0, 0},
                   {16, 0, 0, 0},  {32, 0, 0, 0}};
  int64_t cur[JP2G_NUM_OPTS], win[JP2G_NUM_OPTS];
  std::memcpy(cur, saved, sizeof cur);
  cur[JP2G_OPT_MQ_HEAVY] = 0;
  double win_ms = 1e300;
  for (const Mq& m : mq) {
    cur[JP2G_OPT_MQ_BLOCKS_PER_WARP] = m.bpw;
    cur[JP2G_OPT_MQ_WARPS_PER_SM] = m.wps;
    cur[JP2G_OPT_MQ_PIPES_PER_SM] = m.pipes;
    cur[JP2G_OPT_MQ_CHAINS_PER_PAIR] = m.chains;
    const double t = time_candidate(cur);
    if (t < 0) return fail(cur, t);
    if (t < win_ms) {
      win_ms = t;
      std::memcpy(win, cur, sizeof win);
    }
  }
  // stage 2: device wave size under the chosen schedule
  std::memcpy(cur, win, sizeof cur);
  for (int64_t wb : {20000ll, 40000ll, 80000ll, 160000ll, 240000ll}) {
    if (wb == win[JP2G_OPT_WAVE_BLOCKS]) continue;
    cur[JP2G_OPT_WAVE_BLOCKS] = wb;
    const double t = time_candidate(cur);
    if (t < 0) return fail(cur, t);
    if (t < win_ms) {
      win_ms = t;
      win[JP2G_OPT_WAVE_BLOCKS] = wb;
    }
  }
  for (int i = 0; i < JP2G_NUM_OPTS; ++i) jp2g_set_option(c, i, win[i]);
  if (best) std::memcpy(best, win, sizeof win);
  if (best_ms) *best_ms = win_ms;
  return JP2G_OK;
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
  int k = std::min(n, (int)kNumStages + 4);
  for (int i = 0; i < k; ++i) ms[i] = c->stage_ms[i];
  return k;
}

int jp2g_counters(jp2g_ctx* c, uint64_t* out, int n) {
  if (!c || !out) return 0;
  int k = std::min(n, 8);
  for (int i = 0; i < k; ++i) out[i] = c->counters[i];
  return k;
}

static int debug_coefficients(jp2g_ctx* c, const uint8_t* px, uint32_t w, uint32_t h, uint32_t ncomp,
                              uint8_t quality, uint32_t comp, int32_t* plane, bool raw);

int jp2g_debug_coefficients(jp2g_ctx* c, const uint8_t* px, uint32_t w, uint32_t h,
                            uint32_t ncomp, uint8_t quality, uint32_t comp, int32_t* plane) {
  return debug_coefficients(c, px, w, h, ncomp, quality, comp, plane, false);
}

int jp2g_debug_coefficients_f32(jp2g_ctx* c, const uint8_t* px, uint32_t w, uint32_t h, uint32_t ncomp,
                                uint8_t quality, uint32_t comp, float* plane) {
  if (c && quality >= 100) return set_err(c, JP2G_INVALID_INPUT, "f32 coefficients exist only for lossy qualities");
  return debug_coefficients(c, px, w, h, ncomp, quality, comp, reinterpret_cast<int32_t*>(plane), true);
}

static int debug_coefficients(jp2g_ctx* c, const uint8_t* px, uint32_t w, uint32_t h, uint32_t ncomp,
                              uint8_t quality, uint32_t comp, int32_t* plane, bool raw) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!px || !plane) return set_err(c, JP2G_INVALID_INPUT, "null pointer");
  if (comp >= ncomp) return set_err(c, JP2G_INVALID_INPUT, "component index out of range");
  cudaSetDevice(c->device);
  PageJob j;
  j.host_px = px;
  j.w = w;
  j.h = h;
  j.ncomp = ncomp;
  j.quality = quality;
  WaveDebug dbg;
  dbg.stop_after_dwt = true;
  dbg.raw_coefficients = raw;
  int rc = encode_one(c, &j, &dbg);
  if (rc) return rc;
  const PagePlan& p = j.plan;
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
  PageJob j;
  j.host_px = px;
  j.w = w;
  j.h = h;
  j.ncomp = ncomp;
  j.quality = quality;
  std::vector<BlockOut> res;
  std::vector<BlockKeep> keep;
  WaveDebug dbg;
  dbg.res = &res;
  dbg.keep = &keep;
  int rc = encode_one(c, &j, &dbg);
  if (rc) return rc;
  const PagePlan& p = j.plan;
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

int jp2g_debug_assemble_device(jp2g_ctx* c, uint32_t w, uint32_t h, uint32_t ncomp, uint8_t quality, int format,
                               const uint16_t* npasses, const uint8_t* zbp, const uint32_t* seg_len,
                               const uint8_t* body, uint32_t nblocks, uint8_t** out, size_t* out_len) {
  if (!c) return JP2G_INVALID_INPUT;
  std::lock_guard<std::mutex> lk(c->mu);
  if (!out || !out_len || (nblocks > 0 && (!npasses || !zbp || !seg_len)))
    return set_err(c, JP2G_INVALID_INPUT, "null pointer");
  cudaSetDevice(c->device);
  PageJob j;
  Failure f{};
  if (!build_plan(w, h, (int)ncomp, quality, format, &j.plan, &f)) return set_err(c, f.code, f.msg);
  if (nblocks != j.plan.nblocks) return set_err(c, JP2G_INVALID_INPUT, "block count does not match the plan");
  std::vector<BlockKeep> keep(std::max<uint32_t>(nblocks, 1));
  std::vector<uint32_t> offsets((size_t)nblocks + 1, 0);
  for (uint32_t i = 0; i < nblocks; ++i) {
    BlockKeep k{};
    k.npasses = npasses[i];
    k.zbp = zbp[i];
    k.seg_len = npasses[i] ? seg_len[i] : 0;
    k.body_len = k.seg_len;
    keep[i] = k;
    offsets[i + 1] = offsets[i] + k.body_len;
  }
  const uint32_t total = offsets[nblocks];
  if (total > 0 && !body) return set_err(c, JP2G_INVALID_INPUT, "null body");
  if (!reserve(c, c->keep, keep.size() * sizeof(BlockKeep)) || !reserve(c, c->offsets, offsets.size() * 4) ||
      !reserve(c, c->body, std::max<uint32_t>(total, 1)) ||
      !cuda_ok(c, cudaMemcpyAsync(c->keep.p, keep.data(), keep.size() * sizeof(BlockKeep), cudaMemcpyHostToDevice,
                                  c->stream), "H2D keep") ||
      !cuda_ok(c, cudaMemcpyAsync(c->offsets.p, offsets.data(), offsets.size() * 4, cudaMemcpyHostToDevice, c->stream),
               "H2D offsets") ||
      (total > 0 && !cuda_ok(c, cudaMemcpyAsync(c->body.p, body, total, cudaMemcpyHostToDevice, c->stream), "H2D body")))
    return JP2G_ENCODE_FAILED;
  std::vector<PageJob*> live{&j};
  if (int rc = run_tier2(c, live, dptr<BlockKeep>(c->keep), dptr<uint32_t>(c->offsets), dptr<uint8_t>(c->body), total))
    return rc;
  if (j.status != kOk) return set_err(c, j.status, j.err);
  return finish_output(c, JP2G_OK, j, out, out_len);
}

int jp2g_debug_assemble(uint32_t w, uint32_t h, uint32_t ncomp, uint8_t quality, int format,
                        const uint16_t* npasses, const uint8_t* zbp, const uint32_t* seg_len,
                        const uint8_t* body, uint32_t nblocks, uint8_t** out, size_t* out_len) {
  if (!out || !out_len || (nblocks > 0 && (!npasses || !zbp || !seg_len))) return JP2G_INVALID_INPUT;
  PagePlan p;
  Failure f{};
  if (!build_plan(w, h, (int)ncomp, quality, format, &p, &f)) return f.code;
  if (nblocks != p.nblocks) return JP2G_INVALID_INPUT;
  std::vector<BlockKeep> keep(nblocks);
  std::vector<uint32_t> offsets((size_t)nblocks + 1, 0);
  for (uint32_t i = 0; i < nblocks; ++i) {
    BlockKeep k{};
    k.npasses = npasses[i];
    k.zbp = zbp[i];
    k.seg_len = npasses[i] ? seg_len[i] : 0;
    k.body_len = k.seg_len;
    keep[i] = k;
    offsets[i + 1] = offsets[i] + k.body_len;
  }
  if (offsets[nblocks] > 0 && !body) return JP2G_INVALID_INPUT;
  std::vector<uint8_t> cs;
  if (!assemble_codestream(p, keep.data(), body, offsets.data(), &cs, &f)) return f.code;
  *out = static_cast<uint8_t*>(std::malloc(std::max<size_t>(cs.size(), 1)));
  if (!*out) return JP2G_ENCODE_FAILED;
  std::memcpy(*out, cs.data(), cs.size());
  *out_len = cs.size();
  return JP2G_OK;
}

int jp2g_debug_plan(uint32_t w, uint32_t h, uint32_t ncomp, uint8_t quality, int* levels, int* cbw,
                    int* nquant, int* quants, uint32_t* nblocks, double* lambdas) {
  if (!levels || !cbw || !nquant || !quants || !nblocks || !lambdas) return JP2G_INVALID_INPUT;
  PagePlan p;
  Failure f{};
  if (!build_plan(w, h, (int)ncomp, quality, 0, &p, &f)) return f.code;
  *levels = p.levels;
  *cbw = p.cbw;
  *nquant = (int)p.quants.size();
  for (size_t i = 0; i < p.quants.size() && i < 32; ++i) {
    quants[4 * i + 0] = p.quants[i].res;
    quants[4 * i + 1] = p.quants[i].orient;
    quants[4 * i + 2] = p.quants[i].exponent;
    quants[4 * i + 3] = p.quants[i].mantissa;
  }
  *nblocks = p.nblocks;
  lambdas[0] = p.lambda_raw;
  lambdas[1] = p.lambda_floor;
  return JP2G_OK;
}

// Host-only: the Tier-1 tables the device uses, for checking against the
// reference's literal tables without a GPU.
void jp2g_debug_context_labels(uint8_t* zc, uint8_t* sc, uint8_t* spb) {
  jp2g::context_labels_from_logic(zc, sc, spb);
}

void jp2g_tables(uint8_t* zc, uint8_t* sc, uint8_t* spb, uint32_t* mq) {
  build_t1_tables(zc, sc, spb, mq);
}

}  // extern "C"
