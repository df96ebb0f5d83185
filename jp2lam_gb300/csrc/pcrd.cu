// PCRD rate control on the device, then compaction of the retained bytes.
//
// Replaces curves_from_tier1_layout / raw_records_for_block
// (src/encode/backend/native/rate.rs:43-180), build_hull_curve and
// prune_to_convex_hull (src/dwt/pcrd.rs:151-252), the pass-kind-aware
// distortion model (pcrd.rs:669-802), calibrate_lambda / choose_block_point
// (pcrd.rs:406-424, 1493-1514) and truncate_layout_passes
// (src/encode/backend/native/backend.rs:834-897).
//
// Kernel 1 (one thread per code-block) builds the block's rate-distortion
// curve from its pass records, prunes it to the convex hull and folds the
// largest finite positive hull slope into its (page, component) maximum.
// Kernel 2 turns that maximum into the component's lambda exactly as the
// reference calibrates it, keeps the deepest hull point whose slope is at
// least lambda, and records the retained segment length and body bytes.
// All f64 arithmetic uses explicit round-to-nearest intrinsics in the
// reference's association order.
#include <cuda_runtime.h>

#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {

namespace {

constexpr int kMaxPts = 128;  // 1 + maximum pass count handled per block
constexpr uint8_t kHullTooLong = 255;

__device__ __forceinline__ double rd_slope(uint32_t ab, double ad, uint32_t bb, double bd) {
  // pcrd.rs:539-554 (bytes never decrease along a curve).
  double db = (double)(bb - ab);
  double dd = __dsub_rn(bd, ad);
  if (db == 0.0) return dd > 0.0 ? __longlong_as_double(0x7ff0000000000000ll) : 0.0;
  return __ddiv_rn(dd, db);
}

// Cumulative byte count after pass i (t1.rs:580-607): the numbytes()
// snapshot for every pass but the last, which absorbs the termination bytes.
__device__ __forceinline__ uint32_t cum_len(const PassRec* pr, uint32_t n, uint32_t i,
                                            uint32_t total) {
  if (i + 1 < n) return pr[i].snap;
  uint32_t prev = n >= 2 ? pr[n - 2].snap : 0u;
  return total >= prev ? total : prev;
}

__global__ void pcrd_hull_kernel(PcrdArgs a) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nblocks) return;
  const BlockDesc d = a.blocks[b];
  const BlockOut o = a.res[b];
  const CompParam cp = a.comps[d.comp_key];
  const uint32_t n = o.npasses;
  if (n + 1 > (uint32_t)kMaxPts) {
    a.hull_n[b] = kHullTooLong;
    return;
  }
  if (cp.lossless || n == 0) {
    a.hull_n[b] = 0;
    return;
  }
  const BandParam bp = a.bands[d.band_param];
  const PassRec* pr = a.passes + d.pass_off;
  // class_distortion_weight (src/profile.rs:141-154)
  double cw_base = o.cls == 0 ? 2.5 : (o.cls == 1 ? 1.5 : 1.0);
  double block_w = bp.is_ll ? __dmul_rn(cw_base, 1.1) : cw_base;

  // The hull as a stack of points (bytes hb, distortion hd, pass count hp)
  // with hs[k] the slope from point k-1 to point k, computed once when
  // point k is pushed or its predecessor popped: the same operands as
  // recomputing both slopes at every comparison, so the same bits, with
  // about half the f64 divisions. The top point and its slope stay in
  // registers.
  uint32_t hb[kMaxPts];
  double hd[kMaxPts], hs[kMaxPts];
  uint16_t hp[kMaxPts];
  int hn = 1;
  hb[0] = 0; hd[0] = 0.0; hp[0] = 0; hs[0] = 0.0;
  uint32_t tb = 0;
  double td = 0.0, ts = 0.0;
  double cum_d = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    const PassRec r = pr[i];
    // estimate_pass_distortion_delta_pass_kind_aware with visibility 1.0
    int bpl = r.bitplane < 30 ? r.bitplane : 30;
    double plane = __dmul_rn((double)(1ull << bpl), bp.quant_step);
    double energy = __dmul_rn(plane, plane);
    double contrib;
    if (r.kind == 0) contrib = __dmul_rn((double)r.ns, energy);
    else if (r.kind == 1) contrib = __dmul_rn(__dmul_rn((double)r.sig_before, energy), 0.25);
    else contrib = __dmul_rn(__dmul_rn((double)r.ns, energy), 0.85);
    double raw = __dmul_rn(__dmul_rn(__dmul_rn(bp.subband_weight, bp.band_bias), block_w), contrib);
    // apply_contrast_masking_to_delta(raw, 1.0, ..): the blended weight is
    // exactly 1.0 for visibility 1.0, so the delta is raw (or 0).
    double delta = raw <= 0.0 ? 0.0 : raw;
    delta = __dmul_rn(delta, cp.comp_weight);
    cum_d = __dadd_rn(cum_d, delta);
    uint32_t cum = cum_len(pr, n, i, o.payload_len) + 2u;  // HEADER_OVERHEAD_BYTES
    // push, after popping the top while the slope does not strictly
    // decrease (the slope into the new point >= the slope into the top)
    double sn = rd_slope(tb, td, cum, cum_d);
    while (hn >= 2 && sn >= ts) {
      --hn;
      tb = hb[hn - 1];
      td = hd[hn - 1];
      ts = hs[hn - 1];
      sn = rd_slope(tb, td, cum, cum_d);
    }
    hb[hn] = cum; hd[hn] = cum_d; hp[hn] = (uint16_t)(i + 1); hs[hn] = sn; ++hn;
    tb = cum; td = cum_d; ts = sn;
  }
  // hull slopes and the component's largest finite positive slope
  double mx = 0.0;
  uint16_t* outp = a.hull_passes + d.pass_off;
  double* outs = a.hull_slope + d.pass_off;
  for (int i = 1; i < hn; ++i) {
    const double s = hs[i];
    outp[i - 1] = hp[i];
    outs[i - 1] = s;
    if (isfinite(s) && s > mx) mx = s;
  }
  a.hull_n[b] = (uint8_t)(hn - 1);
  if (mx > 0.0) atomicMax(a.comp_max_slope + d.comp_key, (unsigned long long)__double_as_longlong(mx));
}

__global__ void pcrd_select_kernel(PcrdArgs a) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nblocks) return;
  const BlockDesc d = a.blocks[b];
  const BlockOut o = a.res[b];
  const CompParam cp = a.comps[d.comp_key];
  const uint32_t n = o.npasses;
  BlockKeep k{};
  k.zbp = o.zbp;
  k.status = o.status;
  uint32_t keep = 0;
  if (a.hull_n[b] == kHullTooLong) k.status = 3;
  if (n > 0 && k.status == 0) {
    if (cp.lossless) {
      keep = n;
    } else {
      double lambda = cp.lambda_raw;
      double maxs = __longlong_as_double((long long)a.comp_max_slope[d.comp_key]);
      if (maxs > 0.0) {
        double target = __dmul_rn(maxs, 1.2);
        if (!(target >= cp.lambda_floor)) lambda = __dmul_rn(cp.lambda_raw, __ddiv_rn(target, cp.lambda_floor));
      }
      const uint16_t* hp = a.hull_passes + d.pass_off;
      const double* hs = a.hull_slope + d.pass_off;
      for (int i = 0; i < a.hull_n[b]; ++i) {
        if (hs[i] >= lambda) keep = hp[i];
        else break;
      }
    }
  }
  if (keep > n) keep = n;
  if (keep > 0) {
    const PassRec* pr = a.passes + d.pass_off;
    uint32_t seg = cum_len(pr, n, keep - 1, o.payload_len);
    k.seg_len = seg;
    k.body_len = seg < o.payload_len ? seg : o.payload_len;
  }
  k.npasses = (uint16_t)keep;
  a.keep[b] = k;
}

// ---------------------------------------------------------- compaction -----
constexpr int kScanT = 1024;

__global__ void scan_partial_kernel(const uint32_t* in, uint32_t stride, uint32_t n, uint32_t* out,
                                    uint32_t* sums) {
  __shared__ uint32_t warp_tot[32];
  const uint32_t i = blockIdx.x * kScanT + threadIdx.x;
  const uint32_t v = i < n ? in[(size_t)i * stride] : 0u;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t y = warp_tot[lane];
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += t;
    }
    warp_tot[lane] = y;
  }
  __syncthreads();
  const uint32_t excl = x - v + (wid > 0 ? warp_tot[wid - 1] : 0u);
  if (i < n) out[i] = excl;
  if (threadIdx.x == kScanT - 1) sums[blockIdx.x] = excl + v;
}

__global__ void scan_sums_kernel(uint32_t* sums, uint32_t nparts, uint32_t* out, uint32_t n) {
  // one warp: nparts is n / 1024
  const int lane = threadIdx.x;
  uint32_t run = 0;
  for (uint32_t p0 = 0; p0 < nparts; p0 += 32) {
    const uint32_t p = p0 + lane;
    const uint32_t v = p < nparts ? sums[p] : 0u;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    if (p < nparts) sums[p] = run + x - v;
    run += __shfl_sync(0xffffffffu, x, 31);
  }
  if (lane == 0) out[n] = run;
}

__global__ void scan_add_kernel(uint32_t* out, uint32_t n, const uint32_t* sums) {
  const uint32_t i = blockIdx.x * kScanT + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

__global__ void copy_bodies_kernel(const BlockDesc* blocks, const BlockKeep* keep, uint32_t n,
                                   const uint8_t* src, uint8_t* dst, const uint32_t* offsets) {
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const uint32_t off = offsets[warp];
  const uint32_t len = keep[warp].body_len;
  const uint8_t* s = src + blocks[warp].out_off;
  for (uint32_t i = lane; i < len; i += 32) dst[off + i] = s[i];
}

}  // namespace

void launch_pcrd(const PcrdArgs& a, cudaStream_t st) {
  if (a.nblocks == 0) return;
  cudaMemsetAsync(a.comp_max_slope, 0, sizeof(unsigned long long) * a.ncomp_keys, st);
  // one warp per CTA: a page's blocks spread over all SMs, whose few f64
  // units bound the hull's divisions
  const int t = 32;
  const uint32_t g = (a.nblocks + t - 1) / t;
  pcrd_hull_kernel<<<g, t, 0, st>>>(a);
  pcrd_select_kernel<<<g, t, 0, st>>>(a);
}

void launch_scan_u32(const uint32_t* in, uint32_t stride, uint32_t n, uint32_t* out,
                     uint32_t* scratch, cudaStream_t st) {
  if (n == 0) {
    cudaMemsetAsync(out, 0, sizeof(uint32_t), st);
    return;
  }
  const uint32_t parts = (n + kScanT - 1) / kScanT;
  scan_partial_kernel<<<parts, kScanT, 0, st>>>(in, stride, n, out, scratch);
  scan_sums_kernel<<<1, 32, 0, st>>>(scratch, parts, out, n);
  if (parts > 1) scan_add_kernel<<<parts, kScanT, 0, st>>>(out, n, scratch);
}

void launch_compact(const BlockDesc* blocks, const BlockKeep* keep, uint32_t nblocks,
                    const uint8_t* src, uint8_t* dst, uint32_t* offsets, uint32_t* scratch,
                    cudaStream_t st) {
  static_assert(sizeof(BlockKeep) == 12, "body_len is read as every third word");
  launch_scan_u32(reinterpret_cast<const uint32_t*>(keep) + 1, 3, nblocks, offsets, scratch, st);
  if (nblocks == 0) return;
  const uint32_t threads = 256;
  const uint32_t grid = (uint32_t)(((uint64_t)nblocks * 32 + threads - 1) / threads);
  copy_bodies_kernel<<<grid, threads, 0, st>>>(blocks, keep, nblocks, src, dst, offsets);
}

}  // namespace jp2g
