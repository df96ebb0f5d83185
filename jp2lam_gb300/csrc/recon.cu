// Decoder-side reconstruction of an encoded page on the device, for the
// quality metrics of jp2g_encode_with_psnr.
//
// Follows compute_quality_metrics (src/encode/backend/native/backend.rs:
// 305-433): each code-block's quantised coefficients are truncated to the
// last bit-plane its retained passes reach and dequantised at the midpoint
// (dequantize_truncated_coeff, backend.rs:628-639), the inverse 9/7 runs
// level by level, rows then columns (src/dwt/irrev97.rs:639-796), the
// inverse ICT and level shift give 8-bit samples (clamped), and the page's
// PSNR and mean 8x8 luma SSIM (mssim_8x8, backend.rs:911-959) come from
// them. Every f32 step is the reference's operation in its order without
// contraction (built with --fmad=false), so the reconstructed samples equal
// the oracle's; only the f64 sums run in a different order.
#include <cuda_runtime.h>

#include <vector>

#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {

namespace {

__constant__ float kRAlpha = -1.586134342059924f;
__constant__ float kRBeta = -0.052980118572961f;
__constant__ float kRGamma = 0.882911075530934f;
__constant__ float kRDelta = 0.443506852043971f;
__constant__ float kRK = 1.230174104914001f;
__constant__ float kRInvK = 1.0f / 1.230174104914001f;

// Whole-sample symmetric extension (src/dwt/irrev97.rs:523-536).
__device__ __forceinline__ int sym_at(int i, int n) {
  if (n <= 1) return 0;
  if (i >= 0 && i < n) return i;
  const int period = 2 * (n - 1);
  int k = i % period;
  if (k < 0) k += period;
  return k >= n ? period - k : k;
}

// Code-block samples -> midpoint dequantised f32 in the component's plane.
__global__ void recon_dequant_kernel(ReconArgs r) {
  const int lane = threadIdx.x & 31;
  const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= r.nblocks) return;
  const BlockDesc d = r.blocks[b];
  const ReconBlock rb = r.rblocks[b];
  const uint32_t kept = r.keep[b].npasses;
  const int last_bp = kept ? r.passes[d.pass_off + kept - 1].bitplane : -1;
  const int32_t* q = r.coef + (size_t)d.coef_slot * r.cbw * r.cbh;
  float* out = r.plane + (size_t)rb.comp * r.width * r.height;
  for (int i = lane; i < d.w * d.h; i += 32) {
    const int y = i / d.w, x = i - y * d.w;
    const int32_t v = q[y * r.cbw + x];
    float o = 0.0f;
    if (last_bp >= 0) {
      const uint32_t a = v < 0 ? 0u - (uint32_t)v : (uint32_t)v;
      const uint32_t t = (a >> last_bp) << last_bp;
      if (t != 0) o = __fmul_rn(__fmul_rn(v >= 0 ? 1.0f : -1.0f, __fadd_rn((float)t, 0.5f)), rb.step);
    }
    out[(size_t)(rb.y0 + y) * r.width + rb.x0 + x] = o;
  }
}

__device__ __forceinline__ float lifted(float x, float c, float l, float rr) {
  return __fadd_rn(x, __fmul_rn(c, __fadd_rn(l, rr)));
}

// The job holding global index g (rows or tiles) of a level's launch.
__device__ __forceinline__ const IdwtJob& job_of(const IdwtJob* jobs, uint32_t njobs, uint32_t g, bool tiles) {
  uint32_t lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if ((tiles ? jobs[mid].tile_base : jobs[mid].row_base) <= g) lo = mid;
    else hi = mid;
  }
  return jobs[lo];
}

// Inverse 1-D transform of one row (rw samples, low half first) of a job's
// plane into the same row of its tmp, interleaved: a warp per row, each
// lifting step's positions in parallel.
//  9/7 (src/dwt/irrev97.rs:639-796): scale by K / 1/K, then the four
//    lifting steps x[j] += c (x[j-1] + x[j+1]) over whole-sample symmetric
//    extension, each rounded as written.
//  5/3 (src/dwt/rev53.rs:96-129, 419-497): even samples
//    s[i] - ((d[i-1] + d[i] + 2) >> 2) with the edges clamped, then odd
//    samples d[i] + ((e[i] + e[i+1]) >> 1), or d[i] + e[i] at the right edge.
__global__ void idwt_rows_kernel(const IdwtJob* jobs, uint32_t njobs, uint32_t total_rows) {
  const int lane = threadIdx.x & 31;
  const uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (g >= total_rows) return;
  const IdwtJob& jb = job_of(jobs, njobs, g, false);
  const uint32_t y = g - jb.row_base;
  const int n = (int)jb.rw, sn = (n + 1) / 2, dn = n - sn;
  if (jb.reversible) {
    const int32_t* x = static_cast<const int32_t*>(jb.plane) + (size_t)y * jb.stride;
    int32_t* t = static_cast<int32_t*>(jb.tmp) + (size_t)y * jb.stride;
    if (n == 1) {
      if (lane == 0) t[0] = x[0];
      return;
    }
    for (int i = lane; i < sn; i += 32) {
      const int l = min(max(i - 1, 0), dn - 1), r = min(i, dn - 1);
      t[2 * i] = x[i] - ((x[sn + l] + x[sn + r] + 2) >> 2);
    }
    __syncwarp();
    for (int i = lane; i < dn; i += 32)
      t[2 * i + 1] = i + 1 < sn ? x[sn + i] + ((t[2 * i] + t[2 * i + 2]) >> 1) : x[sn + i] + t[2 * i];
  } else {
    const float* x = static_cast<const float*>(jb.plane) + (size_t)y * jb.stride;
    float* t = static_cast<float*>(jb.tmp) + (size_t)y * jb.stride;
    if (n == 1) {
      if (lane == 0) t[0] = __fmul_rn(x[0], kRK);
      return;
    }
    for (int i = lane; i < n; i += 32) {
      const float v = i & 1 ? x[sn + (i >> 1)] : x[i >> 1];
      t[i] = __fmul_rn(v, i & 1 ? kRInvK : kRK);
    }
    __syncwarp();
    const float c[4] = {-kRDelta, -kRGamma, -kRBeta, -kRAlpha};
    #pragma unroll
    for (int s = 0; s < 4; ++s) {
      for (int j = (s & 1) + 2 * lane; j < n; j += 64)
        t[j] = lifted(t[j], c[s], t[sym_at(j - 1, n)], t[sym_at(j + 1, n)]);
      __syncwarp();
    }
  }
}

// Inverse 1-D transform of the columns of a job's tmp (low half of the rows
// first) into its plane, interleaved. A CTA takes 32 columns x 64 output
// rows and the 4 (9/7) or 2 (5/3) rows of halo each side in shared memory;
// positions beyond the column's ends are loaded from their mirror images.
// Whole-sample symmetric extension commutes with each lifting step (a
// position and its mirror have the same parity and mirrored neighbours, and
// l + r = r + l exactly), so every kept row equals the reference's value;
// the 5/3 edge clamps are the same extension. The halo rows, whose outer
// neighbours are missing, are not written.
constexpr int kTileRows = kIdwtTileRows;
__global__ void __launch_bounds__(256) idwt_cols_kernel(const IdwtJob* jobs, uint32_t njobs, uint32_t total_tiles) {
  __shared__ float sh[(kTileRows + 8) * 33];
  const uint32_t g = blockIdx.x;
  if (g >= total_tiles) return;
  const IdwtJob& jb = job_of(jobs, njobs, g, true);
  const uint32_t tiles_x = (jb.rw + 31) / 32, t = g - jb.tile_base;
  const int tx = (int)(t % tiles_x), ty = (int)(t / tiles_x);
  const int lane = threadIdx.x & 31, ry = threadIdx.x >> 5;  // 8 row groups
  const int x = tx * 32 + lane;
  const bool col = x < (int)jb.rw;
  const int n = (int)jb.rh, sn = (n + 1) / 2;
  const size_t stride = jb.stride;
  const int r0 = ty * kTileRows;
  if (jb.reversible) {
    const int32_t* src = static_cast<const int32_t*>(jb.tmp) + x;
    int32_t* dst = static_cast<int32_t*>(jb.plane) + x;
    int32_t* si = reinterpret_cast<int32_t*>(sh);
    if (n == 1) {
      if (ry == 0 && col) dst[0] = src[0];
      return;
    }
    constexpr int halo = 2, m = kTileRows + 2 * halo;
    for (int li = ry; li < m; li += 8) {
      const int p = sym_at(r0 - halo + li, n);
      si[li * 33 + lane] = col ? src[(size_t)(p & 1 ? sn + (p >> 1) : p >> 1) * stride] : 0;
    }
    __syncthreads();
    for (int li = 1 + ry; li < m - 1; li += 8)  // even positions (r0 is even)
      if (!(li & 1)) si[li * 33 + lane] -= (si[(li - 1) * 33 + lane] + si[(li + 1) * 33 + lane] + 2) >> 2;
    __syncthreads();
    for (int li = 1 + ry; li < m - 1; li += 8)
      if (li & 1) si[li * 33 + lane] += (si[(li - 1) * 33 + lane] + si[(li + 1) * 33 + lane]) >> 1;
    __syncthreads();
    for (int li = halo + ry; li < halo + kTileRows; li += 8) {
      const int i = r0 + li - halo;
      if (col && i < n) dst[(size_t)i * stride] = si[li * 33 + lane];
    }
  } else {
    const float* src = static_cast<const float*>(jb.tmp) + x;
    float* dst = static_cast<float*>(jb.plane) + x;
    if (n == 1) {
      if (ry == 0 && col) dst[0] = __fmul_rn(src[0], kRK);
      return;
    }
    constexpr int halo = 4, m = kTileRows + 2 * halo;
    for (int li = ry; li < m; li += 8) {
      const int p = sym_at(r0 - halo + li, n);
      const float v = col ? src[(size_t)(p & 1 ? sn + (p >> 1) : p >> 1) * stride] : 0.0f;
      sh[li * 33 + lane] = __fmul_rn(v, p & 1 ? kRInvK : kRK);
    }
    __syncthreads();
    const float c[4] = {-kRDelta, -kRGamma, -kRBeta, -kRAlpha};
    #pragma unroll
    for (int s = 0; s < 4; ++s) {
      for (int li = 1 + ry; li < m - 1; li += 8)
        if ((li & 1) == (s & 1))
          sh[li * 33 + lane] = lifted(sh[li * 33 + lane], c[s], sh[(li - 1) * 33 + lane], sh[(li + 1) * 33 + lane]);
      __syncthreads();
    }
    for (int li = halo + ry; li < halo + kTileRows; li += 8) {
      const int i = r0 + li - halo;
      if (col && i < n) dst[(size_t)i * stride] = sh[li * 33 + lane];
    }
  }
}

__device__ __forceinline__ float clamp255(float v) { return fminf(fmaxf(v, 0.0f), 255.0f); }

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(~0u, v, o);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  return s;
}

// Decoded samples: squared error against the original pixels, and the
// original and decoded luma (BT.601 for sRGB) for SSIM.
__global__ void recon_pixels_kernel(ReconArgs r) {
  __shared__ double sh[8];
  const size_t n = (size_t)r.width * r.height;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < n) {
    if (r.ncomp == 1) {
      const float dec = clamp255(__fadd_rn(r.plane[i], 128.0f));
      const float orig = (float)r.px[i];
      const float diff = __fadd_rn(dec, -orig);
      e = (double)__fmul_rn(diff, diff);
      r.luma_dec[i] = dec;
      r.luma_orig[i] = orig;
    } else {
      const float yc = r.plane[i], cb = r.plane[n + i], cr = r.plane[2 * n + i];
      // inverse ICT (ISO/IEC 15444-1 G.2) and level shift, backend.rs:392-400
      const float R = clamp255(__fadd_rn(__fadd_rn(yc, __fmul_rn(1.402f, cr)), 128.0f));
      const float G = clamp255(
          __fadd_rn(__fadd_rn(__fadd_rn(yc, -__fmul_rn(0.34413f, cb)), -__fmul_rn(0.71414f, cr)), 128.0f));
      const float B = clamp255(__fadd_rn(__fadd_rn(yc, __fmul_rn(1.772f, cb)), 128.0f));
      const float o0 = (float)r.px[3 * i], o1 = (float)r.px[3 * i + 1], o2 = (float)r.px[3 * i + 2];
      const float dr = __fadd_rn(R, -o0), dg = __fadd_rn(G, -o1), db = __fadd_rn(B, -o2);
      e = (double)__fadd_rn(__fadd_rn(__fmul_rn(dr, dr), __fmul_rn(dg, dg)), __fmul_rn(db, db));
      r.luma_dec[i] = __fadd_rn(__fadd_rn(__fmul_rn(0.299f, R), __fmul_rn(0.587f, G)), __fmul_rn(0.114f, B));
      r.luma_orig[i] = __fadd_rn(__fadd_rn(__fmul_rn(0.299f, o0), __fmul_rn(0.587f, o1)), __fmul_rn(0.114f, o2));
    }
  }
  const double s = block_sum(e, sh);
  if (threadIdx.x == 0) atomicAdd(&r.stats[0], s);
}

// SSIM of one 8x8 luma block per thread (sums in the reference's order).
__global__ void recon_ssim_kernel(ReconArgs r) {
  __shared__ double sh[8];
  const int bc = r.width / 8, br = r.height / 8;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (k < bc * br) {
    const int by = k / bc, bx = k - by * bc;
    double sx = 0, sy = 0, sxx = 0, syy = 0, sxy = 0;
    for (int dy = 0; dy < 8; ++dy)
      for (int dx = 0; dx < 8; ++dx) {
        const size_t i = (size_t)(by * 8 + dy) * r.width + bx * 8 + dx;
        const double x = r.luma_orig[i], y = r.luma_dec[i];
        sx = __dadd_rn(sx, x);
        sy = __dadd_rn(sy, y);
        sxx = __dadd_rn(sxx, __dmul_rn(x, x));
        syy = __dadd_rn(syy, __dmul_rn(y, y));
        sxy = __dadd_rn(sxy, __dmul_rn(x, y));
      }
    const double n = 64.0, C1 = 6.5025, C2 = 58.5225;
    const double ux = __ddiv_rn(sx, n), uy = __ddiv_rn(sy, n);
    const double vx = fmax(__dadd_rn(__ddiv_rn(sxx, n), -__dmul_rn(ux, ux)), 0.0);
    const double vy = fmax(__dadd_rn(__ddiv_rn(syy, n), -__dmul_rn(uy, uy)), 0.0);
    const double cxy = __dadd_rn(__ddiv_rn(sxy, n), -__dmul_rn(ux, uy));
    const double num = __dmul_rn(__dadd_rn(__dmul_rn(__dmul_rn(2.0, ux), uy), C1), __dadd_rn(__dmul_rn(2.0, cxy), C2));
    const double den = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)), C1),
                                 __dadd_rn(__dadd_rn(vx, vy), C2));
    v = __ddiv_rn(num, den);
  }
  const double s = block_sum(v, sh);
  if (threadIdx.x == 0) atomicAdd(&r.stats[1], s);
}

// ------------------------------------------------------------- decoding --
__device__ __forceinline__ uint8_t clamp_int(int32_t v) { return (uint8_t)min(max(v + 128, 0), 255); }
__device__ __forceinline__ uint8_t clamp_round(float v) {
  return (uint8_t)(int)fminf(fmaxf(roundf(__fadd_rn(v, 128.0f)), 0.0f), 255.0f);
}

// Inverse RCT (src/simd/scalar.rs:216-228) or ICT (scalar.rs:201-214), the
// level shift and clamp (finalize, scalar.rs:230-242) of one sample of one
// page, written interleaved.
__global__ void dec_pixels_kernel(const PixJob* jobs, uint32_t njobs, uint64_t total) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  uint32_t lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (jobs[mid].pix_base <= g) lo = mid;
    else hi = mid;
  }
  const PixJob& jb = jobs[lo];
  const size_t n = jb.npx, i = g - jb.pix_base;
  uint8_t* out = jb.px + (size_t)jb.ncomp * i;
  if (jb.reversible) {
    const int32_t* q = jb.planes;
    if (jb.ncomp == 3 && jb.mct) {
      const int32_t yy = q[i], db = q[n + i], dr = q[2 * n + i];
      const int32_t gg = yy - ((db + dr) >> 2);
      out[0] = clamp_int(dr + gg);
      out[1] = clamp_int(gg);
      out[2] = clamp_int(db + gg);
    } else {
      for (uint32_t c = 0; c < jb.ncomp; ++c) out[c] = clamp_int(q[c * n + i]);
    }
  } else {
    const float* f = reinterpret_cast<const float*>(jb.planes);
    if (jb.ncomp == 3 && jb.mct) {
      const float yy = f[i], cb = f[n + i], cr = f[2 * n + i];
      out[0] = clamp_round(__fadd_rn(yy, __fmul_rn(1.402f, cr)));
      out[1] = clamp_round(__fadd_rn(__fadd_rn(yy, -__fmul_rn(0.34413f, cb)), -__fmul_rn(0.71414f, cr)));
      out[2] = clamp_round(__fadd_rn(yy, __fmul_rn(1.772f, cb)));
    } else {
      for (uint32_t c = 0; c < jb.ncomp; ++c) out[c] = clamp_round(f[c * n + i]);
    }
  }
}

}  // namespace

void launch_idwt_level(const IdwtJob* jobs, uint32_t njobs, uint32_t total_rows, uint32_t total_tiles,
                       cudaStream_t st) {
  if (njobs == 0) return;
  if (total_rows) idwt_rows_kernel<<<(unsigned)(((size_t)total_rows * 32 + 255) / 256), 256, 0, st>>>(jobs, njobs, total_rows);
  if (total_tiles) idwt_cols_kernel<<<total_tiles, 256, 0, st>>>(jobs, njobs, total_tiles);
}

void launch_dec_pixels(const PixJob* jobs, uint32_t njobs, uint64_t total_px, cudaStream_t st) {
  if (njobs == 0 || total_px == 0) return;
  dec_pixels_kernel<<<(unsigned)((total_px + 255) / 256), 256, 0, st>>>(jobs, njobs, total_px);
}

void launch_recon(const ReconArgs& r, const std::pair<int, int>* ladder, int levels, cudaStream_t st) {
  const size_t n = (size_t)r.width * r.height;
  cudaMemsetAsync(r.plane, 0, n * r.ncomp * sizeof(float), st);
  cudaMemsetAsync(r.stats, 0, 2 * sizeof(double), st);
  if (r.nblocks) recon_dequant_kernel<<<(unsigned)(((size_t)r.nblocks * 32 + 255) / 256), 256, 0, st>>>(r);
  // every component of a level in one launch, each with its own tmp plane
  std::vector<IdwtJob> jobs;
  std::vector<uint32_t> first(levels + 2, 0), rows(levels + 2, 0), tiles(levels + 2, 0);
  for (int l = 1; l <= levels; ++l) {
    first[l] = (uint32_t)jobs.size();
    const uint32_t rw = (uint32_t)ladder[l].first, rh = (uint32_t)ladder[l].second;
    for (int c = 0; c < r.ncomp && rw && rh; ++c) {
      IdwtJob j{};
      j.plane = r.plane + (size_t)c * n;
      j.tmp = r.tmp + (size_t)c * n;
      j.stride = r.width;
      j.rw = rw;
      j.rh = rh;
      j.reversible = 0;
      j.row_base = rows[l];
      j.tile_base = tiles[l];
      rows[l] += rh;
      tiles[l] += ((rw + 31) / 32) * ((rh + kIdwtTileRows - 1) / kIdwtTileRows);
      jobs.push_back(j);
    }
  }
  first[levels + 1] = (uint32_t)jobs.size();
  if (!jobs.empty()) cudaMemcpyAsync(r.jobs, jobs.data(), jobs.size() * sizeof(IdwtJob), cudaMemcpyHostToDevice, st);
  for (int l = 1; l <= levels; ++l)
    launch_idwt_level(r.jobs + first[l], first[l + 1] - first[l], rows[l], tiles[l], st);
  recon_pixels_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(r);
  const int nb8 = (int)(r.width / 8) * (int)(r.height / 8);
  if (nb8 > 0) recon_ssim_kernel<<<(unsigned)((nb8 + 255) / 256), 256, 0, st>>>(r);
}

}  // namespace jp2g
