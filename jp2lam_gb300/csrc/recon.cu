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

// Inverse 1-D 9/7 of row y (rw samples, low half first): a warp per row,
// each step's positions in parallel, through the row's slice of `tmp`.
__global__ void recon_rows_kernel(float* plane, float* tmp, int stride, int rw, int rh) {
  const int lane = threadIdx.x & 31;
  const int y = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (y >= rh) return;
  float* x = plane + (size_t)y * stride;
  float* t = tmp + (size_t)y * stride;
  const int n = rw;
  if (n < 2) {
    if (n == 1 && lane == 0) x[0] = __fmul_rn(x[0], kRK);
    return;
  }
  const int sn = (n + 1) / 2;
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
  for (int i = lane; i < n; i += 32) x[i] = t[i];
}

// Inverse 1-D 9/7 of every column x < rw over rh rows: a thread per column
// (neighbouring threads read neighbouring samples of a row), through `tmp`.
__global__ void recon_cols_kernel(float* plane, float* tmp, int stride, int rw, int rh) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= rw) return;
  float* p = plane + x;
  float* t = tmp + x;
  const int n = rh;
  if (n < 2) {
    if (n == 1) p[0] = __fmul_rn(p[0], kRK);
    return;
  }
  const int sn = (n + 1) / 2;
  for (int i = 0; i < n; ++i) {
    const float v = i & 1 ? p[(size_t)(sn + (i >> 1)) * stride] : p[(size_t)(i >> 1) * stride];
    t[(size_t)i * stride] = __fmul_rn(v, i & 1 ? kRInvK : kRK);
  }
  const float c[4] = {-kRDelta, -kRGamma, -kRBeta, -kRAlpha};
  #pragma unroll
  for (int s = 0; s < 4; ++s)
    for (int j = s & 1; j < n; j += 2)
      t[(size_t)j * stride] =
          lifted(t[(size_t)j * stride], c[s], t[(size_t)sym_at(j - 1, n) * stride], t[(size_t)sym_at(j + 1, n) * stride]);
  for (int i = 0; i < n; ++i) p[(size_t)i * stride] = t[(size_t)i * stride];
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
// Reconstruction of a decoded codestream (reconstruct, src/decode/
// reconstruct.rs:24-304): the inverse 5/3 (src/dwt/rev53.rs:96-129 and
// 419-497: per level rows then columns; even samples first,
// s[i] - ((d[i-1] + d[i] + 2) >> 2) with the edges clamped, then odd samples
// d[i] + ((e[i] + e[i+1]) >> 1), or d[i] + e[i] at the right edge) and
// inverse RCT, or the inverse 9/7 above and inverse ICT; the level shift and
// the 8-bit clamp (finalize, src/simd/scalar.rs:216-242).

// Inverse 1-D 5/3 of row y: a warp per row, through the row's slice of tmp.
__global__ void dec53_rows_kernel(int32_t* plane, int32_t* tmp, int stride, int rw, int rh) {
  const int lane = threadIdx.x & 31;
  const int y = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (y >= rh || rw <= 1) return;
  int32_t* x = plane + (size_t)y * stride;
  int32_t* t = tmp + (size_t)y * stride;
  const int sn = (rw + 1) / 2, dn = rw - sn;
  for (int i = lane; i < sn; i += 32) {
    const int l = min(max(i - 1, 0), dn - 1), r = min(i, dn - 1);
    t[2 * i] = x[i] - ((x[sn + l] + x[sn + r] + 2) >> 2);
  }
  __syncwarp();
  for (int i = lane; i < dn; i += 32)
    t[2 * i + 1] = i + 1 < sn ? x[sn + i] + ((t[2 * i] + t[2 * i + 2]) >> 1) : x[sn + i] + t[2 * i];
  __syncwarp();
  for (int i = lane; i < rw; i += 32) x[i] = t[i];
}

// Inverse 1-D 5/3 of every column x < rw: a thread per column.
__global__ void dec53_cols_kernel(int32_t* plane, int32_t* tmp, int stride, int rw, int rh) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= rw || rh <= 1) return;
  int32_t* p = plane + x;
  int32_t* t = tmp + x;
  const size_t s = (size_t)stride;
  const int sn = (rh + 1) / 2, dn = rh - sn;
  for (int i = 0; i < sn; ++i) {
    const int l = min(max(i - 1, 0), dn - 1), r = min(i, dn - 1);
    t[2 * i * s] = p[i * s] - ((p[(sn + l) * s] + p[(sn + r) * s] + 2) >> 2);
  }
  for (int i = 0; i < dn; ++i)
    t[(2 * i + 1) * s] =
        i + 1 < sn ? p[(sn + i) * s] + ((t[2 * i * s] + t[(2 * i + 2) * s]) >> 1) : p[(sn + i) * s] + t[2 * i * s];
  for (int i = 0; i < rh; ++i) p[i * s] = t[i * s];
}

__device__ __forceinline__ uint8_t clamp_int(int32_t v) { return (uint8_t)min(max(v + 128, 0), 255); }
__device__ __forceinline__ uint8_t clamp_round(float v) {
  return (uint8_t)(int)fminf(fmaxf(roundf(__fadd_rn(v, 128.0f)), 0.0f), 255.0f);
}

// Inverse RCT (src/simd/scalar.rs:216-228) or ICT (scalar.rs:201-214) and
// the interleaved 8-bit samples.
__global__ void dec_pixels_kernel(DecodeArgs a) {
  const size_t n = (size_t)a.width * a.height;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (a.reversible) {
    const int32_t* q = a.plane;
    if (a.ncomp == 3 && a.mct) {
      const int32_t yy = q[i], db = q[n + i], dr = q[2 * n + i];
      const int32_t g = yy - ((db + dr) >> 2);
      a.px[3 * i] = clamp_int(dr + g);
      a.px[3 * i + 1] = clamp_int(g);
      a.px[3 * i + 2] = clamp_int(db + g);
    } else {
      for (int c = 0; c < a.ncomp; ++c) a.px[a.ncomp * i + c] = clamp_int(q[c * n + i]);
    }
  } else {
    const float* f = reinterpret_cast<const float*>(a.plane);
    if (a.ncomp == 3 && a.mct) {
      const float yy = f[i], cb = f[n + i], cr = f[2 * n + i];
      a.px[3 * i] = clamp_round(__fadd_rn(yy, __fmul_rn(1.402f, cr)));
      a.px[3 * i + 1] = clamp_round(__fadd_rn(__fadd_rn(yy, -__fmul_rn(0.34413f, cb)), -__fmul_rn(0.71414f, cr)));
      a.px[3 * i + 2] = clamp_round(__fadd_rn(yy, __fmul_rn(1.772f, cb)));
    } else {
      for (int c = 0; c < a.ncomp; ++c) a.px[a.ncomp * i + c] = clamp_round(f[c * n + i]);
    }
  }
}

}  // namespace

void launch_decode_reconstruct(const DecodeArgs& a, const std::pair<int, int>* ladder, int levels, cudaStream_t st) {
  const size_t n = (size_t)a.width * a.height;
  for (int c = 0; c < a.ncomp; ++c)
    for (int l = 1; l <= levels; ++l) {
      const int rw = ladder[l].first, rh = ladder[l].second;
      if (rw == 0 || rh == 0) continue;
      const unsigned rows_grid = (unsigned)(((size_t)rh * 32 + 255) / 256), cols_grid = (unsigned)((rw + 127) / 128);
      if (a.reversible) {
        int32_t* plane = a.plane + (size_t)c * n;
        dec53_rows_kernel<<<rows_grid, 256, 0, st>>>(plane, a.tmp, (int)a.width, rw, rh);
        dec53_cols_kernel<<<cols_grid, 128, 0, st>>>(plane, a.tmp, (int)a.width, rw, rh);
      } else {
        float* plane = reinterpret_cast<float*>(a.plane) + (size_t)c * n;
        float* tmp = reinterpret_cast<float*>(a.tmp);
        recon_rows_kernel<<<rows_grid, 256, 0, st>>>(plane, tmp, (int)a.width, rw, rh);
        recon_cols_kernel<<<cols_grid, 128, 0, st>>>(plane, tmp, (int)a.width, rw, rh);
      }
    }
  dec_pixels_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a);
}

void launch_recon(const ReconArgs& r, const std::pair<int, int>* ladder, int levels, cudaStream_t st) {
  const size_t n = (size_t)r.width * r.height;
  cudaMemsetAsync(r.plane, 0, n * r.ncomp * sizeof(float), st);
  cudaMemsetAsync(r.stats, 0, 2 * sizeof(double), st);
  if (r.nblocks) recon_dequant_kernel<<<(unsigned)(((size_t)r.nblocks * 32 + 255) / 256), 256, 0, st>>>(r);
  for (int c = 0; c < r.ncomp; ++c) {
    float* plane = r.plane + (size_t)c * n;
    for (int l = 1; l <= levels; ++l) {
      const int rw = ladder[l].first, rh = ladder[l].second;
      if (rw == 0 || rh == 0) continue;
      recon_rows_kernel<<<(unsigned)(((size_t)rh * 32 + 255) / 256), 256, 0, st>>>(plane, r.tmp, (int)r.width, rw, rh);
      recon_cols_kernel<<<(unsigned)((rw + 127) / 128), 128, 0, st>>>(plane, r.tmp, (int)r.width, rw, rh);
    }
  }
  recon_pixels_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(r);
  const int nb8 = (int)(r.width / 8) * (int)(r.height / 8);
  if (nb8 > 0) recon_ssim_kernel<<<(unsigned)((nb8 + 255) / 256), 256, 0, st>>>(r);
}

}  // namespace jp2g
