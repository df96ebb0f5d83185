// Colour transform + one level of the 2-D forward DWT + deadzone quantiser,
// over shared-memory tiles with a symmetric-extension halo.
//
// Replaces, for one decomposition level:
//   level_shift / forward_rct_component / forward_ict_component
//     (src/simd/scalar.rs:135-195)                      [first level only]
//   forward_53_2d_in_place (src/dwt/rev53.rs:34-75)      [reversible]
//   forward_97_2d_in_place (src/dwt/irrev97.rs:51-82)    [irreversible]
//   quantize_97_coefficients (src/encode/backend/native/backend.rs:519-587)
//
// A CTA owns a TW x TH tile of the level's interleaved input. It loads the
// tile plus a HALO-sample border (mirrored at the region edges), runs the
// vertical lifting steps over every column, then the horizontal steps over
// the centre rows, and writes the four subbands: LL to the next level's
// plane (or, at the last level, into code-block storage) and HL/LH/HH,
// quantised, straight into their 64x64 code-block slots. Whole-sample
// symmetric extension commutes with the lifting steps, so every output
// equals the reference's whole-row/whole-column lifting bit for bit; the
// f32 arithmetic uses explicit round-to-nearest intrinsics so nothing is
// contracted into an FMA.
#include <cuda_runtime.h>

#include <type_traits>

#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {

namespace {

// ISO 15444-1 Annex F.4.8.2 lifting constants (src/dwt/irrev97.rs:10-15).
__constant__ float kAlpha = -1.586134342059924f;
__constant__ float kBeta = -0.052980118572961f;
__constant__ float kGamma = 0.882911075530934f;
__constant__ float kDelta = 0.443506852043971f;
__constant__ float kK = 1.230174104914001f;
__constant__ float kInvK = 1.0f / 1.230174104914001f;

constexpr int TW = 128;
constexpr int TH = 64;
constexpr int NT = 256;

// Whole-sample symmetric extension (src/dwt/irrev97.rs:523-536).
__device__ __forceinline__ int sym(int i, int n) {
  if (n <= 1) return 0;
  if (i >= 0 && i < n) return i;
  int period = 2 * (n - 1);
  int k = i % period;
  if (k < 0) k += period;
  return k >= n ? period - k : k;
}

__device__ __forceinline__ float lift97(float x, float c, float l, float r) {
  return __fadd_rn(x, __fmul_rn(c, __fadd_rn(l, r)));
}

__device__ __forceinline__ int32_t quantize(float v, float step) {
  // src/simd/scalar.rs:100-106: trunc(v / step), saturating.
  return __float2int_rz(__fdiv_rn(v, step));
}

template <bool REV>
struct Cfg {
  using T = typename std::conditional<REV, int32_t, float>::type;
  static constexpr int HALO = REV ? 2 : 4;
  static constexpr int SW = TW + 2 * HALO;
  static constexpr int SH = TH + 2 * HALO;
  static constexpr int PITCH = SW + 1;
};

// Reads one sample of the level's input, applying the DC level shift and
// the component transform when the input is the page's pixels.
template <bool REV>
__device__ __forceinline__ typename Cfg<REV>::T load_sample(const DwtLevelArgs& a, int comp,
                                                            int gx, int gy) {
  using T = typename Cfg<REV>::T;
  if (a.from_pixels) {
    const uint8_t* row = a.px + (size_t)gy * a.px_pitch;
    if (!a.mct) {
      return (T)((int)row[(size_t)gx * a.ncomp + comp] - 128);
    }
    int r = (int)row[(size_t)gx * 3 + 0] - 128;
    int g = (int)row[(size_t)gx * 3 + 1] - 128;
    int b = (int)row[(size_t)gx * 3 + 2] - 128;
    if (REV) {  // RCT (src/simd/scalar.rs:173-195)
      int v = comp == 0 ? ((r + 2 * g + b) >> 2) : (comp == 1 ? b - g : r - g);
      return (T)v;
    } else {  // ICT (src/simd/scalar.rs:149-171), evaluated left to right
      float rf = (float)r, gf = (float)g, bf = (float)b;
      float v;
      if (comp == 0)
        v = __fadd_rn(__fadd_rn(__fmul_rn(0.299f, rf), __fmul_rn(0.587f, gf)), __fmul_rn(0.114f, bf));
      else if (comp == 1)
        v = __fadd_rn(__fadd_rn(__fmul_rn(-0.16875f, rf), __fmul_rn(-0.33126f, gf)), __fmul_rn(0.5f, bf));
      else
        v = __fsub_rn(__fsub_rn(__fmul_rn(0.5f, rf), __fmul_rn(0.41869f, gf)), __fmul_rn(0.08131f, bf));
      return (T)v;
    }
  }
  const T* src = reinterpret_cast<const T*>(a.src);
  return src[(size_t)comp * a.src_comp + (size_t)gy * a.src_pitch + gx];
}

template <bool REV>
__global__ void __launch_bounds__(NT) dwt_level_kernel(DwtLevelArgs a) {
  using C = Cfg<REV>;
  using T = typename C::T;
  constexpr int HALO = C::HALO, SW = C::SW, SH = C::SH, P = C::PITCH;
  constexpr int TX = 32, TY = NT / 32;
  __shared__ T s[SH * P];

  const int comp = blockIdx.z;
  const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
  const int rw = a.rw, rh = a.rh;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;

  // ---- load tile + halo (mirrored at the region borders) ----
  const bool inner_x = x0 - HALO >= 0 && x0 - HALO + SW <= rw;
  for (int ly = ty; ly < SH; ly += TY) {
    int gy = y0 - HALO + ly;
    if ((unsigned)gy >= (unsigned)rh) gy = sym(gy, rh);
    for (int lx = tx; lx < SW; lx += TX) {
      int gx = x0 - HALO + lx;
      if (!inner_x && (unsigned)gx >= (unsigned)rw) gx = sym(gx, rw);
      s[ly * P + lx] = load_sample<REV>(a, comp, gx, gy);
    }
  }
  __syncthreads();

  if (!a.no_transform) {
    // ---- vertical pass over every tile column ----
    // A step updates rows of one parity from their two neighbours; rows in
    // [1, SH-2] are updated (the halo shrinks by one row per step). Tile
    // origins and HALO are even, so local parity equals image parity.
    if (rh >= 2) {
      if constexpr (REV) {
        // predict on odd rows, update on even rows (rev53.rs:419-497)
        #pragma unroll
        for (int step = 0; step < 2; ++step) {
          const int first = step == 0 ? 1 : 2;
          for (int ly = first + 2 * ty; ly <= SH - 2; ly += 2 * TY)
            for (int lx = tx; lx < SW; lx += TX) {
              int32_t up = s[(ly - 1) * P + lx], dn = s[(ly + 1) * P + lx];
              if (step == 0) s[ly * P + lx] -= (up + dn) >> 1;
              else s[ly * P + lx] += (up + dn + 2) >> 2;
            }
          __syncthreads();
        }
      } else {
        // alpha (odd), beta (even), gamma (odd), delta (even), then scale
        // (irrev97.rs:261-336)
        #pragma unroll
        for (int step = 0; step < 4; ++step) {
          const int first = (step & 1) ? 2 : 1;
          const float c = step == 0 ? kAlpha : step == 1 ? kBeta : step == 2 ? kGamma : kDelta;
          for (int ly = first + 2 * ty; ly <= SH - 2; ly += 2 * TY)
            for (int lx = tx; lx < SW; lx += TX)
              s[ly * P + lx] = lift97(s[ly * P + lx], c, s[(ly - 1) * P + lx], s[(ly + 1) * P + lx]);
          __syncthreads();
        }
        for (int ly = ty; ly < SH; ly += TY) {
          const float k = (ly & 1) ? kK : kInvK;
          for (int lx = tx; lx < SW; lx += TX) s[ly * P + lx] = __fmul_rn(s[ly * P + lx], k);
        }
        __syncthreads();
      }
    } else {
      if constexpr (!REV) {  // height 1: scale by 1/K (irrev97.rs:271-275)
        for (int ly = ty; ly < SH; ly += TY)
          for (int lx = tx; lx < SW; lx += TX) s[ly * P + lx] = __fmul_rn(s[ly * P + lx], kInvK);
        __syncthreads();
      }
    }
    // ---- horizontal pass over the centre rows ----
    if (rw >= 2) {
      if constexpr (REV) {
        #pragma unroll
        for (int step = 0; step < 2; ++step) {
          const int first = step == 0 ? 1 : 2;
          for (int r = ty; r < TH; r += TY) {
            T* row = s + (HALO + r) * P;
            for (int lx = first + 2 * tx; lx <= SW - 2; lx += 2 * TX) {
              int32_t l = row[lx - 1], rr = row[lx + 1];
              if (step == 0) row[lx] -= (l + rr) >> 1;
              else row[lx] += (l + rr + 2) >> 2;
            }
          }
          __syncthreads();
        }
      } else {
        #pragma unroll
        for (int step = 0; step < 4; ++step) {
          const int first = (step & 1) ? 2 : 1;
          const float c = step == 0 ? kAlpha : step == 1 ? kBeta : step == 2 ? kGamma : kDelta;
          for (int r = ty; r < TH; r += TY) {
            T* row = s + (HALO + r) * P;
            for (int lx = first + 2 * tx; lx <= SW - 2; lx += 2 * TX)
              row[lx] = lift97(row[lx], c, row[lx - 1], row[lx + 1]);
          }
          __syncthreads();
        }
        // the column scale (1/K even, K odd) is applied as the samples are
        // written out
      }
    } else {
      if constexpr (!REV) {  // width 1: scale by 1/K (irrev97.rs:95-97)
        for (int r = ty; r < TH; r += TY)
          for (int lx = tx; lx < SW; lx += TX) s[(HALO + r) * P + lx] = __fmul_rn(s[(HALO + r) * P + lx], kInvK);
        __syncthreads();
      }
    }
  }

  // ---- write subbands ----
  // Within a tile row, the first TW/2 columns of the loop take the even
  // (low) samples and the rest the odd (high) ones, so each warp writes a
  // contiguous run of one band row.
  const int cbs = __ffs(a.cbw) - 1, cbhs = __ffs(a.cbh) - 1;  // code-blocks are 2^k
  const int cbw = a.cbw, cbh = a.cbh;
  const bool col_scale = !REV && !a.no_transform && rw >= 2;
  for (int ly = ty; ly < TH; ly += TY) {
    const int gy = y0 + ly;
    if (gy >= rh) break;
    const T* row = s + (HALO + ly) * P + HALO;
    for (int j = tx; j < TW; j += TX) {
      const int lx = a.no_transform ? j : (j < TW / 2 ? 2 * j : 2 * (j - TW / 2) + 1);
      const int gx = x0 + lx;
      if (gx >= rw) continue;
      T v = row[lx];
      if constexpr (!REV) {
        if (col_scale) v = __fmul_rn(v, (lx & 1) ? kK : kInvK);
      }
      int orient, u, vv;
      if (a.no_transform) {
        orient = 0; u = gx; vv = gy;
      } else {
        orient = ((gy & 1) << 1) | (gx & 1);  // LL, HL, LH, HH
        u = gx >> 1; vv = gy >> 1;
      }
      if (orient == 0 && a.ll != nullptr) {
        T* ll = reinterpret_cast<T*>(a.ll);
        ll[(size_t)comp * a.ll_comp + (size_t)vv * a.ll_pitch + u] = v;
        continue;
      }
      const DwtBandOut& bo = a.band[comp][orient];
      const uint32_t blk = bo.first_block + (uint32_t)(vv >> cbhs) * bo.ncbx + (uint32_t)(u >> cbs);
      int32_t q;
      if constexpr (REV) q = v;
      else q = quantize(v, bo.step);
      a.coef[((size_t)blk << (cbs + cbhs)) + (size_t)((vv & (cbh - 1)) << cbs) + (u & (cbw - 1))] = q;
    }
  }
}

// ---------------------------------------------------------------------------
// Register-resident tile kernel (every level with a region of at least 2x2).
//
// A CTA of 288 threads owns a TW x TH = 128 x 64 tile plus a 4-sample halo
// (a 136 x 72 shared-memory tile). Lifting runs on per-thread register
// arrays of 40 samples (32 outputs plus 4 halo samples on each side, so
// every lifting step sees its true neighbours):
//   vertical:   272 jobs = 136 columns x 2 row halves,
//   horizontal: 256 jobs = 64 rows x 4 column quarters.
// Lanes take consecutive columns (vertical) or consecutive rows
// (horizontal); the odd shared-memory pitch keeps both conflict-free. Every
// job reads its 40 samples before a barrier and writes its 32 outputs after
// it, so overlapping halos read the pre-step values. The epilogue walks each
// subband's 64 x 32 part of the tile in row order, applies the column scale
// (9/7), quantises and stores whole code-block rows.
constexpr int RT = 288;
constexpr int RH = 4;             // halo
constexpr int RN = 40;            // samples per register job (32 + 2 * RH)
constexpr int RSW = TW + 2 * RH;  // 136
constexpr int RSH = TH + 2 * RH;  // 72
constexpr int RP = RSW + 1;       // shared-memory pitch

template <bool REV, typename T>
__device__ __forceinline__ void lift_regs(T (&x)[RN]) {
  if constexpr (REV) {
    // predict on odd samples, update on even ones (rev53.rs:419-497)
    #pragma unroll
    for (int i = 1; i < RN - 1; i += 2) x[i] -= (x[i - 1] + x[i + 1]) >> 1;
    #pragma unroll
    for (int i = 2; i < RN - 1; i += 2) x[i] += (x[i - 1] + x[i + 1] + 2) >> 2;
  } else {
    // alpha (odd), beta (even), gamma (odd), delta (even) (irrev97.rs:261-336)
    #pragma unroll
    for (int i = 1; i < RN - 1; i += 2) x[i] = lift97(x[i], kAlpha, x[i - 1], x[i + 1]);
    #pragma unroll
    for (int i = 2; i < RN - 2; i += 2) x[i] = lift97(x[i], kBeta, x[i - 1], x[i + 1]);
    #pragma unroll
    for (int i = 3; i < RN - 2; i += 2) x[i] = lift97(x[i], kGamma, x[i - 1], x[i + 1]);
    #pragma unroll
    for (int i = 4; i < RN - 4; i += 2) x[i] = lift97(x[i], kDelta, x[i - 1], x[i + 1]);
  }
}

// One value of the level's input: the page's pixels (level shift and
// RCT/ICT applied) or the previous level's LL plane.
template <bool REV>
struct TileSrc {
  using T = typename Cfg<REV>::T;
  const uint8_t* px;
  size_t px_pitch;
  const T* ll;
  size_t ll_pitch;
  int ncomp, comp, mct, from_pixels;
  __device__ __forceinline__ T at(int gx, int gy) const {
    if (from_pixels) {
      const uint8_t* row = px + (size_t)gy * px_pitch;
      if (!mct) return (T)((int)row[(size_t)gx * ncomp + comp] - 128);
      const uint8_t* q = row + (size_t)gx * 3;
      const int r = (int)q[0] - 128, g = (int)q[1] - 128, b = (int)q[2] - 128;
      if constexpr (REV) {  // RCT (src/simd/scalar.rs:173-195)
        return (T)(comp == 0 ? ((r + 2 * g + b) >> 2) : (comp == 1 ? b - g : r - g));
      } else {  // ICT (src/simd/scalar.rs:149-171), evaluated left to right
        const float rf = (float)r, gf = (float)g, bf = (float)b;
        if (comp == 0)
          return __fadd_rn(__fadd_rn(__fmul_rn(0.299f, rf), __fmul_rn(0.587f, gf)), __fmul_rn(0.114f, bf));
        if (comp == 1)
          return __fadd_rn(__fadd_rn(__fmul_rn(-0.16875f, rf), __fmul_rn(-0.33126f, gf)), __fmul_rn(0.5f, bf));
        return __fsub_rn(__fsub_rn(__fmul_rn(0.5f, rf), __fmul_rn(0.41869f, gf)), __fmul_rn(0.08131f, bf));
      }
    }
    return ll[(size_t)gy * ll_pitch + gx];
  }
};

// One tile of one level (see the comment above RT). The level's arguments
// are read once into registers: the caller's copy may live in global memory.
template <bool REV>
__device__ __forceinline__ void dwt_tile(const DwtLevelArgs& args, int comp, int x0, int y0,
                                         typename Cfg<REV>::T* s) {
  using T = typename Cfg<REV>::T;
  const int rw = args.rw, rh = args.rh;
  const int tid = threadIdx.x;
  TileSrc<REV> src;
  src.from_pixels = args.from_pixels;
  src.px = args.px;
  src.px_pitch = args.px_pitch;
  src.ncomp = args.ncomp;
  src.comp = comp;
  src.mct = args.mct;
  src.ll = reinterpret_cast<const T*>(args.src) + (size_t)comp * args.src_comp;
  src.ll_pitch = args.src_pitch;
  T* const ll_out = args.ll ? reinterpret_cast<T*>(args.ll) + (size_t)comp * args.ll_comp : nullptr;
  const size_t ll_pitch = args.ll_pitch;
  int32_t* const coef = args.coef;
  const int cbw = args.cbw, cbh = args.cbh;

  // ---- load tile + halo (mirrored at the region borders) ----
  {
    const int tx = tid & 31, ty = tid >> 5, nty = RT / 32;
    const bool inner_x = x0 - RH >= 0 && x0 - RH + RSW <= rw;
    for (int ly = ty; ly < RSH; ly += nty) {
      int gy = y0 - RH + ly;
      if ((unsigned)gy >= (unsigned)rh) gy = sym(gy, rh);
      for (int lx = tx; lx < RSW; lx += 32) {
        int gx = x0 - RH + lx;
        if (!inner_x && (unsigned)gx >= (unsigned)rw) gx = sym(gx, rw);
        s[ly * RP + lx] = src.at(gx, gy);
      }
    }
  }
  __syncthreads();

  // ---- vertical lifting: column lx, rows [32 h, 32 h + 40) ----
  {
    T x[RN];
    const int job = tid;  // 272 jobs, 288 threads
    const bool active = job < 2 * RSW;
    const int h = job >= RSW ? 1 : 0, lx = job - h * RSW, r0 = 32 * h;
    if (active) {
      #pragma unroll
      for (int i = 0; i < RN; ++i) x[i] = s[(r0 + i) * RP + lx];
    }
    __syncthreads();
    if (active) {
      lift_regs<REV>(x);
      #pragma unroll
      for (int i = RH; i < RN - RH; ++i) {
        T v = x[i];
        if constexpr (!REV) v = __fmul_rn(v, (i & 1) ? kK : kInvK);  // rows: 1/K even, K odd
        s[(r0 + i) * RP + lx] = v;
      }
    }
  }
  __syncthreads();

  // ---- horizontal lifting: row RH + r, columns [32 q, 32 q + 40) ----
  {
    T x[RN];
    const int job = tid;  // 256 jobs
    const bool active = job < 4 * TH;
    const int q = job / TH, r = job - q * TH, c0 = 32 * q;
    T* row = s + (RH + r) * RP;
    if (active) {
      #pragma unroll
      for (int i = 0; i < RN; ++i) x[i] = row[c0 + i];
    }
    __syncthreads();
    if (active) {
      lift_regs<REV>(x);
      #pragma unroll
      for (int i = RH; i < RN - RH; ++i) row[c0 + i] = x[i];
    }
  }
  __syncthreads();

  // ---- epilogue: each subband's 64 x 32 part, rows in order ----
  const int cbs = __ffs(cbw) - 1, cbhs = __ffs(cbh) - 1;
  const int u0 = x0 >> 1, v0 = y0 >> 1;
  #pragma unroll 1
  for (int band = 0; band < 4; ++band) {  // LL, HL, LH, HH
    const int bw = (band & 1) ? rw >> 1 : (rw + 1) >> 1;
    const int bh = (band & 2) ? rh >> 1 : (rh + 1) >> 1;
    const int cols = min(64, bw - u0), rows = min(32, bh - v0);
    if (cols <= 0 || rows <= 0) continue;
    const T* sb = s + (RH + (band >> 1)) * RP + RH + (band & 1);
    const float cscale = (band & 1) ? kK : kInvK;  // columns: 1/K even, K odd (9/7)
    if (band == 0 && ll_out != nullptr) {
      for (int idx = tid; idx < 32 * 64; idx += RT) {
        const int rr = idx >> 6, cc = idx & 63;
        if (rr >= rows || cc >= cols) continue;
        T val = sb[2 * rr * RP + 2 * cc];
        if constexpr (!REV) val = __fmul_rn(val, cscale);
        ll_out[(size_t)(v0 + rr) * ll_pitch + u0 + cc] = val;
      }
      continue;
    }
    const DwtBandOut bo = args.band[comp][band];
    for (int idx = tid; idx < 32 * 64; idx += RT) {
      const int rr = idx >> 6, cc = idx & 63;
      if (rr >= rows || cc >= cols) continue;
      T val = sb[2 * rr * RP + 2 * cc];
      const int u = u0 + cc, v = v0 + rr;
      const uint32_t blk = bo.first_block + (uint32_t)(v >> cbhs) * bo.ncbx + (uint32_t)(u >> cbs);
      int32_t qv;
      if constexpr (REV) qv = val;
      else qv = quantize(__fmul_rn(val, cscale), bo.step);
      coef[((size_t)blk << (cbs + cbhs)) + ((size_t)(v & (cbh - 1)) << cbs) + (u & (cbw - 1))] = qv;
    }
  }
}

// Flat tile list over many pages: the CTA finds its page by binary search
// over the tile bases, then its component and tile position.
template <bool REV>
__global__ void __launch_bounds__(RT) dwt_batch_kernel(const DwtLevelArgs* __restrict__ args,
                                                       const uint32_t* __restrict__ tile_base,
                                                       uint32_t npages) {
  __shared__ typename Cfg<REV>::T s[RSH * RP];
  const uint32_t t = blockIdx.x;
  uint32_t lo = 0, hi = npages;  // tile_base[lo] <= t < tile_base[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (tile_base[mid] <= t) lo = mid;
    else hi = mid;
  }
  const DwtLevelArgs& a = args[lo];
  const uint32_t local = t - tile_base[lo];
  const uint32_t ntx = (uint32_t)(a.rw + TW - 1) / TW, nty = (uint32_t)(a.rh + TH - 1) / TH;
  const uint32_t comp = local / (ntx * nty), rem = local - comp * ntx * nty;
  const uint32_t ty = rem / ntx, tx = rem - ty * ntx;
  dwt_tile<REV>(a, (int)comp, (int)tx * TW, (int)ty * TH, s);
}

}  // namespace

uint32_t dwt_tiles(int rw, int rh, int ncomp) {
  return (uint32_t)((rw + TW - 1) / TW) * (uint32_t)((rh + TH - 1) / TH) * (uint32_t)ncomp;
}

void launch_dwt_batch(const DwtLevelArgs* d_args, const uint32_t* d_tile_base, uint32_t npages,
                      uint32_t ntiles, bool reversible, cudaStream_t st) {
  if (npages == 0 || ntiles == 0) return;
  if (reversible) dwt_batch_kernel<true><<<ntiles, RT, 0, st>>>(d_args, d_tile_base, npages);
  else dwt_batch_kernel<false><<<ntiles, RT, 0, st>>>(d_args, d_tile_base, npages);
}

void launch_dwt_level(const DwtLevelArgs& a, bool reversible, cudaStream_t st) {
  // zero levels, or a one-sample-wide/high region (its own scaling rules);
  // every other level goes through launch_dwt_batch
  dim3 grid((a.rw + TW - 1) / TW, (a.rh + TH - 1) / TH, a.ncomp);
  if (reversible) dwt_level_kernel<true><<<grid, NT, 0, st>>>(a);
  else dwt_level_kernel<false><<<grid, NT, 0, st>>>(a);
}

}  // namespace jp2g
