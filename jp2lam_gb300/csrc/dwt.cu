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
  __shared__ T s[SH * P];

  const int comp = blockIdx.z;
  const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
  const int rw = a.rw, rh = a.rh;
  const int tid = threadIdx.x;

  // ---- load tile + halo (mirrored at the region borders) ----
  for (int i = tid; i < SH * SW; i += NT) {
    int ly = i / SW, lx = i - ly * SW;
    int gy = sym(y0 - HALO + ly, rh), gx = sym(x0 - HALO + lx, rw);
    s[ly * P + lx] = load_sample<REV>(a, comp, gx, gy);
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
        for (int step = 0; step < 2; ++step) {
          const int first = step == 0 ? 1 : 2;
          const int nrows = (SH - 2 - first) / 2 + 1;
          for (int i = tid; i < nrows * SW; i += NT) {
            int r = i / SW, lx = i - r * SW;
            int ly = first + 2 * r;
            int32_t up = s[(ly - 1) * P + lx], dn = s[(ly + 1) * P + lx];
            if (step == 0) s[ly * P + lx] -= (up + dn) >> 1;
            else s[ly * P + lx] += (up + dn + 2) >> 2;
          }
          __syncthreads();
        }
      } else {
        // alpha (odd), beta (even), gamma (odd), delta (even), then scale
        // (irrev97.rs:261-336)
        for (int step = 0; step < 4; ++step) {
          const int first = (step & 1) ? 2 : 1;
          const int nrows = (SH - 2 - first) / 2 + 1;
          const float c = step == 0 ? kAlpha : step == 1 ? kBeta : step == 2 ? kGamma : kDelta;
          for (int i = tid; i < nrows * SW; i += NT) {
            int r = i / SW, lx = i - r * SW;
            int ly = first + 2 * r;
            s[ly * P + lx] = lift97(s[ly * P + lx], c, s[(ly - 1) * P + lx], s[(ly + 1) * P + lx]);
          }
          __syncthreads();
        }
        for (int i = tid; i < SH * SW; i += NT) {
          int ly = i / SW, lx = i - ly * SW;
          s[ly * P + lx] = __fmul_rn(s[ly * P + lx], (ly & 1) ? kK : kInvK);
        }
        __syncthreads();
      }
    } else {
      if constexpr (!REV) {  // height 1: scale by 1/K (irrev97.rs:271-275)
        for (int i = tid; i < SH * SW; i += NT) {
          int ly = i / SW, lx = i - ly * SW;
          s[ly * P + lx] = __fmul_rn(s[ly * P + lx], kInvK);
        }
        __syncthreads();
      }
    }
    // ---- horizontal pass over the centre rows ----
    if (rw >= 2) {
      if constexpr (REV) {
        for (int step = 0; step < 2; ++step) {
          const int first = step == 0 ? 1 : 2;
          const int ncols = (SW - 2 - first) / 2 + 1;
          for (int i = tid; i < ncols * TH; i += NT) {
            int r = i / ncols, ci = i - r * ncols;
            int ly = HALO + r, lx = first + 2 * ci;
            int32_t l = s[ly * P + lx - 1], rr = s[ly * P + lx + 1];
            if (step == 0) s[ly * P + lx] -= (l + rr) >> 1;
            else s[ly * P + lx] += (l + rr + 2) >> 2;
          }
          __syncthreads();
        }
      } else {
        for (int step = 0; step < 4; ++step) {
          const int first = (step & 1) ? 2 : 1;
          const int ncols = (SW - 2 - first) / 2 + 1;
          const float c = step == 0 ? kAlpha : step == 1 ? kBeta : step == 2 ? kGamma : kDelta;
          for (int i = tid; i < ncols * TH; i += NT) {
            int r = i / ncols, ci = i - r * ncols;
            int ly = HALO + r, lx = first + 2 * ci;
            s[ly * P + lx] = lift97(s[ly * P + lx], c, s[ly * P + lx - 1], s[ly * P + lx + 1]);
          }
          __syncthreads();
        }
        for (int i = tid; i < TH * SW; i += NT) {
          int r = i / SW, lx = i - r * SW;
          s[(HALO + r) * P + lx] = __fmul_rn(s[(HALO + r) * P + lx], (lx & 1) ? kK : kInvK);
        }
        __syncthreads();
      }
    } else {
      if constexpr (!REV) {  // width 1: scale by 1/K (irrev97.rs:95-97)
        for (int i = tid; i < TH * SW; i += NT) {
          int r = i / SW, lx = i - r * SW;
          s[(HALO + r) * P + lx] = __fmul_rn(s[(HALO + r) * P + lx], kInvK);
        }
        __syncthreads();
      }
    }
  }

  // ---- write subbands ----
  // Within a tile row, the first TW/2 threads take the even (low) columns and
  // the rest the odd (high) ones, so each warp writes a contiguous run of one
  // band row.
  const int cbw = a.cbw, cbh = a.cbh;
  const size_t slot = (size_t)cbw * cbh;
  for (int i = tid; i < TH * TW; i += NT) {
    int ly = i / TW, j = i - ly * TW;
    int lx = a.no_transform ? j : (j < TW / 2 ? 2 * j : 2 * (j - TW / 2) + 1);
    int gy = y0 + ly, gx = x0 + lx;
    if (gy >= rh || gx >= rw) continue;
    T v = s[(HALO + ly) * P + HALO + lx];
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
    uint32_t blk = bo.first_block + (uint32_t)(vv / cbh) * bo.ncbx + (uint32_t)(u / cbw);
    int32_t q;
    if constexpr (REV) q = v;
    else q = quantize(v, bo.step);
    a.coef[(size_t)blk * slot + (size_t)(vv % cbh) * cbw + (u % cbw)] = q;
  }
}

}  // namespace

void launch_dwt_level(const DwtLevelArgs& a, bool reversible, cudaStream_t st) {
  dim3 grid((a.rw + TW - 1) / TW, (a.rh + TH - 1) / TH, a.ncomp);
  if (reversible) dwt_level_kernel<true><<<grid, NT, 0, st>>>(a);
  else dwt_level_kernel<false><<<grid, NT, 0, st>>>(a);
}

}  // namespace jp2g
