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
  // src/simd/scalar.rs:100-106: trunc(v / step), saturating. Plan steps are
  // floored at 1e-6 (backend.rs:602-620); a zero step asks for the
  // unquantised coefficient's bits instead (jp2g_debug_coefficients_f32).
  if (step == 0.0f) return __float_as_int(v);
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
// A CTA of 288 threads owns a TW x TH = 128 x 64 tile of the level's input
// plus a 4-sample border, mirrored at the region edges:
//   1. vertical: 272 jobs = 136 columns x 2 row halves. A job reads the
//      samples its 32 outputs depend on straight from global memory (the
//      page's pixels with the level shift and RCT/ICT applied, or the
//      previous level's LL plane), lifts them in registers and writes the
//      32 outputs to shared memory, even tile rows in smem rows 0-31 and odd
//      ones in rows 32-63.
//   2. horizontal: 256 jobs = 4 column quarters x 64 rows. The 32 rows of a
//      warp share one parity (and read 32 consecutive smem rows, odd pitch:
//      no bank conflict), so a warp produces two subbands, LL/HL from even
//      rows or LH/HH from odd ones. A job lifts 40 samples of its row,
//      applies the 9/7 column scale, quantises its 16 low and 16 high
//      outputs and stores each run as four 16-byte vectors into a
//      code-block row (or the next LL plane, whose pitch is a multiple of
//      16 samples). Code-blocks are 32 or 64 wide and runs start at
//      multiples of 16, so a run never crosses a code-block; samples past
//      the band edge land in the slot's unused columns (or the plane's
//      padding), which nothing reads.
// Lifting runs in wavefront order: a step is applied as soon as the two
// neighbours it reads are final, so samples leave the register set early.
// Whole-sample symmetric extension commutes with the lifting steps, so every
// output equals the reference's whole-row/whole-column lifting bit for bit.
constexpr int RT = 288;
constexpr int RH = 4;             // border
constexpr int RN = 40;            // samples per register job (32 + 2 * RH)
constexpr int RSW = TW + 2 * RH;  // 136 columns of vertical jobs
constexpr int RP = RSW + 1;       // shared-memory pitch (odd)

// Samples x[LO..HI] of a job are read; they determine outputs x[4..35].
template <bool REV>
struct JobRange {
  static constexpr int LO = REV ? 2 : 0;
  static constexpr int HI = REV ? 36 : 38;
};

// Lifts x in wavefront order and hands every output to emit(i, value),
// i = 4..35, in the order 5, 4, 7, 6, ..., 35, 34.
template <bool REV, typename T, typename Emit>
__device__ __forceinline__ void lift_wave(T (&x)[RN], Emit&& emit) {
  if constexpr (REV) {
    // predict on odd samples, update on even ones (rev53.rs:419-497)
    #pragma unroll
    for (int k = 3; k <= 35; k += 2) {
      x[k] -= (x[k - 1] + x[k + 1]) >> 1;
      if (k >= 5) {
        x[k - 1] += (x[k - 2] + x[k] + 2) >> 2;
        emit(k, x[k]);
        emit(k - 1, x[k - 1]);
      }
    }
  } else {
    // alpha (odd), beta (even), gamma (odd), delta (even) (irrev97.rs:261-336)
    #pragma unroll
    for (int k = 1; k <= 37; k += 2) {
      x[k] = lift97(x[k], kAlpha, x[k - 1], x[k + 1]);
      if (k >= 3) x[k - 1] = lift97(x[k - 1], kBeta, x[k - 2], x[k]);
      if (k >= 5) x[k - 2] = lift97(x[k - 2], kGamma, x[k - 3], x[k - 1]);
      if (k >= 7) {
        x[k - 3] = lift97(x[k - 3], kDelta, x[k - 4], x[k - 2]);
        emit(k - 2, x[k - 2]);
        emit(k - 3, x[k - 3]);
      }
    }
  }
}

// b - 128 as a float, exactly: the bits of 2^23 + b minus 2^23 + 128.
__device__ __forceinline__ float byte_centered(uint32_t b) {
  return __fsub_rn(__uint_as_float(0x4B000000u | b), 8388736.0f);
}

// One column of the level's input. KIND 0: the previous LL plane; 1: pixels,
// one byte per sample; 2: three interleaved bytes through RCT/ICT.
template <bool REV, int KIND>
struct ColumnSrc {
  using T = typename Cfg<REV>::T;
  const uint8_t* px;  // KIND 1, 2: the column's first byte in row 0
  const T* ll;        // KIND 0: the column's sample in row 0
  size_t pitch;       // bytes (pixels) or samples (LL plane) per row
  int comp;
  float c0, c1, c2;   // the component's ICT row (KIND 2, irreversible)
  __device__ __forceinline__ T operator()(int gy) const {
    if constexpr (KIND == 0) {
      return ll[(size_t)gy * pitch];
    } else if constexpr (KIND == 1) {
      const uint32_t b = px[(size_t)gy * pitch];
      if constexpr (REV) return (int)b - 128;
      else return byte_centered(b);
    } else {
      const uint8_t* q = px + (size_t)gy * pitch;
      const uint32_t r8 = q[0], g8 = q[1], b8 = q[2];
      if constexpr (REV) {  // RCT (src/simd/scalar.rs:173-195)
        const int r = (int)r8 - 128, g = (int)g8 - 128, b = (int)b8 - 128;
        return comp == 0 ? ((r + 2 * g + b) >> 2) : (comp == 1 ? b - g : r - g);
      } else {  // ICT (src/simd/scalar.rs:149-171), evaluated left to right
        return __fadd_rn(__fadd_rn(__fmul_rn(c0, byte_centered(r8)), __fmul_rn(c1, byte_centered(g8))),
                         __fmul_rn(c2, byte_centered(b8)));
      }
    }
  }
};

// Vertical job: rows y_first + LO .. y_first + HI of one column, lifted, the
// 32 outputs (9/7: scaled 1/K on even rows, K on odd ones) written to col.
template <bool REV, int KIND>
__device__ __forceinline__ void vertical_job(const ColumnSrc<REV, KIND>& src, int y_first, int rh,
                                             typename Cfg<REV>::T* col) {
  using T = typename Cfg<REV>::T;
  constexpr int LO = JobRange<REV>::LO, HI = JobRange<REV>::HI;
  T x[RN];
  if (y_first + LO >= 0 && y_first + HI < rh) {
    #pragma unroll
    for (int i = LO; i <= HI; ++i) x[i] = src(y_first + i);
  } else {
    #pragma unroll
    for (int i = LO; i <= HI; ++i) x[i] = src(sym(y_first + i, rh));
  }
  lift_wave<REV>(x, [&](int i, T v) {
    if constexpr (!REV) v = __fmul_rn(v, (i & 1) ? kK : kInvK);
    col[((i & 1) * 32 + ((i - 4) >> 1)) * RP] = v;
  });
}

__device__ __forceinline__ void store_run(uint32_t* dst, const uint32_t (&v)[16]) {
  uint4* d = reinterpret_cast<uint4*>(dst);
  #pragma unroll
  for (int m = 0; m < 4; ++m) d[m] = make_uint4(v[4 * m], v[4 * m + 1], v[4 * m + 2], v[4 * m + 3]);
}

// First sample of code-block row v, column u (a multiple of 16) of a band.
__device__ __forceinline__ uint32_t* slot_at(int32_t* coef, const DwtBandOut& b, int v, int u, int cbs,
                                             int cbhs) {
  const uint32_t blk = b.first_block + (uint32_t)(v >> cbhs) * b.ncbx + (uint32_t)(u >> cbs);
  return reinterpret_cast<uint32_t*>(coef + ((size_t)blk << (cbs + cbhs)) +
                                     ((size_t)(v & ((1 << cbhs) - 1)) << cbs) + (u & ((1 << cbs) - 1)));
}

// One tile of one level (see the comment above RT). The level's arguments
// are read as needed: the caller's copy lives in global memory.
template <bool REV>
__device__ __forceinline__ void dwt_tile(const DwtLevelArgs& args, int comp, int x0, int y0,
                                         typename Cfg<REV>::T* s) {
  using T = typename Cfg<REV>::T;
  constexpr int LO = JobRange<REV>::LO, HI = JobRange<REV>::HI;
  const int rw = args.rw, rh = args.rh;
  const int tid = threadIdx.x;

  // ---- 1. vertical jobs: column lx, rows [32 h, 32 h + 40) of the tile ----
  if (tid < 2 * RSW) {
    const int h = tid >= RSW ? 1 : 0, lx = tid - h * RSW;
    int gx = x0 - RH + lx;
    if ((unsigned)gx >= (unsigned)rw) gx = sym(gx, rw);
    const int y_first = y0 - RH + 32 * h;
    T* col = s + 16 * h * RP + lx;
    if (!args.from_pixels) {
      ColumnSrc<REV, 0> src{};
      src.ll = reinterpret_cast<const T*>(args.src) + (size_t)comp * args.src_comp + gx;
      src.pitch = args.src_pitch;
      vertical_job<REV, 0>(src, y_first, rh, col);
    } else if (!args.mct) {
      ColumnSrc<REV, 1> src{};
      src.px = args.px + (size_t)gx * args.ncomp + comp;
      src.pitch = args.px_pitch;
      vertical_job<REV, 1>(src, y_first, rh, col);
    } else {
      ColumnSrc<REV, 2> src{};
      src.px = args.px + (size_t)gx * 3;
      src.pitch = args.px_pitch;
      src.comp = comp;
      src.c0 = comp == 0 ? 0.299f : comp == 1 ? -0.16875f : 0.5f;
      src.c1 = comp == 0 ? 0.587f : comp == 1 ? -0.33126f : -0.41869f;
      src.c2 = comp == 0 ? 0.114f : comp == 1 ? 0.5f : -0.08131f;
      vertical_job<REV, 2>(src, y_first, rh, col);
    }
  }
  __syncthreads();

  // ---- 2. horizontal jobs: tile row 2 lane + p, columns [32 q, 32 q + 40) ----
  const int warp = tid >> 5, lane = tid & 31;
  if (warp >= 8) return;
  const int p = warp & 1, q = warp >> 1;
  const T* row = s + (p * 32 + lane) * RP + 32 * q;
  T x[RN];
  #pragma unroll
  for (int i = LO; i <= HI; ++i) x[i] = row[i];

  const int cbs = __ffs(args.cbw) - 1, cbhs = __ffs(args.cbh) - 1;
  const int v = (y0 >> 1) + lane;  // band row
  const int u = (x0 >> 1) + 16 * q;  // first band column of both runs
  const bool row_ok = y0 + 2 * lane + p < rh;
  const bool lo_ok = row_ok && u < ((rw + 1) >> 1), hi_ok = row_ok && u < (rw >> 1);
  T* const ll_out = args.ll ? reinterpret_cast<T*>(args.ll) + (size_t)comp * args.ll_comp : nullptr;
  const DwtBandOut bhi = args.band[comp][p ? 3 : 1];  // HL or HH
  uint32_t lo[16], hi[16];
  if (p == 0 && ll_out != nullptr) {
    // even rows of an intermediate level: LL to the next plane, unquantised
    lift_wave<REV>(x, [&](int i, T val) {
      if (i & 1) {
        if constexpr (REV) hi[(i - 5) >> 1] = (uint32_t)val;
        else hi[(i - 5) >> 1] = (uint32_t)quantize(__fmul_rn(val, kK), bhi.step);
      } else {
        if constexpr (REV) lo[(i - 4) >> 1] = (uint32_t)val;
        else lo[(i - 4) >> 1] = __float_as_uint(__fmul_rn(val, kInvK));
      }
    });
    if (lo_ok) store_run(reinterpret_cast<uint32_t*>(ll_out + (size_t)v * args.ll_pitch + u), lo);
  } else {
    const DwtBandOut blo = args.band[comp][p ? 2 : 0];  // LL (last level) or LH
    lift_wave<REV>(x, [&](int i, T val) {
      if (i & 1) {
        if constexpr (REV) hi[(i - 5) >> 1] = (uint32_t)val;
        else hi[(i - 5) >> 1] = (uint32_t)quantize(__fmul_rn(val, kK), bhi.step);
      } else {
        if constexpr (REV) lo[(i - 4) >> 1] = (uint32_t)val;
        else lo[(i - 4) >> 1] = (uint32_t)quantize(__fmul_rn(val, kInvK), blo.step);
      }
    });
    if (lo_ok) store_run(slot_at(args.coef, blo, v, u, cbs, cbhs), lo);
  }
  if (hi_ok) store_run(slot_at(args.coef, bhi, v, u, cbs, cbhs), hi);
}

// Flat tile list over many pages: the CTA finds its page by binary search
// over the tile bases, then its component and tile position.
template <bool REV>
__global__ void __launch_bounds__(RT) dwt_batch_kernel(const DwtLevelArgs* __restrict__ args,
                                                       const uint32_t* __restrict__ tile_base,
                                                       uint32_t npages) {
  __shared__ typename Cfg<REV>::T s[TH * RP];
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
