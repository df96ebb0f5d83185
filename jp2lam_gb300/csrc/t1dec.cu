// Tier-1 decoding on the device: the MQ decoder and the three decoding
// passes of every code-block (decode_codeblock, src/decode/t1.rs:87-210;
// the MQ decoder of src/mq/mod.rs; the context rules of src/tier1/*).
//
// Decoding is sequential within a code-block (every decoded bit changes the
// contexts of the samples after it), so one lane of a warp runs a block's
// decoder while the warp's other lanes wait; a CTA holds 8 such warps.
//  - State: significance, sign, visited and refined flags as 64-bit row
//    masks in shared memory (a row per mask, zero rows above and below).
//    A stripe's rows (4, plus the rows above and below for significance and
//    sign) are held in registers while the stripe is coded, so a sample's
//    neighbourhood is a few shifts.
//  - Skipping: each pass visits only the columns of a stripe that can hold
//    a decision: significance propagation the columns with an insignificant
//    sample next to a significant one (recomputed when a decision makes a
//    sample significant), refinement the columns with a significant
//    unvisited sample, cleanup the columns with an unvisited insignificant
//    one. Samples are still decided in the standard's scan order.
//  - Magnitudes: the decoded bits of a bit-plane are gathered as row masks;
//    after each bit-plane the whole warp ORs them into the component plane
//    (lane l owns columns l and l + 32). At the end it writes the block's
//    signed coefficients (reversible codestreams) or their midpoint
//    dequantised values (irreversible: sign * (|q| + 0.5) * step,
//    src/simd/scalar.rs:122-129) in place.
#include <cuda_runtime.h>

#include <cstring>

#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {

namespace {

constexpr int kDecWarps = 8;
constexpr int kCtxZC0 = 0, kCtxMR = 14, kCtxAGG = 17, kCtxUNI = 18;

struct DecTables {
  uint8_t zc[4 * 512];
  uint8_t sc[256];
  uint8_t spb[256];
  uint32_t mq[94];  // qe | next-MPS index << 16 | next-LPS index << 24; index = 2 state + MPS
};
__constant__ DecTables c_dec;

struct WarpState {
  uint64_t sig[66], sgn[66], vis[66], ref[66];  // row y at y + 1
  uint64_t bits[64];                             // the current bit-plane's decoded 1 bits
  uint8_t ctx[20];
};

// The MQ decoder (ISO/IEC 15444-1 C.3; src/mq/mod.rs): bytes beyond the
// segment read as 0xFF.
struct MqDecoder {
  const uint8_t* b;
  uint32_t n, bp;
  uint32_t a, c, ct;
  uint8_t* ctx;
  __device__ uint32_t at(uint32_t i) const { return i < n ? b[i] : 0xffu; }
  __device__ void bytein() {
    const uint32_t next = at(bp + 1);
    if (at(bp) == 0xffu) {
      if (next > 0x8fu) {
        c += 0xff00u;
        ct = 8;
      } else {
        ++bp;
        c += next << 9;
        ct = 7;
      }
    } else {
      ++bp;
      c += next << 8;
      ct = 8;
    }
  }
  __device__ void init(const uint8_t* data, uint32_t len, uint8_t* contexts) {
    b = data;
    n = len;
    bp = 0;
    ctx = contexts;
    c = n == 0 ? (0xffu << 16) : ((uint32_t)b[0] << 16);
    ct = 0;
    bytein();
    c <<= 7;
    ct = ct >= 7 ? ct - 7 : 0;
    a = 0x8000u;
  }
  __device__ __forceinline__ uint32_t decode(int cx) {
    const uint32_t st = ctx[cx], e = c_dec.mq[st];
    const uint32_t qe = e & 0xffffu, mps = st & 1u;
    uint32_t bit;
    a -= qe;
    if ((c >> 16) < qe) {
      const bool mps_path = a < qe;
      a = qe;
      ctx[cx] = (uint8_t)(mps_path ? (e >> 16) & 0xffu : e >> 24);
      bit = mps_path ? mps : mps ^ 1u;
    } else {
      c -= qe << 16;
      if ((a & 0x8000u) == 0) {
        const bool lps_path = a < qe;
        ctx[cx] = (uint8_t)(lps_path ? e >> 24 : (e >> 16) & 0xffu);
        bit = lps_path ? mps ^ 1u : mps;
      } else {
        return mps;
      }
    }
    // renormalise: shift until a >= 0x8000, reading a byte whenever the bit
    // count runs out first (the one-bit-at-a-time loop of C.3.3, in runs)
    uint32_t n = (uint32_t)__clz(a) - 16u;  // 0 < a < 0x8000 here
    while (n > ct) {
      a <<= ct;
      c <<= ct;
      n -= ct;
      ct = 0;
      bytein();
    }
    a <<= n;
    c <<= n;
    ct -= n;
    return bit;
  }
};

// Bits x-1, x, x+1 of a row mask (bit 0 = column x - 1).
__device__ __forceinline__ uint32_t win3(uint64_t row, int x) {
  return (uint32_t)(x == 0 ? row << 1 : row >> (x - 1)) & 7u;
}
__device__ __forceinline__ uint64_t spread(uint64_t m) { return m | (m << 1) | (m >> 1); }
__device__ __forceinline__ uint64_t above(int x) { return x >= 63 ? 0ull : ~0ull << (x + 1); }

// One stripe's state while it is coded: S/G rows k-1 .. k+4, V/R rows k .. k+3,
// B the stripe's decoded 1 bits of the current bit-plane.
struct Stripe {
  uint64_t S[6], G[6], V[4], R[4], B[4];
};

struct BlockDecoder {
  WarpState& s;
  MqDecoder mq;
  const uint8_t* zc;
  uint64_t wmask;

  // A pass loads (and writes back) only the masks it uses: significance
  // and visited always, signs for the passes that decode signs, refined for
  // the refinement pass (fewer live registers, more decoders per SM).
  template <bool kSigns, bool kRefined>
  __device__ void load(int k, Stripe& t) const {
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      t.S[i] = s.sig[k + i];
      if (kSigns) t.G[i] = s.sgn[k + i];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      t.V[i] = s.vis[k + 1 + i];
      if (kRefined) t.R[i] = s.ref[k + 1 + i];
      t.B[i] = 0;
    }
  }
  template <bool kSigns, bool kRefined>
  __device__ void store(int k, const Stripe& t) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (kSigns) {  // the passes that can make samples significant
        s.sig[k + 1 + i] = t.S[i + 1];
        s.sgn[k + 1 + i] = t.G[i + 1];
        s.vis[k + 1 + i] = t.V[i];
      }
      if (kRefined) s.ref[k + 1 + i] = t.R[i];
      s.bits[k + i] |= t.B[i];
    }
  }

  // Neighbour-significance index of (x, k + r) (bit 0 NW, 1 N, 2 NE, 3 W,
  // 5 E, 6 SW, 7 S, 8 SE; src/tier1/consts.rs).
  template <int r>
  __device__ __forceinline__ uint32_t nmask(const Stripe& t, int x) const {
    const uint32_t up = win3(t.S[r], x), mid = win3(t.S[r + 1], x), dn = win3(t.S[r + 2], x);
    return up | ((mid & 1u) << 3) | ((mid & 4u) << 3) | (dn << 6);
  }

  // Sign of a newly significant sample (src/tier1/helpers.rs:52-88).
  template <int r>
  __device__ __forceinline__ void sign(Stripe& t, int x) {
    const uint64_t bx = 1ull << x;
    const uint32_t sw = win3(t.S[r + 1], x), gw = win3(t.G[r + 1], x);  // bit 0 west, bit 2 east
    const uint32_t ws = sw & 1u, wg = gw & 1u, es = sw >> 2, eg = gw >> 2;
    const uint32_t ns = (uint32_t)(t.S[r] >> x) & 1u, ng = (uint32_t)(t.G[r] >> x) & 1u;
    const uint32_t ss = (uint32_t)(t.S[r + 2] >> x) & 1u, sg = (uint32_t)(t.G[r + 2] >> x) & 1u;
    const uint32_t lu = (ws << 3) | (ws & wg) | (ns << 1) | ((ns & ng) << 4) | (es << 5) | ((es & eg) << 2) |
                        (ss << 7) | ((ss & sg) << 6);
    const uint32_t neg = mq.decode(c_dec.sc[lu]) ^ c_dec.spb[lu];
    t.S[r + 1] |= bx;
    if (neg) t.G[r + 1] |= bx;
  }

  // Columns of the stripe with an insignificant sample next to a
  // significant one.
  __device__ __forceinline__ uint64_t sig_candidates(const Stripe& t, int lim) const {
    uint64_t m = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (r < lim) m |= ~t.S[r + 1] & (spread(t.S[r]) | spread(t.S[r + 2]) | (t.S[r + 1] << 1) | (t.S[r + 1] >> 1));
    return m & wmask;
  }

  template <int r>
  __device__ __forceinline__ bool sig_one(Stripe& t, int x, uint64_t bx) {
    if (t.S[r + 1] & bx) return false;
    const uint32_t nm = nmask<r>(t, x);
    if (!nm) return false;
    const uint32_t bit = mq.decode(zc[nm]);
    t.V[r] |= bx;
    if (!bit) return false;
    t.B[r] |= bx;
    sign<r>(t, x);
    return true;
  }

  __device__ void sigpass(int k, int lim) {
    Stripe t;
    load<true, false>(k, t);
    uint64_t cols = sig_candidates(t, lim);
    while (cols) {
      const int x = __ffsll((long long)cols) - 1;
      const uint64_t bx = 1ull << x;
      bool grew = sig_one<0>(t, x, bx);
      if (lim > 1) grew |= sig_one<1>(t, x, bx);
      if (lim > 2) grew |= sig_one<2>(t, x, bx);
      if (lim > 3) grew |= sig_one<3>(t, x, bx);
      cols &= above(x);
      if (grew) cols = sig_candidates(t, lim) & above(x);
    }
    store<true, false>(k, t);
  }

  template <int r>
  __device__ __forceinline__ void ref_one(Stripe& t, int x, uint64_t bx) {
    if (!(t.S[r + 1] & ~t.V[r] & bx)) return;
    const int cx = (t.R[r] & bx) ? kCtxMR + 2 : (nmask<r>(t, x) ? kCtxMR + 1 : kCtxMR);
    if (mq.decode(cx)) t.B[r] |= bx;
    t.R[r] |= bx;
  }

  __device__ void refpass(int k, int lim) {
    Stripe t;
    load<false, true>(k, t);
    uint64_t cols = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (r < lim) cols |= t.S[r + 1] & ~t.V[r];
    cols &= wmask;
    while (cols) {
      const int x = __ffsll((long long)cols) - 1;
      const uint64_t bx = 1ull << x;
      ref_one<0>(t, x, bx);
      if (lim > 1) ref_one<1>(t, x, bx);
      if (lim > 2) ref_one<2>(t, x, bx);
      if (lim > 3) ref_one<3>(t, x, bx);
      cols &= above(x);
    }
    store<false, true>(k, t);
  }

  template <int r>
  __device__ __forceinline__ void cleanup_one(Stripe& t, int x, uint64_t bx) {
    if ((t.S[r + 1] | t.V[r]) & bx) return;
    const uint32_t nm = nmask<r>(t, x);
    if (mq.decode(nm ? zc[nm] : kCtxZC0)) {
      t.B[r] |= bx;
      sign<r>(t, x);
    }
  }

  __device__ void cleanup(int k, int lim) {
    Stripe t;
    load<true, false>(k, t);
    uint64_t busy = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (r < lim) busy |= t.S[r + 1] | t.V[r];
    uint64_t cols = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (r < lim) cols |= ~(t.S[r + 1] | t.V[r]);
    cols &= wmask;
    while (cols) {
      const int x = __ffsll((long long)cols) - 1;
      const uint64_t bx = 1ull << x;
      cols &= above(x);
      // a full stripe's column with nothing significant or visited in it or
      // around it is coded as a run (src/tier1/flags.rs:219-235)
      if (lim == 4 && !(busy & bx) && win3(t.S[0] | t.S[1] | t.S[2] | t.S[3] | t.S[4] | t.S[5], x) == 0) {
        if (mq.decode(kCtxAGG) == 0) continue;
        int rl = (int)mq.decode(kCtxUNI) << 1;
        rl |= (int)mq.decode(kCtxUNI);
        if (rl == 0) {
          t.B[0] |= bx;
          sign<0>(t, x);
          cleanup_one<1>(t, x, bx);
          cleanup_one<2>(t, x, bx);
          cleanup_one<3>(t, x, bx);
        } else if (rl == 1) {
          t.B[1] |= bx;
          sign<1>(t, x);
          cleanup_one<2>(t, x, bx);
          cleanup_one<3>(t, x, bx);
        } else if (rl == 2) {
          t.B[2] |= bx;
          sign<2>(t, x);
          cleanup_one<3>(t, x, bx);
        } else {
          t.B[3] |= bx;
          sign<3>(t, x);
        }
      } else {
        cleanup_one<0>(t, x, bx);
        if (lim > 1) cleanup_one<1>(t, x, bx);
        if (lim > 2) cleanup_one<2>(t, x, bx);
        if (lim > 3) cleanup_one<3>(t, x, bx);
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) t.V[r] = 0;
    store<true, false>(k, t);
  }
};

// H decoders per warp: with H = 2 each half-warp decodes its own block
// (its lane 0 running the chain, its 16 lanes merging), so two chains share
// a warp's instruction stream: more decoders per SM for batches, at some
// cost to each chain where the two diverge.
template <int H>
__global__ void __launch_bounds__(kDecWarps * 32) t1_decode_kernel(const DecBlock* blocks, uint32_t nblocks,
                                                                     const uint8_t* data, int32_t* planes) {
  constexpr int HL = 32 / H;  // lanes per decoder
  constexpr int NX = 64 / HL;  // columns each lane merges
  __shared__ WarpState st_all[kDecWarps * H];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int half = lane / HL, hl = lane % HL;
  const uint32_t hmask = H == 1 ? 0xffffffffu : (0xffffu << (16 * half));
  const uint32_t blk = (blockIdx.x * kDecWarps + wid) * H + half;
  if (blk >= nblocks) return;
  WarpState& s = st_all[wid * H + half];
  const DecBlock d = blocks[blk];
  for (int i = hl; i < 66; i += HL) s.sig[i] = s.sgn[i] = s.vis[i] = s.ref[i] = 0;
  for (int i = hl; i < 64; i += HL) s.bits[i] = 0;
  // initial context states (src/mq/mod.rs:195-200)
  for (int i = hl; i < 20; i += HL) s.ctx[i] = i == kCtxUNI ? 92 : i == kCtxAGG ? 6 : i == kCtxZC0 ? 8 : 0;
  int32_t* plane = planes + d.plane_off;
  const int w = d.w, h = d.h;
  __syncwarp(hmask);
  BlockDecoder dec{s, {}, c_dec.zc + (d.orient & 3) * 512, w == 64 ? ~0ull : (1ull << w) - 1};
  if (hl == 0 && d.npasses > 0) dec.mq.init(data + d.data_off, d.data_len, s.ctx);
  // pass sequence: cleanup of the top bit-plane, then significance,
  // refinement and cleanup per bit-plane until the block's passes end
  const int top = (int)d.mb - (int)d.zbp - 1;  // checked on the host: 0..30
  int remaining = d.npasses;
  for (int bp = top; bp >= 0 && remaining > 0; --bp) {
    if (hl == 0) {
      if (bp < top) {
        for (int k = 0; k < h; k += 4) dec.sigpass(k, min(4, h - k));
        if (--remaining > 0) {
          for (int k = 0; k < h; k += 4) dec.refpass(k, min(4, h - k));
          if (--remaining > 0) {
            for (int k = 0; k < h; k += 4) dec.cleanup(k, min(4, h - k));
            --remaining;
          }
        }
      } else {
        for (int k = 0; k < h; k += 4) dec.cleanup(k, min(4, h - k));
        --remaining;
      }
    } else {
      remaining -= bp < top ? min(3, remaining) : 1;
    }
    __syncwarp(hmask);
    const int32_t one = (int32_t)(1u << bp);
    for (int y = 0; y < h; ++y) {
      const uint64_t bits = s.bits[y];
      if (!bits) continue;
      int32_t* row = plane + (size_t)y * d.stride;
#pragma unroll
      for (int m = 0; m < NX; ++m) {
        const int x = hl + HL * m;
        if (x < w && ((bits >> x) & 1u)) row[x] |= one;
      }
    }
    __syncwarp(hmask);
    for (int i = hl; i < 64; i += HL) s.bits[i] = 0;
    __syncwarp(hmask);
  }
  // signed coefficients, or their midpoint dequantised values
  for (int y = 0; y < h; ++y) {
    const uint64_t neg = s.sgn[y + 1];
    int32_t* row = plane + (size_t)y * d.stride;
#pragma unroll
    for (int m = 0; m < NX; ++m) {
      const int x = hl + HL * m;
      if (x >= w) continue;
      const int32_t mag = row[x];
      const bool n = (neg >> x) & 1u;
      if (d.reversible) {
        row[x] = n ? -mag : mag;
      } else {
        float v = 0.0f;
        if (mag != 0) v = __fmul_rn(__fmul_rn(n ? -1.0f : 1.0f, __fadd_rn((float)(uint32_t)mag, 0.5f)), d.step);
        row[x] = __float_as_int(v);
      }
    }
  }
}

}  // namespace

bool upload_decode_tables(const uint8_t* zc, const uint8_t* sc, const uint8_t* spb, const uint32_t* mq) {
  DecTables t;
  memcpy(t.zc, zc, sizeof t.zc);
  memcpy(t.sc, sc, sizeof t.sc);
  memcpy(t.spb, spb, sizeof t.spb);
  memcpy(t.mq, mq, sizeof t.mq);
  return cudaMemcpyToSymbol(c_dec, &t, sizeof t) == cudaSuccess;
}

void launch_t1_decode(const DecBlock* blocks, uint32_t nblocks, const uint8_t* data, int32_t* planes, int per_warp,
                      cudaStream_t st) {
  if (nblocks == 0) return;
  if (per_warp == 2) {
    const uint32_t per_cta = kDecWarps * 2;
    t1_decode_kernel<2><<<(nblocks + per_cta - 1) / per_cta, kDecWarps * 32, 0, st>>>(blocks, nblocks, data, planes);
  } else {
    t1_decode_kernel<1><<<(nblocks + kDecWarps - 1) / kDecWarps, kDecWarps * 32, 0, st>>>(blocks, nblocks, data,
                                                                                           planes);
  }
}

}  // namespace jp2g
