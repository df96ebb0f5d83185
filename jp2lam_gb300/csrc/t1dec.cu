// Tier-1 decoding on the device: the MQ decoder and the three decoding
// passes of every code-block (decode_tile_components / the block decoder of
// src/decode/t1.rs:87-210, MqDecoder of src/mq/mod.rs, the context rules of
// src/tier1/*).
//
// Decoding is sequential within a code-block (every decoded bit changes the
// contexts of the samples after it), so one lane of a warp decodes one
// block, its significance, visited, refined and sign states held as 64-bit
// row masks in shared memory (a row per mask and row, zero rows above and
// below), from which a sample's neighbourhood is a few shifts. The decoded
// magnitudes accumulate in the component plane; at the end the whole warp
// writes the block's signed coefficients (reversible codestreams) or their
// midpoint dequantised values (irreversible: sign * (|q| + 0.5) * step,
// src/simd/scalar.rs:122-129) in place.
#include <cuda_runtime.h>

#include <cstring>

#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {

namespace {

constexpr int kDecWarps = 4;
constexpr int kCtxZC0 = 0, kCtxMR = 14, kCtxAGG = 17, kCtxUNI = 18;

struct DecTables {
  uint8_t zc[4 * 512];
  uint8_t sc[256];
  uint8_t spb[256];
  uint32_t mq[94];  // qe | next-MPS index << 16 | next-LPS index << 24; index = 2 state + MPS
};
__constant__ DecTables c_dec;

struct BlockState {
  uint64_t sig[66], vis[66], ref[66], sgn[66];  // row y at y + 1
  uint8_t ctx[20];
};

// The MQ decoder (ISO/IEC 15444-1 C.3; src/mq/mod.rs): bytes beyond the
// segment read as 0xFF.
struct MqDecoder {
  const uint8_t* b;
  uint32_t n, bp;
  uint32_t a, c, ct;
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
  __device__ void init(const uint8_t* data, uint32_t len) {
    b = data;
    n = len;
    bp = 0;
    c = n == 0 ? (0xffu << 16) : ((uint32_t)b[0] << 16);
    ct = 0;
    bytein();
    c <<= 7;
    ct = ct >= 7 ? ct - 7 : 0;
    a = 0x8000u;
  }
  __device__ uint32_t decode(uint8_t* ctx, int cx) {
    const uint32_t st = ctx[cx], e = c_dec.mq[st];
    const uint32_t qe = e & 0xffffu, mps = st & 1u;
    uint32_t bit;
    a -= qe;
    if ((c >> 16) < qe) {
      const uint32_t post = a;
      a = qe;
      if (post < qe) {
        ctx[cx] = (uint8_t)((e >> 16) & 0xffu);
        bit = mps;
      } else {
        ctx[cx] = (uint8_t)(e >> 24);
        bit = mps ^ 1u;
      }
    } else {
      c -= qe << 16;
      if ((a & 0x8000u) == 0) {
        if (a < qe) {
          ctx[cx] = (uint8_t)(e >> 24);
          bit = mps ^ 1u;
        } else {
          ctx[cx] = (uint8_t)((e >> 16) & 0xffu);
          bit = mps;
        }
      } else {
        bit = mps;
      }
    }
    while (a < 0x8000u) {
      if (ct == 0) bytein();
      a <<= 1;
      c <<= 1;
      --ct;
    }
    return bit;
  }
};

// Bits x-1, x, x+1 of a row mask (bit 0 = column x - 1).
__device__ __forceinline__ uint32_t win3(uint64_t row, int x) {
  return (uint32_t)(x == 0 ? row << 1 : row >> (x - 1)) & 7u;
}

struct BlockDecoder {
  BlockState& s;
  MqDecoder mq;
  int w, h;
  const uint8_t* zc;
  int32_t* plane;  // the block's first sample; rows `stride` apart
  uint32_t stride;

  // Neighbour-significance index (bit 0 NW, 1 N, 2 NE, 3 W, 5 E, 6 SW, 7 S,
  // 8 SE) of sample (x, y) in the current state.
  __device__ uint32_t nmask(int x, int y) const {
    const uint32_t up = win3(s.sig[y], x), mid = win3(s.sig[y + 1], x), dn = win3(s.sig[y + 2], x);
    return up | ((mid & 1u) << 3) | ((mid & 4u) << 3) | (dn << 6);
  }
  __device__ bool bit_at(const uint64_t* m, int x, int y) const { return (m[y + 1] >> x) & 1u; }
  __device__ void set(uint64_t* m, int x, int y) { m[y + 1] |= 1ull << x; }
  __device__ void clear(uint64_t* m, int x, int y) { m[y + 1] &= ~(1ull << x); }
  __device__ void add_magnitude(int x, int y, uint32_t one) { plane[(size_t)y * stride + x] |= (int32_t)one; }

  // Sign of a newly significant sample (src/tier1/helpers.rs:52-88).
  __device__ void decode_sign(int x, int y) {
    const uint32_t ws = x > 0 && bit_at(s.sig, x - 1, y), wg = x > 0 && bit_at(s.sgn, x - 1, y);
    const uint32_t es = x + 1 < w && bit_at(s.sig, x + 1, y), eg = x + 1 < w && bit_at(s.sgn, x + 1, y);
    const uint32_t ns = (s.sig[y] >> x) & 1u, ng = (s.sgn[y] >> x) & 1u;
    const uint32_t ss = (s.sig[y + 2] >> x) & 1u, sg = (s.sgn[y + 2] >> x) & 1u;
    const uint32_t lu = (ws << 3) | (ws & wg) | (ns << 1) | ((ns & ng) << 4) | (es << 5) | ((es & eg) << 2) |
                        (ss << 7) | ((ss & sg) << 6);
    const uint32_t sign = mq.decode(s.ctx, c_dec.sc[lu]) ^ c_dec.spb[lu];
    set(s.sig, x, y);
    if (sign) set(s.sgn, x, y);
  }

  __device__ void sigpass_step(int x, int y, uint32_t one) {
    if (bit_at(s.sig, x, y)) return;
    const uint32_t nm = nmask(x, y);
    if (nm == 0) return;
    const uint32_t bit = mq.decode(s.ctx, zc[nm]);
    set(s.vis, x, y);
    if (bit) {
      add_magnitude(x, y, one);
      decode_sign(x, y);
    }
  }
  __device__ void refpass_step(int x, int y, uint32_t one) {
    if (!bit_at(s.sig, x, y) || bit_at(s.vis, x, y)) return;
    const int cx = bit_at(s.ref, x, y) ? kCtxMR + 2 : (nmask(x, y) ? kCtxMR + 1 : kCtxMR);
    if (mq.decode(s.ctx, cx)) add_magnitude(x, y, one);
    set(s.ref, x, y);
  }
  __device__ void cleanup_step(int x, int y, uint32_t one) {
    if (bit_at(s.sig, x, y) || bit_at(s.vis, x, y)) {
      clear(s.vis, x, y);
      return;
    }
    const uint32_t nm = nmask(x, y);
    const uint32_t bit = mq.decode(s.ctx, nm ? zc[nm] : kCtxZC0);
    clear(s.vis, x, y);
    if (bit) {
      add_magnitude(x, y, one);
      decode_sign(x, y);
    }
  }
  // A full stripe's column with nothing significant or visited in it or
  // around it codes as a run (src/tier1/flags.rs:219-235).
  __device__ bool clean(int x, int k) const {
    for (int r = 0; r < 4; ++r)
      if (bit_at(s.sig, x, k + r) || bit_at(s.vis, x, k + r) || nmask(x, k + r)) return false;
    return true;
  }

  __device__ void sigpass(int bp) {
    const uint32_t one = 1u << bp;
    for (int k = 0; k < h; k += 4) {
      const int lim = min(4, h - k);
      for (int x = 0; x < w; ++x)
        for (int r = 0; r < lim; ++r) sigpass_step(x, k + r, one);
    }
  }
  __device__ void refpass(int bp) {
    const uint32_t one = 1u << bp;
    for (int k = 0; k < h; k += 4) {
      const int lim = min(4, h - k);
      for (int x = 0; x < w; ++x)
        for (int r = 0; r < lim; ++r) refpass_step(x, k + r, one);
    }
  }
  __device__ void cleanup(int bp) {
    const uint32_t one = 1u << bp;
    for (int k = 0; k < h; k += 4) {
      const int lim = min(4, h - k);
      for (int x = 0; x < w; ++x) {
        if (lim == 4 && clean(x, k)) {
          if (mq.decode(s.ctx, kCtxAGG) == 0) continue;
          int rl = (int)mq.decode(s.ctx, kCtxUNI) << 1;
          rl |= (int)mq.decode(s.ctx, kCtxUNI);
          add_magnitude(x, k + rl, one);
          decode_sign(x, k + rl);
          clear(s.vis, x, k + rl);
          for (int r = rl + 1; r < 4; ++r) cleanup_step(x, k + r, one);
        } else {
          for (int r = 0; r < lim; ++r) cleanup_step(x, k + r, one);
        }
      }
    }
    for (int y = 0; y < h; ++y) s.vis[y + 1] = 0;
  }
};

__global__ void __launch_bounds__(kDecWarps * 32) t1_decode_kernel(DecodeArgs a) {
  __shared__ BlockState st_all[kDecWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t blk = blockIdx.x * kDecWarps + wid;
  if (blk >= a.nblocks) return;
  BlockState& s = st_all[wid];
  const DecBlock d = a.blocks[blk];
  for (int i = lane; i < 66; i += 32) s.sig[i] = s.vis[i] = s.ref[i] = s.sgn[i] = 0;
  int32_t* plane = a.plane + (size_t)d.comp * a.width * a.height + (size_t)d.y0 * a.width + d.x0;
  __syncwarp();
  if (lane == 0 && d.npasses > 0) {
    for (int i = 0; i < 20; ++i) s.ctx[i] = 0;
    s.ctx[kCtxUNI] = 92;  // src/mq/mod.rs:195-200
    s.ctx[kCtxAGG] = 6;
    s.ctx[kCtxZC0] = 8;
    BlockDecoder dec{s, {}, d.w, d.h, c_dec.zc + (d.orient & 3) * 512, plane, a.width};
    dec.mq.init(a.data + d.data_off, d.data_len);
    const int top = (int)d.mb - (int)d.zbp - 1;  // checked on the host: 0..30
    int remaining = d.npasses;
    dec.cleanup(top);
    --remaining;
    for (int bp = top - 1; bp >= 0 && remaining > 0; --bp) {
      dec.sigpass(bp);
      if (--remaining == 0) break;
      dec.refpass(bp);
      if (--remaining == 0) break;
      dec.cleanup(bp);
      --remaining;
    }
  }
  __syncwarp();
  // signed coefficients, or their midpoint dequantised values
  for (int i = lane; i < d.w * d.h; i += 32) {
    const int y = i / d.w, x = i - y * d.w;
    int32_t* p = plane + (size_t)y * a.width + x;
    const int32_t m = *p;
    const bool neg = (s.sgn[y + 1] >> x) & 1u;
    if (a.reversible) {
      *p = neg ? -m : m;
    } else {
      float v = 0.0f;
      if (m != 0) v = __fmul_rn(__fmul_rn(neg ? -1.0f : 1.0f, __fadd_rn((float)(uint32_t)m, 0.5f)), d.step);
      *p = __float_as_int(v);
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

void launch_t1_decode(const DecodeArgs& a, cudaStream_t st) {
  if (a.nblocks == 0) return;
  t1_decode_kernel<<<(a.nblocks + kDecWarps - 1) / kDecWarps, kDecWarps * 32, 0, st>>>(a);
}

}  // namespace jp2g
