// EBCOT Tier-1 encoder: one warp per code-block, single MQ termination per
// block, per-pass numbytes() snapshots for rate control.
//
// Replaces analyze_codeblock (src/encode/backend/native/t1.rs:215-258) and
// encode_codeblock_single_term (t1.rs:508-658) with its passes (SP
// t1.rs:805-905, MR t1.rs:914-965, cleanup t1.rs:977-1197) and the MQ coder
// (src/mq/mod.rs:163-432).
//
// State lives in shared memory as 64-bit row masks (bit x = column x):
// significance and coefficient sign (with a zero row above and below),
// visited, refined, and a window of magnitude bit-planes built once per block
// by warp ballots. The whole warp loads the block and builds the masks; lane 0
// then walks the passes in the reference's exact scan order (4-row stripes,
// columns left to right, rows top to bottom) and drives the MQ coder, using
// the masks to jump straight to the columns a pass can touch. The byte stream
// goes directly to the block's payload slot in global memory.
#include <cuda_runtime.h>

#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {

namespace {

constexpr int kWarps = 4;
constexpr int kNBP = 16;  // magnitude bit-planes held in shared memory at once

// Context numbers (src/mq/mod.rs:5-10).
constexpr int kCtxAGG = 17, kCtxUNI = 18;

struct Tables {
  uint8_t zc[4 * 512];
  uint8_t sc[256];
  uint8_t spb[256];
  uint32_t mq[94];  // qe | nmps << 16 | nlps << 24
};

// Built on the host from the standard's rules and copied in at launch.
__constant__ Tables c_tables;

struct WarpState {
  uint64_t bp[kNBP][64];  // magnitude bit-plane window
  uint64_t sig[68];       // row y at index y+1; rows -1 and h.. stay zero
  uint64_t sgn[68];       // coefficient sign, same indexing
  uint64_t vis[64];
  uint64_t ref[64];
  uint8_t ctx[20];
};

struct Mq {
  uint32_t a, c, ct;
  int pos;        // index of the last written byte; 0 is the pre-byte
  uint32_t last;  // value of that byte
  uint8_t* out;   // out[k] holds byte k+1
  int cap;
  int ovf;
};

__device__ __forceinline__ void mq_emit(Mq& m, uint32_t b) {
  ++m.pos;
  m.last = b & 0xffu;
  if (m.pos <= m.cap) m.out[m.pos - 1] = (uint8_t)m.last;
  else m.ovf = 1;
}

// BYTEOUT with carry propagation and 0xFF bit stuffing (src/mq/mod.rs:382-404).
__device__ __forceinline__ void mq_byteout(Mq& m) {
  if (m.last == 0xffu) {
    mq_emit(m, m.c >> 20);
    m.c &= 0xfffffu;
    m.ct = 7;
  } else if ((m.c & 0x8000000u) == 0) {
    mq_emit(m, m.c >> 19);
    m.c &= 0x7ffffu;
    m.ct = 8;
  } else {
    m.last = (m.last + 1) & 0xffu;
    if (m.pos >= 1 && m.pos <= m.cap) m.out[m.pos - 1] = (uint8_t)m.last;
    if (m.last == 0xffu) {
      m.c &= 0x7ffffffu;
      mq_emit(m, m.c >> 20);
      m.c &= 0xfffffu;
      m.ct = 7;
    } else {
      mq_emit(m, m.c >> 19);
      m.c &= 0x7ffffu;
      m.ct = 8;
    }
  }
}

// RENORME: shift until A >= 0x8000, emitting a byte whenever CT runs out.
__device__ __forceinline__ void mq_renorm(Mq& m) {
  uint32_t n = __clz(m.a) - 16;
  m.a <<= n;
  while (n >= m.ct) {
    m.c <<= m.ct;
    n -= m.ct;
    mq_byteout(m);
  }
  m.c <<= n;
  m.ct -= n;
}

__device__ __forceinline__ void mq_encode(Mq& m, uint8_t* ctx, int cx, uint32_t bit) {
  uint32_t st = ctx[cx];
  uint32_t e = c_tables.mq[st];
  uint32_t qe = e & 0xffffu;
  m.a -= qe;
  if (bit == (st & 1u)) {
    if ((m.a & 0x8000u) == 0) {
      if (m.a < qe) m.a = qe;
      else m.c += qe;
      ctx[cx] = (uint8_t)((e >> 16) & 0xff);
      mq_renorm(m);
    } else {
      m.c += qe;
    }
  } else {
    if (m.a < qe) m.c += qe;
    else m.a = qe;
    ctx[cx] = (uint8_t)(e >> 24);
    mq_renorm(m);
  }
}

__device__ __forceinline__ void mq_flush(Mq& m) {  // src/mq/mod.rs:244-250, 373-379
  uint32_t t = m.c + m.a;
  m.c |= 0xffffu;
  if (m.c >= t) m.c -= 0x8000u;
  m.c <<= m.ct;
  mq_byteout(m);
  m.c <<= m.ct;
  mq_byteout(m);
}

__device__ __forceinline__ uint32_t win3(uint64_t r, int x) {
  return x == 0 ? (uint32_t)((r << 1) & 7u) : (uint32_t)((r >> (x - 1)) & 7u);
}

// Neighbour significance mask (NW N NE W . E SW S SE -> bits 0..8).
__device__ __forceinline__ uint32_t nmask(const uint64_t* S, int x, int y) {
  return win3(S[y], x) | ((win3(S[y + 1], x) & 5u) << 3) | (win3(S[y + 2], x) << 6);
}

// Sign-context index from the four cardinal neighbours
// (src/tier1/helpers.rs:52-88, src/tier1/flags.rs:237-296).
__device__ __forceinline__ uint32_t sign_lu(const uint64_t* S, const uint64_t* G, int x, int y) {
  uint32_t lu = 0;
  uint64_t mid = S[y + 1], gm = G[y + 1];
  if (x > 0 && ((mid >> (x - 1)) & 1)) lu |= 8u | (uint32_t)((gm >> (x - 1)) & 1);
  if ((S[y] >> x) & 1) lu |= 2u | ((uint32_t)((G[y] >> x) & 1) << 4);
  if (x < 63 && ((mid >> (x + 1)) & 1)) lu |= 32u | ((uint32_t)((gm >> (x + 1)) & 1) << 2);
  if ((S[y + 2] >> x) & 1) lu |= 128u | ((uint32_t)((G[y + 2] >> x) & 1) << 6);
  return lu;
}

struct Block {
  int w, h;
  uint64_t valid;
  const uint8_t* zc;
};

// Codes the sign of a sample that just became significant and marks it.
__device__ __forceinline__ void code_sign(Mq& m, WarpState& ws, int x, int y) {
  uint32_t lu = sign_lu(ws.sig, ws.sgn, x, y);
  uint32_t s = (uint32_t)((ws.sgn[y + 1] >> x) & 1);
  mq_encode(m, ws.ctx, c_tables.sc[lu], s ^ c_tables.spb[lu]);
  ws.sig[y + 1] |= 1ull << x;
}

// Significance propagation (t1.rs:805-905).
__device__ uint32_t sig_pass(Mq& m, WarpState& ws, const Block& b, const uint64_t* bpm) {
  uint32_t ns = 0;
  uint64_t* S = ws.sig;
  for (int k = 0; k < b.h; k += 4) {
    const int lim = min(4, b.h - k);
    int x = 0;
    while (x < b.w) {
      uint64_t any = 0, all = ~0ull;
      for (int r = 0; r < lim + 2; ++r) any |= S[k + r];
      for (int r = 0; r < lim; ++r) all &= S[k + 1 + r];
      uint64_t cand = (any | (any << 1) | (any >> 1)) & ~all & b.valid & (~0ull << x);
      if (cand == 0) break;
      x = __ffsll((long long)cand) - 1;
      const uint64_t bx = 1ull << x;
      for (int ci = 0; ci < lim; ++ci) {
        const int y = k + ci;
        if (S[y + 1] & bx) continue;
        uint32_t nm = nmask(S, x, y);
        if (nm == 0) continue;
        uint32_t bit = (uint32_t)((bpm[y] >> x) & 1);
        mq_encode(m, ws.ctx, b.zc[nm], bit);
        ws.vis[y] |= bx;
        if (bit) {
          code_sign(m, ws, x, y);
          ++ns;
        }
      }
      ++x;
    }
  }
  return ns;
}

// Magnitude refinement (t1.rs:914-965).
__device__ void ref_pass(Mq& m, WarpState& ws, const Block& b, const uint64_t* bpm) {
  uint64_t* S = ws.sig;
  for (int k = 0; k < b.h; k += 4) {
    const int lim = min(4, b.h - k);
    uint64_t col = 0;
    for (int ci = 0; ci < lim; ++ci) col |= S[k + ci + 1] & ~ws.vis[k + ci];
    while (col) {
      const int x = __ffsll((long long)col) - 1;
      col &= col - 1;
      const uint64_t bx = 1ull << x;
      for (int ci = 0; ci < lim; ++ci) {
        const int y = k + ci;
        if (!(S[y + 1] & ~ws.vis[y] & bx)) continue;
        int cx = (ws.ref[y] & bx) ? 16 : (nmask(S, x, y) ? 15 : 14);  // helpers.rs:36-50
        mq_encode(m, ws.ctx, cx, (uint32_t)((bpm[y] >> x) & 1));
        ws.ref[y] |= bx;
      }
    }
  }
}

// Regular (non run-length) cleanup step; returns true if the sample became
// significant (t1.rs:1150-1197).
__device__ __forceinline__ bool cl_sample(Mq& m, WarpState& ws, const Block& b,
                                          const uint64_t* bpm, int x, int y) {
  const uint64_t bx = 1ull << x;
  if ((ws.sig[y + 1] | ws.vis[y]) & bx) return false;
  uint32_t nm = nmask(ws.sig, x, y);
  uint32_t bit = (uint32_t)((bpm[y] >> x) & 1);
  mq_encode(m, ws.ctx, nm ? b.zc[nm] : 0, bit);
  if (bit) code_sign(m, ws, x, y);
  return bit != 0;
}

// Columns of a full stripe that qualify for run-length coding: no sample
// significant or visited, no significant neighbour (flags.rs:219-235).
__device__ __forceinline__ uint64_t clean_cols(const WarpState& ws, int k, uint64_t valid) {
  uint64_t sv = 0, any = 0;
  for (int ci = 0; ci < 4; ++ci) sv |= ws.sig[k + ci + 1] | ws.vis[k + ci];
  for (int r = 0; r < 6; ++r) any |= ws.sig[k + r];
  return ~(sv | any | (any << 1) | (any >> 1)) & valid;
}

// Cleanup pass (t1.rs:977-1148).
__device__ uint32_t cleanup_pass(Mq& m, WarpState& ws, const Block& b, const uint64_t* bpm) {
  uint32_t ns = 0;
  const int full = b.h & ~3;
  for (int k = 0; k < full; k += 4) {
    uint64_t clean = clean_cols(ws, k, b.valid);
    for (int x = 0; x < b.w; ++x) {
      const uint64_t bx = 1ull << x;
      if (clean & bx) {
        uint32_t nib = (uint32_t)((bpm[k] >> x) & 1) | ((uint32_t)((bpm[k + 1] >> x) & 1) << 1) |
                       ((uint32_t)((bpm[k + 2] >> x) & 1) << 2) | ((uint32_t)((bpm[k + 3] >> x) & 1) << 3);
        if (nib == 0) {
          mq_encode(m, ws.ctx, kCtxAGG, 0);
          continue;
        }
        const int rl = __ffs(nib) - 1;
        mq_encode(m, ws.ctx, kCtxAGG, 1);
        mq_encode(m, ws.ctx, kCtxUNI, (uint32_t)(rl >> 1) & 1);
        mq_encode(m, ws.ctx, kCtxUNI, (uint32_t)rl & 1);
        code_sign(m, ws, x, k + rl);
        ++ns;
        for (int ci = rl + 1; ci < 4; ++ci) ns += cl_sample(m, ws, b, bpm, x, k + ci);
        clean = clean_cols(ws, k, b.valid);
      } else {
        bool changed = false;
        for (int ci = 0; ci < 4; ++ci) {
          bool s = cl_sample(m, ws, b, bpm, x, k + ci);
          ns += s;
          changed |= s;
        }
        if (changed) clean = clean_cols(ws, k, b.valid);
      }
    }
  }
  if (full < b.h) {  // partial stripe: never run-length coded
    const int lim = b.h - full;
    for (int x = 0; x < b.w; ++x)
      for (int ci = 0; ci < lim; ++ci) ns += cl_sample(m, ws, b, bpm, x, full + ci);
  }
  for (int y = 0; y < b.h; ++y) ws.vis[y] = 0;  // clear_visited_all
  return ns;
}

// Builds bit-planes [base, base+kNBP) of the block's magnitudes, one ballot
// per row half.
__device__ void build_planes(WarpState& ws, const int32_t* blk, int cbw, int w, int h, int base,
                             int top, int lane) {
  for (int y = 0; y < h; ++y) {
    int32_t v0 = lane < w ? blk[y * cbw + lane] : 0;
    int32_t v1 = lane + 32 < w ? blk[y * cbw + lane + 32] : 0;
    uint32_t m0 = v0 < 0 ? (uint32_t)(-(int64_t)v0) : (uint32_t)v0;
    uint32_t m1 = v1 < 0 ? (uint32_t)(-(int64_t)v1) : (uint32_t)v1;
    for (int p = base; p < top && p < base + kNBP; ++p) {
      uint32_t lo = __ballot_sync(0xffffffffu, (m0 >> p) & 1);
      uint32_t hi = __ballot_sync(0xffffffffu, (m1 >> p) & 1);
      if (lane == 0) ws.bp[p - base][y] = (uint64_t)lo | ((uint64_t)hi << 32);
    }
  }
}

__global__ void __launch_bounds__(kWarps * 32) t1_kernel(T1Args a) {
  __shared__ WarpState states[kWarps];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  WarpState& ws = states[wid];
  const uint32_t gwarp = blockIdx.x * kWarps + wid;
  const uint32_t nwarps = gridDim.x * kWarps;

  for (uint32_t bi = gwarp; bi < a.nblocks; bi += nwarps) {
    const BlockDesc d = a.blocks[bi];
    const int w = d.w, h = d.h;
    const int32_t* blk = a.coef + (size_t)d.coef_slot * a.cbw * a.cbh;

    // ---- analysis: max magnitude, non-zero count, signs ----
    uint32_t mx = 0, nnz = 0;
    for (int y = 0; y < h; ++y) {
      int32_t v0 = lane < w ? blk[y * a.cbw + lane] : 0;
      int32_t v1 = lane + 32 < w ? blk[y * a.cbw + lane + 32] : 0;
      uint32_t m0 = v0 < 0 ? (uint32_t)(-(int64_t)v0) : (uint32_t)v0;
      uint32_t m1 = v1 < 0 ? (uint32_t)(-(int64_t)v1) : (uint32_t)v1;
      mx = max(mx, max(m0, m1));
      nnz += __popc(__ballot_sync(0xffffffffu, v0 != 0)) + __popc(__ballot_sync(0xffffffffu, v1 != 0));
      uint32_t s0 = __ballot_sync(0xffffffffu, v0 < 0), s1 = __ballot_sync(0xffffffffu, v1 < 0);
      if (lane == 0) ws.sgn[y + 1] = (uint64_t)s0 | ((uint64_t)s1 << 32);
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    const int mbp = mx == 0 ? 0 : 32 - __clz(mx);
    const int zbp = d.mb > mbp ? d.mb - mbp : 0;
    // classify_from_nonzero_fraction (src/profile.rs:122-130), in f32.
    const float frac = __fdiv_rn((float)nnz, (float)(w * h));
    const int cls = mbp == 0 ? 0 : (frac <= 0.05f ? 0 : (frac <= 0.30f ? 1 : 2));
    const uint32_t npasses = mbp == 0 ? 0u : 1u + 3u * (uint32_t)(mbp - 1);

    if (mbp == 0 || npasses > a.pass_cap) {
      if (lane == 0) {
        BlockOut o{};
        o.payload_len = 0;
        o.npasses = 0;
        o.mbp = (uint8_t)mbp;
        o.zbp = (uint8_t)zbp;
        o.cls = (uint8_t)cls;
        o.status = mbp == 0 ? 0 : 2;
        a.res[bi] = o;
      }
      __syncwarp();
      continue;
    }

    // ---- state init ----
    for (int i = lane; i < 68; i += 32) ws.sig[i] = 0;
    if (lane == 0) { ws.sgn[0] = 0; }
    for (int i = h + 1 + lane; i < 68; i += 32) ws.sgn[i] = 0;
    for (int i = lane; i < 64; i += 32) { ws.vis[i] = 0; ws.ref[i] = 0; }
    if (lane < 20) ws.ctx[lane] = 0;
    __syncwarp();
    if (lane == 0) {  // src/mq/mod.rs:195-200
      ws.ctx[kCtxUNI] = 92;
      ws.ctx[kCtxAGG] = 6;
      ws.ctx[0] = 8;
    }
    int base = mbp > kNBP ? mbp - kNBP : 0;
    build_planes(ws, blk, a.cbw, w, h, base, mbp, lane);
    __syncwarp();

    Mq m{0x8000u, 0u, 12u, 0, 0u, a.out + d.out_off, (int)d.out_cap, 0};
    Block b{w, h, w == 64 ? ~0ull : ((1ull << w) - 1), c_tables.zc + d.orient * 512};
    PassRec* pr = a.passes + d.pass_off;
    uint32_t sig_so_far = 0;
    int pi = 0;

    for (int p = mbp - 1; p >= 0; --p) {
      if (p < base) {
        base = p + 1 > kNBP ? p + 1 - kNBP : 0;
        build_planes(ws, blk, a.cbw, w, h, base, p + 1, lane);
        __syncwarp();
      }
      if (lane == 0) {
        const uint64_t* bpm = ws.bp[p - base];
        if (p == mbp - 1) {
          uint32_t ns = cleanup_pass(m, ws, b, bpm);
          pr[pi++] = PassRec{(uint32_t)m.pos, ns, 0u, 2, (uint8_t)p, 0};
          sig_so_far += ns;
        } else {
          const uint32_t before = sig_so_far;
          uint32_t sp = sig_pass(m, ws, b, bpm);
          pr[pi++] = PassRec{(uint32_t)m.pos, sp, before, 0, (uint8_t)p, 0};
          sig_so_far += sp;
          ref_pass(m, ws, b, bpm);
          pr[pi++] = PassRec{(uint32_t)m.pos, 0u, before, 1, (uint8_t)p, 0};
          uint32_t cl = cleanup_pass(m, ws, b, bpm);
          pr[pi++] = PassRec{(uint32_t)m.pos, cl, sig_so_far, 2, (uint8_t)p, 0};
          sig_so_far += cl;
        }
      }
      __syncwarp();
    }

    if (lane == 0) {
      mq_flush(m);
      BlockOut o{};
      o.payload_len = (uint32_t)(m.last == 0xffu ? m.pos - 1 : m.pos);  // take_bytes
      o.npasses = (uint16_t)npasses;
      o.mbp = (uint8_t)mbp;
      o.zbp = (uint8_t)zbp;
      o.cls = (uint8_t)cls;
      o.status = m.ovf ? 1 : 0;
      a.res[bi] = o;
    }
    __syncwarp();
  }
}

}  // namespace

bool upload_t1_tables(const uint8_t* zc, const uint8_t* sc, const uint8_t* spb,
                      const uint32_t* mq) {
  Tables t;
  memcpy(t.zc, zc, sizeof t.zc);
  memcpy(t.sc, sc, sizeof t.sc);
  memcpy(t.spb, spb, sizeof t.spb);
  memcpy(t.mq, mq, sizeof t.mq);
  return cudaMemcpyToSymbol(c_tables, &t, sizeof t) == cudaSuccess;
}

void launch_t1(const T1Args& a, int num_sms, cudaStream_t st) {
  if (a.nblocks == 0) return;
  uint32_t need = (a.nblocks + kWarps - 1) / kWarps;
  uint32_t grid = need;
  uint32_t cap = (uint32_t)num_sms * 16;  // persistent: several CTAs per SM
  if (grid > cap) grid = cap;
  t1_kernel<<<grid, kWarps * 32, 0, st>>>(a);
}

}  // namespace jp2g
