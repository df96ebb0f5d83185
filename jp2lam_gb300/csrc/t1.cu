// EBCOT Tier-1 encoder, single MQ termination per code-block, per-pass
// numbytes() snapshots for rate control.
//
// Replaces analyze_codeblock (src/encode/backend/native/t1.rs:215-258) and
// encode_codeblock_single_term (t1.rs:508-658) with its passes (SP
// t1.rs:805-905, MR t1.rs:914-965, cleanup t1.rs:977-1197) and the MQ coder
// (src/mq/mod.rs:163-432).
//
// The work is split where the dependencies allow:
//
// 1. t1_analyze_kernel (warp per block): max magnitude, non-zero count ->
//    magnitude bit-planes, zero bit-planes, block class.
// 2. t1_model_kernel (warp per (block, bit-plane)): the significance state
//    at the start of bit-plane p is known in closed form (|q| >> (p+1) != 0),
//    and so is the refinement history (|q| >> (p+2) != 0), so every
//    bit-plane's three passes are modelled independently. Within a
//    bit-plane, significance propagation is the least fixpoint of a
//    monotone system over 64-bit row masks in which each sample only looks
//    at samples earlier in the scan order (stripe by stripe); refinement and
//    cleanup are then data-parallel. The warp emits the (context, bit)
//    symbols of each stripe in exact scan order with a prefix sum over the
//    columns (one lane per column), into a per-bit-plane symbol slot.
// 3. t1_mq_kernel (lane per block): runs the MQ coder over a block's symbol
//    streams, top bit-plane first, recording numbytes() after every pass
//    and writing the byte stream to the block's payload slot.
#include <cuda_runtime.h>

#include <algorithm>

#include <cstring>

#include "jp2g_internal.h"
#include "kernels.h"
#include "t1_logic.h"

namespace jp2g {

namespace {

// Context numbers (src/mq/mod.rs:5-10).
constexpr int kCtxAGG = 17, kCtxUNI = 18;
constexpr int kModelWarps = 4;  // 7 KB of shared memory each: 6 CTAs per SM
constexpr int kMqWarps = 4;

struct Tables {
  uint8_t zc[4 * 512];
  uint8_t sc[256];
  uint8_t spb[256];
  uint32_t mq[94];  // qe | nmps << 16 | nlps << 24
};

// Built on the host from the standard's rules, copied in by upload_t1_tables.
__constant__ Tables c_tables;

// ---------------------------------------------------------------- analyze --
__global__ void t1_analyze_kernel(T1Args a) {
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= a.nblocks) return;
  const BlockDesc d = a.blocks[warp];
  const int w = d.w, h = d.h;
  const int32_t* blk = a.coef + (size_t)d.coef_slot * a.cbw * a.cbh;
  uint32_t mx = 0, nnz = 0;
  for (int y = 0; y < h; ++y) {
    int32_t v0 = lane < w ? blk[y * a.cbw + lane] : 0;
    int32_t v1 = lane + 32 < w ? blk[y * a.cbw + lane + 32] : 0;
    uint32_t m0 = v0 < 0 ? 0u - (uint32_t)v0 : (uint32_t)v0;
    uint32_t m1 = v1 < 0 ? 0u - (uint32_t)v1 : (uint32_t)v1;
    mx = max(mx, max(m0, m1));
    nnz += (v0 != 0) + (v1 != 0);
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  nnz = __reduce_add_sync(0xffffffffu, nnz);
  if (lane != 0) return;
  const int mbp = mx == 0 ? 0 : 32 - __clz(mx);
  // classify_from_nonzero_fraction (src/profile.rs:122-130), in f32.
  const float frac = __fdiv_rn((float)nnz, (float)(w * h));
  BlockOut o{};
  o.mbp = (uint8_t)mbp;
  o.zbp = (uint8_t)(d.mb > mbp ? d.mb - mbp : 0);
  o.cls = (uint8_t)(mbp == 0 ? 0 : (frac <= 0.05f ? 0 : (frac <= 0.30f ? 1 : 2)));
  uint32_t np = mbp == 0 ? 0u : 1u + 3u * (uint32_t)(mbp - 1);
  o.status = np > a.pass_cap ? 2 : 0;
  o.npasses = o.status ? 0 : (uint16_t)np;
  a.res[warp] = o;
  a.nplanes[warp] = o.status ? 0u : (uint32_t)mbp;
}

// 32x32 bit-matrix transpose in registers: on entry bit j of t[i] is
// element (i, j); on exit bit i of t[j] is.
__device__ __forceinline__ void transpose32(uint32_t (&t)[32]) {
  #pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const uint32_t m = s == 16 ? 0x0000ffffu : (s == 8 ? 0x00ff00ffu : (s == 4 ? 0x0f0f0f0fu : (s == 2 ? 0x33333333u : 0x55555555u)));
    #pragma unroll
    for (int i = 0; i < 32; ++i) {
      if (i & s) continue;
      const uint32_t x = ((t[i] >> s) ^ t[i + s]) & m;
      t[i] ^= x << s;
      t[i + s] ^= x;
    }
  }
}

// One warp per code-block: lists the block's items and writes, for every
// bit-plane p it codes, the column masks the modelling kernel starts from:
// significant before the plane (|q| >> (p+1) != 0) and the magnitude bit p,
// plus the block's sign masks. A lane reads 32 rows of one column, and a
// transpose in registers turns 32 magnitudes into 32 bit-plane masks, so
// every coefficient is read once per block instead of once per plane.
// Layout: planes[((item * 2 + {0: S, 1: B}) * 2 + half) * 64 + column],
// signs[(block * 2 + half) * 64 + column], half 0 = rows 0-31.
__global__ void __launch_bounds__(256) t1_planes_kernel(T1Args a) {
  const int lane = threadIdx.x & 31;
  const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= a.nblocks) return;
  const uint32_t np = a.nplanes[b], base = a.plane_base[b];
  for (uint32_t j = lane; j < np; j += 32) a.items[base + j] = b;
  const BlockDesc d = a.blocks[b];
  const int w = d.w, h = d.h, mbp = (int)np;
  const int32_t* blk = a.coef + (size_t)d.coef_slot * a.cbw * a.cbh;
  #pragma unroll 1
  for (int col = 0; col < 2; ++col) {
    const int x = lane + 32 * col;
    #pragma unroll 1
    for (int half = 0; half < 2; ++half) {
      uint32_t t[32], sg = 0;
      #pragma unroll
      for (int i = 0; i < 32; ++i) {
        const int y = 32 * half + i;
        const int32_t q = y < h && x < w ? blk[y * a.cbw + x] : 0;
        t[i] = q < 0 ? 0u - (uint32_t)q : (uint32_t)q;
        sg |= q < 0 ? 1u << i : 0u;
      }
      a.signs[((size_t)b * 2 + half) * 64 + x] = sg;
      if (mbp == 0) continue;
      transpose32(t);
      uint32_t above = 0;  // rows with a bit above plane k
      #pragma unroll
      for (int k = 31; k >= 0; --k) {
        if (k < mbp) {
          const size_t item = base + (uint32_t)(mbp - 1 - k);
          a.planes[((item * 2 + 0) * 2 + half) * 64 + x] = above;
          a.planes[((item * 2 + 1) * 2 + half) * 64 + x] = t[k];
        }
        above |= t[k];
      }
    }
  }
}

// Modelling works on the code-block in column layout: lane L owns columns
// L ("A") and L + 32 ("B"), and every per-sample state of a column is a
// 64-bit mask with bit y = row y. Vertical neighbours are then shifts of the
// lane's own masks, horizontal ones a shuffle from the adjacent lane, and one
// logic operation handles 64 samples.
constexpr uint64_t kRow0 = 0x1111111111111111ull;  // first row of each stripe
constexpr uint64_t kRow3 = 0x8888888888888888ull;  // last row of each stripe

__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
  const uint32_t lo = __shfl_sync(~0u, (uint32_t)v, src);
  const uint32_t hi = __shfl_sync(~0u, (uint32_t)(v >> 32), src);
  return (uint64_t)hi << 32 | lo;
}

// The masks of the columns west and east of this lane's columns A and B.
struct Side {
  uint64_t wa, ea, wb, eb;
};
__device__ __forceinline__ Side sides(uint64_t a, uint64_t b, int lane) {
  const int up = (lane + 31) & 31, dn = (lane + 1) & 31;
  Side r;
  r.wa = shfl64(a, up);                   // column L - 1 (none for lane 0)
  r.wb = shfl64(lane == 31 ? a : b, up);  // column L + 31 (lane 0: column 31)
  r.ea = shfl64(lane == 0 ? b : a, dn);   // column L + 1 (lane 31: column 32)
  r.eb = shfl64(b, dn);                   // column L + 33 (none for lane 31)
  if (lane == 0) r.wa = 0;
  if (lane == 31) r.eb = 0;
  return r;
}

// Neighbourhood of every sample of a column at the moment it is coded in a
// pass: samples coded earlier in the pass (the column to the west, the row
// above in the same column, and the row above the stripe) in their state
// after it (f), the others in their state before it (p); the row below the
// stripe is taken before the pass. fc/pc: this column; fw/pw: the column to
// the west; fe/pe: to the east.
struct Hood {
  uint64_t nw, n, ne, w, e, sw, s, se;
};
__device__ __forceinline__ Hood hood(uint64_t fc, uint64_t pc, uint64_t fw, uint64_t pw, uint64_t fe, uint64_t pe) {
  Hood h;
  h.n = fc << 1;
  h.s = pc >> 1;
  h.w = fw;
  h.e = pe;
  h.nw = fw << 1;
  h.ne = ((pe << 1) & ~kRow0) | ((fe << 1) & kRow0);
  h.sw = ((fw >> 1) & ~kRow3) | ((pw >> 1) & kRow3);
  h.se = pe >> 1;
  return h;
}

__device__ __forceinline__ uint64_t pick(uint64_t m, uint64_t a, uint64_t b) { return (a & m) | (b & ~m); }

// Symbol planes of one column: which pass codes each sample, its primary
// symbol (context << 1 | magnitude bit) and its sign symbol, as bit-planes.
enum Plane {
  kPlV = 0,   // coded in significance propagation
  kPlS,       // coded in magnitude refinement (significant before the plane)
  kPlC,       // coded in cleanup
  kPlB,       // magnitude bit of the plane
  kPlClean,   // bit 4s: the column's part of stripe s is a cleanup run
  kPlP0,      // primary context, bits 0..4
  kPlP1,
  kPlP2,
  kPlP3,
  kPlP4,
  kPlM0,      // sign context - 8, bits 0..2
  kPlM1,
  kPlM2,
  kPlX,       // sign ^ sign prediction
  kNumPlanes
};

// Shared memory of one warp: the planes of its 64 columns, split in the
// 32-bit halves of rows 0-31 and 32-63 (bank-conflict-free per half).
struct ModelSmem {
  uint32_t pl[kNumPlanes][2][64];
};

// Nibble (4 rows of stripe s) of a half-plane, s counted within the half.
__device__ __forceinline__ uint32_t nib(uint32_t v, int s) { return (v >> (4 * s)) & 0xfu; }
// The 4 bits of a nibble spread to bit 0 of each byte.
__device__ __forceinline__ uint32_t spread4(uint32_t n) { return (n * 0x00204081u) & 0x01010101u; }

// Symbols of one column of one stripe: the column's counts per pass.
__device__ __forceinline__ uint32_t column_counts(uint32_t v, uint32_t sm, uint32_t c, uint32_t b, uint32_t cl) {
  const uint32_t sp = __popc(v) + __popc(v & b), mr = __popc(sm);
  uint32_t cln;
  if (cl) {
    if (b == 0) {
      cln = 1;
    } else {
      const uint32_t after = 0xfu & ~((2u << (__ffs(b) - 1)) - 1u);
      cln = 4 + __popc(after) + __popc(after & b);
    }
  } else {
    cln = __popc(c) + __popc(c & b);
  }
  return sp | (mr << 11) | (cln << 21);
}

// Exclusive prefix of v over the warp's lanes; *total = the warp's sum.
__device__ __forceinline__ uint32_t warp_offset(uint32_t v, int lane, uint32_t* total) {
  uint32_t x = v;
  #pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  *total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

// Writes the symbols of one column of one stripe into the three streams.
__device__ __forceinline__ void emit_column(uint32_t v, uint32_t sm, uint32_t c, uint32_t b, uint32_t cl,
                                            uint32_t prim, uint32_t sgn, uint8_t*& osp, uint8_t*& omr,
                                            uint8_t*& ocl) {
  int first = 0;  // rows consumed by a cleanup run
  if (cl) {
    if (b == 0) {
      *ocl++ = (uint8_t)((uint32_t)kCtxAGG << 1);
      first = 4;
    } else {
      const int rl = __ffs(b) - 1;
      ocl[0] = (uint8_t)(((uint32_t)kCtxAGG << 1) | 1u);
      ocl[1] = (uint8_t)(((uint32_t)kCtxUNI << 1) | ((uint32_t)rl >> 1));
      ocl[2] = (uint8_t)(((uint32_t)kCtxUNI << 1) | ((uint32_t)rl & 1u));
      ocl[3] = (uint8_t)(sgn >> (8 * rl));  // sign of the run's first significant sample
      ocl += 4;
      first = rl + 1;
    }
  }
  // every row in the same predicated code: the lanes of a warp code
  // samples of different passes at the same row
  #pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint32_t bit = (b >> r) & 1u;
    const bool im = (sm >> r) & 1u;
    const bool iv = (v >> r) & 1u;
    const bool ic = r >= first && ((c >> r) & 1u);
    uint8_t* o = im ? omr : (iv ? osp : ocl);
    if (im | iv | ic) o[0] = (uint8_t)(prim >> (8 * r));
    if ((iv | ic) && bit) o[1] = (uint8_t)(sgn >> (8 * r));
    omr += im ? 1 : 0;
    osp += iv ? 1 + bit : 0;
    ocl += ic ? 1 + bit : 0;
  }
}

// One warp per (code-block, bit-plane) item.
//
// 1. Column masks of the plane: significant before it (|q| >> (p+1) != 0),
//    magnitude bit p, refinement history (|q| >> (p+2) != 0), sign.
// 2. Significance propagation: the visited (V) and newly significant (N)
//    samples are the least fixpoint of the pass's visiting rule, iterated
//    over the whole block; each round also fills every newly significant
//    sample's run of magnitude-1 samples below it with one carry-propagating
//    addition, so only horizontal chains take extra rounds. The scan order
//    makes the rule causal, so the fixpoint is the sequential pass's result.
// 3. Cleanup masks, run-length columns and, bit-sliced, every sample's
//    symbols: zero-coding label with the neighbourhood of the pass that codes
//    it, refinement context, sign context and prediction bit.
// 4. Emission, stripe by stripe: each sample is coded in exactly one pass
//    (SP if visited, MR if significant before, else cleanup or a cleanup
//    run), so each lane writes its two columns' symbols into the three
//    streams (SP | MR | cleanup, whose starts are known from the totals) at
//    offsets from two packed warp scans.
__global__ void __launch_bounds__(kModelWarps * 32, 5) t1_model_kernel(T1Args a) {
  __shared__ ModelSmem sm_all[kModelWarps];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  ModelSmem& sm = sm_all[wid];
  const uint32_t nwarps = gridDim.x * kModelWarps;
  const int xa = lane, xb = lane + 32;

  for (uint32_t item = blockIdx.x * kModelWarps + wid; item < a.nitems; item += nwarps) {
    const uint32_t blkno = a.items[item];
    const BlockDesc d = a.blocks[blkno];
    const int w = d.w, h = d.h;
    const int mbp = a.res[blkno].mbp;
    const int j = (int)(item - a.plane_base[blkno]);
    const int p = mbp - 1 - j;
    const bool top = j == 0;
    const uint64_t rows = h >= 64 ? ~0ull : ((1ull << h) - 1);
    const uint64_t vA = xa < w ? rows : 0, vB = xb < w ? rows : 0;

    // ---- 1. column masks (made by t1_planes_kernel) ----
    auto ld = [&](const uint32_t* v, size_t row0, int x) {
      return (uint64_t)v[row0 + x] | (uint64_t)v[row0 + 64 + x] << 32;
    };
    const size_t pi = (size_t)item * 256;
    const uint64_t SA = ld(a.planes, pi, xa), SB = ld(a.planes, pi, xb);
    const uint64_t BA = ld(a.planes, pi + 128, xa), BB = ld(a.planes, pi + 128, xb);
    const uint64_t RA = top ? 0 : ld(a.planes, pi - 256, xa), RB = top ? 0 : ld(a.planes, pi - 256, xb);
    const uint64_t GA = ld(a.signs, (size_t)blkno * 128, xa), GB = ld(a.signs, (size_t)blkno * 128, xb);
    const Side sS = sides(SA, SB, lane);

    // ---- 2. significance propagation ----
    uint64_t NA = 0, NB = 0, VA = 0, VB = 0;
    if (!top) {
      // parts of the visiting rule on states before the pass: S below, E,
      // SE, NE (rows 1-3 of a stripe), SW (row 3)
      const uint64_t invA = (SA >> 1) | sS.ea | (sS.ea >> 1) | ((sS.ea << 1) & ~kRow0) | ((sS.wa >> 1) & kRow3);
      const uint64_t invB = (SB >> 1) | sS.eb | (sS.eb >> 1) | ((sS.eb << 1) & ~kRow0) | ((sS.wb >> 1) & kRow3);
      const uint64_t MA = BA & ~SA & vA, MB = BB & ~SB & vB;  // samples that turn significant when visited
      for (;;) {  // N grows every round until it is stable: at most 4096 rounds
        const uint64_t FA = SA | NA, FB = SB | NB;
        const Side f = sides(FA, FB, lane);
        VA = (invA | (FA << 1) | f.wa | (f.wa << 1) | ((f.wa >> 1) & ~kRow3) | ((f.ea << 1) & kRow0)) & ~SA & vA;
        VB = (invB | (FB << 1) | f.wb | (f.wb << 1) | ((f.wb >> 1) & ~kRow3) | ((f.eb << 1) & kRow0)) & ~SB & vB;
        uint64_t nA = VA & BA, nB = VB & BB;
        nA |= MA & ~(MA + nA);  // the run of M below each new sample
        nB |= MB & ~(MB + nB);
        const bool changed = nA != NA || nB != NB;
        NA = nA;
        NB = nB;
        if (!__any_sync(~0u, changed)) break;
      }
    }

    // ---- 3. cleanup masks and the symbol planes ----
    const uint64_t SNA = SA | NA, SNB = SB | NB;                // after SP
    const uint64_t CA = ~SNA & ~VA & vA, CB = ~SNB & ~VB & vB;  // coded in cleanup
    const uint64_t QA = CA & BA, QB = CB & BB;                  // significant in cleanup
    const uint64_t FA = SNA | QA, FB = SNB | QB;                // after cleanup
    const Side sSN = sides(SNA, SNB, lane), sF = sides(FA, FB, lane), sG = sides(GA, GB, lane);
    uint32_t ns_sp = __popcll(NA) + __popcll(NB), ns_cl = __popcll(QA) + __popcll(QB);
    uint32_t n_sp = __popcll(VA) + __popcll(VB) + ns_sp, sig_before = __popcll(SA) + __popcll(SB);
    #pragma unroll
    for (int col = 0; col < 2; ++col) {
      const uint64_t S = col ? SB : SA, B = col ? BB : BA, R = col ? RB : RA, G = col ? GB : GA;
      const uint64_t V = col ? VB : VA, SN = col ? SNB : SNA, C = col ? CB : CA, F = col ? FB : FA;
      const uint64_t valid = col ? vB : vA;
      const uint64_t Sw = col ? sS.wb : sS.wa, Se = col ? sS.eb : sS.ea;
      const uint64_t SNw = col ? sSN.wb : sSN.wa, SNe = col ? sSN.eb : sSN.ea;
      const uint64_t Fw = col ? sF.wb : sF.wa, Fe = col ? sF.eb : sF.ea;
      const uint64_t Gw = col ? sG.wb : sG.wa, Ge = col ? sG.eb : sG.ea;
      // cleanup runs (flags.rs:219-235): a full stripe of the column with
      // nothing significant or visited in it or around it (west column and
      // row above after cleanup, east column and row below before it)
      const uint64_t T = SN | V | Fw | SNe | (((Fw | F | Fe) << 1) & kRow0) | (((SNw | SN | SNe) >> 1) & kRow3);
      const uint64_t busy = (T | (T >> 1) | (T >> 2) | (T >> 3)) & kRow0;
      const uint64_t clean = ~busy & kRow0 & (valid >> 3);
      // neighbourhood at coding time: SP samples see the SP frames, the
      // others the cleanup frames
      const Hood hs = hood(SN, S, SNw, Sw, SNe, Se);
      const Hood hc = hood(F, SN, Fw, SNw, Fe, SNe);
      Hood hd;
      hd.nw = pick(V, hs.nw, hc.nw);
      hd.n = pick(V, hs.n, hc.n);
      hd.ne = pick(V, hs.ne, hc.ne);
      hd.w = pick(V, hs.w, hc.w);
      hd.e = pick(V, hs.e, hc.e);
      hd.sw = pick(V, hs.sw, hc.sw);
      hd.s = pick(V, hs.s, hc.s);
      hd.se = pick(V, hs.se, hc.se);
      uint64_t l[4], m[3], x;
      zc_label_planes(hd.nw, hd.n, hd.ne, hd.w, hd.e, hd.sw, hd.s, hd.se, (int)d.orient, l);
      sign_planes(hd.n, hd.s, hd.w, hd.e, G << 1, G >> 1, Gw, Ge, m, &x);
      // refinement context (helpers.rs:36-50): 16 after a first refinement,
      // else 15 with a significant neighbour (state after SP), else 14
      const uint64_t nb = (SN << 1) | (SN >> 1) | SNw | (SNw << 1) | (SNw >> 1) | SNe | (SNe << 1) | (SNe >> 1);
      const uint64_t mr1 = S & ~R;  // contexts 14 and 15: binary 0111x
      uint64_t out[kNumPlanes];
      out[kPlV] = V;
      out[kPlS] = S;
      out[kPlC] = C;
      out[kPlB] = B;
      out[kPlClean] = clean;
      out[kPlP0] = pick(S, mr1 & nb, l[0]);
      out[kPlP1] = pick(S, mr1, l[1]);
      out[kPlP2] = pick(S, mr1, l[2]);
      out[kPlP3] = pick(S, mr1, l[3]);
      out[kPlP4] = S & R;
      out[kPlM0] = m[0];
      out[kPlM1] = m[1];
      out[kPlM2] = m[2];
      out[kPlX] = x ^ G;
      const int xc = col ? xb : xa;
      #pragma unroll
      for (int k = 0; k < kNumPlanes; ++k) {
        sm.pl[k][0][xc] = (uint32_t)out[k];
        sm.pl[k][1][xc] = (uint32_t)(out[k] >> 32);
      }
    }
    n_sp = __reduce_add_sync(~0u, n_sp);
    sig_before = __reduce_add_sync(~0u, sig_before);
    ns_sp = __reduce_add_sync(~0u, ns_sp);
    ns_cl = __reduce_add_sync(~0u, ns_cl);
    __syncwarp();

    // ---- 4. emission, stripe by stripe ----
    uint8_t* out = a.sym + (size_t)item * a.sym_slot;
    uint32_t pos_sp = 0, pos_mr = n_sp, pos_cl = n_sp + sig_before;
    const int nstripes = (h + 3) >> 2;
    for (int half = 0; half < 2 && 8 * half < nstripes; ++half) {
      uint32_t qa[kNumPlanes], qb[kNumPlanes];
      #pragma unroll
      for (int k = 0; k < kNumPlanes; ++k) {
        qa[k] = sm.pl[k][half][xa];
        qb[k] = sm.pl[k][half][xb];
      }
      const int send = min(8, nstripes - 8 * half);
      for (int s = 0; s < send; ++s) {
        const uint32_t vA4 = nib(qa[kPlV], s), sA4 = nib(qa[kPlS], s), cA4 = nib(qa[kPlC], s),
                       bA4 = nib(qa[kPlB], s), lA = nib(qa[kPlClean], s) & 1u;
        const uint32_t vB4 = nib(qb[kPlV], s), sB4 = nib(qb[kPlS], s), cB4 = nib(qb[kPlC], s),
                       bB4 = nib(qb[kPlB], s), lB = nib(qb[kPlClean], s) & 1u;
        uint32_t totA, totB;
        const uint32_t offA = warp_offset(column_counts(vA4, sA4, cA4, bA4, lA), lane, &totA);
        const uint32_t offB = warp_offset(column_counts(vB4, sB4, cB4, bB4, lB), lane, &totB);
        // primary and sign symbols of the 4 rows, one per byte
        uint32_t primA = spread4(bA4), primB = spread4(bB4);
        #pragma unroll
        for (int k = 0; k < 5; ++k) {
          primA |= spread4(nib(qa[kPlP0 + k], s)) << (k + 1);
          primB |= spread4(nib(qb[kPlP0 + k], s)) << (k + 1);
        }
        uint32_t sgnA = 0x10101010u | spread4(nib(qa[kPlX], s)), sgnB = 0x10101010u | spread4(nib(qb[kPlX], s));
        #pragma unroll
        for (int k = 0; k < 3; ++k) {
          sgnA |= spread4(nib(qa[kPlM0 + k], s)) << (k + 1);
          sgnB |= spread4(nib(qb[kPlM0 + k], s)) << (k + 1);
        }
        uint8_t* osp = out + pos_sp + (offA & 0x7ffu);
        uint8_t* omr = out + pos_mr + ((offA >> 11) & 0x3ffu);
        uint8_t* ocl = out + pos_cl + (offA >> 21);
        emit_column(vA4, sA4, cA4, bA4, lA, primA, sgnA, osp, omr, ocl);
        osp = out + pos_sp + (totA & 0x7ffu) + (offB & 0x7ffu);
        omr = out + pos_mr + ((totA >> 11) & 0x3ffu) + ((offB >> 11) & 0x3ffu);
        ocl = out + pos_cl + (totA >> 21) + (offB >> 21);
        emit_column(vB4, sB4, cB4, bB4, lB, primB, sgnB, osp, omr, ocl);
        pos_sp += (totA & 0x7ffu) + (totB & 0x7ffu);
        pos_mr += ((totA >> 11) & 0x3ffu) + ((totB >> 11) & 0x3ffu);
        pos_cl += (totA >> 21) + (totB >> 21);
      }
    }
    if (lane == 0) {
      ItemRec rec;
      rec.n_sp = n_sp;
      rec.n_mr = sig_before;
      rec.n_cl = pos_cl - (n_sp + sig_before);
      rec.ns_sp = ns_sp;
      rec.ns_cl = ns_cl;
      rec.sig_before = sig_before;
      rec.bitplane = (uint32_t)p;
      rec.pad = 0;
      a.item_rec[item] = rec;
    }
    __syncwarp();
  }
}

// --------------------------------------------------------------------- MQ --
// The coder runs one code-block per lane. Every step is written without
// data-dependent branches (conditional exchange, renormalisation and byte
// output are predicated), so the 32 lanes of a warp, each coding a different
// block, stay converged; only pass boundaries and stream refills branch.
//
// Per context the shared table holds the full probability-state entry
// (qe | MPS << 16 | next-MPS index << 17 | next-LPS index << 24), so one load
// yields qe and the MPS; the state table T is only consulted to move a
// context to its next state.
struct Mq {
  uint32_t a, c, ct;
  int pos;        // index of the last written byte; 0 is the pre-byte
  uint32_t last;  // value of that byte
  uint8_t* out;   // out[k] holds byte k+1
  int cap;
  int ovf;
};

// BYTEOUT (src/mq/mod.rs:382-404) as straight-line code: a carry into the
// previous byte is applied first, then one byte is emitted (7 bits after an
// 0xFF, 8 otherwise).
__device__ __forceinline__ void mq_byteout(Mq& m) {
  const bool carry = m.last != 0xffu && (m.c & 0x8000000u) != 0;
  if (carry) {
    m.last = (m.last + 1) & 0xffu;
    if (m.pos >= 1 && m.pos <= m.cap) m.out[m.pos - 1] = (uint8_t)m.last;
    if (m.last == 0xffu) m.c &= 0x7ffffffu;
  }
  const bool big = m.last == 0xffu;
  const uint32_t byte = (big ? (m.c >> 20) : (m.c >> 19)) & 0xffu;
  m.c &= big ? 0xfffffu : 0x7ffffu;
  m.ct = big ? 7u : 8u;
  ++m.pos;
  m.last = byte;
  if (m.pos <= m.cap) m.out[m.pos - 1] = (uint8_t)byte;
  else m.ovf = 1;
}

// Probability-state entry of a context, in shared memory: x = qe |
// (leading zeros of qe in 16 bits) << 16 | MPS << 20; y = index of the next
// state after an MPS renormalisation | index after an LPS << 8 (indices
// into the 94-entry table of (state, MPS) pairs).
//
// One MQ symbol (C.2.4-C.2.7) with the decisions folded: after A -= qe the
// coder keeps A (and adds qe to C) exactly when (A < qe) equals "LPS", and
// otherwise takes qe (C unchanged). A stays >= 0x8000 between symbols and qe
// <= 0x5601, so a kept A is either >= 0x8000 (no renormalisation) or in
// [0x29ff, 0x8000) (a shift of 1 or 2), while a taken qe shifts by its
// stored leading-zero count. The context moves to its next state exactly
// when the shift is non-zero. Returns the context's new entry.
__device__ __forceinline__ uint2 mq_step(Mq& m, uint2 e, uint32_t sym, const uint2* T) {
  const uint32_t qe = e.x & 0xffffu;
  const uint32_t lps = ((e.x >> 20) ^ sym) & 1u;
  const uint32_t a = m.a - qe;
  const bool take_a = (a < qe) == (lps != 0);
  uint32_t n = take_a ? (a < 0x4000u ? 2u : (a < 0x8000u ? 1u : 0u)) : ((e.x >> 16) & 15u);
  m.c += take_a ? qe : 0u;
  m.a = (take_a ? a : qe) << n;
  uint2 ne = e;
  if (n) ne = T[lps ? (e.y >> 8) : (e.y & 0xffu)];
  if (n >= m.ct) {
    do {
      m.c <<= m.ct;
      n -= m.ct;
      mq_byteout(m);
    } while (n >= m.ct);
  }
  m.c <<= n;
  m.ct -= n;
  return ne;
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

// Symbol i (0..15) of a 16-byte chunk.
__device__ __forceinline__ uint32_t chunk_sym(const uint4& q, int i) {
  const uint32_t w = i < 8 ? (i < 4 ? q.x : q.y) : (i < 12 ? q.z : q.w);
  return (w >> (8 * (i & 3))) & 0xffu;
}

// Codes all 16 symbols of a chunk, the next symbol's context entry loaded
// one step ahead of its use, capturing numbytes() after symbols e0 - 1 and
// e1 - 1 (pass ends; outside 1..16 they capture nothing) with predicated
// selects, so lanes of a warp at different pass ends stay converged.
__device__ __forceinline__ void mq_chunk16_at(Mq& m, uint2* ce, const uint2* T, const uint4 q, int e0,
                                              int e1, uint32_t& p0, uint32_t& p1) {
  uint32_t sym = q.x & 0xffu;
  uint2 e = ce[32 * (sym >> 1)];
  #pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint32_t symn = i < 15 ? chunk_sym(q, i + 1) : 0u;
    const uint32_t cx = sym >> 1, cxn = symn >> 1;
    uint2 en = i < 15 ? ce[32 * cxn] : make_uint2(0u, 0u);
    const uint2 ne = mq_step(m, e, sym, T);
    ce[32 * cx] = ne;
    if (cxn == cx) en = ne;
    e = en;
    sym = symn;
    p0 = e0 == i + 1 ? (uint32_t)m.pos : p0;
    p1 = e1 == i + 1 ? (uint32_t)m.pos : p1;
  }
}

// Per-block MQ coding over the symbol streams of the block's bit-planes.
// Blocks go `bpw` to a warp, one per lane: 32 when enough blocks are in
// flight to fill the GPU, 1 when a single page leaves it mostly idle and the
// longest block's serial chain sets the time (lanes of a warp diverge on
// every byte emitted, which lengthens each lane's chain).
// The 94 state entries in the layout mq_step uses.
__device__ __forceinline__ void load_mq_table(uint2* T) {
  for (int i = threadIdx.x; i < 94; i += blockDim.x) {
    // (qe | nmps << 16 | nlps << 24) -> the entry layout of mq_step
    const uint32_t v = c_tables.mq[i];
    const uint32_t qe = v & 0xffffu;
    T[i] = make_uint2(qe | ((uint32_t)(__clz(qe) - 16) << 16) | ((uint32_t)(i & 1) << 20),
                      ((v >> 16) & 0xffu) | (((v >> 24) & 0xffu) << 8));
  }
}

// MQ-codes code-block b on the calling lane; ce is the lane's context
// column (context c at ce[32 * c]).
__device__ __forceinline__ void mq_code_block(const T1Args& a, uint32_t b, uint2* ce, const uint2* T) {
  BlockOut o = a.res[b];
  const int mbp = o.status ? 0 : o.mbp;
  if (mbp == 0) return;
  const BlockDesc d = a.blocks[b];
  // contexts: state 0 except UNI 46, AGG 3, ZC 4 (src/mq/mod.rs:195-200)
  for (int c = 0; c < 19; ++c) ce[32 * c] = T[0];
  ce[32 * kCtxUNI] = T[92];
  ce[32 * kCtxAGG] = T[6];
  ce[0] = T[8];
  Mq m{0x8000u, 0u, 12u, 0, 0u, a.out + d.out_off, (int)d.out_cap, 0};
  PassRec* pr = a.passes + d.pass_off;
  const uint32_t base = a.plane_base[b];
  int pi = 0;
  uint32_t nsym = 0;
  // One flat loop over the chunks of all items (bit-planes), so lanes of a
  // warp coding different blocks stay in the same code; the next item's
  // record and first chunks are fetched during the current item's last
  // chunk.
  ItemRec r = a.item_rec[base];
  ItemRec rn = mbp > 1 ? a.item_rec[base + 1] : r;
  const uint4* src = reinterpret_cast<const uint4*>(a.sym + (size_t)base * a.sym_slot);
  uint4 c0 = src[0], c1 = src[1], c2 = src[2];  // the slot and buffer are padded for these reads
  uint4 n0 = c0, n1 = c0, n2 = c0;
  int j = 0, lo = 0, kp = 0;
  auto item_total = [](const ItemRec& x) { return (int)(x.n_sp + x.n_mr + x.n_cl); };
  // pass ends of item j: SP | MR | CL, or CL alone for the first item
  auto end_of = [&](int k) {
    if (j == 0) return item_total(r);
    return k == 0 ? (int)r.n_sp : (k == 1 ? (int)(r.n_sp + r.n_mr) : item_total(r));
  };
  auto record = [&](int k, uint32_t pos) {  // numbytes() after pass k
    const uint8_t bp = (uint8_t)r.bitplane;
    if (j == 0 || k == 2)
      pr[pi] = PassRec{pos, r.ns_cl, j == 0 ? 0u : r.sig_before + r.ns_sp, 2, bp, 0};
    else if (k == 0)
      pr[pi] = PassRec{pos, r.ns_sp, r.sig_before, 0, bp, 0};
    else
      pr[pi] = PassRec{pos, 0u, r.sig_before, 1, bp, 0};
    ++pi;
  };
  int npass = 1, total = item_total(r);
  nsym = (uint32_t)total;
  for (;;) {
    // passes of item j that end at its first symbol
    while (kp < npass - 1 && end_of(kp) == lo) record(kp++, (uint32_t)m.pos);
    const int cnt = min(16, total - lo);
    const bool last = lo + cnt >= total;
    if (last && j + 1 < mbp) {
      const uint4* ns = reinterpret_cast<const uint4*>(a.sym + (size_t)(base + j + 1) * a.sym_slot);
      n0 = ns[0];
      n1 = ns[1];
      n2 = ns[2];
    }
    const uint4 q = c0;
    c0 = c1;
    c1 = c2;
    c2 = src[(lo >> 4) + 3];  // 48 bytes ahead: inside the slot or the buffer's pad
    const int e0 = kp < npass - 1 ? end_of(kp) - lo : -1;
    const int e1 = kp + 1 < npass - 1 ? end_of(kp + 1) - lo : -1;
    uint32_t p0 = 0, p1 = 0;
    if (cnt == 16) {
      mq_chunk16_at(m, ce, T, q, e0, e1, p0, p1);
    } else {
      for (int i = 0; i < cnt; ++i) {
        const uint32_t sym = chunk_sym(q, i);
        const uint32_t cx = sym >> 1;
        ce[32 * cx] = mq_step(m, ce[32 * cx], sym, T);
        p0 = e0 == i + 1 ? (uint32_t)m.pos : p0;
        p1 = e1 == i + 1 ? (uint32_t)m.pos : p1;
      }
    }
    if (e0 >= 1 && e0 <= cnt) {
      record(kp++, p0);
      if (e1 >= 1 && e1 <= cnt) record(kp++, p1);
    }
    lo += cnt;
    if (!last) continue;
    record(npass == 1 ? 0 : 2, (uint32_t)m.pos);  // cleanup: the item's last pass
    if (++j == mbp) break;
    r = rn;
    if (j + 1 < mbp) rn = a.item_rec[base + j + 1];
    src = reinterpret_cast<const uint4*>(a.sym + (size_t)(base + j) * a.sym_slot);
    c0 = n0;
    c1 = n1;
    c2 = n2;
    lo = 0;
    kp = 0;
    npass = 3;
    total = item_total(r);
    nsym += (uint32_t)total;
  }
  mq_flush(m);
  o.payload_len = (uint32_t)(m.last == 0xffu ? m.pos - 1 : m.pos);  // take_bytes
  o.status = m.ovf ? 1 : 0;
  a.res[b] = o;
  atomicAdd(a.sym_count, (unsigned long long)nsym);
}

// ------------------------------------------------- two-warp MQ pipeline --
// For one code-block at a time, the MQ coder splits into two chains: the
// interval and context-state chain (A register, probability states) and the
// code register chain (C register, byte output). The first never depends on
// the second, so a producer warp runs it over 16-symbol chunks, handing each
// symbol's (qe added to C | shift << 16) to a consumer warp that runs the C
// chain, writes the bytes and records numbytes() at every pass end, one
// chunk behind. All lanes of a chain (the whole warp, or one half-warp when
// a pair codes two blocks at once) run the same chain on the same values, so
// their byte stores coincide and only the chain's first lane writes the
// handoff. Chains pull blocks, heaviest first, from an atomic counter.
constexpr int kPipes = 4;  // pipelines (warp pairs) per CTA
constexpr uint32_t kPipeEnd = 0xffffffffu;

struct PipeChunk {
  uint32_t block;  // code-block, or kPipeEnd
  uint16_t item;   // item (bit-plane) index within the block
  uint16_t lo;     // first symbol of the chunk within the item
  uint32_t count;  // symbols in the chunk, 0..16
  uint32_t flags;  // 1: first chunk of the block, 2: last of its item, 4: last of the block
  uint32_t a_end;  // A after the block's last symbol (flags & 4)
  uint32_t op[16];
};

// Barrier `id` of one producer/consumer pair (64 threads). With two chains
// per warp the halves of a warp may arrive apart, so that form uses the
// barrier that does not require a converged warp.
template <int H>
__device__ __forceinline__ void pipe_bar(int id) {
  if constexpr (H == 1) asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory");
  else asm volatile("barrier.sync %0, 64;" ::"r"(id) : "memory");
}

// State entry with its successors: x = qe | leading zeros of qe << 16 |
// MPS << 20, y and z the x of the states after an MPS and an LPS
// renormalisation, w their indices (MPS | LPS << 8).
__device__ __forceinline__ void load_fat_table(uint4* F) {
  for (int i = threadIdx.x; i < 94; i += blockDim.x) {
    auto xs = [](int k) {
      const uint32_t v = c_tables.mq[k], qe = v & 0xffffu;
      return qe | ((uint32_t)(__clz(qe) - 16) << 16) | ((uint32_t)(k & 1) << 20);
    };
    const uint32_t v = c_tables.mq[i], nm = (v >> 16) & 0xffu, nl = (v >> 24) & 0xffu;
    F[i] = make_uint4(xs(i), xs((int)nm), xs((int)nl), nm | (nl << 8));
  }
}

// Interval/state step of one symbol whose context state index is
// ci[32 * cx] (the calling lane's own copy of the context states); returns
// the symbol's C operation (see mq_step for the folded decisions).
__device__ __forceinline__ uint32_t phase_a_one(uint32_t& A, uint32_t* ci, const uint4* F, uint32_t sym) {
  const uint32_t cx = sym >> 1, cur = ci[32 * cx];
  const uint4 f = F[cur];
  const uint32_t qe = f.x & 0xffffu;
  const uint32_t lps = ((f.x >> 20) ^ sym) & 1u;
  const uint32_t a = A - qe;
  const bool take_a = (a < qe) == (lps != 0);
  const uint32_t n = take_a ? ((a < 0x4000u ? 1u : 0u) + (a < 0x8000u ? 1u : 0u)) : ((f.x >> 16) & 15u);
  A = (take_a ? a : qe) << n;
  ci[32 * cx] = n ? (lps ? (f.w >> 8) : (f.w & 0xffu)) : cur;
  return (take_a ? qe : 0u) | (n << 16);
}

// The same over a full chunk: the next state's qe comes from the current
// entry (no load on the chain), context indices are read two symbols ahead
// and forwarded when a context repeats.
__device__ __forceinline__ void phase_a_chunk(uint32_t& A, uint32_t* ci, const uint4* F, const uint4 q,
                                              uint32_t (&op)[16]) {
  uint32_t sy[16];
  #pragma unroll
  for (int i = 0; i < 16; ++i) sy[i] = chunk_sym(q, i);
  uint32_t cur = ci[32 * (sy[0] >> 1)];
  uint4 f = F[cur];
  uint32_t idx_next = ci[32 * (sy[1] >> 1)];
  uint4 fl_next = F[idx_next];
  #pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint32_t cx = sy[i] >> 1;
    uint32_t raw2 = 0;
    if (i + 2 < 16) raw2 = ci[32 * (sy[i + 2] >> 1)];  // before this symbol's update
    const uint32_t qe = f.x & 0xffffu;
    const uint32_t lps = ((f.x >> 20) ^ sy[i]) & 1u;
    const uint32_t a = A - qe;
    const bool take_a = (a < qe) == (lps != 0);
    const uint32_t n = take_a ? ((a < 0x4000u ? 1u : 0u) + (a < 0x8000u ? 1u : 0u)) : ((f.x >> 16) & 15u);
    A = (take_a ? a : qe) << n;
    op[i] = (take_a ? qe : 0u) | (n << 16);
    const uint32_t newidx = n ? (lps ? (f.w >> 8) : (f.w & 0xffu)) : cur;
    const uint32_t newx = n ? (lps ? f.z : f.y) : f.x;
    ci[32 * cx] = newidx;
    if (i + 1 < 16) {
      const uint4 L = F[newidx];
      const uint32_t cxn = sy[i + 1] >> 1;
      if (cxn == cx) {
        f = make_uint4(newx, L.y, L.z, L.w);
        cur = newidx;
      } else {
        f = fl_next;
        cur = idx_next;
      }
      if (i + 2 < 16) {
        idx_next = (sy[i + 2] >> 1) == cx ? newidx : raw2;
        fl_next = F[idx_next];
      }
    }
  }
}

// Code-register step of one symbol's operation (byte output as needed).
__device__ __forceinline__ void phase_c_one(Mq& m, uint32_t op) {
  m.c += op & 0xffffu;
  uint32_t n = op >> 16;
  if (n >= m.ct) {
    do {
      m.c <<= m.ct;
      n -= m.ct;
      mq_byteout(m);
    } while (n >= m.ct);
  }
  m.c <<= n;
  m.ct -= n;
}

// CTAs below pipe_ctas are pipelines that pull the `heavy` heaviest blocks;
// the CTAs above code the remaining (lighter) blocks 32 to a warp, one per
// lane, which costs the schedulers far fewer issue slots per symbol.
//
// H chains per warp pair: with H = 2 the two half-warps of each warp run the
// chains of two different code-blocks in the same instruction stream (each
// half pulls its own blocks), so a symbol costs about half the issue slots
// of H = 1 (all 32 lanes on one chain), at the price of executing both
// halves' byte-output branches. A half with nothing left keeps taking part
// in the pair's barriers with empty chunks until both halves are done.
template <int H>
__global__ void __launch_bounds__(kPipes * 64, 2) t1_mq_pipe_kernel(T1Args a, uint32_t* next, uint32_t pipe_ctas,
                                                                uint32_t heavy) {
  constexpr int HL = 32 / H;  // lanes per chain
  __shared__ uint4 F[94];
  __shared__ PipeChunk slots[kPipes][2][H];
  // Context state indices: every lane keeps its own copy (context c of a
  // lane at [pipe][c][lane]). The lanes of a chain compute identical values,
  // but a shared copy would be read and written by all of them with nothing
  // ordering one lane's write after another lane's read of the same symbol;
  // private copies make the chain correct however the lanes are scheduled.
  __shared__ uint32_t ci_all[kPipes][19][32];
  if (blockIdx.x >= pipe_ctas) {
    __shared__ uint2 T[94];
    __shared__ uint2 ce_all[kPipes * 2][20 * 32];
    load_mq_table(T);
    __syncthreads();
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const uint32_t slot = heavy + ((blockIdx.x - pipe_ctas) * (kPipes * 2) + (uint32_t)w) * 32u + (uint32_t)l;
    if (slot < a.nblocks) mq_code_block(a, a.mq_order[slot], &ce_all[w][l], T);
    return;
  }
  load_fat_table(F);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int half = lane / HL, hl = lane % HL;  // this lane's chain, its lane within it
  const uint32_t hmask = H == 1 ? 0xffffffffu : (((1u << HL) - 1u) << (HL * half));
  // producers are warps 0..kPipes-1 and consumers the warps above, so the
  // (heavier) producer chains spread over the SM's schedulers
  const int pipe = warp % kPipes;
  const int bar = 1 + pipe;
  if (warp < kPipes) {
    // ---- producer: interval and state chain ----
    uint32_t* ci = &ci_all[pipe][0][lane];
    uint32_t b = kPipeEnd, base = 0, A = 0x8000u;
    int mbp = 0, j = 0, lo = 0, total = 0;
    bool exhausted = false;  // the block queue is empty for this chain
    const uint4* src = nullptr;
    uint4 c0 = make_uint4(0, 0, 0, 0), c1 = c0, c2 = c0;
    auto start_item = [&]() {
      const ItemRec r = a.item_rec[base + j];
      total = (int)(r.n_sp + r.n_mr + r.n_cl);
      lo = 0;
      src = reinterpret_cast<const uint4*>(a.sym + (size_t)(base + j) * a.sym_slot);
      c0 = src[0];
      c1 = src[1];
      c2 = src[2];  // the slot and the buffer are padded for these reads
    };
    for (uint32_t k = 0;; ++k) {
      PipeChunk& s = slots[pipe][k & 1][half];
      uint32_t flags = 0;
      while (b == kPipeEnd && !exhausted) {
        uint32_t t = 0;
        if (hl == 0) t = atomicAdd(next, 1u);
        t = __shfl_sync(hmask, t, half * HL);
        if (t >= heavy) {
          exhausted = true;
          break;
        }
        const uint32_t cand = a.mq_order[t];
        const BlockOut o = a.res[cand];
        const int m_ = o.status ? 0 : o.mbp;
        if (m_ == 0) continue;
        b = cand;
        mbp = m_;
        j = 0;
        base = a.plane_base[b];
        A = 0x8000u;
        // contexts: state 0 except UNI 46, AGG 3, ZC 4 (src/mq/mod.rs:195-200)
        #pragma unroll
        for (int x = 0; x < 19; ++x) ci[32 * x] = x == kCtxUNI ? 92u : (x == kCtxAGG ? 6u : (x == 0 ? 8u : 0u));
        flags = 1;
        start_item();
      }
      const bool idle = b == kPipeEnd;
      if (idle) {
        if (hl == 0) s.block = kPipeEnd;
      } else {
        const int cnt = min(16, total - lo);
        if (cnt == 16) {
          const uint4 q = c0;
          c0 = c1;
          c1 = c2;
          c2 = src[(lo >> 4) + 3];  // 48 bytes ahead: inside the slot or the buffer's pad
          uint32_t op[16];
          phase_a_chunk(A, ci, F, q, op);
          if (hl == 0) {
            #pragma unroll
            for (int i = 0; i < 16; ++i) s.op[i] = op[i];
          }
        } else {
          const uint4 q = c0;
          for (int i = 0; i < cnt; ++i) {
            const uint32_t o = phase_a_one(A, ci, F, chunk_sym(q, i));
            if (hl == 0) s.op[i] = o;
          }
        }
        if (hl == 0) {
          s.block = b;
          s.item = (uint16_t)j;
          s.lo = (uint16_t)lo;
          s.count = (uint32_t)cnt;
        }
        lo += cnt;
        if (lo >= total) {
          flags |= 2;
          if (++j == mbp) {
            flags |= 4;
            if (hl == 0) s.a_end = A;
            b = kPipeEnd;
          } else {
            start_item();
          }
        }
        if (hl == 0) s.flags = flags;
      }
      const bool all_idle = __all_sync(0xffffffffu, idle);
      pipe_bar<H>(bar);
      if (all_idle) break;
    }
  } else {
    // ---- consumer: code register chain, bytes and pass records ----
    Mq m{0x8000u, 0u, 12u, 0, 0u, nullptr, 0, 0};
    BlockOut o{};
    PassRec* pr = nullptr;
    ItemRec r{};
    uint32_t base = 0, nsym = 0;
    int pi = 0, npass = 1, kp = 0;
    int end[3] = {0, 0, 0};
    auto snapshot = [&](int k, int item) {  // numbytes() after pass k
      const uint8_t bp = (uint8_t)r.bitplane;
      if (npass == 1 || k == 2)
        pr[pi] = PassRec{(uint32_t)m.pos, r.ns_cl, item == 0 ? 0u : r.sig_before + r.ns_sp, 2, bp, 0};
      else if (k == 0)
        pr[pi] = PassRec{(uint32_t)m.pos, r.ns_sp, r.sig_before, 0, bp, 0};
      else
        pr[pi] = PassRec{(uint32_t)m.pos, 0u, r.sig_before, 1, bp, 0};
      ++pi;
    };
    for (uint32_t k = 0;; ++k) {
      __syncwarp();  // the halves meet before the pair's barrier
      pipe_bar<H>(bar);
      const PipeChunk& s = slots[pipe][k & 1][half];
      const uint32_t blk = s.block;
      if (__all_sync(0xffffffffu, blk == kPipeEnd)) break;
      if (blk == kPipeEnd) continue;  // this chain is idle in this round
      const uint32_t flags = s.flags;
      const int item = s.item, lo = s.lo, cnt = (int)s.count;
      if (flags & 1) {
        const BlockDesc d = a.blocks[blk];
        o = a.res[blk];
        m = Mq{0x8000u, 0u, 12u, 0, 0u, a.out + d.out_off, (int)d.out_cap, 0};
        pr = a.passes + d.pass_off;
        pi = 0;
        nsym = 0;
        base = a.plane_base[blk];
      }
      if (lo == 0) {
        r = a.item_rec[base + item];
        const int total = (int)(r.n_sp + r.n_mr + r.n_cl);
        npass = item == 0 ? 1 : 3;
        end[0] = item == 0 ? total : (int)r.n_sp;
        end[1] = (int)(r.n_sp + r.n_mr);
        end[2] = total;
        nsym += (uint32_t)total;
        kp = 0;
        while (kp < npass - 1 && end[kp] == 0) snapshot(kp++, item);
      }
      const int hi = lo + cnt;
      if (cnt == 16 && (kp == npass - 1 || end[kp] >= hi)) {
        uint32_t op[16];
        #pragma unroll
        for (int i = 0; i < 16; ++i) op[i] = s.op[i];
        #pragma unroll
        for (int i = 0; i < 16; ++i) phase_c_one(m, op[i]);
      } else {
        for (int i = 0; i < cnt; ++i) {
          phase_c_one(m, s.op[i]);
          while (kp < npass - 1 && end[kp] == lo + i + 1) snapshot(kp++, item);
        }
      }
      while (kp < npass - 1 && end[kp] == hi) snapshot(kp++, item);
      if (flags & 2) snapshot(npass == 1 ? 0 : 2, item);
      if (flags & 4) {
        m.a = s.a_end;
        mq_flush(m);
        o.payload_len = (uint32_t)(m.last == 0xffu ? m.pos - 1 : m.pos);  // take_bytes
        o.status = m.ovf ? 1 : 0;
        if (hl == 0) {
          a.res[blk] = o;
          atomicAdd(a.sym_count, (unsigned long long)nsym);
        }
      }
    }
  }
}

// Static mapping: warp w codes blocks order[w * bpw + lane], lanes < bpw.
__global__ void __launch_bounds__(kMqWarps * 32) t1_mq_kernel(T1Args a, int bpw) {
  __shared__ uint2 T[94];
  __shared__ uint2 ce_all[kMqWarps][20 * 32];
  load_mq_table(T);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  if (lane >= bpw) return;
  const uint32_t slot = (blockIdx.x * kMqWarps + wid) * (uint32_t)bpw + (uint32_t)lane;
  if (slot >= a.nblocks) return;
  mq_code_block(a, a.mq_order ? a.mq_order[slot] : slot, &ce_all[wid][lane], T);
}

// Persistent form for one block per warp: a fixed number of warps per SM
// take the next block of the order (heaviest first) until none is left, so
// the longest chains start first and share their schedulers with few others.
__global__ void __launch_bounds__(kMqWarps * 32) t1_mq_pull_kernel(T1Args a, uint32_t* next) {
  __shared__ uint2 T[94];
  __shared__ uint2 ce_all[kMqWarps][20 * 32];
  load_mq_table(T);
  __syncthreads();
  if ((threadIdx.x & 31) != 0) return;
  uint2* ce = &ce_all[threadIdx.x >> 5][0];
  for (;;) {
    const uint32_t slot = atomicAdd(next, 1u);
    if (slot >= a.nblocks) return;
    mq_code_block(a, a.mq_order[slot], ce, T);
  }
}

}  // namespace

// The bit-sliced context formation evaluated on single samples, in the
// layout of the context tables (jp2g_debug_context_labels).
void context_labels_from_logic(uint8_t* zc, uint8_t* sc, uint8_t* spb) {
  for (int o = 0; o < 4; ++o)
    for (uint32_t f = 0; f < 512; ++f) {
      uint32_t l[4];
      zc_label_planes<uint32_t>(f & 1u, (f >> 1) & 1u, (f >> 2) & 1u, (f >> 3) & 1u, (f >> 5) & 1u,
                                (f >> 6) & 1u, (f >> 7) & 1u, (f >> 8) & 1u, o, l);
      zc[o * 512 + f] = (uint8_t)((l[0] & 1u) | (l[1] & 1u) << 1 | (l[2] & 1u) << 2 | (l[3] & 1u) << 3);
    }
  // sign index: bit 3 W, 0 W negative, 1 N, 4 N negative, 5 E, 2 E negative, 7 S, 6 S negative
  for (uint32_t f = 0; f < 256; ++f) {
    uint32_t m[3], x;
    sign_planes<uint32_t>((f >> 1) & 1u, (f >> 7) & 1u, (f >> 3) & 1u, (f >> 5) & 1u, (f >> 4) & 1u, (f >> 6) & 1u,
                          f & 1u, (f >> 2) & 1u, m, &x);
    sc[f] = (uint8_t)(8u + ((m[0] & 1u) | (m[1] & 1u) << 1 | (m[2] & 1u) << 2));
    spb[f] = (uint8_t)(x & 1u);
  }
}

bool upload_t1_tables(const uint8_t* zc, const uint8_t* sc, const uint8_t* spb,
                      const uint32_t* mq) {
  Tables t;
  memcpy(t.zc, zc, sizeof t.zc);
  memcpy(t.sc, sc, sizeof t.sc);
  memcpy(t.spb, spb, sizeof t.spb);
  memcpy(t.mq, mq, sizeof t.mq);
  return cudaMemcpyToSymbol(c_tables, &t, sizeof t) == cudaSuccess;
}

void launch_t1_analyze(const T1Args& a, cudaStream_t st) {
  if (a.nblocks == 0) return;
  const uint32_t threads = 256;
  const uint32_t grid = (uint32_t)(((uint64_t)a.nblocks * 32 + threads - 1) / threads);
  t1_analyze_kernel<<<grid, threads, 0, st>>>(a);
}

void launch_t1_planes(const T1Args& a, cudaStream_t st) {
  if (a.nblocks == 0) return;
  t1_planes_kernel<<<(uint32_t)(((uint64_t)a.nblocks * 32 + 255) / 256), 256, 0, st>>>(a);
}

void launch_t1_model(const T1Args& a, int num_sms, cudaStream_t st) {
  if (a.nitems == 0) return;
  uint32_t need = (a.nitems + kModelWarps - 1) / kModelWarps;
  uint32_t cap = (uint32_t)num_sms * 6 * 4;  // CTAs loop over the items
  t1_model_kernel<<<need < cap ? need : cap, kModelWarps * 32, 0, st>>>(a);
}

int mq_blocks_per_warp(const T1Args& a, int num_sms, int bpw) {
  // Automatic: up to 48 blocks per SM, one block per chain (the caller
  // pulls or pipelines them); beyond that, as few blocks per warp (at least
  // 2) as keep about 24 latency-bound warps per SM, since the lanes of a
  // warp diverge.
  if (bpw <= 0 || bpw > 32) {
    const uint32_t sms = (uint32_t)num_sms;
    if (a.nblocks <= sms * 48u) return 1;
    bpw = (int)std::min<uint32_t>(32u, std::max<uint32_t>(2u, (a.nblocks + sms * 24u - 1) / (sms * 24u)));
  }
  return bpw;
}

void launch_t1_mq(const T1Args& a, int num_sms, int bpw, cudaStream_t st) {
  if (a.nblocks == 0) return;
  bpw = mq_blocks_per_warp(a, num_sms, bpw);
  const uint32_t per_cta = (uint32_t)bpw * kMqWarps;
  t1_mq_kernel<<<(a.nblocks + per_cta - 1) / per_cta, kMqWarps * 32, 0, st>>>(a, bpw);
}

void launch_t1_mq_pipe(const T1Args& a, int num_sms, int pipes_per_sm, int chains, uint32_t heavy, uint32_t* next,
                       cudaStream_t st) {
  if (a.nblocks == 0) return;
  cudaMemsetAsync(next, 0, sizeof(uint32_t), st);
  heavy = heavy == 0 ? a.nblocks : std::min(heavy, a.nblocks);
  chains = chains == 2 || chains == 4 ? chains : 1;
  const uint32_t per_pipe_cta = (uint32_t)kPipes * (uint32_t)chains;  // blocks a CTA codes at once
  const uint32_t pipe_ctas = std::max<uint32_t>(
      1u, std::min<uint32_t>((uint32_t)num_sms * (uint32_t)pipes_per_sm / kPipes,
                             (heavy + per_pipe_cta - 1) / per_pipe_cta));
  const uint32_t per_cta = kPipes * 2 * 32;
  const uint32_t packed_ctas = (a.nblocks - heavy + per_cta - 1) / per_cta;
  if (chains == 4)
    t1_mq_pipe_kernel<4><<<pipe_ctas + packed_ctas, kPipes * 64, 0, st>>>(a, next, pipe_ctas, heavy);
  else if (chains == 2)
    t1_mq_pipe_kernel<2><<<pipe_ctas + packed_ctas, kPipes * 64, 0, st>>>(a, next, pipe_ctas, heavy);
  else
    t1_mq_pipe_kernel<1><<<pipe_ctas + packed_ctas, kPipes * 64, 0, st>>>(a, next, pipe_ctas, heavy);
}

void launch_t1_mq_pull(const T1Args& a, int num_sms, int warps_per_sm, uint32_t* next, cudaStream_t st) {
  if (a.nblocks == 0) return;
  cudaMemsetAsync(next, 0, sizeof(uint32_t), st);
  const uint32_t ctas = std::min<uint32_t>((uint32_t)num_sms * (uint32_t)warps_per_sm / kMqWarps,
                                           (a.nblocks + kMqWarps - 1) / kMqWarps);
  t1_mq_pull_kernel<<<std::max<uint32_t>(ctas, 1u), kMqWarps * 32, 0, st>>>(a, next);
}

namespace {
constexpr uint32_t kOrderBuckets = 1024;

// Bucket of a block: its MQ symbol count / 64, clamped, reversed so that
// bucket 0 holds the largest blocks.
__device__ __forceinline__ uint32_t order_bucket(const T1Args& a, uint32_t b) {
  const uint32_t i0 = a.plane_base[b], i1 = a.plane_base[b + 1];
  uint32_t n = 0;
  for (uint32_t i = i0; i < i1; ++i) {
    const ItemRec r = a.item_rec[i];
    n += r.n_sp + r.n_mr + r.n_cl;
  }
  const uint32_t k = min(n >> 6, kOrderBuckets - 1);
  return kOrderBuckets - 1 - k;
}

__global__ void order_hist_kernel(T1Args a, uint32_t* key, uint32_t* hist) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nblocks) return;
  const uint32_t k = order_bucket(a, b);
  key[b] = k;
  atomicAdd(hist + k, 1u);
}

// One CTA of 1024 threads: exclusive scan of the bucket counts into cursors.
__global__ void order_scan_kernel(const uint32_t* hist, uint32_t* cursor) {
  __shared__ uint32_t warp_tot[32];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const uint32_t v = hist[t];
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t y = warp_tot[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t z = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += z;
    }
    warp_tot[lane] = y;
  }
  __syncthreads();
  cursor[t] = x - v + (wid > 0 ? warp_tot[wid - 1] : 0u);
}

__global__ void order_scatter_kernel(uint32_t n, const uint32_t* key, uint32_t* cursor, uint32_t* order) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  order[atomicAdd(cursor + key[b], 1u)] = b;
}
}  // namespace

void launch_mq_order(const T1Args& a, uint32_t* order, uint32_t* scratch, cudaStream_t st) {
  if (a.nblocks == 0) return;
  uint32_t* hist = scratch;
  uint32_t* cursor = scratch + kOrderBuckets;
  uint32_t* key = scratch + 2 * kOrderBuckets;
  cudaMemsetAsync(hist, 0, kOrderBuckets * sizeof(uint32_t), st);
  const uint32_t g = (a.nblocks + 255) / 256;
  order_hist_kernel<<<g, 256, 0, st>>>(a, key, hist);
  order_scan_kernel<<<1, kOrderBuckets, 0, st>>>(hist, cursor);
  order_scatter_kernel<<<g, 256, 0, st>>>(a.nblocks, key, cursor, order);
}

}  // namespace jp2g
