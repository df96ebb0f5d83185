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

namespace jp2g {

namespace {

// Context numbers (src/mq/mod.rs:5-10).
constexpr int kCtxAGG = 17, kCtxUNI = 18;
constexpr int kModelWarps = 8;
constexpr int kMqWarps = 4;

struct Tables {
  uint8_t zc[4 * 512];
  uint8_t sc[256];
  uint8_t spb[256];
  uint32_t mq[94];  // qe | nmps << 16 | nlps << 24
};

// Built on the host from the standard's rules, copied in by upload_t1_tables.
__constant__ Tables c_tables;

__device__ __forceinline__ uint64_t westm(uint64_t m) { return m << 1; }   // bit x = m[x-1]
__device__ __forceinline__ uint64_t eastm(uint64_t m) { return m >> 1; }   // bit x = m[x+1]
__device__ __forceinline__ uint64_t dil(uint64_t m) { return m | (m << 1) | (m >> 1); }

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

__global__ void t1_items_kernel(T1Args a) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nblocks) return;
  const uint32_t base = a.plane_base[b], n = a.nplanes[b];
  for (uint32_t j = 0; j < n; ++j) a.items[base + j] = b;
}

// ------------------------------------------------------------------ model --
struct ModelSmem {
  uint64_t S[68];   // significant before this bit-plane; row y at y+1
  uint64_t N[68];   // became significant in SP; row y at y+1
  uint64_t Q[68];   // became significant in CL; row y at y+1
  uint64_t Sn[68];  // coefficient sign; row y at y+1
  uint64_t B[64];   // magnitude bit p
  uint64_t R[64];   // refinement history (|q| >> (p+2) != 0)
  uint64_t V[64];   // visited (coded) in SP
};

// Each lane codes two adjacent columns, xa = 2 lane and xb = 2 lane + 1. A
// row mask is seen through the lane's 4-bit window of columns
// (xa-1, xa, xb, xb+1): bit 0 is the west neighbour of xa, bits 1-2 the
// lane's own columns, bit 3 the east neighbour of xb (0 outside the block).
__device__ __forceinline__ uint32_t win4(uint64_t m, int sh) {  // sh = 2 lane - 1
  return (uint32_t)(sh < 0 ? (m << 1) : (m >> sh)) & 0xfu;
}

// Zero-coding neighbourhood index (bit 0 NW, 1 N, 2 NE, 3 W, 5 E, 6 SW, 7 S,
// 8 SE) of column c (0: xa, 1: xb) from windows of the row above, the row and
// the row below. `f` windows hold the state of samples already visited in
// this pass (west columns, and the rows above in the same column), `p`
// windows the state before the pass (east columns, rows below).
__device__ __forceinline__ uint32_t zc_index(uint32_t up_f, uint32_t up_p, uint32_t f, uint32_t pr,
                                             uint32_t dn_f, uint32_t dn_p, int c) {
  const uint32_t up = ((up_f >> c) & 3u) | ((up_p >> c) & 4u);
  const uint32_t mid = (((f >> c) & 1u) << 3) | (((pr >> c) & 4u) << 3);
  const uint32_t dn = (((dn_f >> c) & 1u) | ((dn_p >> c) & 6u)) << 6;
  return up | mid | dn;
}

// Sign-context index from the four cardinal neighbours' significance and
// sign at the moment the sign is coded (src/tier1/helpers.rs:52-88).
__device__ __forceinline__ uint32_t sign_index(uint32_t sw, uint32_t gw, uint32_t sn, uint32_t gn,
                                               uint32_t se, uint32_t ge, uint32_t ss, uint32_t gs) {
  return (sw << 3) | ((sw & gw) << 0) | (sn << 1) | ((sn & gn) << 4) | (se << 5) | ((se & ge) << 2) |
         (ss << 7) | ((ss & gs) << 6);
}

struct ModelTables {
  const uint8_t* zc;  // orientation row
  const uint8_t* sc;
  const uint8_t* spb;
};

// Sign symbol of column c of a row: m8 is the sample's zero-coding index
// (its N, W, E, S bits are the significance the sign context sees); g, gu,
// gd are the sign windows of the row, the row above and the row below.
__device__ __forceinline__ uint32_t sign_symbol(const ModelTables& t, uint32_t m8, uint32_t g,
                                                uint32_t gu, uint32_t gd, int c) {
  const uint32_t sw = (m8 >> 3) & 1u, sn = (m8 >> 1) & 1u, se = (m8 >> 5) & 1u, ss = (m8 >> 7) & 1u;
  const uint32_t gw = (g >> c) & 1u, ge = (g >> (c + 2)) & 1u;
  const uint32_t gn = (gu >> (c + 1)) & 1u, gs = (gd >> (c + 1)) & 1u;
  const uint32_t lu = sign_index(sw, gw, sn, gn, se, ge, ss, gs);
  return ((uint32_t)t.sc[lu] << 1) | (((g >> (c + 1)) & 1u) ^ t.spb[lu]);
}

// a[i] for a runtime i without indexing a register array (which would move
// the array to local memory).
__device__ __forceinline__ uint32_t pick4(const uint32_t (&a)[4], int i) {
  return i < 2 ? (i == 0 ? a[0] : a[1]) : (i == 2 ? a[2] : a[3]);
}
__device__ __forceinline__ uint32_t pick6(const uint32_t (&a)[6], int i) {
  return i < 3 ? (i == 0 ? a[0] : (i == 1 ? a[1] : a[2])) : (i == 3 ? a[3] : (i == 4 ? a[4] : a[5]));
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

__global__ void __launch_bounds__(kModelWarps * 32, 3) t1_model_kernel(T1Args a) {
  __shared__ ModelSmem sm_all[kModelWarps];
  __shared__ uint8_t s_zc[4 * 512];
  __shared__ uint8_t s_sc[256];
  __shared__ uint8_t s_spb[256];
  for (int i = threadIdx.x; i < 4 * 512; i += blockDim.x) s_zc[i] = c_tables.zc[i];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    s_sc[i] = c_tables.sc[i];
    s_spb[i] = c_tables.spb[i];
  }
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  ModelSmem& s = sm_all[wid];
  const uint32_t nwarps = gridDim.x * kModelWarps;

  for (uint32_t item = blockIdx.x * kModelWarps + wid; item < a.nitems; item += nwarps) {
    const uint32_t b = a.items[item];
    const BlockDesc d = a.blocks[b];
    const int w = d.w, h = d.h;
    const int mbp = a.res[b].mbp;
    const int j = (int)(item - a.plane_base[b]);
    const int p = mbp - 1 - j;
    const bool top = j == 0;
    const uint64_t valid = w == 64 ? ~0ull : ((1ull << w) - 1);
    const int32_t* blk = a.coef + (size_t)d.coef_slot * a.cbw * a.cbh;
    ModelTables t{s_zc + d.orient * 512, s_sc, s_spb};
    const int sh = 2 * lane - 1;  // window of columns 2 lane - 1 .. 2 lane + 2

    // ---- masks for this bit-plane ----
    for (int y = 0; y < h; ++y) {
      int32_t v0 = lane < w ? blk[y * a.cbw + lane] : 0;
      int32_t v1 = lane + 32 < w ? blk[y * a.cbw + lane + 32] : 0;
      uint32_t m0 = v0 < 0 ? 0u - (uint32_t)v0 : (uint32_t)v0;
      uint32_t m1 = v1 < 0 ? 0u - (uint32_t)v1 : (uint32_t)v1;
      uint64_t sg = (uint64_t)__ballot_sync(~0u, (m0 >> (p + 1)) != 0) |
                    ((uint64_t)__ballot_sync(~0u, (m1 >> (p + 1)) != 0) << 32);
      uint64_t bt = (uint64_t)__ballot_sync(~0u, (m0 >> p) & 1) |
                    ((uint64_t)__ballot_sync(~0u, (m1 >> p) & 1) << 32);
      uint64_t rf = (uint64_t)__ballot_sync(~0u, p + 2 < 32 && (m0 >> (p + 2)) != 0) |
                    ((uint64_t)__ballot_sync(~0u, p + 2 < 32 && (m1 >> (p + 2)) != 0) << 32);
      uint64_t sn = (uint64_t)__ballot_sync(~0u, v0 < 0) | ((uint64_t)__ballot_sync(~0u, v1 < 0) << 32);
      if (lane == 0) {
        s.S[y + 1] = sg;
        s.B[y] = bt;
        s.R[y] = rf;
        s.Sn[y + 1] = sn;
      }
    }
    if (lane == 0) {
      s.S[0] = s.Sn[0] = s.N[0] = s.Q[0] = 0;
    }
    for (int y = h + 1 + lane; y < 68; y += 32) s.S[y] = s.Sn[y] = s.N[y] = s.Q[y] = 0;
    __syncwarp();

    uint8_t* out = a.sym + (size_t)item * a.sym_slot;
    uint32_t pos = 0;
    uint32_t n_sp = 0, n_mr = 0, ns_sp = 0, ns_cl = 0;
    uint32_t sig_before = 0;
    for (int y = lane; y < h; y += 32) sig_before += __popcll(s.S[y + 1]);
    sig_before = __reduce_add_sync(~0u, sig_before);

    if (!top) {
      // ---- significance propagation: fixpoint per stripe ----
      uint64_t Fp = 0;  // final SP state of the row above the stripe
      for (int k = 0; k < h; k += 4) {
        uint64_t S0 = s.S[k + 1], S1 = s.S[k + 2], S2 = s.S[k + 3], S3 = s.S[k + 4], D = s.S[k + 5];
        uint64_t B0 = s.B[k], B1 = k + 1 < h ? s.B[k + 1] : 0, B2 = k + 2 < h ? s.B[k + 2] : 0,
                 B3 = k + 3 < h ? s.B[k + 3] : 0;
        uint64_t v0 = valid, v1 = k + 1 < h ? valid : 0, v2 = k + 2 < h ? valid : 0,
                 v3 = k + 3 < h ? valid : 0;
        if (k + 4 > h) D = 0;
        uint64_t N0 = 0, N1 = 0, N2 = 0, N3 = 0, V0, V1, V2, V3;
        for (;;) {
          uint64_t F0 = S0 | N0, F1 = S1 | N1, F2 = S2 | N2, F3 = S3 | N3;
          uint64_t vis0 = dil(Fp) | westm(F0) | eastm(S0) | westm(F1) | S1 | eastm(S1);
          uint64_t vis1 = westm(F0) | F0 | eastm(S0) | westm(F1) | eastm(S1) | westm(F2) | S2 | eastm(S2);
          uint64_t vis2 = westm(F1) | F1 | eastm(S1) | westm(F2) | eastm(S2) | westm(F3) | S3 | eastm(S3);
          uint64_t vis3 = westm(F2) | F2 | eastm(S2) | westm(F3) | eastm(S3) | dil(D);
          V0 = ~S0 & vis0 & v0; V1 = ~S1 & vis1 & v1; V2 = ~S2 & vis2 & v2; V3 = ~S3 & vis3 & v3;
          uint64_t n0 = V0 & B0, n1 = V1 & B1, n2 = V2 & B2, n3 = V3 & B3;
          if (n0 == N0 && n1 == N1 && n2 == N2 && n3 == N3) break;
          N0 = n0; N1 = n1; N2 = n2; N3 = n3;
        }
        if (lane == 0) {
          s.N[k + 1] = N0; s.N[k + 2] = N1; s.N[k + 3] = N2; s.N[k + 4] = N3;
          s.V[k] = V0;
          if (k + 1 < 64) s.V[k + 1] = V1;
          if (k + 2 < 64) s.V[k + 2] = V2;
          if (k + 3 < 64) s.V[k + 3] = V3;
        }
        ns_sp += __popcll(N0) + __popcll(N1) + __popcll(N2) + __popcll(N3);
        // emission in scan order: within the stripe column by column (each
        // lane: its column xa, then xb), rows top to bottom
        const uint64_t F0 = S0 | N0, F1 = S1 | N1, F2 = S2 | N2, F3 = S3 | N3;
        if (V0 | V1 | V2 | V3) {  // same masks in every lane: a uniform skip of empty stripes
          const uint32_t wfp = win4(Fp, sh), wd = win4(D, sh);
          const uint32_t wf[4] = {win4(F0, sh), win4(F1, sh), win4(F2, sh), win4(F3, sh)};
          const uint32_t wp[4] = {win4(S0, sh), win4(S1, sh), win4(S2, sh), win4(S3, sh)};
          const uint32_t wv[4] = {win4(V0, sh), win4(V1, sh), win4(V2, sh), win4(V3, sh)};
          const uint32_t wb[4] = {win4(B0, sh), win4(B1, sh), win4(B2, sh), win4(B3, sh)};
          uint32_t wg[6];
          #pragma unroll
          for (int r = 0; r < 6; ++r) wg[r] = win4(s.Sn[k + r], sh);  // rows k-1 .. k+4
          uint32_t cnt = 0;
          #pragma unroll
          for (int r = 0; r < 4; ++r) cnt += __popc(wv[r] & 6u) + __popc(wv[r] & wb[r] & 6u);
          uint32_t total;
          uint8_t* o = out + pos + warp_offset(cnt, lane, &total);
          pos += total;
          n_sp += total;
          #pragma unroll 1
          for (int c = 0; c < 2; ++c) {
            #pragma unroll
            for (int r = 0; r < 4; ++r) {
              if (!((wv[r] >> (c + 1)) & 1u)) continue;
              const uint32_t uf = r == 0 ? wfp : wf[r > 0 ? r - 1 : 0], up = r == 0 ? wfp : wp[r > 0 ? r - 1 : 0];
              const uint32_t df = r == 3 ? wd : wf[r < 3 ? r + 1 : 3], dp = r == 3 ? wd : wp[r < 3 ? r + 1 : 3];
              const uint32_t m8 = zc_index(uf, up, wf[r], wp[r], df, dp, c);
              const uint32_t bit = (wb[r] >> (c + 1)) & 1u;
              *o++ = (uint8_t)(((uint32_t)t.zc[m8] << 1) | bit);
              if (bit) *o++ = (uint8_t)sign_symbol(t, m8, wg[r + 1], wg[r], wg[r + 2], c);
            }
          }
        }
        Fp = F3;
        if (k + 4 > h) break;
      }
      __syncwarp();
      // ---- magnitude refinement ----
      for (int k = 0; k < h; k += 4) {
        if (!(s.S[k + 1] | s.S[k + 2] | s.S[k + 3] | s.S[k + 4])) continue;  // nothing to refine
        uint32_t wf[6];  // state after SP of rows k-1 .. k+4
        #pragma unroll
        for (int r = 0; r < 6; ++r) wf[r] = win4(s.S[k + r] | s.N[k + r], sh);
        uint32_t ws[4], wr[4], wb[4];
        #pragma unroll
        for (int r = 0; r < 4; ++r) {
          ws[r] = win4(s.S[k + r + 1], sh);
          wr[r] = win4(s.R[k + r], sh);
          wb[r] = win4(s.B[k + r], sh);
        }
        uint32_t cnt = 0;
        #pragma unroll
        for (int r = 0; r < 4; ++r) cnt += __popc(ws[r] & 6u);
        uint32_t total;
        uint8_t* o = out + pos + warp_offset(cnt, lane, &total);
        pos += total;
        n_mr += total;
        #pragma unroll 1
        for (int c = 0; c < 2; ++c) {
          #pragma unroll
          for (int r = 0; r < 4; ++r) {
            if (!((ws[r] >> (c + 1)) & 1u)) continue;
            const uint32_t nb = ((wf[r] >> c) & 7u) | ((wf[r + 1] >> c) & 5u) | ((wf[r + 2] >> c) & 7u);
            const uint32_t cx = ((wr[r] >> (c + 1)) & 1u) ? 16u : (nb ? 15u : 14u);  // helpers.rs:36-50
            *o++ = (uint8_t)((cx << 1) | ((wb[r] >> (c + 1)) & 1u));
          }
        }
      }
    } else {
      for (int y = lane; y < 64; y += 32) s.V[y] = 0;
      for (int y = lane; y < 68; y += 32) s.N[y] = 0;
      __syncwarp();
    }

    // ---- cleanup ----
    {
      uint64_t Gp = 0;  // final state (after this cleanup) of the row above
      const uint32_t start = pos;
      for (int k = 0; k < h; k += 4) {
        const int lim = min(4, h - k);
        uint64_t Gr[4], Vr[4], Br[4], Cr[4], Qr[4], Fr[4], Sg[4];
        for (int r = 0; r < 4; ++r) {
          const bool in = r < lim;
          Gr[r] = in ? (s.S[k + r + 1] | s.N[k + r + 1]) : 0;
          Vr[r] = in ? s.V[k + r] : 0;
          Br[r] = in ? s.B[k + r] : 0;
          Sg[r] = s.Sn[k + r + 1];
          Cr[r] = in ? (~Gr[r] & ~Vr[r] & valid) : 0;
          Qr[r] = Cr[r] & Br[r];
          Fr[r] = Gr[r] | Qr[r];
        }
        const uint64_t Gd = lim == 4 && k + 4 < h ? (s.S[k + 5] | s.N[k + 5]) : 0;  // next stripe, pre-CL
        const uint64_t SgP = s.Sn[k], SgD = s.Sn[k + 5];
        ns_cl += __popcll(Qr[0]) + __popcll(Qr[1]) + __popcll(Qr[2]) + __popcll(Qr[3]);
        if (lane == 0) {
          #pragma unroll
          for (int r = 0; r < 4; ++r)
            if (r < lim) s.Q[k + r + 1] = Qr[r];
        }
        // run-length eligibility of each column (flags.rs:219-235)
        uint64_t clean = 0;
        if (lim == 4) {
          uint64_t busy = Gr[0] | Gr[1] | Gr[2] | Gr[3] | Vr[0] | Vr[1] | Vr[2] | Vr[3];
          uint64_t nbr = dil(Gp) | westm(Fr[0] | Fr[1] | Fr[2] | Fr[3]) |
                         eastm(Gr[0] | Gr[1] | Gr[2] | Gr[3]) | dil(Gd);
          clean = ~(busy | nbr) & valid;
        }
        if (Cr[0] | Cr[1] | Cr[2] | Cr[3]) {  // any sample left to code in this stripe
          const uint32_t wgp = win4(Gp, sh), wgd = win4(Gd, sh), wcl = win4(clean, sh);
          uint32_t wG[4], wF[4], wC[4], wB[4], wsg[6];
          #pragma unroll
          for (int r = 0; r < 4; ++r) {
            wG[r] = win4(Gr[r], sh);
            wF[r] = win4(Fr[r], sh);
            wC[r] = win4(Cr[r], sh);
            wB[r] = win4(Br[r], sh);
          }
          wsg[0] = win4(SgP, sh);
          #pragma unroll
          for (int r = 0; r < 4; ++r) wsg[r + 1] = win4(Sg[r], sh);
          wsg[5] = win4(SgD, sh);
          // per column: candidate rows (4-bit), their bits, run-mode eligibility
          auto col_bits = [&](const uint32_t (&wv)[4], int c) {
            uint32_t m = 0;
            #pragma unroll
            for (int r = 0; r < 4; ++r) m |= ((wv[r] >> (c + 1)) & 1u) << r;
            return m;
          };
          uint32_t cnt = 0;
          #pragma unroll
          for (int c = 0; c < 2; ++c) {
            const uint32_t cmc = col_bits(wC, c), bmc = col_bits(wB, c);
            if ((wcl >> (c + 1)) & 1u) {
              if (bmc == 0) {
                cnt += 1;
              } else {
                const uint32_t after = 0xfu & ~((2u << (__ffs(bmc) - 1)) - 1u);
                cnt += 4 + __popc(after) + __popc(bmc & after);
              }
            } else {
              cnt += __popc(cmc) + __popc(cmc & bmc);
            }
          }
          uint32_t total;
          uint8_t* o = out + pos + warp_offset(cnt, lane, &total);
          pos += total;
          #pragma unroll 1
          for (int c = 0; c < 2; ++c) {
            const uint32_t cmc = col_bits(wC, c), bmc = col_bits(wB, c);
            int first = 0;
            if ((wcl >> (c + 1)) & 1u) {
              if (bmc == 0) {
                *o++ = (uint8_t)((uint32_t)kCtxAGG << 1);
                first = 4;
              } else {
                const int rl = __ffs(bmc) - 1;
                *o++ = (uint8_t)(((uint32_t)kCtxAGG << 1) | 1u);
                *o++ = (uint8_t)(((uint32_t)kCtxUNI << 1) | ((uint32_t)rl >> 1));
                *o++ = (uint8_t)(((uint32_t)kCtxUNI << 1) | ((uint32_t)rl & 1u));
                // sign of the run's first significant sample
                const uint32_t uf = rl == 0 ? wgp : pick4(wF, rl - 1), up = rl == 0 ? wgp : pick4(wG, rl - 1);
                const uint32_t df = rl == 3 ? wgd : pick4(wF, rl + 1), dp = rl == 3 ? wgd : pick4(wG, rl + 1);
                const uint32_t m8 = zc_index(uf, up, pick4(wF, rl), pick4(wG, rl), df, dp, c);
                *o++ = (uint8_t)sign_symbol(t, m8, pick6(wsg, rl + 1), pick6(wsg, rl), pick6(wsg, rl + 2), c);
                first = rl + 1;
              }
            }
            #pragma unroll
            for (int r = 0; r < 4; ++r) {
              if (r < first || !((cmc >> r) & 1u)) continue;
              const uint32_t uf = r == 0 ? wgp : wF[r > 0 ? r - 1 : 0], up = r == 0 ? wgp : wG[r > 0 ? r - 1 : 0];
              const uint32_t df = r == 3 ? wgd : wF[r < 3 ? r + 1 : 3], dp = r == 3 ? wgd : wG[r < 3 ? r + 1 : 3];
              const uint32_t m8 = zc_index(uf, up, wF[r], wG[r], df, dp, c);
              const uint32_t bit = (bmc >> r) & 1u;
              *o++ = (uint8_t)(((uint32_t)t.zc[m8] << 1) | bit);
              if (bit) *o++ = (uint8_t)sign_symbol(t, m8, wsg[r + 1], wsg[r], wsg[r + 2], c);
            }
          }
        }
        Gp = lim == 4 ? Fr[3] : (lim == 3 ? Fr[2] : (lim == 2 ? Fr[1] : Fr[0]));
      }
      if (lane == 0) {
        ItemRec rec;
        rec.n_sp = n_sp;
        rec.n_mr = n_mr;
        rec.n_cl = pos - start;
        rec.ns_sp = ns_sp;
        rec.ns_cl = ns_cl;
        rec.sig_before = sig_before;
        rec.bitplane = (uint32_t)p;
        rec.pad = 0;
        a.item_rec[item] = rec;
      }
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

void launch_t1_items(const T1Args& a, cudaStream_t st) {
  if (a.nblocks == 0) return;
  t1_items_kernel<<<(a.nblocks + 255) / 256, 256, 0, st>>>(a);
}

void launch_t1_model(const T1Args& a, int num_sms, cudaStream_t st) {
  if (a.nitems == 0) return;
  uint32_t need = (a.nitems + kModelWarps - 1) / kModelWarps;
  uint32_t cap = (uint32_t)num_sms * 8;
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
  chains = chains == 2 ? 2 : 1;
  const uint32_t per_pipe_cta = (uint32_t)kPipes * (uint32_t)chains;  // blocks a CTA codes at once
  const uint32_t pipe_ctas = std::max<uint32_t>(
      1u, std::min<uint32_t>((uint32_t)num_sms * (uint32_t)pipes_per_sm / kPipes,
                             (heavy + per_pipe_cta - 1) / per_pipe_cta));
  const uint32_t per_cta = kPipes * 2 * 32;
  const uint32_t packed_ctas = (a.nblocks - heavy + per_cta - 1) / per_cta;
  if (chains == 2)
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
