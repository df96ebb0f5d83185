// Tier-2 on the device: packet headers and codestream assembly.
//
// Replaces build_packet_header / build_packet_sequence_for_components
// (src/encode/backend/native/t2.rs:337-473) with its tag trees (t2.rs:83-229)
// and the codestream/JP2 writers (src/j2k/write.rs:9-77, src/jp2.rs:13-71)
// for the device path: only the finished codestreams cross to the host.
//
// A packet is the bands of one (resolution, component) (one layer, one
// precinct). The bits of a packet header are laid out in parallel:
//  - a tag tree's node values are minima over its leaves (level by level);
//  - with one layer a node's bits are emitted only once, by the first leaf
//    (in raster order) whose walk reaches it: for the inclusion tree every
//    leaf walks, so that is the top-left leaf of the node's region; for the
//    zero bit-plane tree only included leaves walk, so it is the first
//    included leaf of the region (ISO/IEC 15444-1 B.10.2);
//  - so every code-block knows its own header bits (inclusion, zero
//    bit-planes, Table B-4 pass count, Lblock comma code and length,
//    B.10.4-B.10.7), a prefix sum gives their positions, and each thread
//    ORs its bits into an unstuffed big-endian bitstream;
//  - a warp pass cuts the bitstream into bytes, a byte after 0xFF
//    taking only 7 bits (B.10.1), and ends the header with a zero byte when
//    its last byte is 0xFF.
// One CTA per packet: the tag trees and, for the stuffing pass, the
// header's bits are staged in shared memory. The pages are then placed by
// copy jobs of 16 KiB spread over the whole GPU (each packet's header and
// body), and one warp per page writes the host-built marker prefix (JP2
// boxes, SOC..SOD) with Psot and the jp2c box length filled in, and EOC.
#include <cuda_runtime.h>

#include "jp2g_internal.h"
#include "kernels.h"

namespace jp2g {

namespace {

constexpr uint32_t kNone = 0xffffffffu;

__device__ __forceinline__ uint32_t flog2(uint32_t v) { return v == 0 ? 0 : 31 - __clz(v); }

// ORs the n (<= 32) low bits of v, most significant first, into the
// big-endian bitstream at bit position pos.
__device__ __forceinline__ void put_bits(uint32_t* raw, uint32_t pos, uint32_t v, int n) {
  if (n <= 0) return;
  const uint64_t x = (uint64_t)(n == 32 ? v : (v & ((1u << n) - 1u))) << (64 - n - (int)(pos & 31));
  const uint32_t hi = (uint32_t)(x >> 32), lo = (uint32_t)x;
  if (hi) atomicOr(raw + (pos >> 5), hi);
  if (lo) atomicOr(raw + (pos >> 5) + 1, lo);
}

__device__ __forceinline__ uint32_t get_bits(const uint32_t* raw, uint32_t pos, int n) {  // n <= 8
  const uint64_t x = (uint64_t)raw[pos >> 5] << 32 | raw[(pos >> 5) + 1];
  return (uint32_t)(x >> (64 - n - (int)(pos & 31))) & ((1u << n) - 1u);
}

// Table B-4 codeword of a pass count: (value, length).
__device__ __forceinline__ void passes_code(uint32_t n, uint32_t* v, int* len) {
  if (n == 1) { *v = 0; *len = 1; }
  else if (n == 2) { *v = 2; *len = 2; }
  else if (n <= 5) { *v = 0xcu | (n - 3); *len = 4; }
  else if (n <= 36) { *v = 0x1e0u | (n - 6); *len = 9; }
  else { *v = 0xff80u | (min(n, 164u) - 37); *len = 16; }
}

struct LevelGeom {
  uint32_t w[16], off[16];
  int n;
};

// Header bits of leaf (x, y) of a band; when `raw` is set they are written
// at `pos`. Returns the bit count.
__device__ uint32_t leaf_bits(const LevelGeom& g, const T2Node* tree, uint32_t leaf, int x, int y,
                              const BlockKeep& k, uint32_t* raw, uint32_t pos) {
  const uint32_t p0 = pos;
  // inclusion (threshold 1): first-visited nodes down to the first node
  // with no included leaf
  for (int l = g.n - 1; l >= 0; --l) {
    const T2Node nd = tree[g.off[l] + (uint32_t)(y >> l) * g.w[l] + (uint32_t)(x >> l)];
    const bool inc = nd.first_inc != kNone;
    const uint32_t m = (1u << l) - 1u;
    if (((uint32_t)x & m) == 0 && ((uint32_t)y & m) == 0) {
      if (raw && inc) put_bits(raw, pos, 1u, 1);
      ++pos;
    }
    if (!inc) break;
  }
  if (k.npasses == 0) return pos - p0;
  // zero bit-planes (threshold above any value): nodes this leaf reaches
  // first among the included ones emit their value above the parent's as
  // zeros, then a one
  uint32_t parent = 0;
  for (int l = g.n - 1; l >= 0; --l) {
    const T2Node nd = tree[g.off[l] + (uint32_t)(y >> l) * g.w[l] + (uint32_t)(x >> l)];
    if (nd.first_inc == leaf) {
      pos += nd.zmin - parent;
      if (raw) put_bits(raw, pos, 1u, 1);
      ++pos;
    }
    parent = nd.zmin;
  }
  uint32_t cv;
  int cl;
  passes_code(k.npasses, &cv, &cl);
  if (raw) put_bits(raw, pos, cv, cl);
  pos += (uint32_t)cl;
  // Lblock: 3, raised by a comma code until seg_len fits (B.10.7.1)
  const uint32_t need = k.seg_len == 0 ? 0 : flog2(k.seg_len) + 1;
  const uint32_t have = 3 + flog2(k.npasses);
  const uint32_t inc = need > have ? need - have : 0;
  if (raw) {
    for (uint32_t t = 0; t < inc; t += 32) put_bits(raw, pos + t, 0xffffffffu, (int)min(32u, inc - t));
  }
  pos += inc + 1;  // the ones and the terminating zero
  const int nb = (int)(have + inc);
  if (raw) {
    if (nb > 32) {
      put_bits(raw, pos, 0, nb - 32);  // seg_len < 2^32: the top bits are zero
      put_bits(raw, pos + (uint32_t)(nb - 32), k.seg_len, 32);
    } else {
      put_bits(raw, pos, k.seg_len, nb);
    }
  }
  pos += (uint32_t)nb;
  return pos - p0;
}

constexpr int kT2Threads = 256;
constexpr int kT2SmemNodes = 4096;     // tag trees of bands up to ~3,000 code-blocks; then the header bits
constexpr uint32_t kT2Chunk = 16384;   // bytes of output one copy job moves

__global__ void __launch_bounds__(kT2Threads) t2_header_kernel(T2Args a) {
  __shared__ uint64_t sbuf[kT2SmemNodes];
  __shared__ uint32_t wsum[kT2Threads / 32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint32_t pk_id = blockIdx.x;
  const T2Packet pk = a.packets[pk_id];
  uint32_t* raw = a.raw + pk.raw_off;
  uint32_t pos = 1;  // bit 0: the packet is present (t2.rs:337-344)
  if (tid == 0) put_bits(raw, 0, 1u, 1);
  for (uint32_t bi = pk.band0; bi < pk.band0 + pk.nbands; ++bi) {
    const T2Band bd = a.bands[bi];
    const uint32_t n = (uint32_t)bd.ncbx * bd.ncby;
    if (n == 0) continue;
    LevelGeom g;
    {
      uint32_t w = bd.ncbx, h = bd.ncby, off = 0;
      g.n = 0;
      for (;;) {
        g.w[g.n] = w;
        g.off[g.n] = off;
        ++g.n;
        off += w * h;
        if (w * h <= 1 || g.n == 16) break;
        w = (w + 1) / 2;
        h = (h + 1) / 2;
      }
    }
    // the band's tag trees in shared memory when they fit
    const uint32_t nodes = g.off[g.n - 1] + 1;
    T2Node* tree = nodes <= (uint32_t)kT2SmemNodes ? reinterpret_cast<T2Node*>(sbuf) : a.tree + bd.tree_off;
    // leaves, then each level's minima
    for (uint32_t i = tid; i < n; i += kT2Threads) {
      const BlockKeep k = a.keep[bd.first_block + i];
      tree[i] = T2Node{k.zbp, k.npasses > 0 ? i : kNone};
    }
    __syncthreads();
    for (int l = 1; l < g.n; ++l) {
      const uint32_t cw = g.w[l - 1], ch = (g.off[l] - g.off[l - 1]) / cw, w = g.w[l];
      const uint32_t h = (ch + 1) / 2;
      for (uint32_t k = tid; k < w * h; k += kT2Threads) {
        const uint32_t x = k % w, y = k / w;
        uint32_t z = 0xffffffffu, f = kNone;
        for (uint32_t dy = 0; dy < 2; ++dy)
          for (uint32_t dx = 0; dx < 2; ++dx) {
            const uint32_t cx = 2 * x + dx, cy = 2 * y + dy;
            if (cx >= cw || cy >= ch) continue;
            const T2Node c = tree[g.off[l - 1] + cy * cw + cx];
            z = min(z, c.zmin);
            f = min(f, c.first_inc);
          }
        tree[g.off[l] + k] = T2Node{z, f};
      }
      __syncthreads();
    }
    // header bits of the band's blocks, 256 at a time in raster order
    for (uint32_t c0 = 0; c0 < n; c0 += kT2Threads) {
      const uint32_t i = c0 + tid;
      uint32_t cnt = 0;
      BlockKeep k{};
      const int x = (int)(i % bd.ncbx), y = (int)(i / bd.ncbx);
      if (i < n) {
        k = a.keep[bd.first_block + i];
        cnt = leaf_bits(g, tree, i, x, y, k, nullptr, 0);
      }
      uint32_t incl = cnt;
      #pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(~0u, incl, o);
        if (lane >= o) incl += t;
      }
      if (lane == 31) wsum[wid] = incl;
      __syncthreads();
      uint32_t before = 0, total = 0;
      #pragma unroll
      for (int k2 = 0; k2 < kT2Threads / 32; ++k2) {
        before += k2 < wid ? wsum[k2] : 0u;
        total += wsum[k2];
      }
      if (i < n) leaf_bits(g, tree, i, x, y, k, raw, pos + before + incl - cnt);
      pos += total;
      __syncthreads();
    }
  }
  __syncthreads();  // every bit is in `raw`
  // stage the bits in shared memory when they fit
  const uint32_t nbits = pos;
  const uint32_t nwords = (nbits + 31) / 32 + 2;  // the slot has two words of slack
  const uint32_t* rb = raw;
  if (nwords <= 2u * kT2SmemNodes) {
    uint32_t* s32 = reinterpret_cast<uint32_t*>(sbuf);
    for (uint32_t wd = tid; wd < nwords; wd += kT2Threads) s32[wd] = raw[wd];
    __syncthreads();
    rb = s32;
  }
  if (wid != 0) return;
  // bytes: 8 bits each, 7 after a 0xFF byte; a final 0xFF is followed by a
  // zero byte (ISO/IEC 15444-1 B.10.1)
  uint8_t* out = a.hdr + pk.hdr_off;
  uint32_t p = 0, nout = 0;
  bool prev_ff = false;
  while (p < nbits) {
    const uint32_t w0 = prev_ff ? 7u : 8u;
    const uint32_t start = p + (lane == 0 ? 0u : w0 + 8u * (uint32_t)(lane - 1));
    const int width = lane == 0 ? (int)w0 : 8;
    const bool valid = start < nbits;
    const uint32_t byte = valid ? get_bits(rb, start, width) : 0u;
    const uint32_t ff = __ballot_sync(~0u, valid && byte == 0xffu);
    const uint32_t vm = __ballot_sync(~0u, valid);
    const int last = ff ? __ffs(ff) - 1 : 31;  // bytes after a 0xFF need the 7-bit rule
    const uint32_t produced = min((uint32_t)(last + 1), (uint32_t)__popc(vm));
    if ((uint32_t)lane < produced) out[nout + lane] = (uint8_t)byte;
    nout += produced;
    p += w0 + 8u * (produced - 1);
    prev_ff = ff != 0 && produced == (uint32_t)(last + 1);
  }
  if (prev_ff) {
    if (lane == 0) out[nout] = 0;
    ++nout;
  }
  if (lane == 0) a.hdr_len[pk_id] = nout;
}

// Page layout: every packet's place in its page and its number of copy
// jobs, and each page's length.
__global__ void t2_layout_kernel(T2Args a) {
  const uint32_t pg = blockIdx.x * blockDim.x + threadIdx.x;
  if (pg >= a.npages) return;
  const T2Page p = a.pages[pg];
  uint32_t off = p.tmpl_len;
  for (uint32_t k = p.packet0; k < p.packet0 + p.npackets; ++k) {
    const T2Packet pk = a.packets[k];
    const uint32_t len = a.hdr_len[k] + (a.offsets[pk.b1] - a.offsets[pk.b0]);
    a.pkt_off[k] = off;
    a.nchunks[k] = (len + kT2Chunk - 1) / kT2Chunk;
    off += len;
  }
  a.page_len[pg] = off + 2;  // EOC
}

// Copy jobs over the whole GPU: job j moves up to kT2Chunk bytes of one
// packet (its header, then its body) into place.
__global__ void __launch_bounds__(kT2Threads) t2_copy_kernel(T2Args a) {
  const uint32_t njobs = a.chunk_base[a.npackets];
  for (uint32_t job = blockIdx.x; job < njobs; job += gridDim.x) {
    uint32_t lo = 0, hi = a.npackets;  // packet k with chunk_base[k] <= job < chunk_base[k + 1]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) / 2;
      if (a.chunk_base[mid] <= job) lo = mid;
      else hi = mid;
    }
    const uint32_t k = lo;
    const T2Packet pk = a.packets[k];
    uint8_t* o = a.out + a.page_off[pk.page] + a.pkt_off[k];
    const uint32_t hl = a.hdr_len[k];
    const uint8_t* h = a.hdr + pk.hdr_off;
    const uint8_t* b = a.body + a.offsets[pk.b0] - hl;  // body byte i - hl at b[i]
    const uint32_t len = hl + (a.offsets[pk.b1] - a.offsets[pk.b0]);
    const uint32_t from = (job - a.chunk_base[k]) * kT2Chunk, to = min(from + kT2Chunk, len);
    #pragma unroll 4
    for (uint32_t i = from + threadIdx.x; i < to; i += kT2Threads) o[i] = i < hl ? h[i] : b[i];
  }
}

__device__ __forceinline__ void put_be32(uint8_t* o, uint32_t v) {
  o[0] = (uint8_t)(v >> 24);
  o[1] = (uint8_t)(v >> 16);
  o[2] = (uint8_t)(v >> 8);
  o[3] = (uint8_t)v;
}

// One warp per page: the marker prefix with Psot and the jp2c length
// filled in, and EOC.
__global__ void __launch_bounds__(128) t2_pages_kernel(T2Args a) {
  const int lane = threadIdx.x & 31;
  const uint32_t pg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (pg >= a.npages) return;
  const T2Page p = a.pages[pg];
  uint8_t* o = a.out + a.page_off[pg];
  for (uint32_t i = lane; i < p.tmpl_len; i += 32) o[i] = a.tmpl[p.tmpl_off + i];
  __syncwarp();
  const uint32_t len = a.page_len[pg];
  if (lane == 0) {
    const uint32_t payload = len - 2 - p.tmpl_len;
    put_be32(o + p.psot_pos, 12u + 2u + payload);  // SOT segment + SOD + packets (write.rs:54-77)
    if (p.jp2c_pos != kNone) put_be32(o + p.jp2c_pos, len - p.jp2c_pos);  // jp2c box: its header + the codestream
    o[len - 2] = 0xff;
    o[len - 1] = 0xd9;
  }
}

}  // namespace

void launch_t2(const T2Args& a, uint32_t* scan_scratch, int num_sms, cudaStream_t st) {
  if (a.npackets == 0) return;
  t2_header_kernel<<<a.npackets, kT2Threads, 0, st>>>(a);
  t2_layout_kernel<<<(a.npages + 127) / 128, 128, 0, st>>>(a);
  launch_scan_u32(a.page_len, 1, a.npages, a.page_off, scan_scratch, st);
  launch_scan_u32(a.nchunks, 1, a.npackets, a.chunk_base, scan_scratch, st);
  t2_copy_kernel<<<(unsigned)num_sms * 8, kT2Threads, 0, st>>>(a);
  t2_pages_kernel<<<(a.npages + 3) / 4, 128, 0, st>>>(a);
}

}  // namespace jp2g
