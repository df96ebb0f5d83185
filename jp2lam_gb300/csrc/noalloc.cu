// Allocation-free colour transform + DWT + quantiser for callers that cannot
// allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code running inside a
// captured CUDA graph, plug-in hosts that hand the library only
// pre-allocated buffers, and real-time loops that forbid allocator calls
// (which can synchronise the device). For them, jp2g_dwt_noalloc runs the
// first stage of the encoder (level shift + RCT/ICT, all DWT levels, deadzone
// quantisation) into a caller-supplied output buffer, and keeps its only
// scratch (the intermediate LL planes) in the fixed device array below.
//
// The array is file-scope and statically sized, so every GPU that loads this
// library holds it (8 MiB) until the process exits. All calls share it:
// calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race on it and must be serialised by the caller.
// Each level writes every LL element it later reads, so nothing in the array
// has to start at zero and stale contents from earlier calls are harmless.
#include <cuda_runtime.h>

#include <mutex>
#include <type_traits>

#include "../../include/jp2g.h"
#include "jp2g_internal.h"

namespace jp2g {
void set_thread_error(const char* msg);
bool plan_dwt_steps(uint32_t w, uint32_t h, int ncomp, int quality, int* levels, int* lossless,
                    float* steps, int* lo_w, int* lo_h, int* rw, int* rh);
}  // namespace jp2g

namespace {

// Two ping-pong LL planes of kNoAllocPlaneElems 32-bit elements each.
constexpr size_t kNoAllocPlaneElems = size_t(1) << 20;
static __device__ __align__(256) uint32_t g_noalloc_scratch[2 * kNoAllocPlaneElems];

// Host-side address of g_noalloc_scratch per device, resolved with
// cudaGetSymbolAddress while that device is current, together with the
// identity of the CUDA context it was resolved in. The address belongs to
// that context: after cudaDeviceReset (or under another context on the same
// device) it is resolved again, so a stale address is never launched with.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

// Unique id of the calling thread's current CUDA context (0 if none or if
// the driver does not report one). The driver entry points are fetched
// through the runtime, so the library does not link libcuda.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
    looked_up = true;
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

__constant__ float kA = -1.586134342059924f;
__constant__ float kB = -0.052980118572961f;
__constant__ float kG = 0.882911075530934f;
__constant__ float kD = 0.443506852043971f;
__constant__ float kKK = 1.230174104914001f;
__constant__ float kIK = 1.0f / 1.230174104914001f;

constexpr int TW = 128, TH = 64, NT = 256;

struct PlaneArgs {
  int from_pixels;
  const uint8_t* px;
  size_t px_pitch;
  int mct, ncomp;
  const void* src;
  size_t src_pitch, src_comp;
  int rw, rh;
  int no_transform;
  void* ll;  // next LL plane, or nullptr at the last level
  size_t ll_pitch, ll_comp;
  int32_t* out;  // Mallat-layout planes, component-major
  size_t out_pitch, out_comp;
  int lo_w, lo_h;  // size of this level's LL band (band origins)
  float step[4];   // quantiser step per orientation (LL, HL, LH, HH)
};

__device__ __forceinline__ int mirror(int i, int n) {
  if (n <= 1) return 0;
  if (i >= 0 && i < n) return i;
  int period = 2 * (n - 1);
  int k = i % period;
  if (k < 0) k += period;
  return k >= n ? period - k : k;
}

__device__ __forceinline__ float lift(float x, float c, float l, float r) {
  return __fadd_rn(x, __fmul_rn(c, __fadd_rn(l, r)));
}

template <bool REV>
__global__ void __launch_bounds__(NT) dwt_level_plane_kernel(PlaneArgs a) {
  using T = typename std::conditional<REV, int32_t, float>::type;
  constexpr int HALO = REV ? 2 : 4, SW = TW + 2 * HALO, SH = TH + 2 * HALO, P = SW + 1;
  __shared__ T s[SH * P];
  const int comp = blockIdx.z, x0 = blockIdx.x * TW, y0 = blockIdx.y * TH, tid = threadIdx.x;
  const int rw = a.rw, rh = a.rh;
  for (int i = tid; i < SH * SW; i += NT) {
    const int ly = i / SW, lx = i - ly * SW;
    const int gy = mirror(y0 - HALO + ly, rh), gx = mirror(x0 - HALO + lx, rw);
    T v;
    if (a.from_pixels) {
      const uint8_t* row = a.px + (size_t)gy * a.px_pitch;
      if (!a.mct) {
        v = (T)((int)row[(size_t)gx * a.ncomp + comp] - 128);
      } else {
        const int r = (int)row[(size_t)gx * 3] - 128, g = (int)row[(size_t)gx * 3 + 1] - 128,
                  b = (int)row[(size_t)gx * 3 + 2] - 128;
        if constexpr (REV) {
          v = comp == 0 ? ((r + 2 * g + b) >> 2) : (comp == 1 ? b - g : r - g);
        } else {
          const float rf = (float)r, gf = (float)g, bf = (float)b;
          if (comp == 0)
            v = __fadd_rn(__fadd_rn(__fmul_rn(0.299f, rf), __fmul_rn(0.587f, gf)), __fmul_rn(0.114f, bf));
          else if (comp == 1)
            v = __fadd_rn(__fadd_rn(__fmul_rn(-0.16875f, rf), __fmul_rn(-0.33126f, gf)), __fmul_rn(0.5f, bf));
          else
            v = __fsub_rn(__fsub_rn(__fmul_rn(0.5f, rf), __fmul_rn(0.41869f, gf)), __fmul_rn(0.08131f, bf));
        }
      }
    } else {
      v = reinterpret_cast<const T*>(a.src)[(size_t)comp * a.src_comp + (size_t)gy * a.src_pitch + gx];
    }
    s[ly * P + lx] = v;
  }
  __syncthreads();
  if (!a.no_transform) {
    if (rh >= 2) {
      for (int step = 0; step < (REV ? 2 : 4); ++step) {
        const int first = (step & 1) ? 2 : 1, nrows = (SH - 2 - first) / 2 + 1;
        for (int i = tid; i < nrows * SW; i += NT) {
          const int r = i / SW, lx = i - r * SW, ly = first + 2 * r;
          const T up = s[(ly - 1) * P + lx], dn = s[(ly + 1) * P + lx];
          if constexpr (REV) {
            if (step == 0) s[ly * P + lx] -= (up + dn) >> 1;
            else s[ly * P + lx] += (up + dn + 2) >> 2;
          } else {
            const float c = step == 0 ? kA : step == 1 ? kB : step == 2 ? kG : kD;
            s[ly * P + lx] = lift(s[ly * P + lx], c, up, dn);
          }
        }
        __syncthreads();
      }
      if constexpr (!REV) {
        for (int i = tid; i < SH * SW; i += NT) {
          const int ly = i / SW, lx = i - ly * SW;
          s[ly * P + lx] = __fmul_rn(s[ly * P + lx], (ly & 1) ? kKK : kIK);
        }
        __syncthreads();
      }
    } else if constexpr (!REV) {
      for (int i = tid; i < SH * SW; i += NT) s[(i / SW) * P + i % SW] = __fmul_rn(s[(i / SW) * P + i % SW], kIK);
      __syncthreads();
    }
    if (rw >= 2) {
      for (int step = 0; step < (REV ? 2 : 4); ++step) {
        const int first = (step & 1) ? 2 : 1, ncols = (SW - 2 - first) / 2 + 1;
        for (int i = tid; i < ncols * TH; i += NT) {
          const int r = i / ncols, ci = i - r * ncols, ly = HALO + r, lx = first + 2 * ci;
          const T l = s[ly * P + lx - 1], rr = s[ly * P + lx + 1];
          if constexpr (REV) {
            if (step == 0) s[ly * P + lx] -= (l + rr) >> 1;
            else s[ly * P + lx] += (l + rr + 2) >> 2;
          } else {
            const float c = step == 0 ? kA : step == 1 ? kB : step == 2 ? kG : kD;
            s[ly * P + lx] = lift(s[ly * P + lx], c, l, rr);
          }
        }
        __syncthreads();
      }
      if constexpr (!REV) {
        for (int i = tid; i < TH * SW; i += NT) {
          const int r = i / SW, lx = i - r * SW;
          s[(HALO + r) * P + lx] = __fmul_rn(s[(HALO + r) * P + lx], (lx & 1) ? kKK : kIK);
        }
        __syncthreads();
      }
    } else if constexpr (!REV) {
      for (int i = tid; i < TH * SW; i += NT) {
        const int r = i / SW, lx = i - r * SW;
        s[(HALO + r) * P + lx] = __fmul_rn(s[(HALO + r) * P + lx], kIK);
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < TH * TW; i += NT) {
    const int ly = i / TW, j = i - ly * TW;
    const int lx = a.no_transform ? j : (j < TW / 2 ? 2 * j : 2 * (j - TW / 2) + 1);
    const int gy = y0 + ly, gx = x0 + lx;
    if (gy >= rh || gx >= rw) continue;
    const T v = s[(HALO + ly) * P + HALO + lx];
    int orient = 0, px = gx, py = gy;
    if (!a.no_transform) {
      orient = ((gy & 1) << 1) | (gx & 1);
      const int u = gx >> 1, vv = gy >> 1;
      px = u + ((orient & 1) ? a.lo_w : 0);
      py = vv + ((orient & 2) ? a.lo_h : 0);
      if (orient == 0 && a.ll != nullptr) {
        reinterpret_cast<T*>(a.ll)[(size_t)comp * a.ll_comp + (size_t)vv * a.ll_pitch + u] = v;
        continue;
      }
    }
    int32_t q;
    if constexpr (REV) q = v;
    else q = __float2int_rz(__fdiv_rn(v, a.step[orient]));
    a.out[(size_t)comp * a.out_comp + (size_t)py * a.out_pitch + px] = q;
  }
}

int fail(int code, const char* msg) {
  jp2g::set_thread_error(msg);
  return code;
}

}  // namespace

extern "C" int jp2g_dwt_noalloc(const uint8_t* d_px, uint32_t w, uint32_t h, uint32_t ncomp,
                                uint8_t quality, int32_t* d_coef, void* stream) {
  if (!d_px || !d_coef) return fail(JP2G_INVALID_INPUT, "pixel or coefficient pointer is null");
  if (w == 0 || h == 0) return fail(JP2G_INVALID_INPUT, "image dimensions must be non-zero");
  if (ncomp != 1 && ncomp != 3) return fail(JP2G_INVALID_INPUT, "images must have 1 or 3 components");
  int levels = 0, lossless = 0;
  float steps[1 + 3 * 6];
  int lo_w[7], lo_h[7], rw[7], rh[7];
  if (!jp2g::plan_dwt_steps(w, h, (int)ncomp, quality, &levels, &lossless, steps, lo_w, lo_h, rw, rh))
    return fail(JP2G_INVALID_INPUT, "unsupported image parameters");
  // Scratch: the LL plane of every level but the last (the largest is level 1's).
  const size_t ll_elems = ((size_t)w + 1) / 2 * (((size_t)h + 1) / 2) * ncomp;
  if (levels >= 2 && ll_elems > kNoAllocPlaneElems)
    return fail(JP2G_INVALID_INPUT,
                "image too large for the allocation-free path: ceil(w/2)*ceil(h/2)*ncomp must be "
                "<= 1048576 (e.g. 2048x2048 gray, 1182x1182 RGB)");
  if ((size_t)w * h * ncomp > (size_t)1 << 31)
    return fail(JP2G_INVALID_INPUT, "image too large");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(JP2G_ENCODE_FAILED, "no usable current CUDA device");
  void* scratch = nullptr;
  {
    // Set-up once per device (and again for a new context on it): the
    // array's device address, resolved with the device current. The first
    // call on a device does this, so it should come before any stream
    // capture that uses this entry point.
    std::lock_guard<std::mutex> lk(g_setup_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_scratch_ptr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // creates the context if needed
      if (e != cudaSuccess || p == nullptr) return fail(JP2G_ENCODE_FAILED, cudaGetErrorString(e));
      g_scratch_ptr[dev] = p;
      g_scratch_ctx[dev] = current_context_id();
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  uint32_t* planes[2] = {static_cast<uint32_t*>(scratch), static_cast<uint32_t*>(scratch) + kNoAllocPlaneElems};
  PlaneArgs a{};
  a.px = d_px;
  a.px_pitch = (size_t)w * ncomp;
  a.mct = ncomp == 3;
  a.ncomp = (int)ncomp;
  a.out = d_coef;
  a.out_pitch = w;
  a.out_comp = (size_t)w * h;
  const void* src = nullptr;
  size_t src_pitch = 0, src_comp = 0;
  const int nlev = levels == 0 ? 1 : levels;
  for (int l = 1; l <= nlev; ++l) {
    const int res = levels - l + 1;  // resolution whose detail bands this level writes
    a.from_pixels = l == 1;
    a.src = src;
    a.src_pitch = src_pitch;
    a.src_comp = src_comp;
    a.no_transform = levels == 0;
    a.rw = levels == 0 ? (int)w : rw[res];
    a.rh = levels == 0 ? (int)h : rh[res];
    a.lo_w = levels == 0 ? 0 : lo_w[res];
    a.lo_h = levels == 0 ? 0 : lo_h[res];
    a.step[0] = steps[0];  // LL (used at the last level or without a transform)
    for (int o = 1; o < 4; ++o) a.step[o] = levels == 0 ? 0.f : steps[1 + 3 * (res - 1) + (o - 1)];
    if (l < levels) {
      a.ll = planes[(l - 1) & 1];
      a.ll_pitch = (size_t)lo_w[res];
      a.ll_comp = a.ll_pitch * (size_t)lo_h[res];
      src = a.ll;
      src_pitch = a.ll_pitch;
      src_comp = a.ll_comp;
    } else {
      a.ll = nullptr;
    }
    dim3 grid((a.rw + TW - 1) / TW, (a.rh + TH - 1) / TH, ncomp);
    if (lossless) dwt_level_plane_kernel<true><<<grid, NT, 0, st>>>(a);
    else dwt_level_plane_kernel<false><<<grid, NT, 0, st>>>(a);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(JP2G_ENCODE_FAILED, cudaGetErrorString(e));
  return JP2G_OK;
}
