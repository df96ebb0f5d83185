/*
 * jp2g — GB300-native JPEG 2000 encode engine, C ABI.
 *
 * The drop-in boundary for jp2lam's encode path. A Rust (or any FFI) host
 * keeps jp2lam's public types (Image, EncodeOptions, BatchEncoder) and calls
 * these entry points instead of NativeBackend through an extern "C" block.
 * Plain pointers and sizes only.
 *
 * Status codes map 1:1 to jp2lam::Jp2LamError (src/error.rs:7-13):
 *   0 ok, 1 InvalidInput, 2 EncodeFailed, 3 DecodeFailed,
 *   4 UnsupportedFeature, 5 Io.
 * Every entry point validates its arguments before any device work; a failed
 * call leaves a message for jp2g_last_error(). There is no CPU fallback: a
 * context cannot be created without a usable CUDA device.
 */
#ifndef JP2G_H
#define JP2G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct jp2g_ctx jp2g_ctx;

enum {
  JP2G_OK = 0,
  JP2G_INVALID_INPUT = 1,
  JP2G_ENCODE_FAILED = 2,
  JP2G_DECODE_FAILED = 3,
  JP2G_UNSUPPORTED_FEATURE = 4,
  JP2G_IO = 5,
  JP2G_PENDING = 6 /* jp2g_poll only: the result is not ready yet */
};

enum { JP2G_FORMAT_J2K = 0, JP2G_FORMAT_JP2 = 1 };

/* One engine per process and GPU. Owns a CUDA stream and device buffer pools
 * that grow on demand up to `hbm_budget_bytes` (0 = no limit). Under a
 * budget, a device wave whose pools would not fit is retried from empty
 * pools and then split in halves (recursively), and later waves are capped
 * at the size that fitted; only a page that does not fit on its own fails
 * (JP2G_ENCODE_FAILED, "device memory budget exhausted ..."). No
 * jp2g_poll may be waiting when jp2g_destroy is called; queued requests are
 * finished first.
 * Replaces the construction of NativeBackend (src/encode/backend/mod.rs:6-9;
 * src/encode/mod.rs:87). */
int jp2g_create(jp2g_ctx** ctx, int device, uint64_t hbm_budget_bytes);
void jp2g_destroy(jp2g_ctx* ctx);

/* Encode one 8-bit page: ncomp 1 (gray) or 3 (sRGB); `interleaved` selects
 * RGBRGB... (as Image::from_rgb_bytes takes, src/model.rs:87-117) or three
 * planes; quality 0..100 (100 = lossless 5/3); format JP2G_FORMAT_*.
 * On success *out holds a malloc'd J2K/JP2 byte string (free with
 * jp2g_free) byte-identical to jp2lam::encode (src/encode/mod.rs:84-101).
 * Replaces NativeBackend::encode_codestream (src/encode/backend/native/
 * backend.rs:32-40) plus the JP2 wrap (src/jp2.rs:13-50). */
int jp2g_encode(jp2g_ctx* ctx, const uint8_t* px, uint32_t w, uint32_t h, uint32_t ncomp,
                int interleaved, uint8_t quality, int format, uint8_t** out, size_t* out_len);

/* jp2g_encode plus the encode's quality metrics, as encode_with_psnr
 * (src/encode/mod.rs:129-135) computes them (compute_quality_metrics,
 * src/encode/backend/native/backend.rs:305-433): the retained bit-planes of
 * every code-block dequantised at the midpoint, the inverse 9/7, inverse ICT
 * and level shift give the decoded samples, all on the device; *psnr_db is
 * their PSNR against the input (100 when the error is below 1e-10) and *ssim
 * the mean SSIM of 8x8 luma blocks (1.0 when the page has none). Lossless
 * encodes (quality >= 100) give +infinity and 1.0. */
int jp2g_encode_with_psnr(jp2g_ctx* ctx, const uint8_t* px, uint32_t w, uint32_t h, uint32_t ncomp,
                          int interleaved, uint8_t quality, int format, uint8_t** out, size_t* out_len,
                          double* psnr_db, double* ssim);

/* Decodes a J2K or JP2 file as decode_jp2 does (src/decode/mod.rs:56-61):
 * single tile, one quality layer, LRCP, one precinct per resolution, 8-bit
 * gray or 3-component, 64x64 or smaller code-blocks — the codestreams this
 * library and the reference write. The host parses the boxes, the main
 * header and the packet headers; code-block decoding (MQ decoder and the
 * three passes), dequantisation, the inverse DWT and inverse RCT/ICT run on
 * the device. *px (free with jp2g_free) receives w * h * ncomp interleaved
 * samples. Malformed input gives JP2G_DECODE_FAILED, codestreams outside
 * that profile JP2G_UNSUPPORTED_FEATURE, each with a message.
 * flags (both off: the reference decoder's behaviour):
 *   JP2G_DECODE_RCT_CHROMA_EXTRA_BITPLANE counts one more magnitude bit-plane
 *     for the chroma of reversible RCT codestreams (the encoder codes them
 *     with it at quality 100, and QCD does not signal it);
 *   JP2G_DECODE_ACCEPT_EMPTY_SEGMENTS decodes a code-block that has coding
 *     passes but a segment of zero bytes (which the encoder can emit) from an
 *     all-0xFF stream instead of failing as decode/t1.rs:109-111 does. */
enum { JP2G_DECODE_RCT_CHROMA_EXTRA_BITPLANE = 1, JP2G_DECODE_ACCEPT_EMPTY_SEGMENTS = 2 };
int jp2g_decode(jp2g_ctx* ctx, const uint8_t* bytes, size_t n, int flags, uint8_t** px, size_t* px_len,
                uint32_t* w, uint32_t* h, uint32_t* ncomp);

/* jp2g_decode over n files at once (bytes[i], lens[i]): the files share
 * device launches (one Tier-1 decoding launch over all their code-blocks,
 * one inverse-DWT launch pair per level, one for the samples), in rounds
 * that fit the device memory budget. Per file: outs[i]/out_lens[i] (free
 * with jp2g_free), ws/hs/ncomps and status[i]; one file's failure does not
 * fail the others. Returns JP2G_OK or the first failing file's status (its
 * message in jp2g_last_error). Samples equal jp2g_decode's for each file. */
int jp2g_decode_batch(jp2g_ctx* ctx, const uint8_t* const* bytes, const size_t* lens, uint32_t n, int flags,
                      uint8_t** outs, size_t* out_lens, uint32_t* ws, uint32_t* hs, uint32_t* ncomps,
                      int* status);

/* Same as jp2g_encode, but `d_px` is interleaved pixel data already resident
 * in device memory (w * h * ncomp bytes). Used for device-resident batching;
 * the reference has no equivalent entry point (its input is always host
 * memory). */
int jp2g_encode_device(jp2g_ctx* ctx, const uint8_t* d_px, uint32_t w, uint32_t h,
                       uint32_t ncomp, uint8_t quality, int format, uint8_t** out,
                       size_t* out_len);

void jp2g_free(uint8_t* p);

/* One page of a batch or a served request. `px` holds w*h*ncomp 8-bit
 * samples: host memory, or device memory of the context's GPU when
 * on_device != 0 (then interleaved). Gray is ncomp 1; sRGB is ncomp 3,
 * interleaved RGBRGB (interleaved != 0, Image::from_rgb_bytes) or planar.
 * quality 0..255 (>= 100 is lossless, as EncodeOptions::quality);
 * format 0 = J2K, 1 = JP2. */
typedef struct jp2g_request {
  const uint8_t* px;
  uint32_t width, height, ncomp;
  int32_t interleaved;
  int32_t on_device;
  int32_t quality;
  int32_t format;
} jp2g_request;

/* Encodes n pages. Pages are grouped into device waves that share one flat
 * code-block work list (colour+DWT per page, then Tier-1, PCRD and
 * compaction and Tier-2 over all the wave's blocks and packets in single
 * launches; only the finished codestreams are read back). Per page:
 * outs[i]/out_lens[i] receive the codestream (free with jp2g_free) and
 * status[i] its status; one page's failure does not fail the others.
 * Returns JP2G_OK, or the first failing page's status (its message in
 * jp2g_last_error). Output bytes equal jp2g_encode's for each page.
 * Replaces BatchEncoder::encode_one / encode_all and encode_batch
 * (src/batch.rs:39-70, 173), which encode page after page. */
int jp2g_encode_batch(jp2g_ctx* ctx, const jp2g_request* reqs, uint32_t n, uint8_t** outs,
                      size_t* out_lens, int* status);

/* Continuous batching. jp2g_submit validates the request (validate_image,
 * src/plan/validate.rs:4-62, before any device work) and queues it. Queued
 * requests are admitted into device waves of up to JP2G_OPT_WAVE_BLOCKS
 * code-blocks. Without a memory budget, a stager thread admits the next wave
 * and uploads its pixels while a worker thread runs the current one; under
 * a budget, the worker admits each wave as the previous one leaves the
 * device. Another thread completes the finished waves' tickets. The pixel
 * buffer must stay valid until jp2g_poll has returned the ticket's result.
 * jp2g_poll waits up to timeout_ms (< 0: no limit) and returns the
 * request's status with its codestream, or JP2G_PENDING if it is not done
 * (poll again); a returned result releases the ticket. Both calls are
 * thread-safe. No reference counterpart: the reference has no server
 * loop. */
int jp2g_submit(jp2g_ctx* ctx, const jp2g_request* req, uint64_t* ticket);
int jp2g_poll(jp2g_ctx* ctx, uint64_t ticket, uint8_t** out, size_t* out_len, int timeout_ms);

/* Cancels a submitted request. JP2G_OK: it had not been admitted to a device
 * wave and is removed from the queue, or it had already finished and its
 * result is dropped; either way its ticket is released (the pixel buffer
 * may be reused at once; a later jp2g_poll reports an unknown ticket).
 * JP2G_PENDING: its wave is formed (staged, on the device or in Tier-2); the
 * result is dropped, and jp2g_poll on the ticket returns
 * JP2G_ENCODE_FAILED ("request cancelled") once the wave is done -- the
 * pixel buffer must stay valid until then. A poll already waiting on a
 * cancelled request returns that same status. JP2G_INVALID_INPUT: unknown
 * ticket. No reference counterpart: the reference has no request queue. */
int jp2g_cancel(jp2g_ctx* ctx, uint64_t ticket);

/* Tuning knobs (the autotuner sets these):
 * JP2G_OPT_WAVE_BLOCKS        most code-blocks per device wave (default 240000,
 *                             160000 under a memory budget;
 *                             waves never exceed 246,723 64x64 blocks or
 *                             838,860 32x32 blocks, whose payload slots need
 *                             32-bit offsets);
 * JP2G_OPT_MQ_BLOCKS_PER_WARP code-blocks per warp in MQ coding, 1..32, or 0
 *                             for automatic (1 up to 48 blocks per SM, else
 *                             2..32 for about 24 warps per SM);
 * JP2G_OPT_HOST_THREADS       host threads for staging and Tier-2 (0 = all but
 *                             two hardware threads);
 * JP2G_OPT_MQ_WARPS_PER_SM    with one code-block per warp, the warps per SM
 *                             that pull blocks heaviest first (0 = automatic:
 *                             8 up to 16 blocks per SM, else 12; -1 = one warp
 *                             per block, no pulling);
 * JP2G_OPT_MQ_PIPES_PER_SM    when pulling: producer/consumer warp pairs per
 *                             SM that split each block's MQ chain into its
 *                             interval and code-register halves (0 =
 *                             automatic: 8 pairs per SM up to 48 blocks per
 *                             SM; -1 = single-warp pulling);
 * JP2G_OPT_MQ_HEAVY           with pipelines: how many of the heaviest blocks
 *                             they take, the rest being coded 32 to a warp
 *                             (0 = all blocks);
 * JP2G_OPT_MQ_CHAINS_PER_PAIR with pipelines: code-blocks each pair codes at
 *                             once, 1 (all lanes of a warp on one chain), 2
 *                             (one per half-warp: about half the issue slots
 *                             per symbol) or 4 (one per quarter-warp); 0 =
 *                             automatic (1 up to 8 blocks per SM, 2 up to 24,
 *                             else 4 on 4 pairs per SM). */
enum {
  JP2G_OPT_WAVE_BLOCKS = 0,
  JP2G_OPT_MQ_BLOCKS_PER_WARP = 1,
  JP2G_OPT_HOST_THREADS = 2,
  JP2G_OPT_MQ_WARPS_PER_SM = 3,
  JP2G_OPT_MQ_PIPES_PER_SM = 4,
  JP2G_OPT_MQ_HEAVY = 5,
  JP2G_OPT_MQ_CHAINS_PER_PAIR = 6,
  JP2G_NUM_OPTS = 7
};
int jp2g_set_option(jp2g_ctx* ctx, int option, int64_t value);
int jp2g_get_option(jp2g_ctx* ctx, int option, int64_t* value);

/* Autotuner: encodes the caller's sample pages (through jp2g_encode_batch)
 * under each candidate setting of the MQ schedule (automatic; 4, 8 or 16
 * producer/consumer pairs per SM with one or two chains each; 8, 12 or 16
 * pulling warps per SM; 2 to 32 blocks packed per warp), then of the wave
 * size (20,000 to 240,000 code-blocks) under the fastest schedule, and
 * leaves the fastest setting on the context. A candidate's time is the least
 * wall time of `repeats` (1..100) encodes after one untimed encode. Every
 * candidate must reproduce the first encode's codestreams byte for byte; a
 * difference, or a failed encode, restores the previous options and returns
 * JP2G_ENCODE_FAILED.
 * `best` (JP2G_NUM_OPTS entries) and `best_ms` may be NULL. The options it
 * tries apply to the whole context, so call it while no submitted request is
 * in flight. No reference counterpart: the reference has no tunable device
 * schedule. */
int jp2g_autotune(jp2g_ctx* ctx, const jp2g_request* reqs, uint32_t n, int repeats, int64_t* best,
                  double* best_ms);

/* Message of the last failed call on this context (or of the last failed
 * jp2g_create when ctx is NULL). */
const char* jp2g_last_error(jp2g_ctx* ctx);

/* Device stream the context launches on (a cudaStream_t), for callers that
 * time or order their own work against the engine. */
void* jp2g_stream(jp2g_ctx* ctx);

/* Stage timings of the last encode, in milliseconds, measured with CUDA
 * events on the context's stream when timing is enabled (for a batch: the
 * device stages summed over its waves, [6] the host time outside them and
 * [7] the wall time of the call):
 * [0] h2d, [1] dwt (all levels), [2] tier-1, [3] pcrd, [4] compaction,
 * [5] read-back of the codestreams into the callers' buffers, [6] host
 * time after it, [7] total, the tier-1 split [8] analysis and bit-plane
 * masks, [9] context modelling, [10] MQ coding, and [11] device Tier-2
 * (packet headers and assembly, between [4] and [5]). Returns the count. */
int jp2g_set_timing(jp2g_ctx* ctx, int enabled);
int jp2g_stage_times(jp2g_ctx* ctx, float* ms, int n);

/* Work counters of the last encode (or batch): [0] code-blocks,
 * [1] non-empty blocks, [2] coding passes, [3] payload bytes before rate
 * control, [4] bytes retained, [5] kernel launches, [6] coefficient
 * bit-planes (sum over blocks of coefficients x magnitude bit-planes),
 * [7] MQ symbols coded. */
int jp2g_counters(jp2g_ctx* ctx, uint64_t* out, int n);

/* Inspection entry points for parity tests. */
/* Quantised coefficient plane (Mallat layout, w*h int32) of component
 * `comp` after colour transform, DWT and quantisation. */
int jp2g_debug_coefficients(jp2g_ctx* ctx, const uint8_t* px, uint32_t w, uint32_t h,
                            uint32_t ncomp, uint8_t quality, uint32_t comp, int32_t* plane);
/* The same plane before quantisation (lossy qualities only): the f32
 * coefficients of the colour transform and 9/7 DWT, for comparing the
 * pipeline against exact (FP64) lifting. */
int jp2g_debug_coefficients_f32(jp2g_ctx* ctx, const uint8_t* px, uint32_t w, uint32_t h,
                                uint32_t ncomp, uint8_t quality, uint32_t comp, float* plane);
/* Per-block Tier-1 results in codestream order, 8 int32 per block:
 * (mbp, zbp, npasses, payload_len, cls, status, kept_passes, kept_bytes). */
int jp2g_debug_blocks(jp2g_ctx* ctx, const uint8_t* px, uint32_t w, uint32_t h,
                      uint32_t ncomp, uint8_t quality, int32_t* rows, uint32_t cap,
                      uint32_t* nblocks);
/* Host Tier-2 alone (no context, no device; the encoder itself runs Tier-2
 * on the device): packet headers, markers and
 * JP2 boxes of a w x h page whose nblocks code-blocks, in codestream order
 * (resolution, component, band, raster), retain npasses[i] passes in one
 * segment of seg_len[i] bytes, consecutive in `body`, above zbp[i] zero
 * bit-planes. *out is malloc'd (free with jp2g_free). */
int jp2g_debug_assemble(uint32_t w, uint32_t h, uint32_t ncomp, uint8_t quality, int format,
                        const uint16_t* npasses, const uint8_t* zbp, const uint32_t* seg_len,
                        const uint8_t* body, uint32_t nblocks, uint8_t** out, size_t* out_len);
/* Device Tier-2 alone, on the same inputs as jp2g_debug_assemble: the
 * per-block records and bodies go to the device and the packet headers,
 * markers and JP2 boxes are written there (the kernels the encoder runs),
 * so tests can compare the two assemblers byte for byte. */
int jp2g_debug_assemble_device(jp2g_ctx* ctx, uint32_t w, uint32_t h, uint32_t ncomp, uint8_t quality,
                               int format, const uint16_t* npasses, const uint8_t* zbp, const uint32_t* seg_len,
                               const uint8_t* body, uint32_t nblocks, uint8_t** out, size_t* out_len);
/* Encoding plan alone (no context, no device), as EncodingPlan::build makes
 * it (src/plan/mod.rs:116-177): decomposition levels, code-block width,
 * quantiser entries (up to 32, as (resolution, band, exponent, mantissa)),
 * code-blocks of the page, and the PCRD lambda at `quality` and at 1. */
int jp2g_debug_plan(uint32_t w, uint32_t h, uint32_t ncomp, uint8_t quality, int* levels, int* cbw,
                    int* nquant, int* quants, uint32_t* nblocks, double* lambdas);

/* Allocation-free first stage of the encoder: level shift + RCT/ICT, every
 * DWT level and the deadzone quantiser, for callers that cannot allocate
 * device memory -- code recorded into a CUDA graph, plug-in hosts that only
 * lend pre-allocated buffers, and real-time loops that must not call the
 * allocator (cudaMalloc can synchronise the whole device). It has no
 * counterpart in the reference, whose encoder always allocates.
 *
 * d_px: interleaved 8-bit pixels in device memory (w * h * ncomp bytes).
 * d_coef: device buffer of w * h * ncomp int32 that receives the quantised
 * coefficients (the reversible 5/3 coefficients at any quality >= 100) of each
 * component as a w x h plane in subband (Mallat) layout, component after
 * component -- the same values the full encoder codes.
 * stream: a cudaStream_t (NULL = the legacy default stream). The call only
 * enqueues kernels; synchronise the stream before reading d_coef.
 *
 * The call allocates nothing: its scratch (the intermediate LL planes) is
 * one statically sized 8 MiB device array that every GPU loading this
 * library holds until the process exits. Limit: ceil(w/2) * ceil(h/2) *
 * ncomp <= 1048576 whenever the image gets two or more decomposition levels
 * (e.g. 2048x2048 gray or 1182x1182 RGB); larger images are rejected with
 * JP2G_INVALID_INPUT and a message before any device work. All calls share
 * the array, so calls that overlap on the GPU (other streams or threads on
 * the same device) race and must be serialised by the caller. The first call
 * on a device looks up the array's device address for that device (and the
 * first call after the device's context changes, e.g. after
 * cudaDeviceReset, looks it up again); make that call before any stream
 * capture. On failure jp2g_last_error(NULL) holds the message. */
int jp2g_dwt_noalloc(const uint8_t* d_px, uint32_t w, uint32_t h, uint32_t ncomp, uint8_t quality,
                     int32_t* d_coef, void* stream);

/* Host-only, no device needed: the bit-sliced context formation the
 * modelling kernel uses (zero-coding labels of 64 samples per logic
 * operation, sign contexts and prediction bits), evaluated on single samples
 * for every neighbourhood, in the layout of jp2g_tables' zc, sc and spb, so
 * a test can compare it with the tables entry for entry. */
void jp2g_debug_context_labels(uint8_t* zc, uint8_t* sc, uint8_t* spb);

/* Host-only, no device needed: the Tier-1 context tables (zero coding
 * 4x512, sign context 256, sign prediction 256) and the MQ state table
 * (94 entries, qe | next_mps << 16 | next_lps << 24) the kernels use. */
void jp2g_tables(uint8_t* zc, uint8_t* sc, uint8_t* spb, uint32_t* mq);

#ifdef __cplusplus
}
#endif

#endif /* JP2G_H */
