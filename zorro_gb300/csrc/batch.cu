// Batches of movies through the C ABI: a context for one shape class owns
// the device buffers of the correlation stages (sized once, when it is
// created), and zr_submit_batch queues those stages for several movies in
// one set of launches -- xcorrnm2_tri's forward spectra, mnxc2's frame terms
// and pair windows, locatePeak (zorro.py:773-1231) -- the spectra of all
// frames going into one concatenated buffer, every movie's pairs offset by
// its first frame.  zr_poll / zr_wait report completion and copy each
// movie's peak records to the caller's host arrays.  The drift solve
// (zr_logistic_fit, zr_l1_solve) and the later stages (zr_shift_sum,
// zr_dose_filter, zr_tiled_frc) follow per movie through their own entry
// points.  Every value is computed by the same kernels as through the
// per-stage entry points, so a movie's records do not depend on the batch it
// is in.
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace zr {

struct BatchMovieOut {
  zr_peak_result_t* dst;  // caller's host array
  int offset, count;      // records [offset, offset + count) of the batch
};

}  // namespace zr

struct zr_ctx {
  int device;
  zr_batch_limits_t lim;
  long long se;
  // device buffers
  float2 *G, *S, *GM;
  float* terms;
  float* cwin;
  int* pairs;
  zr_peak_result_t* peaks;
  void* specwork;
  size_t specwork_bytes;
  void* xcwork;
  size_t xcwork_bytes;
  // pinned host buffers
  int* h_pairs;
  zr_peak_result_t* h_peaks;
  cudaEvent_t done;
  bool pending;
  int n_records;
  std::vector<zr::BatchMovieOut> outs;
  std::mutex mu;
};

namespace zr {

static int ctx_free(zr_ctx* c) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaSetDevice(c->device);
  void* dptrs[] = {c->G, c->S, c->GM, c->terms, c->cwin, c->pairs, c->peaks, c->specwork, c->xcwork};
  for (void* p : dptrs)
    if (p) cudaFree(p);
  if (c->h_pairs) cudaFreeHost(c->h_pairs);
  if (c->h_peaks) cudaFreeHost(c->h_peaks);
  if (c->done) cudaEventDestroy(c->done);
  cudaSetDevice(dev);
  delete c;
  return ZR_OK;
}

static int check_limits(const zr_batch_limits_t* l) {
  if (!l) return set_error(ZR_EINVAL, "zr_ctx_create: null limits");
  if (!fft_len_ok(l->P0) || !fft_len_ok(l->P1) || !fft_len_ok(l->C0) || !fft_len_ok(l->C1) || l->C0 > l->P0 ||
      l->C1 > l->P1 || l->C0 < 64 || l->C1 < 64 || l->C0 > 4096 || l->C1 > 4096 || l->P0 > 6144 || l->P1 > 6144)
    return set_error(ZR_ESIZE, "zr_ctx_create: P=%dx%d C=%dx%d not supported", l->P0, l->P1, l->C0, l->C1);
  if (l->max_shift < 2 || 2 * l->max_shift > l->C0 || 2 * l->max_shift > l->C1)
    return set_error(ZR_ESIZE, "zr_ctx_create: maxShift %d must satisfy 2 <= maxShift <= C/2", l->max_shift);
  if (l->height < 1 || l->height > l->P0 || l->width < 1 || l->width > l->P1)
    return set_error(ZR_ESIZE, "zr_ctx_create: frames %dx%d must fit the padded %dx%d", l->height, l->width, l->P0,
                     l->P1);
  if (l->max_frames < 2 || l->max_pairs < 1 || l->chunk_frames < 1)
    return set_error(ZR_EINVAL, "zr_ctx_create: max_frames %d, max_pairs %d, chunk_frames %d", l->max_frames,
                     l->max_pairs, l->chunk_frames);
  return ZR_OK;
}

// the finished batch's records to the callers' arrays
static void ctx_deliver(zr_ctx* ctx) {
  for (const BatchMovieOut& o : ctx->outs)
    if (o.count > 0) memcpy(o.dst, ctx->h_peaks + o.offset, (size_t)o.count * sizeof(zr_peak_result_t));
  ctx->pending = false;
}

}  // namespace zr

using namespace zr;

extern "C" int zr_ctx_create(int device, const zr_batch_limits_t* limits, zr_ctx_t** out) {
  if (!out) return set_error(ZR_EINVAL, "zr_ctx_create: null output");
  *out = nullptr;
  ZR_TRY(check_limits(limits));
  int prev = 0;
  ZR_TRY(cuda_check(cudaGetDevice(&prev), "cudaGetDevice"));
  ZR_TRY(zr_init(device));
  ZR_TRY(cuda_check(cudaSetDevice(device), "cudaSetDevice"));
  zr_ctx* c = new zr_ctx();
  c->device = device;
  c->lim = *limits;
  const zr_batch_limits_t& l = c->lim;
  c->se = zr_spectrum_elems(l.C0, l.C1);
  const int w = 2 * l.max_shift;
  c->specwork_bytes = zr_spectra_work_bytes(l.height, l.chunk_frames, l.C1);
  // the correlation passes run in waves that fit their scratch: enough for
  // every pair at once, at most 1.5 GB, at least one job
  const size_t x1 = zr_xcorr_work_bytes(1, l.C1, l.max_shift);
  size_t xw = zr_xcorr_work_bytes(l.max_pairs > 2 * l.max_frames + 1 ? l.max_pairs : 2 * l.max_frames + 1, l.C1,
                                  l.max_shift);
  if (xw > ((size_t)1536 << 20)) xw = (size_t)1536 << 20;
  c->xcwork_bytes = xw > x1 ? xw : x1;
  int rc = ZR_OK;
  auto alloc = [&](void** p, size_t bytes) {
    if (rc == ZR_OK) rc = cuda_check(cudaMalloc(p, bytes > 0 ? bytes : 1), "zr_ctx_create: cudaMalloc");
  };
  alloc((void**)&c->G, (size_t)l.max_frames * c->se * sizeof(float2));
  alloc((void**)&c->S, (size_t)l.max_frames * c->se * sizeof(float2));
  alloc((void**)&c->GM, (size_t)c->se * sizeof(float2));
  alloc((void**)&c->terms, (size_t)(4 * l.max_frames + 1) * w * w * sizeof(float));
  alloc((void**)&c->cwin, (size_t)l.max_pairs * w * w * sizeof(float));
  alloc((void**)&c->pairs, (size_t)2 * l.max_pairs * sizeof(int));
  alloc((void**)&c->peaks, (size_t)l.max_pairs * sizeof(zr_peak_result_t));
  alloc(&c->specwork, c->specwork_bytes);
  alloc(&c->xcwork, c->xcwork_bytes);
  if (rc == ZR_OK)
    rc = cuda_check(cudaMallocHost((void**)&c->h_pairs, (size_t)2 * l.max_pairs * sizeof(int)), "cudaMallocHost");
  if (rc == ZR_OK)
    rc = cuda_check(cudaMallocHost((void**)&c->h_peaks, (size_t)l.max_pairs * sizeof(zr_peak_result_t)),
                    "cudaMallocHost");
  if (rc == ZR_OK) rc = cuda_check(cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming), "cudaEventCreate");
  cudaSetDevice(prev);
  if (rc != ZR_OK) {
    ctx_free(c);
    return rc;
  }
  *out = c;
  return ZR_OK;
}

extern "C" int zr_ctx_destroy(zr_ctx_t* ctx) {
  if (!ctx) return ZR_OK;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->pending) cudaEventSynchronize(ctx->done);
  }
  return ctx_free(ctx);
}

extern "C" int zr_submit_batch(zr_ctx_t* ctx, const zr_batch_movie_t* movies, int n_movies,
                               const zr_peak_params_t* params, void* stream) {
  if (!ctx || !movies || !params) return set_error(ZR_EINVAL, "zr_submit_batch: null argument");
  if (n_movies < 1) return set_error(ZR_EINVAL, "zr_submit_batch: no movies");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (ctx->pending) return set_error(ZR_EINVAL, "zr_submit_batch: the previous batch is still pending (zr_poll)");
  const zr_batch_limits_t& l = ctx->lim;
  int nt = 0, mt = 0;
  for (int m = 0; m < n_movies; m++) {
    const zr_batch_movie_t& mv = movies[m];
    if (!mv.frames.raw || mv.frames.frame_movie || (mv.n_pairs > 0 && (!mv.pairs || !mv.peaks)))
      return set_error(ZR_EINVAL, "zr_submit_batch: movie %d: null frames, pairs or peaks (or a frame map)", m);
    if (mv.frames.height != l.height || mv.frames.width != l.width || mv.frames.n_frames < 1)
      return set_error(ZR_ESIZE, "zr_submit_batch: movie %d has %d frames of %dx%d, the context takes %dx%d", m,
                       mv.frames.n_frames, mv.frames.height, mv.frames.width, l.height, l.width);
    for (int k = 0; k < mv.n_pairs; k++) {
      const int I = mv.pairs[2 * k], J = mv.pairs[2 * k + 1];
      if (I < 0 || J < 0 || I >= mv.frames.n_frames || J >= mv.frames.n_frames)
        return set_error(ZR_EINVAL, "zr_submit_batch: movie %d pair %d (%d, %d) outside its %d frames", m, k, I, J,
                         mv.frames.n_frames);
    }
    nt += mv.frames.n_frames;
    mt += mv.n_pairs;
  }
  if (nt > l.max_frames || mt > l.max_pairs)
    return set_error(ZR_ESIZE, "zr_submit_batch: %d frames and %d pairs, the context holds %d and %d", nt, mt,
                     l.max_frames, l.max_pairs);
  int prev = 0;
  ZR_TRY(cuda_check(cudaGetDevice(&prev), "cudaGetDevice"));
  if (prev != ctx->device) ZR_TRY(cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice"));
  cudaStream_t st = (cudaStream_t)stream;
  const int mS = l.max_shift;
  // the mask spectrum of the frames' area, then every movie's spectra at its offset
  int rc = zr_spectra(&movies[0].frames, nullptr, nullptr, 0, 1, 1, l.P0, l.P1, l.C0, l.C1, ctx->GM, nullptr,
                      ctx->specwork, ctx->specwork_bytes, st);
  int f0 = 0, k0 = 0;
  ctx->outs.clear();
  for (int m = 0; m < n_movies && rc == ZR_OK; m++) {
    const zr_batch_movie_t& mv = movies[m];
    const int n = mv.frames.n_frames;
    for (int c0 = 0; c0 < n && rc == ZR_OK; c0 += l.chunk_frames) {
      const int nc = (n - c0) < l.chunk_frames ? (n - c0) : l.chunk_frames;
      rc = zr_spectra(&mv.frames, nullptr, mv.mean_sub, c0, nc, 0, l.P0, l.P1, l.C0, l.C1,
                      ctx->G + (size_t)(f0 + c0) * ctx->se, ctx->S + (size_t)(f0 + c0) * ctx->se, ctx->specwork,
                      ctx->specwork_bytes, st);
    }
    for (int k = 0; k < mv.n_pairs; k++) {
      ctx->h_pairs[2 * (k0 + k)] = mv.pairs[2 * k] + f0;
      ctx->h_pairs[2 * (k0 + k) + 1] = mv.pairs[2 * k + 1] + f0;
    }
    ctx->outs.push_back(BatchMovieOut{mv.peaks, k0, mv.n_pairs});
    f0 += n;
    k0 += mv.n_pairs;
  }
  if (rc == ZR_OK && mt > 0) {
    rc = cuda_check(cudaMemcpyAsync(ctx->pairs, ctx->h_pairs, (size_t)2 * mt * sizeof(int), cudaMemcpyHostToDevice,
                                    st), "cudaMemcpyAsync(pairs)");
    if (rc == ZR_OK)
      rc = zr_xcorr_terms(ctx->G, ctx->S, ctx->GM, nt, l.C0, l.C1, mS, ctx->terms, ctx->xcwork, ctx->xcwork_bytes,
                          st);
    if (rc == ZR_OK)
      rc = zr_xcorr_pairs(ctx->G, ctx->terms, ctx->pairs, mt, nt, l.C0, l.C1, mS, ctx->cwin, ctx->xcwork,
                          ctx->xcwork_bytes, st);
    if (rc == ZR_OK) rc = zr_locate_peaks(ctx->cwin, mt, mS, params, ctx->peaks, st);
    if (rc == ZR_OK)
      rc = cuda_check(cudaMemcpyAsync(ctx->h_peaks, ctx->peaks, (size_t)mt * sizeof(zr_peak_result_t),
                                      cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync(peaks)");
  }
  if (rc == ZR_OK) rc = cuda_check(cudaEventRecord(ctx->done, st), "cudaEventRecord");
  if (rc == ZR_OK) {
    ctx->pending = true;
    ctx->n_records = mt;
  }
  if (prev != ctx->device) cudaSetDevice(prev);
  return rc;
}

extern "C" int zr_poll(zr_ctx_t* ctx) {
  if (!ctx) return set_error(ZR_EINVAL, "zr_poll: null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!ctx->pending) return 1;
  const cudaError_t e = cudaEventQuery(ctx->done);
  if (e == cudaErrorNotReady) {
    cudaGetLastError();  // not an error: clear it
    return 0;
  }
  ZR_TRY(cuda_check(e, "zr_poll: cudaEventQuery"));
  ctx_deliver(ctx);
  return 1;
}

extern "C" int zr_wait(zr_ctx_t* ctx) {
  if (!ctx) return set_error(ZR_EINVAL, "zr_wait: null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!ctx->pending) return ZR_OK;
  ZR_TRY(cuda_check(cudaEventSynchronize(ctx->done), "zr_wait: cudaEventSynchronize"));
  ctx_deliver(ctx);
  return ZR_OK;
}
