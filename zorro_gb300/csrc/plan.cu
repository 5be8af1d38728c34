// The planner: for one registration shape, time every launch variant of the
// transform kernels on the current device and keep the fastest per transform
// length -- what pyFFTW's FFTW_MEASURE planning does for the reference's
// transforms (pyFFTWPlanner, zorro_util.py:966-1066), with the choices saved
// and restored by the caller like FFTW wisdom (zr_plan_set).
//
// A variant is the number of sequences one CTA transforms (1, 2 or 4) in the
// forward row pass (keyed by P1), the forward column pass (P0), the
// correlation column pass (C0) and the correlation row pass (C1).  Variants
// change only how the work is split between CTAs: every transform computes
// the same values in the same order, so the results do not depend on the
// plan.
//
// Measurement: n_frames synthetic frames of P0 x P1 pseudo-random values in
// the work buffer; the forward spectra of all of them for each of the 3 x 3
// row/column variants, then the correlation windows of all their pairs for
// each of the 3 x 3 column/row variants; each candidate run once to warm up
// and three times timed with CUDA events on ``stream``, its best time kept.
#include <string.h>

#include "common.cuh"
#include "internal.h"

namespace zr {

// pseudo-random frame values in [0, 2): a 32-bit integer hash of the index
__global__ void k_plan_fill(float* __restrict__ v, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned int h = (unsigned int)(i * 2654435761ull) ^ 0x9e3779b9u;
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    v[i] = (float)(h >> 8) * (2.0f / 16777216.0f);
  }
}

struct PlanBufs {
  float* frames;
  double* msub;
  float2 *G, *S, *GM;
  float* terms;
  float* cwin;
  int* pairs;
  void* specwork;
  size_t specwork_bytes;
  void* xcwork;
  size_t xcwork_bytes;
  size_t total;
};

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

static PlanBufs plan_layout(const zr_plan_shape_t* s, char* base) {
  PlanBufs b;
  const int nf = s->n_frames;
  const int w = 2 * s->max_shift;
  const int M = nf * (nf - 1) / 2;
  const long long se = zr_spectrum_elems(s->C0, s->C1);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  b.frames = (float*)take((size_t)nf * s->P0 * s->P1 * sizeof(float));
  b.msub = (double*)take((size_t)nf * sizeof(double));
  b.G = (float2*)take((size_t)nf * se * sizeof(float2));
  b.S = (float2*)take((size_t)nf * se * sizeof(float2));
  b.GM = (float2*)take((size_t)se * sizeof(float2));
  b.terms = (float*)take((size_t)(4 * nf + 1) * w * w * sizeof(float));
  b.cwin = (float*)take((size_t)(M > 0 ? M : 1) * w * w * sizeof(float));
  b.pairs = (int*)take((size_t)2 * (M > 0 ? M : 1) * sizeof(int));
  b.specwork_bytes = zr_spectra_work_bytes(s->P0, nf, s->C1);
  b.specwork = take(b.specwork_bytes);
  const size_t xt = zr_xcorr_work_bytes(2 * nf + 1, s->C1, s->max_shift);
  const size_t xp = zr_xcorr_work_bytes(M > 0 ? M : 1, s->C1, s->max_shift);
  b.xcwork_bytes = xt > xp ? xt : xp;
  b.xcwork = take(b.xcwork_bytes);
  b.total = off;
  return b;
}

static int check_shape(const zr_plan_shape_t* s) {
  if (!s) return set_error(ZR_EINVAL, "zr_plan: null shape");
  if (s->n_frames < 2 || s->n_frames > 64) return set_error(ZR_EINVAL, "zr_plan: n_frames %d not in [2, 64]", s->n_frames);
  if (!fft_len_ok(s->P0) || !fft_len_ok(s->P1) || !fft_len_ok(s->C0) || !fft_len_ok(s->C1) || s->C0 > s->P0 ||
      s->C1 > s->P1 || s->C0 < 64 || s->C1 < 64 || s->C0 > 4096 || s->C1 > 4096 || s->P0 > 6144 || s->P1 > 6144)
    return set_error(ZR_ESIZE, "zr_plan: P=%dx%d C=%dx%d not supported", s->P0, s->P1, s->C0, s->C1);
  if (s->max_shift < 2 || 2 * s->max_shift > s->C0 || 2 * s->max_shift > s->C1)
    return set_error(ZR_ESIZE, "zr_plan: maxShift %d must satisfy 2 <= maxShift <= C/2", s->max_shift);
  return ZR_OK;
}

// best of three timed runs of ``run`` (after one untimed), in ms
template <typename F>
static int time_best(cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, F run, float* ms) {
  ZR_TRY(run());
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    ZR_TRY(cuda_check(cudaEventRecord(e0, st), "cudaEventRecord"));
    ZR_TRY(run());
    ZR_TRY(cuda_check(cudaEventRecord(e1, st), "cudaEventRecord"));
    ZR_TRY(cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize"));
    float t = 0.0f;
    ZR_TRY(cuda_check(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime"));
    if (t < best) best = t;
  }
  *ms = best;
  return ZR_OK;
}

static const int k_variants[3] = {1, 2, 4};

static int plan_measure(const zr_plan_shape_t* s, const PlanBufs& b, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1,
                        zr_plan_choice_t* out) {
  const int nf = s->n_frames;
  const long long npix = (long long)nf * s->P0 * s->P1;
  k_plan_fill<<<1024, 256, 0, st>>>(b.frames, npix);
  ZR_TRY(launched("k_plan_fill"));
  ZR_TRY(cuda_check(cudaMemsetAsync(b.msub, 0, (size_t)nf * sizeof(double), st), "cudaMemsetAsync"));
  zr_frames_t fr;
  memset(&fr, 0, sizeof(fr));
  fr.raw = b.frames;
  fr.raw_type = ZR_F32;
  fr.n_frames = nf;
  fr.height = s->P0;
  fr.width = s->P1;
  ZR_TRY(zr_frame_sums(&fr, b.msub, st));
  ZR_TRY(zr_spectra(&fr, nullptr, nullptr, 0, 1, 1, s->P0, s->P1, s->C0, s->C1, b.GM, nullptr, b.specwork,
                    b.specwork_bytes, st));
  auto spectra = [&]() {
    return zr_spectra(&fr, nullptr, b.msub, 0, nf, 0, s->P0, s->P1, s->C0, s->C1, b.G, b.S, b.specwork,
                      b.specwork_bytes, st);
  };
  float best = 1e30f;
  int br = 0, bc = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      ZR_TRY(tune_set(TUNE_FWD_ROWS, s->P1, k_variants[i]));
      ZR_TRY(tune_set(TUNE_FWD_COLS, s->P0, k_variants[j]));
      float ms = 0.0f;
      ZR_TRY(time_best(st, e0, e1, spectra, &ms));
      out->ms_spectra[i][j] = ms;
      if (ms < best) { best = ms; br = i; bc = j; }
    }
  out->fwd_rows = k_variants[br];
  out->fwd_cols = k_variants[bc];
  ZR_TRY(tune_set(TUNE_FWD_ROWS, s->P1, out->fwd_rows));
  ZR_TRY(tune_set(TUNE_FWD_COLS, s->P0, out->fwd_cols));
  ZR_TRY(spectra());
  // the pairs of all frames
  const int M = nf * (nf - 1) / 2;
  int host_pairs[2 * 64 * 63 / 2];
  int k = 0;
  for (int I = 0; I < nf; I++)
    for (int J = I + 1; J < nf; J++) {
      host_pairs[2 * k] = I;
      host_pairs[2 * k + 1] = J;
      k++;
    }
  ZR_TRY(cuda_check(cudaMemcpyAsync(b.pairs, host_pairs, (size_t)2 * M * sizeof(int), cudaMemcpyHostToDevice, st),
                    "cudaMemcpyAsync"));
  ZR_TRY(cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize"));  // host_pairs is about to go
  ZR_TRY(zr_xcorr_terms(b.G, b.S, b.GM, nf, s->C0, s->C1, s->max_shift, b.terms, b.xcwork, b.xcwork_bytes, st));
  auto pairs = [&]() {
    return zr_xcorr_pairs(b.G, b.terms, b.pairs, M, nf, s->C0, s->C1, s->max_shift, b.cwin, b.xcwork,
                          b.xcwork_bytes, st);
  };
  best = 1e30f;
  br = bc = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      ZR_TRY(tune_set(TUNE_XC_COLS, s->C0, k_variants[i]));
      ZR_TRY(tune_set(TUNE_XC_ROWS, s->C1, k_variants[j]));
      float ms = 0.0f;
      ZR_TRY(time_best(st, e0, e1, pairs, &ms));
      out->ms_pairs[i][j] = ms;
      if (ms < best) { best = ms; br = i; bc = j; }
    }
  out->xc_cols = k_variants[br];
  out->xc_rows = k_variants[bc];
  ZR_TRY(tune_set(TUNE_XC_COLS, s->C0, out->xc_cols));
  ZR_TRY(tune_set(TUNE_XC_ROWS, s->C1, out->xc_rows));
  return cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
}

}  // namespace zr

using namespace zr;

extern "C" size_t zr_plan_work_bytes(const zr_plan_shape_t* shape) {
  if (check_shape(shape) != ZR_OK) return 0;
  return plan_layout(shape, nullptr).total;
}

extern "C" int zr_plan(const zr_plan_shape_t* shape, void* work, size_t work_bytes, void* stream,
                       zr_plan_choice_t* out) {
  ZR_TRY(check_shape(shape));
  if (!work || !out) return set_error(ZR_EINVAL, "zr_plan: null argument");
  const PlanBufs b = plan_layout(shape, (char*)work);
  if (work_bytes < b.total) return set_error(ZR_EWORK, "zr_plan: work buffer %zu < %zu", work_bytes, b.total);
  memset(out, 0, sizeof(*out));
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ZR_TRY(cuda_check(cudaEventCreate(&e0), "cudaEventCreate"));
  int rc = cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
  if (rc == ZR_OK) rc = plan_measure(shape, b, st, e0, e1, out);
  if (rc != ZR_OK) {
    // leave the defaults in place rather than a half-measured plan
    tune_set(TUNE_FWD_ROWS, shape->P1, 0);
    tune_set(TUNE_FWD_COLS, shape->P0, 0);
    tune_set(TUNE_XC_COLS, shape->C0, 0);
    tune_set(TUNE_XC_ROWS, shape->C1, 0);
  }
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return rc;
}

extern "C" int zr_plan_set(const zr_plan_shape_t* shape, const zr_plan_choice_t* choice) {
  ZR_TRY(check_shape(shape));
  if (!choice) return set_error(ZR_EINVAL, "zr_plan_set: null choice");
  ZR_TRY(tune_set(TUNE_FWD_ROWS, shape->P1, choice->fwd_rows));
  ZR_TRY(tune_set(TUNE_FWD_COLS, shape->P0, choice->fwd_cols));
  ZR_TRY(tune_set(TUNE_XC_COLS, shape->C0, choice->xc_cols));
  return tune_set(TUNE_XC_ROWS, shape->C1, choice->xc_rows);
}

extern "C" int zr_plan_get(const zr_plan_shape_t* shape, zr_plan_choice_t* choice) {
  ZR_TRY(check_shape(shape));
  if (!choice) return set_error(ZR_EINVAL, "zr_plan_get: null choice");
  memset(choice, 0, sizeof(*choice));
  choice->fwd_rows = tune_get(TUNE_FWD_ROWS, shape->P1);
  choice->fwd_cols = tune_get(TUNE_FWD_COLS, shape->P0);
  choice->xc_cols = tune_get(TUNE_XC_COLS, shape->C0);
  choice->xc_rows = tune_get(TUNE_XC_ROWS, shape->C1);
  return ZR_OK;
}
