// Gain correction and the outlier-pixel filter (hotpixFilter,
// zorro.py:2497-2672).  The host fits the normal CDF of the unaligned sum's
// histogram (zorro.py:2533-2592); the per-pixel parts run here and are folded
// into two maps so that every later kernel applies the filter while it reads
// a raw frame: corrected = hot_a * (gain * raw) + hot_b (zorro.py:2649).
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace zr {

__global__ void k_gain_sum(FrameSrc f, float* __restrict__ sum, double* __restrict__ total) {
  const long long npix = (long long)f.H * f.W;
  double part = 0.0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(p / f.W), x = (int)(p - (long long)y * f.W);
    float s = 0.0f;
    for (int n = 0; n < f.N; n++) s = __fadd_rn(s, load_corrected(f, n, y, x));
    sum[p] = s;
    part += (double)s;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && total) atomicAdd(total, v);
  }
}

// Same sum, four pixels per thread with vector loads (H*W % 4 == 0).
__global__ void k_gain_sum4(FrameSrc f, float* __restrict__ sum, double* __restrict__ total) {
  const long long n4 = (long long)f.H * f.W / 4;
  double part = 0.0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long long)gridDim.x * blockDim.x) {
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int n = 0; n < f.N; n++) {
      const float4 v = load4_corrected(f, n, 4 * q);
      s = make_float4(__fadd_rn(s.x, v.x), __fadd_rn(s.y, v.y), __fadd_rn(s.z, v.z), __fadd_rn(s.w, v.w));
    }
    reinterpret_cast<float4*>(sum)[q] = s;
    part += (double)s.x + (double)s.y + (double)s.z + (double)s.w;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && total) atomicAdd(total, v);
  }
}

__global__ void k_histogram(const float* __restrict__ v, long long n, double e0, int nbins, unsigned int* __restrict__ counts) {
  extern __shared__ unsigned int hist[];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const double d = (double)v[p] - e0;
    if (d >= 0.0 && d <= (double)nbins) {
      int b = (int)floor(d);
      if (b == nbins) b = nbins - 1;  // the last bin is closed on the right
      atomicAdd(&hist[b], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (hist[i]) atomicAdd(counts + i, hist[i]);
}

// logisticMask, 1 - logisticMask, and the per-frame mean; dead/hot counts.
__global__ void k_hot_lm(const float* __restrict__ sum, long long npix, int nfr, zr_hotpix_params_t p,
                         float* __restrict__ LM, float* __restrict__ CONV, float* __restrict__ MEAN,
                         unsigned int* __restrict__ counts) {
  unsigned int dead = 0, hot = 0;
  const double cl = (double)p.cutoff_lower, cu = (double)p.cutoff_upper;
  const double lrel = (double)(p.cutoff_lower * p.relax), urel = (double)(p.cutoff_upper * p.relax);
  const double K = (double)p.logistic_k;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (long long)gridDim.x * blockDim.x) {
    const float s = sum[i];
    const double sg = ((double)s - p.mu) / p.sigma;
    dead += sg < cl;
    hot += sg > cu;
    const float e1 = expf((float)(K * (sg - lrel)));
    const float e2 = expf((float)(K * (sg - urel)));
    const float s1 = 1.0f / (1.0f + e1);
    const float lm = (1.0f - s1) / (1.0f + e2);
    float conv;
    if (lm < 0.5f || isinf(e2)) conv = 1.0f - lm;
    else conv = (e2 + s1) / (1.0f + e2);
    LM[i] = lm;
    CONV[i] = conv;
    MEAN[i] = s / (float)nfr;
  }
  for (int o = 16; o > 0; o >>= 1) {
    dead += __shfl_down_sync(0xffffffffu, dead, o);
    hot += __shfl_down_sync(0xffffffffu, hot, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (dead) atomicAdd(counts + 0, dead);
    if (hot) atomicAdd(counts + 1, hot);
  }
}

__device__ __forceinline__ int rfl(int i, int n) { return i < 0 ? -i - 1 : (i >= n ? 2 * n - i - 1 : i); }

// PSF fill of singleton outliers and the neighbourly-outlier mask.
__global__ void k_hot_fill(const float* __restrict__ LM, const float* __restrict__ CONV, const float* __restrict__ MEAN,
                           int H, int W, zr_hotpix_params_t p, float* __restrict__ A, float* __restrict__ B,
                           uint8_t* __restrict__ NM, unsigned int* __restrict__ counts) {
  unsigned int nb = 0;
  const long long npix = (long long)H * W;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / W), x = (int)(i - (long long)y * W);
    float cc = 0.0f, pm = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const size_t q = (size_t)rfl(y - a + 1, H) * W + rfl(x - b + 1, W);
        cc = fmaf(p.psf[a * 3 + b], CONV[q], cc);
        pm = fmaf(p.psf[a * 3 + b], MEAN[q], pm);
      }
    const float conv = CONV[i];
    const float nom = conv * cc;
    const bool neigh = nom > p.neighbour_thres;
    const float single = neigh ? 0.0f : conv;
    A[i] = LM[i];
    B[i] = single * pm;
    NM[i] = neigh;
    nb += neigh;
  }
  for (int o = 16; o > 0; o >>= 1) nb += __shfl_down_sync(0xffffffffu, nb, o);
  if ((threadIdx.x & 31) == 0 && nb) atomicAdd(counts + 2, nb);
}

// neighbourFilt for pixels with outlier neighbours (zorro.py:2639-2646); the
// 3x3 slice follows Python slicing: a neighbourhood starting at row or column
// -1 is empty, so those pixels take bestMean.
__global__ void k_hot_neigh(const float* __restrict__ CONV, const float* __restrict__ MEAN, const uint8_t* __restrict__ NM,
                            int H, int W, double best_mean, float* __restrict__ B) {
  const long long npix = (long long)H * W;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (long long)gridDim.x * blockDim.x) {
    if (!NM[i]) continue;
    const int y = (int)(i / W), x = (int)(i - (long long)y * W);
    double nf;
    if (y == 0 || x == 0) {
      nf = best_mean;
    } else {
      const int y1 = min(y + 2, H), x1 = min(x + 2, W);
      int cnt = 0, size = 0, nk = 0;
      double s = 0.0;
      for (int yy = y - 1; yy < y1; yy++)
        for (int xx = x - 1; xx < x1; xx++) {
          const size_t q = (size_t)yy * W + xx;
          size++;
          if (NM[q]) cnt++;
          else { s += (double)MEAN[q]; nk++; }
        }
      const double ratio = (double)cnt / (double)size;
      if (ratio > 0.66 || ratio <= 0.001) nf = best_mean;
      else nf = (double)CONV[i] * (s / (double)nk);
    }
    B[i] = (float)((double)B[i] + nf);
  }
}

}  // namespace zr

using namespace zr;

extern "C" int zr_gain_sum(const zr_frames_t* frames, float* unaligned_sum, double* total, void* stream) {
  if (!frames || !frames->raw || !unaligned_sum) return set_error(ZR_EINVAL, "zr_gain_sum: null argument");
  FrameSrc f = make_src(frames);
  f.ha = nullptr;
  f.hb = nullptr;
  if (f.N <= 0 || f.H <= 0 || f.W <= 0) return set_error(ZR_EINVAL, "zr_gain_sum: empty movie");
  const long long npix = (long long)f.H * f.W;
  if (npix % 4 == 0 && f.fstride % 4 == 0 && ((uintptr_t)unaligned_sum & 15) == 0) {
    int blocks = (int)((npix / 4 + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_gain_sum4<<<blocks, 256, 0, (cudaStream_t)stream>>>(f, unaligned_sum, total);
    return launched("k_gain_sum4");
  }
  int blocks = (int)((npix + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_gain_sum<<<blocks, 256, 0, (cudaStream_t)stream>>>(f, unaligned_sum, total);
  return launched("k_gain_sum");
}

extern "C" int zr_histogram(const float* values, long long n, double first_edge, int nbins, unsigned int* counts,
                            void* stream) {
  if (!values || !counts) return set_error(ZR_EINVAL, "zr_histogram: null argument");
  if (nbins <= 0 || nbins > 32768) return set_error(ZR_ESIZE, "zr_histogram: nbins %d outside [1, 32768]", nbins);
  int blocks = (int)((n + 1023) / 1024);
  if (blocks > 152 * 4) blocks = 152 * 4;
  if (blocks < 1) blocks = 1;
  const size_t smem = (size_t)nbins * sizeof(unsigned int);
  ZR_TRY(cuda_check(cudaFuncSetAttribute(k_histogram, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "hist attr"));
  k_histogram<<<blocks, 512, smem, (cudaStream_t)stream>>>(values, n, first_edge, nbins, counts);
  return launched("k_histogram");
}

extern "C" size_t zr_hotpix_work_bytes(int height, int width) {
  const size_t npix = (size_t)height * width;
  return npix * (3 * sizeof(float) + 1) + 256;
}

extern "C" int zr_hotpix_maps(const float* unaligned_sum, int height, int width, int n_frames,
                              const zr_hotpix_params_t* params, float* hot_a, float* hot_b, unsigned int* counts3,
                              void* work, size_t work_bytes, void* stream) {
  if (!unaligned_sum || !params || !hot_a || !hot_b || !counts3 || !work)
    return set_error(ZR_EINVAL, "zr_hotpix_maps: null argument");
  if (height < 4 || width < 4 || n_frames <= 0) return set_error(ZR_EINVAL, "zr_hotpix_maps: image too small");
  if (work_bytes < zr_hotpix_work_bytes(height, width))
    return set_error(ZR_EWORK, "zr_hotpix_maps: work buffer too small");
  const long long npix = (long long)height * width;
  float* LM = (float*)work;
  float* CONV = LM + npix;
  float* MEAN = CONV + npix;
  uint8_t* NM = (uint8_t*)(MEAN + npix);
  int blocks = (int)((npix + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  cudaStream_t st = (cudaStream_t)stream;
  k_hot_lm<<<blocks, 256, 0, st>>>(unaligned_sum, npix, n_frames, *params, LM, CONV, MEAN, counts3);
  ZR_TRY(launched("k_hot_lm"));
  k_hot_fill<<<blocks, 256, 0, st>>>(LM, CONV, MEAN, height, width, *params, hot_a, hot_b, NM, counts3);
  ZR_TRY(launched("k_hot_fill"));
  k_hot_neigh<<<blocks, 256, 0, st>>>(CONV, MEAN, NM, height, width, params->best_mean, hot_b);
  return launched("k_hot_neigh");
}
