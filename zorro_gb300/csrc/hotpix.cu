// Gain correction and the outlier-pixel filter (hotpixFilter,
// zorro.py:2497-2672).  The host fits the normal CDF of the unaligned sum's
// histogram (zorro.py:2533-2592); the per-pixel parts run here and are folded
// into two maps so that every later kernel applies the filter while it reads
// a raw frame: corrected = hot_a * (gain * raw) + hot_b (zorro.py:2649).
#include <math.h>
#include <stdint.h>
#include <string.h>

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

// Same sum, four pixels per thread (H*W % 4 == 0, aligned vector loads), the
// frames read GS_FRAMES at a time before any is added, so that each thread
// keeps that many loads in flight; the additions stay in frame order.
constexpr int GS_FRAMES = 8;

template <int TYPE>
__global__ void __launch_bounds__(256, 3) k_gain_sum_q(FrameSrc f, float* __restrict__ sum, double* __restrict__ total) {
  const long long n4 = (long long)f.H * f.W / 4;
  double part = 0.0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += (long long)gridDim.x * blockDim.x) {
    const long long p = 4 * q;
    float4 g = make_float4(1.f, 1.f, 1.f, 1.f);
    if (f.gain) g = __ldg(reinterpret_cast<const float4*>(f.gain + p));
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int n0 = 0; n0 < f.N; n0 += GS_FRAMES) {
      uint4 r[GS_FRAMES];
#pragma unroll
      for (int j = 0; j < GS_FRAMES; j++)  // past the last frame: a repeated load, not added
        r[j] = raw_quad<TYPE>(f.raw, (long long)min(n0 + j, f.N - 1) * f.fstride + p);
#pragma unroll
      for (int j = 0; j < GS_FRAMES; j++) {
        if (n0 + j < f.N) {
          float4 v = quad_value<TYPE>(r[j]);
          if (f.gain) v = make_float4(__fmul_rn(g.x, v.x), __fmul_rn(g.y, v.y), __fmul_rn(g.z, v.z), __fmul_rn(g.w, v.w));
          if (f.gdiv != 0.0f)
            v = make_float4(__fdiv_rn(v.x, f.gdiv), __fdiv_rn(v.y, f.gdiv), __fdiv_rn(v.z, f.gdiv),
                            __fdiv_rn(v.w, f.gdiv));
          s = make_float4(__fadd_rn(s.x, v.x), __fadd_rn(s.y, v.y), __fadd_rn(s.z, v.z), __fadd_rn(s.w, v.w));
        }
      }
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

// The same histogram when the first edge is k - 1/2 for an integer k (the
// hot-pixel bins, zorro.py:2530-2533), without float64: the bin of v is
// floor(v - k + 1/2) = floor(v) + [v - floor(v) >= 1/2] - k, exact in float32
// (v - floor(v) is exact for every float32 except just below zero, where the
// rounding cannot cross 1/2), and v equals the last edge exactly when that
// index is nbins and v - floor(v) is 1/2.
__global__ void k_histogram_half(const float* __restrict__ v, long long n, int k, int nbins,
                                 unsigned int* __restrict__ counts) {
  extern __shared__ unsigned int hist[];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float x = __ldg(v + p);
    if (!(fabsf(x) < 1073741824.0f)) continue;  // NaN, inf and values far outside every bin
    const float c = floorf(x);
    const float fr = x - c;
    int b = (int)c + (fr >= 0.5f ? 1 : 0) - k;
    if (b < 0 || b > nbins) continue;
    if (b == nbins) {
      if (fr != 0.5f) continue;
      b = nbins - 1;  // the last bin is closed on the right
    }
    atomicAdd(&hist[b], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (hist[i]) atomicAdd(counts + i, hist[i]);
}

// logisticMask (written as the map a) and 1 - logisticMask; dead/hot counts.
// The logistic exponents K (sigma - c relax), sigma = (s - mu) / sigma_fit,
// are evaluated in float64 as one fused multiply-add each, A s + Cc with
// A = K / sigma_fit and Cc = -K c relax - A mu folded on the host (within a
// few units in the last float64 place of the step-by-step value; the
// exponents are rounded to float32), or step by step as K ((s - mu) rsig -
// c relax) when sigma_fit is 0.  The counts compare the float32 sum with
// s_dead / s_hot, the float32 values where the float64 quotient crosses the
// cut-offs (found on the host with the same float64 operations), which gives
// the counts of the quotient itself without a float64 division per pixel.
__global__ void __launch_bounds__(256) k_hot_lm(const float* __restrict__ sum, long long npix, zr_hotpix_params_t p,
                                                double rsig, double A, double C1, double C2, float s_dead, float s_hot,
                                                float* __restrict__ LM, float* __restrict__ CONV,
                                                unsigned int* __restrict__ counts) {
  unsigned int dead = 0, hot = 0;
  const double lrel = (double)(p.cutoff_lower * p.relax), urel = (double)(p.cutoff_upper * p.relax);
  const double K = (double)p.logistic_k;
  const bool folded = rsig < INFINITY;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (long long)gridDim.x * blockDim.x) {
    const float s = sum[i];
    dead += s < s_dead;
    hot += s >= s_hot;
    float x1, x2;
    if (folded) {
      x1 = (float)fma(A, (double)s, C1);
      x2 = (float)fma(A, (double)s, C2);
    } else {
      const double sg = ((double)s - p.mu) * rsig;
      x1 = (float)(K * (sg - lrel));
      x2 = (float)(K * (sg - urel));
    }
    const float e1 = expf(x1);
    const float e2 = expf(x2);
    const float s1 = 1.0f / (1.0f + e1);
    const float lm = (1.0f - s1) / (1.0f + e2);
    float conv;
    if (lm < 0.5f || isinf(e2)) conv = 1.0f - lm;
    else conv = (e2 + s1) / (1.0f + e2);
    LM[i] = lm;
    CONV[i] = conv;
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

// The PSF fill of singleton outliers, the neighbourly-outlier mask and
// neighbourFilt (zorro.py:2614-2649) for one HF_TY x HF_TX tile of the map b.
// Shared memory holds 1 - logisticMask on the tile and a two-pixel ring, the
// per-frame mean (sum / n_frames) and the mask on a one-pixel ring; positions
// outside the image hold the values at the reflected positions, as
// scipy.ndimage.convolve(mode='reflect') reads them.
//   b = (1 - lm) * [nom <= thres] * psf(mean),  nom = (1 - lm) * psf(1 - lm),
// then for pixels with nom > thres the neighbour term is added: the mean of
// the per-frame means of the in-image 3 x 3 neighbours that are not in the
// mask (Python slicing: a window that starts at row or column -1 is empty),
// times 1 - lm, or bestMean when more than 66 % (or none but the pixel itself
// at 0.1 %) of the window is in the mask; float32 throughout, as np.mean of
// the float32 means and the float32 neighbourFilt array of the reference.
// The PSF sums keep the order of a per-pixel loop (taps row by row).
constexpr int HF_TX = 32, HF_TY = 32;
constexpr int HF_CW = HF_TX + 4, HF_CH = HF_TY + 4;  // 1 - lm, two-pixel ring
constexpr int HF_MW = HF_TX + 2, HF_MH = HF_TY + 2;  // mean and mask, one-pixel ring

__global__ void __launch_bounds__(256) k_hot_fill(const float* __restrict__ CONV, const float* __restrict__ sum,
                                                  int H, int W, int nfr, zr_hotpix_params_t p,
                                                  float* __restrict__ B, unsigned int* __restrict__ counts) {
  __shared__ float cv[HF_CH][HF_CW];
  __shared__ float mn[HF_MH][HF_MW];
  __shared__ uint8_t nm[HF_MH][HF_MW];
  const int ty0 = blockIdx.y * HF_TY, tx0 = blockIdx.x * HF_TX;
  const float fn = (float)nfr;
  const float bm = (float)p.best_mean;
  for (int e = threadIdx.x; e < HF_CH * HF_CW; e += blockDim.x) {
    const int ey = e / HF_CW, ex = e - (e / HF_CW) * HF_CW;
    const int gy = rfl(min(ty0 + ey - 2, H + 1), H), gx = rfl(min(tx0 + ex - 2, W + 1), W);
    cv[ey][ex] = __ldg(CONV + (size_t)gy * W + gx);
  }
  for (int e = threadIdx.x; e < HF_MH * HF_MW; e += blockDim.x) {
    const int ey = e / HF_MW, ex = e - (e / HF_MW) * HF_MW;
    const int gy = rfl(min(ty0 + ey - 1, H), H), gx = rfl(min(tx0 + ex - 1, W), W);
    mn[ey][ex] = __ldg(sum + (size_t)gy * W + gx) / fn;
  }
  __syncthreads();
  // the mask on the tile and its ring (in-image positions only)
  for (int e = threadIdx.x; e < HF_MH * HF_MW; e += blockDim.x) {
    const int ey = e / HF_MW, ex = e - (e / HF_MW) * HF_MW;
    const int gy = ty0 + ey - 1, gx = tx0 + ex - 1;
    uint8_t m = 0;
    if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
      float cc = 0.0f;
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) cc = fmaf(p.psf[a * 3 + b], cv[ey + 2 - a][ex + 2 - b], cc);
      m = (cv[ey + 1][ex + 1] * cc) > p.neighbour_thres;
    }
    nm[ey][ex] = m;
  }
  __syncthreads();
  unsigned int nb = 0;
  for (int e = threadIdx.x; e < HF_TY * HF_TX; e += blockDim.x) {
    const int ly = e / HF_TX, lx = e - (e / HF_TX) * HF_TX;
    const int y = ty0 + ly, x = tx0 + lx;
    if (y >= H || x >= W) continue;
    float pm = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) pm = fmaf(p.psf[a * 3 + b], mn[ly + 2 - a][lx + 2 - b], pm);
    const float conv = cv[ly + 2][lx + 2];
    const bool neigh = nm[ly + 1][lx + 1] != 0;
    const float single = neigh ? 0.0f : conv;
    float bv = single * pm;
    if (neigh) {
      nb++;
      float nf;
      if (y == 0 || x == 0) {
        nf = bm;
      } else {
        const int y1 = min(y + 2, H), x1 = min(x + 2, W);
        int cnt = 0, size = 0, nk = 0;
        float sm = 0.0f;
        for (int yy = y - 1; yy < y1; yy++)
          for (int xx = x - 1; xx < x1; xx++) {
            size++;
            if (nm[yy - ty0 + 1][xx - tx0 + 1]) cnt++;
            else { sm += mn[yy - ty0 + 1][xx - tx0 + 1]; nk++; }
          }
        // cnt / size > 0.66 or <= 0.001 as integers: with size <= 9 no ratio
        // lies within 1/450 of 0.66, and cnt >= 1 (the pixel itself)
        if (50 * cnt > 33 * size || 1000 * cnt <= size) nf = bm;
        else nf = conv * (sm / (float)nk);
      }
      bv = bv + nf;
    }
    B[(size_t)y * W + x] = bv;
  }
  for (int o = 16; o > 0; o >>= 1) nb += __shfl_down_sync(0xffffffffu, nb, o);
  if ((threadIdx.x & 31) == 0 && nb) atomicAdd(counts + 2, nb);
}

// The float32 value t where the float64 test pred(s) = fn((double)s) changes
// from true (below t) to false: pred must be monotone over the float32
// values in their order (-inf ... -0, +0 ... +inf).  Returns the first value
// with pred false, +inf when pred holds up to +inf, NaN when it never holds
// and pred_never_true_means_nan.
static uint32_t order_key(float v) {
  uint32_t u;
  memcpy(&u, &v, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

static float key_value(uint32_t k) {
  const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  float v;
  memcpy(&v, &u, 4);
  return v;
}

template <class P>
static uint64_t first_false(P pred) {
  uint64_t a = order_key(-INFINITY), b = (uint64_t)order_key(INFINITY) + 1;
  while (a < b) {
    const uint64_t m = (a + b) / 2;
    if (pred(key_value((uint32_t)m))) a = m + 1;
    else b = m;
  }
  return a;
}

}  // namespace zr


using namespace zr;

extern "C" int zr_gain_sum(const zr_frames_t* frames, float* unaligned_sum, double* total, void* stream) {
  if (frames && frames->frame_movie)
    return set_error(ZR_EINVAL, "zr_gain_sum: one movie at a time (frame_movie must be NULL)");
  if (!frames || !frames->raw || !unaligned_sum) return set_error(ZR_EINVAL, "zr_gain_sum: null argument");
  FrameSrc f = make_src(frames);
  f.ha = nullptr;
  f.hb = nullptr;
  if (f.N <= 0 || f.H <= 0 || f.W <= 0) return set_error(ZR_EINVAL, "zr_gain_sum: empty movie");
  const long long npix = (long long)f.H * f.W;
  const int vec = f.type == ZR_U8 ? 4 : (f.type == ZR_F32 ? 16 : 8);  // bytes of one pixel quad
  if (npix % 4 == 0 && f.fstride % 4 == 0 && ((uintptr_t)unaligned_sum & 15) == 0 &&
      ((uintptr_t)f.raw % vec) == 0 && ((uintptr_t)f.gain & 15) == 0) {
    int blocks = (int)((npix / 4 + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    cudaStream_t st = (cudaStream_t)stream;
    switch (f.type) {
      case ZR_U8: k_gain_sum_q<ZR_U8><<<blocks, 256, 0, st>>>(f, unaligned_sum, total); break;
      case ZR_U16: k_gain_sum_q<ZR_U16><<<blocks, 256, 0, st>>>(f, unaligned_sum, total); break;
      case ZR_F16: k_gain_sum_q<ZR_F16><<<blocks, 256, 0, st>>>(f, unaligned_sum, total); break;
      default: k_gain_sum_q<ZR_F32><<<blocks, 256, 0, st>>>(f, unaligned_sum, total);
    }
    return launched("k_gain_sum_q");
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
  const double k = first_edge + 0.5;
  if (k == floor(k) && fabs(k) < 4194304.0) {
    ZR_TRY(cuda_check(cudaFuncSetAttribute(k_histogram_half, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "hist attr"));
    k_histogram_half<<<blocks, 512, smem, (cudaStream_t)stream>>>(values, n, (int)k, nbins, counts);
    return launched("k_histogram_half");
  }
  ZR_TRY(cuda_check(cudaFuncSetAttribute(k_histogram, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "hist attr"));
  k_histogram<<<blocks, 512, smem, (cudaStream_t)stream>>>(values, n, first_edge, nbins, counts);
  return launched("k_histogram");
}

extern "C" int zr_hotpix_thresholds(double mu, double sigma, float cutoff_lower, float cutoff_upper, float* s_dead,
                                    float* s_hot) {
  if (!s_dead || !s_hot) return set_error(ZR_EINVAL, "zr_hotpix_thresholds: null argument");
  if (!(sigma >= 0.0)) return set_error(ZR_EINVAL, "zr_hotpix_thresholds: sigma %g is not >= 0", sigma);
  // sigma >= 0 makes (s - mu) / sigma monotone in s, so each cut-off test
  // changes its answer once along the float32 values
  const double cl = (double)cutoff_lower, cu = (double)cutoff_upper;
  const uint64_t end = (uint64_t)order_key(INFINITY) + 1;
  const uint64_t kd = first_false([&](float s) { return ((double)s - mu) / sigma < cl; });
  const uint64_t kh = first_false([&](float s) { return !(((double)s - mu) / sigma > cu); });
  *s_dead = kd >= end ? INFINITY : key_value((uint32_t)kd);  // +inf: only for an infinite cut-off
  *s_hot = kh >= end ? NAN : key_value((uint32_t)kh);         // NaN: no value is hot
  return ZR_OK;
}

extern "C" size_t zr_hotpix_work_bytes(int height, int width) {
  return (size_t)height * width * sizeof(float) + 256;
}

extern "C" int zr_hotpix_maps(const float* unaligned_sum, int height, int width, int n_frames,
                              const zr_hotpix_params_t* params, float* hot_a, float* hot_b, unsigned int* counts3,
                              void* work, size_t work_bytes, void* stream) {
  if (!unaligned_sum || !params || !hot_a || !hot_b || !counts3 || !work)
    return set_error(ZR_EINVAL, "zr_hotpix_maps: null argument");
  if (height < 4 || width < 4 || n_frames <= 0) return set_error(ZR_EINVAL, "zr_hotpix_maps: image too small");
  if (work_bytes < zr_hotpix_work_bytes(height, width))
    return set_error(ZR_EWORK, "zr_hotpix_maps: work buffer too small");
  const zr_hotpix_params_t p = *params;
  float s_dead = 0.0f, s_hot = 0.0f;
  ZR_TRY(zr_hotpix_thresholds(p.mu, p.sigma, p.cutoff_lower, p.cutoff_upper, &s_dead, &s_hot));
  const double mu = p.mu, sigma = p.sigma;
  const double rsig = 1.0 / sigma;
  const double Kd = (double)p.logistic_k;
  const double A = Kd * rsig;
  const double C1 = -(Kd * (double)(p.cutoff_lower * p.relax)) - A * mu;
  const double C2 = -(Kd * (double)(p.cutoff_upper * p.relax)) - A * mu;
  const long long npix = (long long)height * width;
  float* CONV = (float*)work;
  int blocks = (int)((npix + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  cudaStream_t st = (cudaStream_t)stream;
  k_hot_lm<<<blocks, 256, 0, st>>>(unaligned_sum, npix, p, rsig, A, C1, C2, s_dead, s_hot, hot_a, CONV, counts3);
  ZR_TRY(launched("k_hot_lm"));
  const dim3 tiles((width + HF_TX - 1) / HF_TX, (height + HF_TY - 1) / HF_TY);
  k_hot_fill<<<tiles, 256, 0, st>>>(CONV, unaligned_sum, height, width, n_frames, p, hot_b, counts3);
  return launched("k_hot_fill");
}
