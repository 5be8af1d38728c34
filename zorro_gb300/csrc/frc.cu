// Tiled Fourier ring correlation (tiledFRC, zorro.py:2246-2310) and its
// rotational mean (rotmean, zorro_util.py:147-224).
//
// Each box x box tile of the even and odd sums is Hann-windowed; both real
// tiles go through one complex FFT per row (z = e + i o), the column pass
// transforms E and O and accumulates, per frequency and over all tiles, the
// normalised correlation real(E conj O) / sqrt(|O|^2 |E|^2) (float per tile
// and per group of FRC_TPG tiles, the groups summed in double).  The
// reference scales both spectra by 1/box^4 first; the ratio does not depend
// on that scale, so it is left out (it only risks float underflow).  Only
// kx in [0, box/2] is computed: the ratio at (-ky, -kx) equals the one at
// (ky, kx).
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace zr {

constexpr int FRC_NB = 4;
constexpr int FRC_TPG = 8;  // tiles accumulated per CTA of the column pass

// Hann window of apodization('hann', box): radius box/2, circular.  The
// squared radius is exact in float for power-of-two boxes.
__device__ __forceinline__ float hann_at(int y, int x, int B) {
  const float inv = 2.0f / (float)B;
  const float yy = (float)(y - B / 2) * inv, xx = (float)(x - B / 2) * inv;
  const float rr = xx * xx + yy * yy;
  return rr <= 1.0f ? 0.5f * (1.0f + cospif(sqrtf(rr))) : 0.0f;
}

template <int B>
__global__ void __launch_bounds__(fft_threads(B, FRC_NB), fft_minblocks(B))
    k_frc_rows(const float* __restrict__ even, const float* __restrict__ odd, int W, const int* __restrict__ offs,
               int K4, float2* __restrict__ RE, float2* __restrict__ RO, const float2* __restrict__ tw) {
  constexpr int T = fft_threads(B, FRC_NB);
  constexpr int LD = ld_of(B);
  extern __shared__ float2 sm[];
  const int g = blockIdx.x, t = blockIdx.y;
  const int oy = offs[2 * t], ox = offs[2 * t + 1];
  for (int e = threadIdx.x; e < FRC_NB * B; e += T) {
    const int r = e / B, x = e - r * B;
    const int y = g * FRC_NB + r;
    const size_t p = (size_t)(oy + y) * W + ox + x;
    const float h = hann_at(y, x, B);
    sm[r * LD + pidx(x)] = make_float2(h * even[p], h * odd[p]);
  }
  __syncthreads();
  block_fft<B, FRC_NB, T, -1>(sm, tw);
  const size_t base = ((size_t)t * (B / FRC_NB) + g) * K4 * FRC_NB;
  for (int e = threadIdx.x; e < K4 * FRC_NB; e += T) {
    const int k = e / FRC_NB, r = e - k * FRC_NB;
    float2 U = make_float2(0.0f, 0.0f), V = U;
    if (k <= B / 2) {
      const float2 zk = sm[r * LD + pidx(k)];
      const float2 zm = sm[r * LD + pidx((B - k) & (B - 1))];
      U = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
      V = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    }
    RE[base + e] = U;
    RO[base + e] = V;
  }
}

// CTAs per SM that keep a T-thread CTA at <= 128 registers per thread
constexpr int frc_minblocks(int T) { return sm_minb(T); }

template <int B>
__global__ void __launch_bounds__(fft_threads(B, 2 * FRC_NB), frc_minblocks(fft_threads(B, 2 * FRC_NB)))
    k_frc_cols(const float2* __restrict__ RE, const float2* __restrict__ RO, int n_tiles, int K4,
               double* __restrict__ half, const float2* __restrict__ tw) {
  constexpr int T = fft_threads(B, 2 * FRC_NB);
  constexpr int LD = ld_of(B);
  constexpr int PER = (B * FRC_NB + T - 1) / T;
  extern __shared__ float2 sm[];
  const int k0 = blockIdx.x * FRC_NB;
  const int t0 = blockIdx.y * FRC_TPG;
  const int t1 = min(n_tiles, t0 + FRC_TPG);
  float acc[PER];  // at most FRC_TPG tiles per CTA; the groups are summed in double
#pragma unroll
  for (int i = 0; i < PER; i++) acc[i] = 0.0f;
  for (int t = t0; t < t1; t++) {
    const size_t tb = (size_t)t * (B / FRC_NB) * K4 * FRC_NB;
    for (int e = threadIdx.x; e < B * FRC_NB; e += T) {
      const int gg = e / (FRC_NB * FRC_NB), j = e - gg * (FRC_NB * FRC_NB);
      const int c = j / FRC_NB, r = j - c * FRC_NB;
      const int y = gg * FRC_NB + r;
      const size_t idx = tb + ((size_t)gg * K4 + k0) * FRC_NB + j;
      sm[c * LD + pidx(y)] = RE[idx];
      sm[(FRC_NB + c) * LD + pidx(y)] = RO[idx];
    }
    __syncthreads();
    block_fft<B, 2 * FRC_NB, T, -1>(sm, tw);
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int e = threadIdx.x + i * T;
      if (e < B * FRC_NB) {
        const int c = e / B, y = e - c * B;
        // the tile's correlation at this frequency in float (|r| <= 1, the
        // magnitudes taken separately so that their product cannot
        // overflow), the sum over tiles in double
        const float2 E = sm[c * LD + pidx(y)], O = sm[(FRC_NB + c) * LD + pidx(y)];
        const float num = fmaf(E.x, O.x, E.y * O.y);
        const float den = sqrtf(fmaf(O.x, O.x, O.y * O.y)) * sqrtf(fmaf(E.x, E.x, E.y * E.y));
        acc[i] += num / den;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int e = threadIdx.x + i * T;
    if (e < B * FRC_NB) {
      const int c = e / B, y = e - c * B;
      half[((size_t)blockIdx.y * B + y) * K4 + k0 + c] = (double)acc[i];
    }
  }
}

// fftshift + DC normalisation into frc2d, and per-block ring partial sums.
__global__ void k_frc_assemble(const double* __restrict__ half, int ngroups, int B, int K4, int nr,
                               float* __restrict__ frc2d, double* __restrict__ part) {
  extern __shared__ double rs[];  // [2][nr]
  for (int i = threadIdx.x; i < 2 * nr; i += blockDim.x) rs[i] = 0.0;
  __syncthreads();
  const size_t plane = (size_t)B * K4;
  double dc = 0.0;
  for (int g = 0; g < ngroups; g++) dc += half[g * plane];
  const int hb = B / 2;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < B * B; p += gridDim.x * blockDim.x) {
    const int i = p / B, j = p - i * B;
    const int ky = (i + hb) & (B - 1), kx = (j + hb) & (B - 1);
    const size_t q = (kx <= hb) ? (size_t)ky * K4 + kx : (size_t)((B - ky) & (B - 1)) * K4 + (B - kx);
    double v = 0.0;
    for (int g = 0; g < ngroups; g++) v += half[g * plane + q];
    v = v / dc;
    frc2d[p] = (float)v;
    const double xx = j - hb, yy = i - hb;
    const double r = sqrt(xx * xx + yy * yy);
    const double rf = floor(r);
    const double rem = r - rf;
    const int b0 = (int)rf;
    atomicAdd(&rs[b0], v * (1.0 - rem));
    atomicAdd(&rs[nr + b0], 1.0 - rem);
    atomicAdd(&rs[b0 + 1], v * rem);
    atomicAdd(&rs[nr + b0 + 1], rem);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * nr; i += blockDim.x) part[(size_t)blockIdx.x * 2 * nr + i] = rs[i];
}

__global__ void k_frc_rings(const double* __restrict__ part, int nblk, int nr, int nout, double* __restrict__ frc) {
  for (int r = threadIdx.x; r < nout; r += blockDim.x) {
    double s = 0.0, w = 0.0;
    for (int b = 0; b < nblk; b++) {
      s += part[(size_t)b * 2 * nr + r];
      w += part[(size_t)b * 2 * nr + nr + r];
    }
    frc[r] = s / w;
  }
}

constexpr int FRC_ASM_BLOCKS = 64;

template <int B>
static int run_frc(const float* even, const float* odd, int W, const int* offs, int n_tiles, float* frc2d,
                   double* frc, int nr, int nout, void* work, cudaStream_t st) {
  const float2* tw = twiddles();
  if (!tw) return ZR_ECUDA;
  const int K4 = zr_spectrum_pitch(B);
  float2* RE = (float2*)work;
  float2* RO = RE + (size_t)n_tiles * B * K4;
  const int ngroups = (n_tiles + FRC_TPG - 1) / FRC_TPG;
  double* half = (double*)(RO + (size_t)n_tiles * B * K4);
  double* part = half + (size_t)ngroups * B * K4;
  {
    constexpr int T = fft_threads(B, FRC_NB);
    const size_t smem = (size_t)FRC_NB * ld_of(B) * sizeof(float2);
    ZR_TRY(cuda_check(cudaFuncSetAttribute(k_frc_rows<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "frc attr"));
    k_frc_rows<B><<<dim3(B / FRC_NB, n_tiles), T, smem, st>>>(even, odd, W, offs, K4, RE, RO, tw);
    ZR_TRY(launched("k_frc_rows"));
  }
  {
    constexpr int T = fft_threads(B, 2 * FRC_NB);
    const size_t smem = (size_t)2 * FRC_NB * ld_of(B) * sizeof(float2);
    ZR_TRY(cuda_check(cudaFuncSetAttribute(k_frc_cols<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "frc attr"));
    k_frc_cols<B><<<dim3(K4 / FRC_NB, ngroups), T, smem, st>>>(RE, RO, n_tiles, K4, half, tw);
    ZR_TRY(launched("k_frc_cols"));
  }
  k_frc_assemble<<<FRC_ASM_BLOCKS, 512, 2 * nr * sizeof(double), st>>>(half, ngroups, B, K4, nr, frc2d, part);
  ZR_TRY(launched("k_frc_assemble"));
  k_frc_rings<<<1, 512, 0, st>>>(part, FRC_ASM_BLOCKS, nr, nout, frc);
  return launched("k_frc_rings");
}

}  // namespace zr

using namespace zr;

extern "C" size_t zr_frc_work_bytes(int n_tiles, int box) {
  const size_t K4 = zr_spectrum_pitch(box);
  const int nr = (int)ceil(sqrt((double)(box / 2) * (box / 2) * 2.0)) + 1;
  const size_t ngroups = (n_tiles + FRC_TPG - 1) / FRC_TPG;
  return 2 * (size_t)n_tiles * box * K4 * sizeof(float2) + ngroups * box * K4 * sizeof(double) +
         (size_t)FRC_ASM_BLOCKS * 2 * (nr + 1) * sizeof(double);
}

extern "C" int zr_tiled_frc(const float* even, const float* odd, int height, int width, int box, const int* offsets,
                            int n_tiles, float* frc2d, double* frc, int nrings, void* work, size_t work_bytes,
                            void* stream) {
  if (!even || !odd || !offsets || !frc2d || !frc) return set_error(ZR_EINVAL, "zr_tiled_frc: null argument");
  if (n_tiles <= 0) return set_error(ZR_EINVAL, "zr_tiled_frc: no tiles (image smaller than the FRC box)");
  if (box != 128 && box != 256 && box != 512 && box != 1024)
    return set_error(ZR_ESIZE, "zr_tiled_frc: box %d not supported (128..1024, power of two)", box);
  const int nr_full = (int)ceil(sqrt((double)(box / 2) * (box / 2) * 2.0)) + 1;
  if (nrings <= 0 || nrings > nr_full) return set_error(ZR_EINVAL, "zr_tiled_frc: nrings must be in [1, %d]", nr_full);
  if (work_bytes < zr_frc_work_bytes(n_tiles, box))
    return set_error(ZR_EWORK, "zr_tiled_frc: work buffer %zu < %zu", work_bytes, zr_frc_work_bytes(n_tiles, box));
  (void)height;
  cudaStream_t st = (cudaStream_t)stream;
  switch (box) {
    case 128: return run_frc<128>(even, odd, width, offsets, n_tiles, frc2d, frc, nr_full, nrings, work, st);
    case 256: return run_frc<256>(even, odd, width, offsets, n_tiles, frc2d, frc, nr_full, nrings, work, st);
    case 512: return run_frc<512>(even, odd, width, offsets, n_tiles, frc2d, frc, nr_full, nrings, work, st);
    default: return run_frc<1024>(even, odd, width, offsets, n_tiles, frc2d, frc, nr_full, nrings, work, st);
  }
}
