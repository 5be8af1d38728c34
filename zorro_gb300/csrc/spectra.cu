// Forward spectra of the masked frames (xcorrnm2_tri, zorro.py:814-925).
//
// The reference transforms m*I and (m*I)^2 as two complex P0 x P1 FFTs per
// frame and keeps the four corners (FFTCrop, zorro.py:901-914).  Here both
// real images go through ONE complex FFT per row (z = u + i u^2, untangled by
// Hermitian symmetry), only the C1/2+1 non-negative kx columns the crop keeps
// are written, and the column pass keeps only the C0+1 cropped ky rows.
//
// Row-pass output layout (scratch): [frame][y/4][K4][y%4] complex, so that
// the row pass (4 rows per CTA) and the column pass (4 columns per CTA) both
// move whole 128-byte lines.
#include <stdio.h>

#include "common.cuh"
#include "internal.h"

namespace zr {

constexpr int NBR = 4;  // rows per group of the row-pass output layout
// rows per CTA of the row pass and columns per CTA of the column pass: the
// defaults (two CTAs share an SM at 4096 points), or the planner's choice of
// 1, 2 or 4 per transform length (tune_get)
constexpr int FR_DEFAULT = 2, FC_DEFAULT = 2;
// CTAs per SM to ask the register allocator for: 128 registers a thread
constexpr int minb_of(int T) { return sm_minb(T); }

template <int P1, int FR>
__global__ void __launch_bounds__(fft_threads(P1, FR), minb_of(fft_threads(P1, FR)))
    k_fwd_rows(FrameSrc f, const float* __restrict__ mask, const double* __restrict__ mean_sub,
               double inv_area, int frame0, int mode, int rows, int cols, int C1, int K4, int H4,
               float2* __restrict__ RU, float2* __restrict__ RV, const float2* __restrict__ tw) {
  constexpr int T = fft_threads(P1, FR);
  constexpr int LD = ld_of(P1);
  extern __shared__ float2 sm[];
  // frames vary fastest so that concurrent CTAs read the same rows of the
  // gain and hot-pixel maps through L2
  const int g = blockIdx.y;
  const int nl = blockIdx.x;
  const int n = frame0 + nl;
  float mu = 0.0f;
  if (mode == 0 && mean_sub) mu = (float)(mean_sub[n] * inv_area);
  if (mode == 0 && !mask && (f.fstride & 3) == 0 && (f.mstride & 3) == 0) {
    // 4 pixels per thread and step: aligned vector loads of the raw frame and
    // every map; the unaligned head (< 4 pixels) and tail go pixel by pixel
    // FR_UNR quads per thread are fetched before any is used, so that several
    // loads per thread are in flight
    constexpr int NQ = FR * (P1 / 4);
    constexpr int FR_UNR = 4;
    for (int e0 = threadIdx.x; e0 < NQ; e0 += T * FR_UNR) {
      Px4 px[FR_UNR];
#pragma unroll
      for (int u = 0; u < FR_UNR; u++) {
        const int e = e0 + u * T;
        if (e < NQ) {
          const int r = e / (P1 / 4), q = e - r * (P1 / 4);
          const int y = g * FR + r;
          if (y < rows) {
            const long long p0 = (long long)y * f.W;
            const int x = (int)((4 - (p0 & 3)) & 3) + 4 * q;
            if (x + 3 < cols) fetch4(f, n, p0 + x, px[u]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < FR_UNR; u++) {
        const int e = e0 + u * T;
        if (e >= NQ) continue;
        const int r = e / (P1 / 4), q = e - r * (P1 / 4);
        const int y = g * FR + r;
        float2* srow = sm + r * LD;
        if (y >= rows) {
#pragma unroll
          for (int j = 0; j < 4; j++) srow[pidx(4 * q + j)] = make_float2(0.0f, 0.0f);
          continue;
        }
        const long long p0 = (long long)y * f.W;
        const int off = (int)((4 - (p0 & 3)) & 3);  // first x with (p0 + x) % 4 == 0
        const int x = off + 4 * q;
        if (x + 3 < cols) {
          const float4 v = finish4(f, px[u]);
          const float u0 = v.x - mu, u1 = v.y - mu, u2 = v.z - mu, u3 = v.w - mu;
          srow[pidx(x)] = make_float2(u0, u0 * u0);
          srow[pidx(x + 1)] = make_float2(u1, u1 * u1);
          srow[pidx(x + 2)] = make_float2(u2, u2 * u2);
          srow[pidx(x + 3)] = make_float2(u3, u3 * u3);
        } else {
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const int xx = x + j;
            if (xx < P1) {
              float2 z = make_float2(0.0f, 0.0f);
              if (xx < cols) {
                const float u = load_corrected(f, n, y, xx) - mu;
                z = make_float2(u, u * u);
              }
              srow[pidx(xx)] = z;
            }
          }
        }
        if (q == 0) {
          for (int xx = 0; xx < off; xx++) {
            float2 z = make_float2(0.0f, 0.0f);
            if (xx < cols) {
              const float u = load_corrected(f, n, y, xx) - mu;
              z = make_float2(u, u * u);
            }
            srow[pidx(xx)] = z;
          }
        }
      }
    }
  } else {
    for (int e = threadIdx.x; e < FR * P1; e += T) {
      const int r = e / P1, x = e - (e / P1) * P1;
      const int y = g * FR + r;
      float2 z = make_float2(0.0f, 0.0f);
      if (y < rows && x < cols) {
        const float m = mask ? __ldg(mask + (size_t)y * P1 + x) : 1.0f;
        if (mode == 0) {
          const float u = m * (load_corrected(f, n, y, x) - mu);
          z = make_float2(u, u * u);
        } else {
          z.x = m;
        }
      }
      sm[r * LD + pidx(x)] = z;
    }
  }
  __syncthreads();
  block_fft<P1, FR, T, -1>(sm, tw);
  const int half = C1 / 2;
  for (int e = threadIdx.x; e < K4 * FR; e += T) {
    const int k = e / FR, r = e - (e / FR) * FR;
    const int y = g * FR + r;
    const size_t o = (((size_t)nl * H4 + (y >> 2)) * K4 + k) * NBR + (y & 3);
    float2 U = make_float2(0.0f, 0.0f), V = U;
    if (k <= half) {
      const float2 zk = sm[r * LD + pidx(k)];
      const float2 zm = sm[r * LD + pidx(k == 0 ? 0 : P1 - k)];
      U = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
      V = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    }
    RU[o] = U;
    if (mode == 0) RV[o] = V;
  }
}

template <int P0, int FC>
__global__ void __launch_bounds__(fft_threads(P0, FC), minb_of(fft_threads(P0, FC)))
    k_fwd_cols(const float2* __restrict__ RU, const float2* __restrict__ RV, int rows, int C0, int K4, int H4,
               long long spec_elems, float2* __restrict__ G, float2* __restrict__ S,
               const float2* __restrict__ tw) {
  constexpr int T = fft_threads(P0, FC);
  constexpr int LD = ld_of(P0);
  extern __shared__ float2 sm[];
  const int k0 = blockIdx.x * FC;
  const int nl = blockIdx.y;
  const float2* R = (blockIdx.z == 0 ? RU : RV) + (size_t)nl * H4 * K4 * NBR;
  float2* out = (blockIdx.z == 0 ? G : S) + (size_t)nl * spec_elems;
  // element y of column k0 + c: row y of the row-pass output, zero past the
  // frame (the zero padding to P0)
  block_fft_from<P0, FC, T, -1>(sm, tw, [&](int c, int y) {
    return y < rows ? __ldg(R + ((size_t)(y >> 2) * K4 + k0 + c) * NBR + (y & 3)) : make_float2(0.0f, 0.0f);
  });
  const int hc = C0 / 2;
  const int RP = C0 + 4;
  // rows C0 + 1 .. C0 + 3 pad the column to its pitch: written as zeros, so
  // that every element of a spectrum is defined (zr_pack_half scans them all)
  for (int e = threadIdx.x; e < RP * FC; e += T) {
    const int c = e / RP, r = e - c * RP;
    const int ky = r < hc ? r : (r < C0 ? P0 - C0 + r : hc);
    out[(size_t)(k0 + c) * RP + r] = r <= C0 ? sm[c * LD + pidx(ky)] : make_float2(0.0f, 0.0f);
  }
}

__global__ void k_frame_sums(FrameSrc f, double* __restrict__ sums) {
  const int n = blockIdx.y;
  const long long npix = (long long)f.H * f.W;
  float acc = 0.0f;
  double dacc = 0.0;
  int cnt = 0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(p / f.W), x = (int)(p - (long long)y * f.W);
    acc += load_corrected(f, n, y, x);
    if (++cnt == 64) { dacc += acc; acc = 0.0f; cnt = 0; }
  }
  dacc += acc;
  for (int o = 16; o > 0; o >>= 1) dacc += __shfl_down_sync(0xffffffffu, dacc, o);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dacc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) atomicAdd(sums + n, v);
  }
}

template <int P, int FR>
static int launch_rows_v(const FrameSrc& f, const float* mask, const double* mean_sub, double inv_area,
                         int frame0, int nfr, int mode, int rows, int cols, int C1, int K4, int H4,
                         float2* RU, float2* RV, const float2* tw, cudaStream_t st) {
  constexpr int T = fft_threads(P, FR);
  const size_t smem = (size_t)FR * ld_of(P) * sizeof(float2);
  ZR_TRY(cuda_check(cudaFuncSetAttribute(k_fwd_rows<P, FR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "k_fwd_rows attr"));
  k_fwd_rows<P, FR><<<dim3(nfr, (rows + FR - 1) / FR), T, smem, st>>>(f, mask, mean_sub, inv_area, frame0, mode,
                                                                       rows, cols, C1, K4, H4, RU, RV, tw);
  return launched("k_fwd_rows");
}

template <int P>
static int launch_rows(const FrameSrc& f, const float* mask, const double* mean_sub, double inv_area,
                       int frame0, int nfr, int mode, int rows, int cols, int C1, int K4, int H4,
                       float2* RU, float2* RV, const float2* tw, cudaStream_t st) {
  switch (tune_get(TUNE_FWD_ROWS, P)) {
    case 1: return launch_rows_v<P, 1>(f, mask, mean_sub, inv_area, frame0, nfr, mode, rows, cols, C1, K4, H4, RU, RV, tw, st);
    case 4: return launch_rows_v<P, 4>(f, mask, mean_sub, inv_area, frame0, nfr, mode, rows, cols, C1, K4, H4, RU, RV, tw, st);
    default:
      return launch_rows_v<P, FR_DEFAULT>(f, mask, mean_sub, inv_area, frame0, nfr, mode, rows, cols, C1, K4, H4, RU,
                                          RV, tw, st);
  }
}

template <int P, int FC>
static int launch_cols_v(const float2* RU, const float2* RV, int rows, int C0, int K4, int H4, long long se,
                         int nfr, int nz, float2* G, float2* S, const float2* tw, cudaStream_t st) {
  constexpr int T = fft_threads(P, FC);
  const size_t smem = (size_t)FC * ld_of(P) * sizeof(float2);
  ZR_TRY(cuda_check(cudaFuncSetAttribute(k_fwd_cols<P, FC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "k_fwd_cols attr"));
  k_fwd_cols<P, FC><<<dim3(K4 / FC, nfr, nz), T, smem, st>>>(RU, RV, rows, C0, K4, H4, se, G, S, tw);
  return launched("k_fwd_cols");
}

template <int P>
static int launch_cols(const float2* RU, const float2* RV, int rows, int C0, int K4, int H4, long long se,
                       int nfr, int nz, float2* G, float2* S, const float2* tw, cudaStream_t st) {
  switch (tune_get(TUNE_FWD_COLS, P)) {
    case 1: return launch_cols_v<P, 1>(RU, RV, rows, C0, K4, H4, se, nfr, nz, G, S, tw, st);
    case 4: return launch_cols_v<P, 4>(RU, RV, rows, C0, K4, H4, se, nfr, nz, G, S, tw, st);
    default: return launch_cols_v<P, FC_DEFAULT>(RU, RV, rows, C0, K4, H4, se, nfr, nz, G, S, tw, st);
  }
}

#define ZR_POW2_DISPATCH(L, CALL)                  \
  switch (L) {                                     \
    case 64: { constexpr int LL = 64; CALL; } break;     \
    case 128: { constexpr int LL = 128; CALL; } break;   \
    case 256: { constexpr int LL = 256; CALL; } break;   \
    case 512: { constexpr int LL = 512; CALL; } break;   \
    case 1024: { constexpr int LL = 1024; CALL; } break; \
    case 1536: { constexpr int LL = 1536; CALL; } break; \
    case 2048: { constexpr int LL = 2048; CALL; } break; \
    case 3072: { constexpr int LL = 3072; CALL; } break; \
    case 4096: { constexpr int LL = 4096; CALL; } break; \
    case 6144: { constexpr int LL = 6144; CALL; } break; \
    default: return set_error(ZR_ESIZE, "transform length %d not supported (powers of two 64..4096, 1536, 3072, 6144)", (int)(L)); \
  }

}  // namespace zr

using namespace zr;

extern "C" int zr_spectrum_pitch(int C1) { return ((C1 / 2 + 1) + 3) & ~3; }

extern "C" long long zr_spectrum_elems(int C0, int C1) { return (long long)(C0 + 4) * zr_spectrum_pitch(C1); }

extern "C" size_t zr_spectra_work_bytes(int height, int n_frames, int C1) {
  const size_t H4 = (size_t)(height + 3) / 4;
  return 2 * (size_t)n_frames * H4 * zr_spectrum_pitch(C1) * 4 * sizeof(float2);
}

extern "C" int zr_frame_sums(const zr_frames_t* frames, double* sums, void* stream) {
  if (!frames || !sums || !frames->raw) return set_error(ZR_EINVAL, "zr_frame_sums: null argument");
  FrameSrc f = make_src(frames);
  if (f.N <= 0 || f.H <= 0 || f.W <= 0) return set_error(ZR_EINVAL, "zr_frame_sums: empty movie");
  const long long npix = (long long)f.H * f.W;
  int bx = (int)((npix + 256 * 64 - 1) / (256 * 64));
  if (bx > 1024) bx = 1024;
  k_frame_sums<<<dim3(bx, f.N), 256, 0, (cudaStream_t)stream>>>(f, sums);
  return launched("k_frame_sums");
}

extern "C" int zr_spectra(const zr_frames_t* frames, const float* mask, const double* mean_sub, int frame0,
                          int n_frames, int mode, int P0, int P1, int C0, int C1, void* G, void* S, void* work,
                          size_t work_bytes, void* stream) {
  if (!frames || !G || (mode == 0 && (!S || !frames->raw)))
    return set_error(ZR_EINVAL, "zr_spectra: null argument");
  if (!fft_len_ok(P0) || !fft_len_ok(P1) || !fft_len_ok(C0) || !fft_len_ok(C1) || C0 > P0 || C1 > P1 || C0 < 64 ||
      C1 < 64 || P0 > 6144 || P1 > 6144 || C0 > 4096 || C1 > 4096)
    return set_error(ZR_ESIZE,
                     "zr_spectra: P=%dx%d C=%dx%d must be powers of two or 3 x 2^k with 64 <= C <= P, P <= 6144, "
                     "C <= 4096", P0, P1, C0, C1);
  FrameSrc f = make_src(frames);
  if (f.H > P0 || f.W > P1) return set_error(ZR_EINVAL, "zr_spectra: frame %dx%d larger than padded %dx%d", f.H, f.W, P0, P1);
  if (n_frames <= 0 || frame0 < 0 || (mode == 0 && frame0 + n_frames > f.N))
    return set_error(ZR_EINVAL, "zr_spectra: frame range [%d,%d) outside movie of %d frames", frame0, frame0 + n_frames, f.N);
  const int rows = (mode == 1 && mask) ? P0 : f.H;
  const int cols = (mode == 1 && mask) ? P1 : f.W;
  const int H4 = (rows + 3) / 4;
  const int K4 = zr_spectrum_pitch(C1);
  const size_t need = (size_t)(mode == 0 ? 2 : 1) * n_frames * H4 * K4 * 4 * sizeof(float2);
  if (!work || work_bytes < need)
    return set_error(ZR_EWORK, "zr_spectra: work buffer %zu bytes < %zu needed", work_bytes, need);
  const float2* tw = twiddles();
  if (!tw) return ZR_ECUDA;
  float2* RU = (float2*)work;
  float2* RV = RU + (size_t)n_frames * H4 * K4 * 4;
  cudaStream_t st = (cudaStream_t)stream;
  const double inv_area = 1.0 / ((double)f.H * f.W);
  ZR_POW2_DISPATCH(P1, ZR_TRY((launch_rows<LL>(f, mask, mean_sub, inv_area, frame0, n_frames, mode, rows, cols, C1,
                                                K4, H4, RU, RV, tw, st))));
  const long long se = zr_spectrum_elems(C0, C1);
  ZR_POW2_DISPATCH(P0, ZR_TRY((launch_cols<LL>(RU, RV, rows, C0, K4, H4, se, n_frames, mode == 0 ? 2 : 1,
                                                (float2*)G, (float2*)S, tw, st))));
  return ZR_OK;
}
