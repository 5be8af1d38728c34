// Dose-weighted sum (doseFilter, zorro.py:2349-2494), the Unblur filter:
//
//   filtSum = | IFFT( sum_n FFT(pad_sym(frame_n)) * thres_n(q) * filt_n(q) ) |[:H, :W]
//   filt_n(q)  = exp(-0.5 * dose_end_n / critDose(q)),
//   critDose(q) = vs * (A q^B + C)   (the value at the Nyquist corner is
//                 replaced by the square of its left neighbour, zorro.py:2422),
//   thres_n(q) = exp(-(q / thresQ_n)^order).
//
// The filters are real and even in frequency, so the accumulated spectrum is
// Hermitian: only kx in [0, P1/2] is kept.  Two aligned frames share one
// complex row FFT; the column pass applies each frame's filter and
// accumulates in shared memory; the inverse column pass keeps only the H
// output rows and the final row pass packs two rows per complex inverse FFT.
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace zr {

// rows per CTA of the forward row pass and columns per CTA of the inverse
// column pass
#ifndef ZR_DS_NBR
#define ZR_DS_NBR 4
#endif
constexpr int DS_NBR = ZR_DS_NBR;
// rows (columns) per CTA for a transform of length L: two for the 6144-point
// transforms, whose four-row tiles would not fit the register file
__host__ __device__ constexpr int ds_nbr(int L) { return L > 4096 ? 2 : DS_NBR; }
// CTAs per SM to ask the register allocator for: 128 registers a thread
constexpr int ds_minb(int T) { return sm_minb(T); }


__device__ __forceinline__ int sym_idx(int i, int n) {
  int m = i % (2 * n);
  return m < n ? m : 2 * n - 1 - m;
}

template <int P1>
__global__ void __launch_bounds__(fft_threads(P1, ds_nbr(P1)), ds_minb(fft_threads(P1, ds_nbr(P1))))
    k_dose_rows(const float* __restrict__ img, int N, int H, int W, int f0, int K4, int P0,
                float2* __restrict__ RW, const float2* __restrict__ tw) {
  constexpr int T = fft_threads(P1, ds_nbr(P1));
  constexpr int LD = ld_of(P1);
  extern __shared__ float2 sm[];
  const int g = blockIdx.x;
  const int pl = blockIdx.y;              // frame pair within the chunk
  const int na = f0 + 2 * pl, nb = na + 1;
  const float* ia = img + (size_t)na * H * W;
  const float* ib = img + (size_t)(nb < N ? nb : na) * H * W;
  // element x of row r: the symmetric padding of the two frames' row; every
  // pass but the last, which pairs X[k] with X[P1 - k] in registers
  constexpr int NB = ds_nbr(P1);
  constexpr int RL = last_radix(P1), NSL = P1 / RL;
  block_fft_from<P1, NB, T, -1, NSL>(sm, tw, [&](int r, int x) {
    const int yy = g * NB + r;
    const int ys = yy < H ? yy : (yy < 2 * H ? 2 * H - 1 - yy : sym_idx(yy, H));
    const int xs = x < W ? x : (x < 2 * W ? 2 * W - 1 - x : sym_idx(x, W));
    const size_t p = (size_t)ys * W + xs;
    return make_float2(__ldg(ia + p), nb < N ? __ldg(ib + p) : 0.0f);
  });
  // output: column-major per frame, [frame][kx][ky]
  const size_t fa = (size_t)(2 * pl) * K4 * P0;
  const size_t fb = fa + (size_t)K4 * P0;
  const int y0 = g * NB;
  fft_last_paired<P1, NB, T, -1>(sm, tw, [&](int r, int k0, const float2* x0, int k1, const float2* x1) {
    auto put = [&](int k, float2 zk, float2 zm) {
      const size_t o = (size_t)k * P0 + y0 + r;
      RW[fa + o] = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
      if (nb < N) RW[fb + o] = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    };
#pragma unroll
    for (int q = 0; q < RL; q++) {
      const int m0 = k0 + q * NSL, m1 = k1 + q * NSL;
      if (m0 <= P1 / 2) put(m0, x0[q], k0 > 0 ? x1[RL - 1 - q] : x0[(RL - q) % RL]);
      if (m1 <= P1 / 2) put(m1, x1[q], k0 > 0 ? x0[RL - 1 - q] : x1[RL - 1 - q]);
    }
  });
  // the pitch's columns past P1/2 are zero
  for (int e = threadIdx.x; e < NB * (K4 - P1 / 2 - 1); e += T) {
    const int r = e % NB, k = P1 / 2 + 1 + e / NB;
    const size_t o = (size_t)k * P0 + y0 + r;
    RW[fa + o] = make_float2(0.0f, 0.0f);
    if (nb < N) RW[fb + o] = make_float2(0.0f, 0.0f);
  }
}

__device__ __forceinline__ float crit_dose(const zr_dose_params_t& p, int fy, int fx) {
  const float q = sqrtf((float)fx * (float)fx * (p.inv_ps_x * p.inv_ps_x) + (float)fy * (float)fy * (p.inv_ps_y * p.inv_ps_y));
  return p.voltage_scaling * (p.crit_a * powf(q, p.crit_b) + p.crit_c);
}

__device__ __forceinline__ void dose_weight(const zr_dose_params_t& p, int P0, int P1, int ky, int kx, float dose_end,
                                            float tq, float& w) {
  const int fy = ky < P0 / 2 ? ky : ky - P0;
  const int fx = kx;
  const float q = sqrtf((float)fx * (float)fx * (p.inv_ps_x * p.inv_ps_x) + (float)fy * (float)fy * (p.inv_ps_y * p.inv_ps_y));
  float crit;
  if (ky == P0 / 2 && kx == P1 / 2) {
    const float c = crit_dose(p, fy, P1 / 2 - 1);
    crit = c * c;
  } else {
    crit = p.voltage_scaling * (p.crit_a * powf(q, p.crit_b) + p.crit_c);
  }
  const float filt = expf((-0.5f * dose_end) / crit);
  const float thres = expf(-powf(q / tq, p.cutoff_order));
  w = thres * filt;
}

// One column kx per CTA: for every frame, the column's forward FFT, times the
// frame's filter, accumulated in registers (each thread owns P0/T rows).
constexpr int DS_CT = 256;

template <int P0>
__global__ void __launch_bounds__(DS_CT, 2)
    k_dose_cols(const float2* __restrict__ RW, int f0, int nfr, int K4, int P1, zr_dose_params_t prm,
                const float* __restrict__ thres_q, const float* __restrict__ dose_end, int first,
                float2* __restrict__ ACC, float* __restrict__ FM, const float2* __restrict__ tw) {
  constexpr int LD = ld_of(P0);
  constexpr int PER = P0 / DS_CT;
  extern __shared__ float2 sm[];
  // per-element constants of this column: 1/critDose(q) and log2(q)
  float* inv_crit = reinterpret_cast<float*>(sm + LD);
  float* lq = inv_crit + P0;
  const int kx = blockIdx.x;
  const bool live = kx <= P1 / 2;
  for (int y = threadIdx.x; y < P0 && live; y += DS_CT) {
    const int fy = y < P0 / 2 ? y : y - P0;
    const float q = sqrtf((float)kx * (float)kx * (prm.inv_ps_x * prm.inv_ps_x) +
                          (float)fy * (float)fy * (prm.inv_ps_y * prm.inv_ps_y));
    float crit;
    if (y == P0 / 2 && kx == P1 / 2) {
      const float c = crit_dose(prm, fy, P1 / 2 - 1);
      crit = c * c;  // zorro.py:2422
    } else {
      crit = prm.voltage_scaling * (prm.crit_a * powf(q, prm.crit_b) + prm.crit_c);
    }
    inv_crit[y] = 1.0f / crit;
    lq[y] = log2f(q);
  }
  float2 acc[PER];
  float fm[PER];
#pragma unroll
  for (int j = 0; j < PER; j++) {
    const int y = threadIdx.x + j * DS_CT;
    acc[j] = first ? make_float2(0.0f, 0.0f) : ACC[(size_t)kx * P0 + y];
    fm[j] = (first || !prm.normalize) ? 0.0f : FM[(size_t)kx * P0 + y];
  }
  const float LOG2E = 1.4426950408889634f;
  // the last pass's butterfly j = thread holds elements j + r P0/R: with
  // P0/R = DS_CT those are exactly the thread's accumulator rows, so the
  // spectrum is weighted and summed straight from its registers
  constexpr bool ACC_DIRECT = P0 / last_radix(P0) == DS_CT && last_radix(P0) == PER;
  for (int nl = 0; nl < nfr; nl++) {
    const float2* col = RW + ((size_t)nl * K4 + kx) * P0;
    // filt = exp(-0.5 D / crit), thres = exp(-(q / thresQ)^order)
    const float cd = (-0.5f * dose_end[f0 + nl]) * LOG2E;
    const float ltq = log2f(thres_q[f0 + nl]);
    auto accumulate = [&](int j, int y, float2 F) {
      const float filt = exp2f(cd * inv_crit[y]);
      const float thres = exp2f(-LOG2E * exp2f(prm.cutoff_order * (lq[y] - ltq)));
      const float w = thres * filt;
      acc[j] = make_float2(acc[j].x + F.x * w, acc[j].y + F.y * w);
      if (prm.normalize) fm[j] += w;
    };
    __syncthreads();  // the previous frame's spectrum has been read
    if constexpr (ACC_DIRECT) {
      block_fft_from<P0, 1, DS_CT, -1>(
          sm, tw, [&](int, int y) { return __ldg(col + y); },
          all_out([&](int, int y, int r, float2 F) {
            if (live) accumulate(r, y, F);
          }));
    } else {
      block_fft_from<P0, 1, DS_CT, -1>(sm, tw, [&](int, int y) { return __ldg(col + y); });
      if (!live) continue;
#pragma unroll
      for (int j = 0; j < PER; j++) {
        const int y = threadIdx.x + j * DS_CT;
        accumulate(j, y, sm[pidx(y)]);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < PER; j++) {
    const int y = threadIdx.x + j * DS_CT;
    ACC[(size_t)kx * P0 + y] = acc[j];
    if (prm.normalize) FM[(size_t)kx * P0 + y] = fm[j];
  }
}

// Inverse column pass, keeping rows [0, H).
template <int P0>
__global__ void __launch_bounds__(fft_threads(P0, ds_nbr(P0)), ds_minb(fft_threads(P0, ds_nbr(P0))))
    k_dose_icols(const float2* __restrict__ ACC, const float* __restrict__ FM, int normalize, int K4, int H,
                 float2* __restrict__ T2, const float2* __restrict__ tw) {
  constexpr int T = fft_threads(P0, ds_nbr(P0));
  constexpr int LD = ld_of(P0);
  extern __shared__ float2 sm[];
  const int k0 = blockIdx.x * ds_nbr(P0);
  block_fft_from<P0, ds_nbr(P0), T, 1>(sm, tw, [&](int c, int y) {
    float2 v = __ldg(ACC + (size_t)(k0 + c) * P0 + y);
    if (normalize) {
      const float s = 1.0f / (__ldg(FM + (size_t)(k0 + c) * P0 + y) + 1.0f);
      v = make_float2(v.x * s, v.y * s);
    }
    return v;
  });
  for (int e = threadIdx.x; e < H * ds_nbr(P0); e += T) {
    const int y = e / ds_nbr(P0), c = e - y * ds_nbr(P0);
    T2[(size_t)y * K4 + k0 + c] = sm[c * LD + pidx(y)];
  }
}

// Real-output inverse row pass (two rows per complex FFT), |.|, crop, scale.
template <int P1>
__global__ void __launch_bounds__(fft_threads(P1, 2), fft_minblocks(P1))
    k_dose_irows(const float2* __restrict__ T2, int K4, int H, int W, float scale, float* __restrict__ out,
                 const float2* __restrict__ tw) {
  constexpr int T = fft_threads(P1, 2);
  constexpr int LD = ld_of(P1);
  extern __shared__ float2 sm[];
  const int y0 = blockIdx.x * 4;
  block_fft_from<P1, 2, T, 1>(sm, tw, [&](int p, int i) {
    const int a0 = y0 + 2 * p, a1 = a0 + 1;
    return packed_rows<P1>(a0 < H ? T2 + (size_t)a0 * K4 : nullptr, a1 < H ? T2 + (size_t)a1 * K4 : nullptr, i);
  });
  for (int e = threadIdx.x; e < 4 * W; e += T) {
    const int q = e / W, x = e - q * W;
    const int y = y0 + q;
    if (y >= H) continue;
    const float2 v = sm[(q >> 1) * LD + pidx(x)];
    out[(size_t)y * W + x] = fabsf(((q & 1) ? v.y : v.x) * scale);
  }
}

template <int P>
static int set_smem(const void* fn, size_t smem) {
  return cuda_check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "dose attr");
}

#define ZR_DOSE_DISPATCH(L, CALL)                               \
  switch (L) {                                                  \
    case 256: { constexpr int LL = 256; CALL; } break;          \
    case 512: { constexpr int LL = 512; CALL; } break;          \
    case 1024: { constexpr int LL = 1024; CALL; } break;        \
    case 1536: { constexpr int LL = 1536; CALL; } break;        \
    case 2048: { constexpr int LL = 2048; CALL; } break;        \
    case 3072: { constexpr int LL = 3072; CALL; } break;        \
    case 4096: { constexpr int LL = 4096; CALL; } break;        \
    case 6144: { constexpr int LL = 6144; CALL; } break;        \
    default: return set_error(ZR_ESIZE, "dose filter size %d not supported", (int)(L)); \
  }

template <int P1>
static int dose_rows(const float* img, int N, int H, int W, int f0, int npairs, int K4, int P0, float2* RW,
                     const float2* tw, cudaStream_t st) {
  const size_t smem = (size_t)ds_nbr(P1) * ld_of(P1) * sizeof(float2);
  ZR_TRY(set_smem<P1>((const void*)k_dose_rows<P1>, smem));
  k_dose_rows<P1><<<dim3(P0 / ds_nbr(P1), npairs), fft_threads(P1, ds_nbr(P1)), smem, st>>>(img, N, H, W, f0, K4, P0,
                                                                                            RW, tw);
  return launched("k_dose_rows");
}

template <int P0>
static int dose_cols(const float2* RW, int f0, int nfr, int K4, int P1, const zr_dose_params_t& prm,
                     const float* tq, const float* de, int first, float2* ACC, float* FM, const float2* tw,
                     cudaStream_t st) {
  const size_t smem = (size_t)ld_of(P0) * sizeof(float2) + (size_t)2 * P0 * sizeof(float);
  ZR_TRY(set_smem<P0>((const void*)k_dose_cols<P0>, smem));
  k_dose_cols<P0><<<K4, DS_CT, smem, st>>>(RW, f0, nfr, K4, P1, prm, tq, de, first, ACC, FM, tw);
  return launched("k_dose_cols");
}

template <int P0>
static int dose_icols(const float2* ACC, const float* FM, int normalize, int K4, int H, float2* T2, const float2* tw,
                      cudaStream_t st) {
  const size_t smem = (size_t)ds_nbr(P0) * ld_of(P0) * sizeof(float2);
  ZR_TRY(set_smem<P0>((const void*)k_dose_icols<P0>, smem));
  k_dose_icols<P0><<<K4 / ds_nbr(P0), fft_threads(P0, ds_nbr(P0)), smem, st>>>(ACC, FM, normalize, K4, H, T2, tw);
  return launched("k_dose_icols");
}

template <int P1>
static int dose_irows(const float2* T2, int K4, int H, int W, float scale, float* out, const float2* tw,
                      cudaStream_t st) {
  const size_t smem = (size_t)2 * ld_of(P1) * sizeof(float2);
  ZR_TRY(set_smem<P1>((const void*)k_dose_irows<P1>, smem));
  k_dose_irows<P1><<<(H + 3) / 4, fft_threads(P1, 2), smem, st>>>(T2, K4, H, W, scale, out, tw);
  return launched("k_dose_irows");
}

}  // namespace zr

using namespace zr;

static size_t dose_fixed_bytes(int P0, int P1) {
  const size_t K4 = zr_spectrum_pitch(P1);
  return (size_t)P0 * K4 * (2 * sizeof(float2) + sizeof(float));
}

static size_t dose_frame_bytes(int P0, int P1) { return (size_t)P0 * zr_spectrum_pitch(P1) * sizeof(float2); }

extern "C" size_t zr_dose_work_bytes(int P0, int P1, int n_frames) {
  return dose_fixed_bytes(P0, P1) + (size_t)n_frames * dose_frame_bytes(P0, P1);
}

extern "C" int zr_dose_filter(const float* aligned, int N, int H, int W, const zr_dose_params_t* params,
                              const float* thres_q, const float* dose_end, int P0, int P1, float* filt_sum,
                              void* work, size_t work_bytes, void* stream) {
  if (!aligned || !params || !thres_q || !dose_end || !filt_sum || !work)
    return set_error(ZR_EINVAL, "zr_dose_filter: null argument");
  if (N <= 0 || H <= 0 || W <= 0 || H > P0 || W > P1) return set_error(ZR_EINVAL, "zr_dose_filter: bad sizes");
  if (!fft_len_ok(P0) || !fft_len_ok(P1) || P0 < 256 || P1 < 256 || P0 > 6144 || P1 > 6144 || P0 == 8192 ||
      P1 == 8192)
    return set_error(ZR_ESIZE,
                     "zr_dose_filter: padded size %dx%d must be a power of two in [256, 4096], 1536, 3072 or 6144", P0,
                     P1);
  const size_t fixed = dose_fixed_bytes(P0, P1), per = dose_frame_bytes(P0, P1);
  if (work_bytes < fixed + 2 * per)
    return set_error(ZR_EWORK, "zr_dose_filter: work buffer %zu < %zu", work_bytes, fixed + 2 * per);
  int chunk = (int)((work_bytes - fixed) / per);
  chunk &= ~1;
  if (chunk > N + (N & 1)) chunk = N + (N & 1);
  const float2* tw = twiddles();
  if (!tw) return ZR_ECUDA;
  const int K4 = zr_spectrum_pitch(P1);
  float2* ACC = (float2*)work;
  float2* T2 = ACC + (size_t)P0 * K4;
  float* FM = (float*)(T2 + (size_t)P0 * K4);
  float2* RW = (float2*)(FM + (size_t)P0 * K4);
  cudaStream_t st = (cudaStream_t)stream;
  for (int f0 = 0; f0 < N; f0 += chunk) {
    const int nfr = (N - f0) < chunk ? (N - f0) : chunk;
    const int npairs = (nfr + 1) / 2;
    ZR_DOSE_DISPATCH(P1, ZR_TRY((dose_rows<LL>(aligned, N, H, W, f0, npairs, K4, P0, RW, tw, st))));
    ZR_DOSE_DISPATCH(P0, ZR_TRY((dose_cols<LL>(RW, f0, nfr, K4, P1, *params, thres_q, dose_end, f0 == 0, ACC, FM,
                                                tw, st))));
  }
  ZR_DOSE_DISPATCH(P0, ZR_TRY((dose_icols<LL>(ACC, FM, params->normalize, K4, H, T2, tw, st))));
  // abs(IFFT2.execute(...)) at zorro.py:2484-2488: FFTW's inverse carries no 1/N
  const float scale = 1.0f;
  ZR_DOSE_DISPATCH(P1, ZR_TRY((dose_irows<LL>(T2, K4, H, W, scale, filt_sum, tw, st))));
  return ZR_OK;
}
