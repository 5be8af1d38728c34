// Fourier binning of a movie (binStack with binKernel='fourier',
// zorro.py:1826-1904): per frame, the H x W DFT, the corners kept to
// Hb x Wb (rows [0, Hb/2) and [H - Hb/2, H), columns likewise), times
// normConst = 1/(Hb Wb), the unscaled Hb x Wb inverse DFT, and its real part.
//
// Frame sizes are arbitrary (K2 super-resolution frames are 7676 x 7420), so
// a length-n DFT with n <= 8192 is Bluestein's: with the chirp
// c_m = exp(i pi m^2/n),
//     X_k = conj(c_k) sum_j (x_j conj(c_j)) c_{k-j},
// a linear convolution done as a circular one of power-of-two length
// M >= 2n - 1 with the shared-memory engine (forward FFT, product with the
// transformed chirp, unscaled inverse, 1/M).  Longer sides (the 11520-pixel
// width of K3 super-resolution frames) would need M = 32768, more than one
// CTA's shared memory holds; they are transformed directly by the mixed-radix
// engine when they divide its twiddle table (2^a 3^b 5^c, b <= 2, c <= 1:
// 9216, 10240, 11520, 12288, 15360 and 16384).  An inverse DFT is the
// conjugate of the forward DFT of the conjugate.
//
// Passes (one frame at a time, scratch in ``work``):
//   rows     two real rows per complex Bluestein DFT of length W, split by
//            Hermitian symmetry, columns kx in [0, Wb/2] kept   -> R [H][Kb]
//   transpose                                                  -> Ct [Kb][H]
//   columns  Bluestein DFT of length H, the Hb crop rows plus row +Hb/2, the
//            real part that the reference's real() keeps made explicit (the
//            cropped spectrum's Nyquist row and column averaged with their
//            mirrors), Bluestein inverse of length Hb, times 1/(Hb Wb)  -> Ci [Kb][Hb]
//   transpose                                                  -> Ri [Hb][Kb]
//   rows     the Hermitian row completed from kx in [0, Wb/2], Bluestein
//            inverse of length Wb, real part                    -> out [Hb][Wb]
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace zr {

constexpr int BN_T = 512;

__host__ __device__ constexpr int bn_pow2_at_least(int v) {
  int m = 1;
  while (m < v) m <<= 1;
  return m;
}

// c_m = exp(i pi m^2 / n): m^2 is reduced mod 2n in integers, so the angle is
// exact before the (double) sincospi.
__device__ __forceinline__ float2 chirp(long long m, int n) {
  const long long q = (m * m) % (2LL * n);
  double s, c;
  sincospi((double)q / (double)n, &s, &c);
  return make_float2((float)c, (float)s);
}

// Per length n: the chirp c[0..n) and the length-M transform of the symmetric
// sequence b (b_m = c_m, b_{M-m} = c_m for 0 < m < n, zero between).
template <int M>
__global__ void __launch_bounds__(BN_T) k_bluestein_plan(int n, float2* __restrict__ c, float2* __restrict__ bhat,
                                                        const float2* __restrict__ tw) {
  extern __shared__ float2 sm[];
  for (int m = threadIdx.x; m < M; m += BN_T) {
    float2 v = make_float2(0.0f, 0.0f);
    if (m < n) v = chirp(m, n);
    else if (m > M - n) v = chirp(M - m, n);
    sm[pidx(m)] = v;
  }
  for (int m = threadIdx.x; m < n; m += BN_T) c[m] = chirp(m, n);
  __syncthreads();
  block_fft<M, 1, BN_T, -1>(sm, tw);
  for (int m = threadIdx.x; m < M; m += BN_T) bhat[m] = sm[pidx(m)];
}

// Forward DFT of length n of the values already in sm[pidx(j)] (j < n; the
// rest must be zero): X_k = conj(c_k) (IFFT(FFT(x conj(c)) bhat))_k / M, left
// in sm[pidx(k)] for k < n.  All threads call; ends synchronised.
//
// With n == M (a length the engine transforms directly) it is the plain
// forward FFT of the n values; ``c`` and ``bhat`` are not read.
template <int M>
__device__ void bluestein_inplace(float2* sm, int n, const float2* __restrict__ c, const float2* __restrict__ bhat,
                                  const float2* __restrict__ tw) {
  if (n == M) {
    __syncthreads();
    block_fft<M, 1, BN_T, -1>(sm, tw);
    return;
  }
  for (int j = threadIdx.x; j < n; j += BN_T) sm[pidx(j)] = cmulc(sm[pidx(j)], __ldg(c + j));
  __syncthreads();
  block_fft<M, 1, BN_T, -1>(sm, tw);
  for (int k = threadIdx.x; k < M; k += BN_T) sm[pidx(k)] = cmul(sm[pidx(k)], __ldg(bhat + k));
  __syncthreads();
  block_fft<M, 1, BN_T, 1>(sm, tw);
  const float inv = 1.0f / (float)M;
  for (int k = threadIdx.x; k < n; k += BN_T) {
    const float2 v = cmulc(sm[pidx(k)], __ldg(c + k));
    sm[pidx(k)] = make_float2(v.x * inv, v.y * inv);
  }
  __syncthreads();
}

// Row pass: rows 2q and 2q+1 of the frame packed as x = a + i b.
template <int M>
__global__ void __launch_bounds__(BN_T) k_bin_rows(FrameSrc f, int n_frame, int W, int H, int Kb,
                                                  const float2* __restrict__ c, const float2* __restrict__ bhat,
                                                  float2* __restrict__ R, const float2* __restrict__ tw) {
  extern __shared__ float2 sm[];
  const int ya = 2 * blockIdx.x, yb = ya + 1;
  for (int m = threadIdx.x; m < M; m += BN_T) {
    float2 v = make_float2(0.0f, 0.0f);
    if (m < W) {
      v.x = load_corrected(f, n_frame, ya, m);
      if (yb < H) v.y = load_corrected(f, n_frame, yb, m);
    }
    sm[pidx(m)] = v;
  }
  __syncthreads();
  bluestein_inplace<M>(sm, W, c, bhat, tw);
  // split: A_k = (Z_k + conj(Z_{-k})) / 2, B_k = (Z_k - conj(Z_{-k})) / (2i)
  for (int k = threadIdx.x; k < Kb; k += BN_T) {
    const float2 z = sm[pidx(k)], zm = sm[pidx(k == 0 ? 0 : W - k)];
    R[(size_t)ya * Kb + k] = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
    if (yb < H) R[(size_t)yb * Kb + k] = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
  }
}

// 32 x 32 tiled transpose of a rows x cols complex matrix.
__global__ void k_bin_transpose(const float2* __restrict__ in, int rows, int cols, float2* __restrict__ out) {
  __shared__ float2 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int r = r0 + i, cc = c0 + threadIdx.x;
    if (r < rows && cc < cols) t[i][threadIdx.x] = in[(size_t)r * cols + cc];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int cc = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && cc < cols) out[(size_t)cc * rows + r] = t[threadIdx.x][i];
  }
}

// Column pass for column kx of the kept half plane.
template <int M1, int M2>
__global__ void __launch_bounds__(BN_T) k_bin_cols(const float2* __restrict__ Ct, int H, int Hb, int Kb, int Wb,
                                                  const float2* __restrict__ c1, const float2* __restrict__ bh1,
                                                  const float2* __restrict__ c2, const float2* __restrict__ bh2,
                                                  float scale, float2* __restrict__ Ci, const float2* __restrict__ tw) {
  constexpr int MM = M1 > M2 ? M1 : M2;
  extern __shared__ float2 sm[];
  float2* z = sm + ld_of(MM);  // the Hb cropped values of this column
  const int kx = blockIdx.x;
  const int b0 = Hb / 2, b1 = Wb / 2;
  const float2* col = Ct + (size_t)kx * H;
  for (int m = threadIdx.x; m < M1; m += BN_T) sm[pidx(m)] = m < H ? col[m] : make_float2(0.0f, 0.0f);
  __syncthreads();
  bluestein_inplace<M1>(sm, H, c1, bh1, tw);
  // the cropped, Hermitian-completed column: output row i <-> frequency
  // i (i < b0) or i - Hb (i >= b0); F at frequency ky sits at index ky mod H
  for (int i = threadIdx.x; i < Hb; i += BN_T) {
    const int ky = i < b0 ? i : i - Hb;
    const float2 F = sm[pidx(ky < 0 ? ky + H : ky)];
    float2 v;
    if (kx < b1) {
      if (i == b0) {  // frequency -b0: averaged with +b0
        const float2 Fp = sm[pidx(b0)];
        v = make_float2(0.5f * (F.x + Fp.x), 0.5f * (F.y + Fp.y));
      } else {
        v = F;
      }
    } else {  // the Nyquist column: F(ky, -b1) = conj(F(-ky, b1)) averaged with F(ky, b1)
      if (i == b0) {
        const float2 Fp = sm[pidx(b0)];
        v = make_float2(Fp.x, 0.0f);
      } else {
        const float2 Fm = sm[pidx(ky == 0 ? 0 : (-ky < 0 ? -ky + H : -ky))];
        v = make_float2(0.5f * (F.x + Fm.x), 0.5f * (F.y - Fm.y));
      }
    }
    z[i] = v;
  }
  __syncthreads();
  // inverse of length Hb: conj(DFT(conj(z)))
  for (int m = threadIdx.x; m < M2; m += BN_T) sm[pidx(m)] = m < Hb ? cconj(z[m]) : make_float2(0.0f, 0.0f);
  __syncthreads();
  bluestein_inplace<M2>(sm, Hb, c2, bh2, tw);
  for (int i = threadIdx.x; i < Hb; i += BN_T) {
    const float2 v = sm[pidx(i)];
    Ci[(size_t)kx * Hb + i] = make_float2(v.x * scale, -v.y * scale);
  }
}

// Final rows: the Hermitian row of length Wb from kx in [0, Wb/2], inverse,
// real part.
template <int M>
__global__ void __launch_bounds__(BN_T) k_bin_irows(const float2* __restrict__ Ri, int Kb, int Wb,
                                                   const float2* __restrict__ c, const float2* __restrict__ bhat,
                                                   float* __restrict__ out, const float2* __restrict__ tw) {
  extern __shared__ float2 sm[];
  const int i = blockIdx.x;
  const float2* row = Ri + (size_t)i * Kb;
  const int b1 = Wb / 2;
  for (int m = threadIdx.x; m < M; m += BN_T) {
    float2 v = make_float2(0.0f, 0.0f);
    if (m <= b1) v = row[m];
    else if (m < Wb) v = cconj(row[Wb - m]);
    sm[pidx(m)] = cconj(v);  // inverse = conj(DFT(conj(.)))
  }
  __syncthreads();
  bluestein_inplace<M>(sm, Wb, c, bhat, tw);
  for (int x = threadIdx.x; x < Wb; x += BN_T) out[(size_t)i * Wb + x] = sm[pidx(x)].x;  // real part
}

template <int M>
static int bn_smem(const void* fn, size_t extra = 0) {
  const size_t smem = (size_t)ld_of(M) * sizeof(float2) + extra;
  return cuda_check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "binning attr");
}

#define ZR_BN_DISPATCH(M, ...)                                     \
  switch (M) {                                                     \
    case 2048: { constexpr int MM = 2048; __VA_ARGS__; } break;    \
    case 4096: { constexpr int MM = 4096; __VA_ARGS__; } break;    \
    case 8192: { constexpr int MM = 8192; __VA_ARGS__; } break;    \
    case 9216: { constexpr int MM = 9216; __VA_ARGS__; } break;    \
    case 10240: { constexpr int MM = 10240; __VA_ARGS__; } break;  \
    case 11520: { constexpr int MM = 11520; __VA_ARGS__; } break;  \
    case 12288: { constexpr int MM = 12288; __VA_ARGS__; } break;  \
    case 15360: { constexpr int MM = 15360; __VA_ARGS__; } break;  \
    case 16384: { constexpr int MM = 16384; __VA_ARGS__; } break;  \
    default: return set_error(ZR_ESIZE, "binning transform of %d points not supported", (int)(M)); \
  }

// Transform length for a side of n pixels: the Bluestein convolution length
// (n <= 8192), n itself when the engine transforms it directly, else 0.
static int bn_len(int n) {
  if (n >= 2 && n <= 8192) return bn_pow2_at_least(2 * n - 1) < 2048 ? 2048 : bn_pow2_at_least(2 * n - 1);
  if (n > 8192 && n <= 16384 && TWN % n == 0 && (n == 9216 || n == 10240 || n == 11520 || n == 12288 ||
                                                  n == 15360 || n == 16384))
    return n;
  return 0;
}

struct BnPlan {
  int n, M;
  float2 *c, *bhat;
};

static size_t bn_plan_bytes(int n) { return ((size_t)n + bn_pow2_at_least(2 * n - 1)) * sizeof(float2); }

template <int M>
static int bn_make_plan(BnPlan& p, const float2* tw, cudaStream_t st) {
  if (p.n == M) return ZR_OK;  // a direct transform: no chirp
  ZR_TRY(bn_smem<M>((const void*)k_bluestein_plan<M>));
  k_bluestein_plan<M><<<1, BN_T, ld_of(M) * sizeof(float2), st>>>(p.n, p.c, p.bhat, tw);
  return launched("k_bluestein_plan");
}

}  // namespace zr

using namespace zr;

extern "C" size_t zr_bin_work_bytes(int H, int W, int Hb, int Wb) {
  const size_t Kb = (size_t)Wb / 2 + 1;
  const size_t plans = bn_plan_bytes(W) + bn_plan_bytes(H) + bn_plan_bytes(Hb) + bn_plan_bytes(Wb);
  return plans + 2 * (size_t)H * Kb * sizeof(float2) + 2 * (size_t)Hb * Kb * sizeof(float2) + 256 * 8;
}

extern "C" int zr_bin_fourier(const zr_frames_t* frames, int Hb, int Wb, float* out, void* work, size_t work_bytes,
                              void* stream) {
  if (!frames || !frames->raw || !out || !work) return set_error(ZR_EINVAL, "zr_bin_fourier: null argument");
  FrameSrc f = make_src(frames);
  const int H = f.H, W = f.W;
  if (f.N <= 0 || H < 2 || W < 2) return set_error(ZR_EINVAL, "zr_bin_fourier: empty movie");
  if (Hb < 2 || Wb < 2 || (Hb & 1) || (Wb & 1) || Hb > H || Wb > W)
    return set_error(ZR_ESIZE, "zr_bin_fourier: binned shape %dx%d must be even and no larger than %dx%d", Hb, Wb,
                     H, W);
  const int MW = bn_len(W), MH = bn_len(H), MHb = bn_len(Hb), MWb = bn_len(Wb);
  if (!MW || !MH || !MHb || !MWb || Hb < 513 || Wb < 513)
    return set_error(ZR_ESIZE,
                     "zr_bin_fourier: frame %dx%d -> %dx%d: every side must be in 513..8192, or one of 9216, 10240, "
                     "11520, 12288, 15360, 16384 (binned sides at least 513)", H, W, Hb, Wb);
  if (work_bytes < zr_bin_work_bytes(H, W, Hb, Wb))
    return set_error(ZR_EWORK, "zr_bin_fourier: work buffer %zu < %zu", work_bytes, zr_bin_work_bytes(H, W, Hb, Wb));
  const float2* tw = twiddles();
  if (!tw) return ZR_ECUDA;
  cudaStream_t st = (cudaStream_t)stream;
  const int Kb = Wb / 2 + 1;
  float2* w = (float2*)work;
  BnPlan pw{W, MW, w, w + W};
  w += W + MW;
  BnPlan ph{H, MH, w, w + H};
  w += H + MH;
  BnPlan phb{Hb, MHb, w, w + Hb};
  w += Hb + MHb;
  BnPlan pwb{Wb, MWb, w, w + Wb};
  w += Wb + MWb;
  float2* R = w;
  float2* Ct = R + (size_t)H * Kb;
  float2* Ci = Ct + (size_t)H * Kb;
  float2* Ri = Ci + (size_t)Hb * Kb;
  ZR_BN_DISPATCH(MW, ZR_TRY((bn_make_plan<MM>(pw, tw, st))));
  ZR_BN_DISPATCH(MH, ZR_TRY((bn_make_plan<MM>(ph, tw, st))));
  ZR_BN_DISPATCH(MHb, ZR_TRY((bn_make_plan<MM>(phb, tw, st))));
  ZR_BN_DISPATCH(MWb, ZR_TRY((bn_make_plan<MM>(pwb, tw, st))));
  const float scale = (float)(1.0 / ((double)Hb * Wb));  // normConst, zorro.py:1881
  for (int n = 0; n < f.N; n++) {
    ZR_BN_DISPATCH(MW, {
      ZR_TRY(bn_smem<MM>((const void*)k_bin_rows<MM>));
      k_bin_rows<MM><<<(H + 1) / 2, BN_T, ld_of(MM) * sizeof(float2), st>>>(f, n, W, H, Kb, pw.c, pw.bhat, R, tw);
      ZR_TRY(launched("k_bin_rows"));
    });
    k_bin_transpose<<<dim3((Kb + 31) / 32, (H + 31) / 32), dim3(32, 8), 0, st>>>(R, H, Kb, Ct);
    ZR_TRY(launched("k_bin_transpose"));
    const int M12 = MH > MHb ? MH : MHb;
    const size_t smem2 = (size_t)ld_of(M12) * sizeof(float2) + (size_t)Hb * sizeof(float2);
    if (smem2 > 227 * 1024) return set_error(ZR_ESIZE, "zr_bin_fourier: column pass needs %zu bytes of shared memory", smem2);
#define ZR_BN_COLS(A, B)                                                                                         \
  if (MH == A && MHb == B) {                                                                                     \
    ZR_TRY(cuda_check(cudaFuncSetAttribute((const void*)k_bin_cols<A, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                           (int)smem2), "binning attr"));                                        \
    k_bin_cols<A, B><<<Kb, BN_T, smem2, st>>>(Ct, H, Hb, Kb, Wb, ph.c, ph.bhat, phb.c, phb.bhat, scale, Ci, tw); \
    ZR_TRY(launched("k_bin_cols"));                                                                              \
  } else
    ZR_BN_COLS(16384, 16384) ZR_BN_COLS(16384, 8192) ZR_BN_COLS(16384, 4096) ZR_BN_COLS(16384, 2048)
    ZR_BN_COLS(8192, 8192) ZR_BN_COLS(8192, 4096) ZR_BN_COLS(8192, 2048)
    ZR_BN_COLS(4096, 4096) ZR_BN_COLS(4096, 2048) ZR_BN_COLS(2048, 2048)
    ZR_BN_COLS(9216, 16384) ZR_BN_COLS(9216, 8192) ZR_BN_COLS(10240, 16384) ZR_BN_COLS(10240, 8192)
    ZR_BN_COLS(11520, 16384) ZR_BN_COLS(11520, 8192) ZR_BN_COLS(12288, 16384) ZR_BN_COLS(12288, 8192)
    ZR_BN_COLS(15360, 16384) ZR_BN_COLS(15360, 8192)
    return set_error(ZR_ESIZE, "zr_bin_fourier: column lengths %d -> %d not supported", H, Hb);
#undef ZR_BN_COLS
    k_bin_transpose<<<dim3((Hb + 31) / 32, (Kb + 31) / 32), dim3(32, 8), 0, st>>>(Ci, Kb, Hb, Ri);
    ZR_TRY(launched("k_bin_transpose"));
    float* o = out + (size_t)n * Hb * Wb;
    ZR_BN_DISPATCH(MWb, {
      ZR_TRY(bn_smem<MM>((const void*)k_bin_irows<MM>));
      k_bin_irows<MM><<<Hb, BN_T, ld_of(MM) * sizeof(float2), st>>>(Ri, Kb, Wb, pwb.c, pwb.bhat, o, tw);
      ZR_TRY(launched("k_bin_irows"));
    });
  }
  return ZR_OK;
}
