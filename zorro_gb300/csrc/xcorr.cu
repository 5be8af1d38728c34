// Masked normalised cross-correlation windows (mnxc2, zorro.py:1014-1097).
//
// Every term of mnxc2 is real(IFFT_C(A * conj(B))) for two cropped spectra A
// and B of real images, and only the +/-maxShift window of it is ever used
// (zorro.py:1090-1092).  With the half-plane spectra of zr_spectra:
//
//   column pass  for each kx in [0, C1/2]: build the C0 products of column kx
//                exactly as the full C0 x C1 cropped product would contribute
//                to real(IFFT) (the Nyquist row/column of the crop is not its
//                own Hermitian mirror, so row ky=-C0/2 averages the -C0/2 and
//                +C0/2 products and column kx=C1/2 uses the mirrored -C1/2
//                values), inverse FFT of length C0, keep the w window rows;
//   row pass     two window rows packed into one complex inverse FFT of length
//                C1 (real-output trick), keep the w window columns, scale by
//                normConst2 (zorro.py:634; the inverse, like the reference's
//                FFTW execute(), carries no 1/N).
//
// The four frame-only terms (CorrTM, CorrBM and the two Denominator IFFTs)
// depend on one frame each, so they are computed once per frame (zr_xcorr_terms)
// instead of once per pair; the pair kernel only transforms the numerator
// G_J conj(G_I) and combines.  Since real(IFFT(A conj(B)))(y, x) =
// real(IFFT(conj(A) B))(-y, -x) for any spectra, CorrTM is CorrBM and DenomT
// is DenomB point-reflected: one transform per frame gives both, over the
// (w+1) x (w+1) window [-maxShift, maxShift]^2 that the reflection needs.
#include "common.cuh"
#include "internal.h"

namespace zr {

// Column pass: columns per CTA (by default fewer for the long 3072 and 4096
// columns; the planner may choose 1, 2 or 4 per length) and threads
// (ZR_XC_EPT elements per thread and pass).
#ifndef ZR_XC_EPT
#define ZR_XC_EPT 32
#endif
#ifndef ZR_XC_MINB
#define ZR_XC_MINB 2
#endif
__host__ __device__ constexpr int xc_nbc_default(int C0) { return C0 >= 3072 ? 1 : 4; }
__host__ __device__ constexpr int xc_threads(int C0, int NBC) { return fft_threads(C0, NBC, ZR_XC_EPT); }
// Row pass: packed row pairs per CTA (default 2; the planner may choose 1,
// 2 or 4), elements per thread and pass
#ifndef ZR_XR_EPT
#define ZR_XR_EPT 32
#endif
constexpr int XC_NBR_DEFAULT = 2;
__host__ __device__ constexpr int xr_threads(int C1, int NBR) { return fft_threads(C1, NBR, ZR_XR_EPT); }
__host__ __device__ constexpr int xr_minb(int T) { return sm_minb(T); }

struct XcJobs {
  const void* G;     // spectra: float2, or __half2 when ``sc`` is set
  const void* S;
  const void* GM;
  const int* pairs;  // kind 1
  const void* G2;    // kind 2: template spectra (triMode 'refine')
  const float* sc;   // half spectra: power-of-two scales, [N] G, [N] S, [1] GM
  int N;
  int kind;          // 0 terms, 1 pairs, 2 frame I against template I
  int job0;
  long long se;      // spectrum elements
  int rows;          // window rows kept by the column pass: w + 1 (terms) or w (pairs)
};

// The two spectra of a job (its product is A conj(B)) and, for half-precision
// spectra, the factor 1 / (scale_A scale_B) that undoes their scaling.
template <typename E>
__device__ __forceinline__ void job_operands(const XcJobs& J, int job, const E*& A, const E*& B, float& unscale) {
  const E* G = (const E*)J.G;
  int ia = 0, ib = 0;  // scale slots
  if (J.kind == 1) {
    const int I = J.pairs[2 * job], Jj = J.pairs[2 * job + 1];
    A = G + (size_t)Jj * J.se;
    B = G + (size_t)I * J.se;
    ia = Jj;
    ib = I;
  } else if (J.kind == 2) {  // base frame I, template (sum_n G_n - G_I) / N
    A = G + (size_t)job * J.se;
    B = (const E*)J.G2 + (size_t)job * J.se;
  } else {
    const int t = job / J.N, n = job - t * J.N;
    const E* GM = (const E*)J.GM;
    switch (t) {
      case 0: A = G + (size_t)n * J.se; B = GM; ia = n; break;                    // CorrBM (and CorrTM)
      case 1: A = (const E*)J.S + (size_t)n * J.se; B = GM; ia = J.N + n; break;  // DenomB (and DenomT)
      default: A = GM; B = GM; ia = 2 * J.N; break;                              // maskProduct
    }
    ib = 2 * J.N;
  }
  unscale = J.sc ? 1.0f / (J.sc[ia] * J.sc[ib]) : 1.0f;
}

// One complex value of a spectrum.
__device__ __forceinline__ float2 load_one(const float2* p) { return __ldg(p); }
__device__ __forceinline__ float2 load_one(const __half2* p) { return __half22float2(__ldg(p)); }
__device__ __forceinline__ float2 to_f2(float2 a) { return a; }
__device__ __forceinline__ float2 to_f2(__half2 a) { return __half22float2(a); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// Value of the cropped product A conj(B) at row ``row`` of column k, as the
// full C0 x C1 product contributes to real(IFFT): regular columns as they
// are, except that row C0/2 averages the -C0/2 and +C0/2 products (the
// latter stored at index C0 of the column); the Nyquist column C1/2 holds
// conj(A) B of the mirrored row; columns past it are zero.
template <int C0, typename E>
__device__ __forceinline__ float2 xc_product(const E* a, const E* b, int row, int k, int half, float us) {
  constexpr int hc = C0 / 2;
  float2 h = make_float2(0.0f, 0.0f);
  if (k < half) {
    h = cmulc(load_one(a + row), load_one(b + row));
    if (k > 0 && row == hc) {
      const float2 h2 = cmulc(load_one(a + C0), load_one(b + C0));
      h = make_float2(0.5f * (h.x + h2.x), 0.5f * (h.y + h2.y));
    }
  } else if (k == half) {
    const int m = row == 0 ? 0 : (row == hc ? C0 : C0 - row);
    h = cmulc(load_one(b + m), load_one(a + m));
  }
  if (sizeof(E) != sizeof(float2)) h = cscale(h, us);  // undo the power-of-two scales (exact)
  return h;
}

// Column pass: CTA (job, column group) transforms NBC columns of the
// job's product.  Jobs vary fastest across the grid, so the CTAs resident at
// one time read the same columns of every spectrum and share them through L2.
// The first radix-16 pass forms the products while it loads its butterflies
// from the (column-major) spectra, so no product buffer passes through shared
// memory; the other passes run in shared memory, and the window rows
// [-maxShift, ...) of the result are kept.
template <int C0, typename E, int NBC>
__global__ void __launch_bounds__(xc_threads(C0, NBC), ZR_XC_MINB)
    k_xc_cols(XcJobs J, int C1, int K4, int mS, float2* __restrict__ Tw, const float2* __restrict__ tw) {
  constexpr int T = xc_threads(C0, NBC);
  constexpr int LD = ld_of(C0);
  constexpr int RP = C0 + 4;  // column pitch of the spectra
  constexpr int R = fft_radix(C0);
  constexpr int LR = C0 / R;
  constexpr int NBF = NBC * LR;
  constexpr int K = (NBF + T - 1) / T;
  static_assert(R < C0, "at least two passes");
  extern __shared__ float2 sm[];
  const int k0 = blockIdx.y * NBC;
  const int jl = blockIdx.x;
  const E *A, *B;
  float us;
  job_operands(J, J.job0 + jl, A, B, us);
  const int half = C1 / 2;
  float2 v[K][R];
#pragma unroll
  for (int i = 0; i < K; i++) {
    const int bf = threadIdx.x + i * T;
    if ((NBF % T) == 0 || bf < NBF) {
      const int b = bf / LR, j = bf - b * LR;
      const int k = k0 + b;
      const E* a = A + (size_t)k * RP;
      const E* bb = B + (size_t)k * RP;
      if (k < half) {
        // every load of the butterfly first (all in bounds), then the products
        E av[R], bv[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
          av[r] = __ldg(a + j + r * LR);
          bv[r] = __ldg(bb + j + r * LR);
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
          float2 h = cmulc(to_f2(av[r]), to_f2(bv[r]));
          if (k > 0 && j + r * LR == C0 / 2) {  // row -C0/2: average with the +C0/2 product
            const float2 h2 = cmulc(load_one(a + C0), load_one(bb + C0));
            h = make_float2(0.5f * (h.x + h2.x), 0.5f * (h.y + h2.y));
          }
          if (sizeof(E) != sizeof(float2)) h = cscale(h, us);  // undo the power-of-two scales (exact)
          v[i][r] = h;
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) v[i][r] = xc_product<C0>(a, bb, j + r * LR, k, half, us);
      }
      dft<R, 1>(v[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < K; i++) {
    const int bf = threadIdx.x + i * T;
    if ((NBF % T) == 0 || bf < NBF) {
      const int b = bf / LR, j = bf - b * LR;
#pragma unroll
      for (int r = 0; r < R; r++) sm[b * LD + pidx(j * R + r)] = v[i][r];
    }
  }
  __syncthreads();
  const int rows = J.rows;
  float2* out = Tw + (size_t)jl * rows * K4;
  fft_pass<C0, NBC, T, 1, R>(sm, tw);
  for (int e = threadIdx.x; e < rows * NBC; e += T) {
    const int a = e / NBC, c = e - a * NBC;
    const int y = a < mS ? a - mS + C0 : a - mS;
    out[(size_t)a * K4 + k0 + c] = sm[c * LD + pidx(y)];
  }
}

template <int C1, int XC_NBR>
__global__ void __launch_bounds__(xr_threads(C1, XC_NBR), xr_minb(xr_threads(C1, XC_NBR)))
    k_xc_rows(XcJobs J, int C0, int K4, int mS, float scale, const float2* __restrict__ Tw,
              const float* __restrict__ terms, float* __restrict__ out, const float2* __restrict__ tw) {
  constexpr int T = xr_threads(C1, XC_NBR);
  constexpr int LD = ld_of(C1);
  extern __shared__ float2 sm[];
  const int w = 2 * mS;
  const int rows = J.rows;  // w + 1 for the frame terms (rows and columns -mS..mS)
  const int jl = blockIdx.y;
  const int job = J.job0 + jl;
  const int arow0 = blockIdx.x * (2 * XC_NBR);
  const float2* src = Tw + (size_t)jl * rows * K4;
  block_fft_from<C1, XC_NBR, T, 1>(sm, tw, [&](int p, int i) {
    const int a0 = arow0 + 2 * p, a1 = a0 + 1;
    return packed_rows<C1>(a0 < rows ? src + (size_t)a0 * K4 : nullptr, a1 < rows ? src + (size_t)a1 * K4 : nullptr, i);
  });
  const size_t w2 = (size_t)w * w;
  const int cols = rows;  // the terms window is square, w + 1 wide
  for (int e = threadIdx.x; e < XC_NBR * 2 * cols; e += T) {
    const int q = e / cols, b = e - q * cols;
    const int p = q >> 1;
    const int a = arow0 + q;
    if (a >= rows) continue;
    const int x = b < mS ? b - mS + C1 : b - mS;
    const float2 yv = sm[p * LD + pidx(x)];
    const float v = ((q & 1) ? yv.y : yv.x) * scale;
    const size_t pix = (size_t)a * w + b;
    if (J.kind == 0) {
      // output slots: CorrTM [0,N), CorrBM [N,2N), DenomT [2N,3N), DenomB [3N,4N), maskProduct 4N
      const int t = job / J.N, n = job - t * J.N;
      const int main_slot = t == 0 ? J.N + n : (t == 1 ? 3 * J.N + n : 4 * J.N);
      if (a < w && b < w) out[(size_t)main_slot * w2 + pix] = v;
      if (t < 2 && a >= 1 && b >= 1) {
        const int refl_slot = t == 0 ? n : 2 * J.N + n;
        out[(size_t)refl_slot * w2 + (size_t)(w - a) * w + (w - b)] = v;
      }
    } else {
      const int I = J.kind == 1 ? J.pairs[2 * job] : job;
      const int Jj = J.kind == 1 ? J.pairs[2 * job + 1] : job;
      const int N = J.N;
      const float ctm = terms[(size_t)I * w2 + pix];
      const float cbm = terms[(size_t)(N + Jj) * w2 + pix];
      const float dt = terms[(size_t)(2 * N + I) * w2 + pix];
      const float db = terms[(size_t)(3 * N + Jj) * w2 + pix];
      const float mp = terms[(size_t)(4 * N) * w2 + pix];
      float den = sqrtf((db - cbm * (cbm / mp)) * (dt - ctm * (ctm / mp)));
      den = (den < 1.0f) ? 1.0f : den;  // np.clip(Denom, 1, inf); NaN stays NaN
      out[(size_t)job * w2 + pix] = (v - ctm * cbm / mp) / den;
    }
  }
}

template <int C0, typename E, int NBC>
static int launch_xc_cols_t(const XcJobs& J, int nj, int C1, int K4, int mS, float2* Tw, const float2* tw,
                            cudaStream_t st) {
  constexpr int T = xc_threads(C0, NBC);
  const size_t smem = (size_t)NBC * ld_of(C0) * sizeof(float2);
  ZR_TRY(cuda_check(cudaFuncSetAttribute(k_xc_cols<C0, E, NBC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem), "k_xc_cols attr"));
  k_xc_cols<C0, E, NBC><<<dim3(nj, K4 / NBC), T, smem, st>>>(J, C1, K4, mS, Tw, tw);
  return launched("k_xc_cols");
}

template <int C0, typename E>
static int launch_xc_cols_e(const XcJobs& J, int nj, int C1, int K4, int mS, float2* Tw, const float2* tw,
                            cudaStream_t st) {
  switch (tune_get(TUNE_XC_COLS, C0)) {
    case 1: return launch_xc_cols_t<C0, E, 1>(J, nj, C1, K4, mS, Tw, tw, st);
    case 2: return launch_xc_cols_t<C0, E, 2>(J, nj, C1, K4, mS, Tw, tw, st);
    case 4: return launch_xc_cols_t<C0, E, 4>(J, nj, C1, K4, mS, Tw, tw, st);
    default: return launch_xc_cols_t<C0, E, xc_nbc_default(C0)>(J, nj, C1, K4, mS, Tw, tw, st);
  }
}

template <int C0>
static int launch_xc_cols(const XcJobs& J, int nj, int C1, int K4, int mS, float2* Tw, const float2* tw,
                          cudaStream_t st) {
  if (J.sc) return launch_xc_cols_e<C0, __half2>(J, nj, C1, K4, mS, Tw, tw, st);
  return launch_xc_cols_e<C0, float2>(J, nj, C1, K4, mS, Tw, tw, st);
}

template <int C1, int NBR>
static int launch_xc_rows_v(const XcJobs& J, int nj, int C0, int K4, int mS, float scale, const float2* Tw,
                            const float* terms, float* out, const float2* tw, cudaStream_t st) {
  constexpr int T = xr_threads(C1, NBR);
  const size_t smem = (size_t)NBR * ld_of(C1) * sizeof(float2);
  ZR_TRY(cuda_check(cudaFuncSetAttribute(k_xc_rows<C1, NBR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "k_xc_rows attr"));
  k_xc_rows<C1, NBR><<<dim3((J.rows + 2 * NBR - 1) / (2 * NBR), nj), T, smem, st>>>(J, C0, K4, mS, scale, Tw,
                                                                                   terms, out, tw);
  return launched("k_xc_rows");
}

template <int C1>
static int launch_xc_rows(const XcJobs& J, int nj, int C0, int K4, int mS, float scale, const float2* Tw,
                          const float* terms, float* out, const float2* tw, cudaStream_t st) {
  switch (tune_get(TUNE_XC_ROWS, C1)) {
    case 1: return launch_xc_rows_v<C1, 1>(J, nj, C0, K4, mS, scale, Tw, terms, out, tw, st);
    case 4: return launch_xc_rows_v<C1, 4>(J, nj, C0, K4, mS, scale, Tw, terms, out, tw, st);
    default: return launch_xc_rows_v<C1, XC_NBR_DEFAULT>(J, nj, C0, K4, mS, scale, Tw, terms, out, tw, st);
  }
}

#define ZR_XC_DISPATCH(L, CALL)                               \
  switch (L) {                                                \
    case 64: { constexpr int LL = 64; CALL; } break;          \
    case 128: { constexpr int LL = 128; CALL; } break;        \
    case 256: { constexpr int LL = 256; CALL; } break;        \
    case 512: { constexpr int LL = 512; CALL; } break;        \
    case 384: { constexpr int LL = 384; CALL; } break;        \
    case 768: { constexpr int LL = 768; CALL; } break;        \
    case 1024: { constexpr int LL = 1024; CALL; } break;      \
    case 1536: { constexpr int LL = 1536; CALL; } break;      \
    case 2048: { constexpr int LL = 2048; CALL; } break;      \
    case 3072: { constexpr int LL = 3072; CALL; } break;      \
    case 4096: { constexpr int LL = 4096; CALL; } break;      \
    default: return set_error(ZR_ESIZE, "crop size %d not supported", (int)(L)); \
  }

static int run_jobs(XcJobs J, int njobs, int C0, int C1, int mS, const float* terms, float* out, void* work,
                    size_t work_bytes, cudaStream_t st) {
  const int K4 = zr_spectrum_pitch(C1);
  const size_t per_job = (size_t)J.rows * K4 * sizeof(float2);
  if (!work || work_bytes < per_job)
    return set_error(ZR_EWORK, "zr_xcorr: work buffer %zu bytes < %zu (one job)", work_bytes, per_job);
  const int wave = (int)((work_bytes / per_job) < (size_t)njobs ? work_bytes / per_job : (size_t)njobs);
  const float2* tw = twiddles();
  if (!tw) return ZR_ECUDA;
  // normConst2 (zorro.py:634, rounded to float32 as there); the reference's
  // inverse FFTs are FFTW executions without 1/N, and so is this one
  const float scale = (float)(1.0 / (((double)C0 * C1) * ((double)C0 * C1)));
  float2* Tw = (float2*)work;
  for (int j0 = 0; j0 < njobs; j0 += wave) {
    const int nj = (njobs - j0) < wave ? (njobs - j0) : wave;
    J.job0 = j0;
    ZR_XC_DISPATCH(C0, ZR_TRY((launch_xc_cols<LL>(J, nj, C1, K4, mS, Tw, tw, st))));
    ZR_XC_DISPATCH(C1, ZR_TRY((launch_xc_rows<LL>(J, nj, C0, K4, mS, scale, Tw, terms, out, tw, st))));
  }
  return ZR_OK;
}

static int check_sizes(int C0, int C1, int mS) {
  if (!fft_len_ok(C0) || !fft_len_ok(C1) || C0 < 64 || C1 < 64 || C0 > 4096 || C1 > 4096)
    return set_error(ZR_ESIZE, "crop %dx%d must be powers of two in [64, 4096] or 3 x 2^k in [384, 3072]", C0, C1);
  if (mS < 2 || 2 * mS > C0 || 2 * mS > C1)
    return set_error(ZR_ESIZE, "maxShift %d must satisfy 2 <= maxShift <= C/2", mS);
  return ZR_OK;
}

// triMode 'refine' (zorro.py:934-954): template I is conj(sum_n G_n - G_I)/N.
// One thread per spectrum element: the frame sum in frame order, then every
// frame's template.
__global__ void k_refine_spectra(const float2* __restrict__ G, int N, long long se, float2* __restrict__ T) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= se) return;
  float sx = 0.0f, sy = 0.0f;
  for (int n = 0; n < N; n++) {
    const float2 g = G[(size_t)n * se + e];
    sx += g.x;
    sy += g.y;
  }
  const float fn = (float)N;
  for (int n = 0; n < N; n++) {
    const float2 g = G[(size_t)n * se + e];
    T[(size_t)n * se + e] = make_float2((sx - g.x) / fn, (sy - g.y) / fn);
  }
}

// The template's frame terms are linear in its spectra: CorrTM and the raw
// DenomT of template I are (sum_n term_n - term_I) / N.  CorrBM, DenomB and
// the mask product are copied.
__global__ void k_refine_terms(const float* __restrict__ terms, int N, int w2, float* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= w2) return;
  const float fn = (float)N;
  for (int t = 0; t < 4; t += 2) {  // CorrTM (slots [0,N)) and DenomT (slots [2N,3N))
    const float* src = terms + (size_t)t * N * w2;
    float s = 0.0f;
    for (int n = 0; n < N; n++) s += src[(size_t)n * w2 + p];
    for (int n = 0; n < N; n++) out[((size_t)t * N + n) * w2 + p] = (s - src[(size_t)n * w2 + p]) / fn;
  }
  for (int n = 0; n < N; n++) {
    out[((size_t)N + n) * w2 + p] = terms[((size_t)N + n) * w2 + p];
    out[((size_t)3 * N + n) * w2 + p] = terms[((size_t)3 * N + n) * w2 + p];
  }
  out[(size_t)4 * N * w2 + p] = terms[(size_t)4 * N * w2 + p];
}

// Half-precision spectra: each spectrum is stored as __half2 times a power of
// two chosen from its largest component, max * scale < 2^15.
__global__ void k_spectrum_absmax(const float2* __restrict__ X, long long se, unsigned int* __restrict__ maxbits) {
  const float2* x = X + (size_t)blockIdx.y * se;
  float m = 0.0f;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < se; e += (long long)gridDim.x * blockDim.x) {
    const float2 v = x[e];
    m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxbits + blockIdx.y, __float_as_uint(m));  // m >= 0: bits order as values
}

__device__ __forceinline__ float half_scale(unsigned int bits) {
  const float m = __uint_as_float(bits);
  if (!(m > 0.0f) || isinf(m)) return 1.0f;
  int ex;
  frexpf(m, &ex);  // m < 2^ex
  return ldexpf(1.0f, 15 - ex);
}

__global__ void k_spectrum_to_half(const float2* __restrict__ X, long long se, const unsigned int* __restrict__ maxbits,
                                   __half2* __restrict__ Y, float* __restrict__ scales) {
  const int n = blockIdx.y;
  const float sc = half_scale(maxbits[n]);
  if (blockIdx.x == 0 && threadIdx.x == 0) scales[n] = sc;
  const float2* x = X + (size_t)n * se;
  __half2* y = Y + (size_t)n * se;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < se; e += (long long)gridDim.x * blockDim.x) {
    const float2 v = x[e];
    y[e] = __floats2half2_rn(v.x * sc, v.y * sc);
  }
}

}  // namespace zr

using namespace zr;

extern "C" int zr_pack_half(const void* spectra, int n_spectra, long long se, void* out, float* scales, void* work,
                            size_t work_bytes, void* stream) {
  if (!spectra || !out || !scales || !work || n_spectra <= 0 || se <= 0)
    return set_error(ZR_EINVAL, "zr_pack_half: bad argument");
  if (work_bytes < (size_t)n_spectra * sizeof(unsigned int))
    return set_error(ZR_EWORK, "zr_pack_half: work buffer %zu < %zu", work_bytes, (size_t)n_spectra * 4);
  cudaStream_t st = (cudaStream_t)stream;
  ZR_TRY(cuda_check(cudaMemsetAsync(work, 0, (size_t)n_spectra * sizeof(unsigned int), st), "zr_pack_half memset"));
  const int blocks = (int)((se + 255) / 256 < 304 ? (se + 255) / 256 : 304);
  k_spectrum_absmax<<<dim3(blocks, n_spectra), 256, 0, st>>>((const float2*)spectra, se, (unsigned int*)work);
  ZR_TRY(launched("k_spectrum_absmax"));
  k_spectrum_to_half<<<dim3(blocks, n_spectra), 256, 0, st>>>((const float2*)spectra, se, (const unsigned int*)work,
                                                               (__half2*)out, scales);
  return launched("k_spectrum_to_half");
}

extern "C" int zr_refine_spectra(const void* G, int N, int C0, int C1, void* templates, void* stream) {
  if (!G || !templates || N <= 0) return set_error(ZR_EINVAL, "zr_refine_spectra: null argument");
  const long long se = zr_spectrum_elems(C0, C1);
  k_refine_spectra<<<(unsigned)((se + 255) / 256), 256, 0, (cudaStream_t)stream>>>((const float2*)G, N, se,
                                                                                    (float2*)templates);
  return launched("k_refine_spectra");
}

extern "C" int zr_refine_terms(const float* terms, int N, int max_shift, float* out, void* stream) {
  if (!terms || !out || N <= 0 || max_shift <= 0) return set_error(ZR_EINVAL, "zr_refine_terms: bad argument");
  const int w2 = 4 * max_shift * max_shift;
  k_refine_terms<<<(w2 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(terms, N, w2, out);
  return launched("k_refine_terms");
}

extern "C" int zr_xcorr_refine(const void* G, const void* templates, const float* refine_terms, int N, int C0,
                               int C1, int max_shift, float* cwin, void* work, size_t work_bytes, void* stream) {
  if (!G || !templates || !refine_terms || !cwin || N <= 0) return set_error(ZR_EINVAL, "zr_xcorr_refine: null argument");
  if (N < 2) return ZR_OK;
  ZR_TRY(check_sizes(C0, C1, max_shift));
  XcJobs J{G, nullptr, nullptr, nullptr, templates, nullptr, N, 2, 0, zr_spectrum_elems(C0, C1), 2 * max_shift};
  return run_jobs(J, N - 1, C0, C1, max_shift, refine_terms, cwin, work, work_bytes, (cudaStream_t)stream);
}

extern "C" size_t zr_xcorr_work_bytes(int n_jobs, int C1, int max_shift) {
  return (size_t)n_jobs * (2 * max_shift + 1) * zr_spectrum_pitch(C1) * sizeof(float2);
}

extern "C" int zr_xcorr_terms(const void* G, const void* S, const void* GM, int N, int C0, int C1, int max_shift,
                              float* terms, void* work, size_t work_bytes, void* stream) {
  if (!G || !S || !GM || !terms || N <= 0) return set_error(ZR_EINVAL, "zr_xcorr_terms: null argument");
  ZR_TRY(check_sizes(C0, C1, max_shift));
  XcJobs J{G, S, GM, nullptr, nullptr, nullptr, N, 0, 0, zr_spectrum_elems(C0, C1), 2 * max_shift + 1};
  return run_jobs(J, 2 * N + 1, C0, C1, max_shift, nullptr, terms, work, work_bytes, (cudaStream_t)stream);
}

extern "C" int zr_xcorr_pairs(const void* G, const float* terms, const int* pairs, int M, int N, int C0, int C1,
                              int max_shift, float* cwin, void* work, size_t work_bytes, void* stream) {
  if (!G || !terms || !pairs || !cwin || N <= 0) return set_error(ZR_EINVAL, "zr_xcorr_pairs: null argument");
  if (M <= 0) return ZR_OK;
  ZR_TRY(check_sizes(C0, C1, max_shift));
  XcJobs J{G, nullptr, nullptr, pairs, nullptr, nullptr, N, 1, 0, zr_spectrum_elems(C0, C1), 2 * max_shift};
  return run_jobs(J, M, C0, C1, max_shift, terms, cwin, work, work_bytes, (cudaStream_t)stream);
}

extern "C" int zr_xcorr_terms_half(const void* G, const void* S, const void* GM, const float* scales, int N, int C0,
                                   int C1, int max_shift, float* terms, void* work, size_t work_bytes, void* stream) {
  if (!G || !S || !GM || !scales || !terms || N <= 0) return set_error(ZR_EINVAL, "zr_xcorr_terms_half: null argument");
  ZR_TRY(check_sizes(C0, C1, max_shift));
  XcJobs J{G, S, GM, nullptr, nullptr, scales, N, 0, 0, zr_spectrum_elems(C0, C1), 2 * max_shift + 1};
  return run_jobs(J, 2 * N + 1, C0, C1, max_shift, nullptr, terms, work, work_bytes, (cudaStream_t)stream);
}

extern "C" int zr_xcorr_pairs_half(const void* G, const float* scales, const float* terms, const int* pairs, int M,
                                   int N, int C0, int C1, int max_shift, float* cwin, void* work, size_t work_bytes,
                                   void* stream) {
  if (!G || !scales || !terms || !pairs || !cwin || N <= 0) return set_error(ZR_EINVAL, "zr_xcorr_pairs_half: null argument");
  if (M <= 0) return ZR_OK;
  ZR_TRY(check_sizes(C0, C1, max_shift));
  XcJobs J{G, nullptr, nullptr, pairs, nullptr, scales, N, 1, 0, zr_spectrum_elems(C0, C1), 2 * max_shift};
  return run_jobs(J, M, C0, C1, max_shift, terms, cwin, work, work_bytes, (cudaStream_t)stream);
}
