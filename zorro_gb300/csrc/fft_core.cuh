// Batched complex FFTs held in shared memory, for sm_103a.
//
// A CTA transforms NB sequences of length L (a power of two, 2..8192) that sit
// in shared memory.  Element i of sequence b lives at s[b*ld(L) + pidx(i)]:
// one padding slot every 8 elements keeps the radix-8 scatter of the first
// pass free of bank conflicts, and the row pitch (ld_of) keeps tiles of 4
// sequences x 4 elements conflict-free.  Each pass is a radix-8 (the last pass radix 2
// or 4 when log2(L) is not a multiple of 3) Stockham step: every thread reads
// its butterflies' inputs into registers, the CTA synchronises, and the
// outputs are written back in place.  No ping-pong buffer is needed.
//
// Twiddles come from a table of W_8192^k = exp(-2 pi i k / 8192) computed in
// double precision on the host and rounded to float (``tw`` argument).
// DIR = -1 is the forward transform, +1 the inverse; neither is normalised.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace zr {

constexpr int TWN = 8192;  // twiddle table length

__host__ __device__ __forceinline__ constexpr int pidx(int i) { return i + (i >> 3); }
// Row pitch of one sequence: the padded length rounded so that pitch = 4
// (mod 16) float2s; then 4 sequences x 4 consecutive elements (the tile the
// row/column passes move per half-warp) fall on 32 distinct banks.
__host__ __device__ __forceinline__ constexpr int ld_of(int L) {
  return (((L + (L >> 3)) + 15) & ~15) + 4;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// multiply by DIR*i
template <int DIR>
__device__ __forceinline__ float2 mul_si(float2 a) {
  return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int R, int DIR>
__device__ __forceinline__ void dft(float2* x);

template <>
__device__ __forceinline__ void dft<2, -1>(float2* x) {
  float2 a = x[0], b = x[1];
  x[0] = cadd(a, b); x[1] = csub(a, b);
}
template <>
__device__ __forceinline__ void dft<2, 1>(float2* x) {
  float2 a = x[0], b = x[1];
  x[0] = cadd(a, b); x[1] = csub(a, b);
}

template <int DIR>
__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3) {
  float2 t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), t3 = mul_si<DIR>(csub(x1, x3));
  x0 = cadd(t0, t2); x2 = csub(t0, t2); x1 = cadd(t1, t3); x3 = csub(t1, t3);
}
template <>
__device__ __forceinline__ void dft<4, -1>(float2* x) { dft4<-1>(x[0], x[1], x[2], x[3]); }
template <>
__device__ __forceinline__ void dft<4, 1>(float2* x) { dft4<1>(x[0], x[1], x[2], x[3]); }

template <int DIR>
__device__ __forceinline__ void dft8(float2* x) {
  const float h = 0.70710678118654752440f;
  float2 e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6];
  float2 o0 = x[1], o1 = x[3], o2 = x[5], o3 = x[7];
  dft4<DIR>(e0, e1, e2, e3);
  dft4<DIR>(o0, o1, o2, o3);
  // o_k *= W8^(DIR' k) with W8 = exp(DIR*i*pi/4)
  float2 w1 = make_float2(h * (o1.x - DIR * o1.y), h * (o1.y + DIR * o1.x));
  float2 w2 = mul_si<DIR>(o2);
  float2 w3 = make_float2(h * (-o3.x - DIR * o3.y), h * (-o3.y + DIR * o3.x));
  x[0] = cadd(e0, o0); x[4] = csub(e0, o0);
  x[1] = cadd(e1, w1); x[5] = csub(e1, w1);
  x[2] = cadd(e2, w2); x[6] = csub(e2, w2);
  x[3] = cadd(e3, w3); x[7] = csub(e3, w3);
}
template <>
__device__ __forceinline__ void dft<8, -1>(float2* x) { dft8<-1>(x); }
template <>
__device__ __forceinline__ void dft<8, 1>(float2* x) { dft8<1>(x); }

// One Stockham pass (radix R, NS = product of the radices already applied),
// then the remaining passes.
template <int L, int NB, int T, int DIR, int NS>
__device__ __forceinline__ void fft_pass(float2* s, const float2* __restrict__ tw) {
  constexpr int R = (L / NS >= 8) ? 8 : (L / NS);
  constexpr int LR = L / R;
  constexpr int NBF = NB * LR;
  constexpr int K = (NBF + T - 1) / T;
  constexpr int LD = ld_of(L);
  constexpr int TWS = TWN / (NS * R);
  float2 v[K][R];
#pragma unroll
  for (int i = 0; i < K; i++) {
    const int bf = threadIdx.x + i * T;
    if ((NBF % T) == 0 || bf < NBF) {
      const int b = bf / LR, j = bf - (bf / LR) * LR;
      const float2* src = s + b * LD;
      const int k = j & (NS - 1);
#pragma unroll
      for (int r = 0; r < R; r++) v[i][r] = src[pidx(j + r * LR)];
      if (NS > 1) {
        // W^(k r) for r = 1 .. R-1: the powers 1, 2, 4 from the table, the
        // others as products of two of them (one extra rounding), which
        // keeps the load/store pipe for the data
        float2 w[R];
        w[1] = __ldg(tw + k * TWS);
        if constexpr (R >= 4) {
          w[2] = __ldg(tw + 2 * k * TWS);
          w[3] = cmul(w[1], w[2]);
        }
        if constexpr (R == 8) {
          w[4] = __ldg(tw + 4 * k * TWS);
          w[5] = cmul(w[1], w[4]);
          w[6] = cmul(w[2], w[4]);
          w[7] = cmul(w[3], w[4]);
        }
#pragma unroll
        for (int r = 1; r < R; r++) {
          float2 ww = w[r];
          if (DIR > 0) ww.y = -ww.y;
          v[i][r] = cmul(v[i][r], ww);
        }
      }
      dft<R, DIR>(v[i]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < K; i++) {
    const int bf = threadIdx.x + i * T;
    if ((NBF % T) == 0 || bf < NBF) {
      const int b = bf / LR, j = bf - (bf / LR) * LR;
      float2* dst = s + b * LD;
      const int k = j & (NS - 1);
      const int base = (j / NS) * NS * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) dst[pidx(base + r * NS)] = v[i][r];
    }
  }
  __syncthreads();
  if constexpr (NS * R < L) fft_pass<L, NB, T, DIR, NS * R>(s, tw);
}

// Transform NB sequences of length L in shared memory (natural order in and
// out).  Must be called by all T threads of the CTA; the caller synchronises
// before (after filling ``s``); the function ends with a barrier.
template <int L, int NB, int T, int DIR>
__device__ __forceinline__ void block_fft(float2* s, const float2* __restrict__ tw) {
  static_assert((L & (L - 1)) == 0 && L >= 2 && L <= TWN, "L must be a power of two <= 8192");
  fft_pass<L, NB, T, DIR, 1>(s, tw);
}

}  // namespace zr
