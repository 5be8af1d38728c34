// Batched complex FFTs held in shared memory, for sm_103a.
//
// A CTA transforms NB sequences of length L (L = 2^a 3^b 5^c dividing TWN,
// e.g. 64..16384, 3 x 2^k and 9 x 2^k) that sit in shared memory.  Element i of sequence b lives at s[b*ld(L) + pidx(i)]:
// one padding slot every 16 elements keeps the radix-16 scatter of the first
// pass free of bank conflicts, and the row pitch (ld_of) keeps tiles of 4
// sequences x 4 elements conflict-free.  Each pass is a radix-16 Stockham
// step (the last pass radix 2, 4 or 8 when log2(L) is not a multiple of 4):
// every thread reads its butterflies' inputs into registers, the CTA
// synchronises, and the outputs are written back in place.  No ping-pong
// buffer is needed.  Lengths with a factor 3 or 5 end with radix-3 / radix-5
// passes.
//
// Twiddles come from a table of W_TWN^k = exp(-2 pi i k / TWN), TWN = 2^14 x
// 3^2 x 5, computed in double precision on the host and rounded to float
// (``tw`` argument); a length-L transform reads every (TWN/L)-th entry, or
// the same values from a contiguous copy for its length (TW_COMPACT below).
// DIR = -1 is the forward transform, +1 the inverse; neither is normalised.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace zr {

constexpr int TWN = 737280;  // twiddle table length: 2^14 * 3^2 * 5

// After the TWN entries the table holds contiguous copies of it for the
// sub-transform lengths M that the passes twiddle with: W_M^j (j < M) at
// tw[TWN + tw_compact_off(M) + j], the same value as tw[j * (TWN / M)], for
// M a power of two up to 16384 (offset M) and M = 3 * 2^a up to 12288
// (offset 32768 + M).  A pass's twiddles W_M^(r k) for the consecutive k of
// a warp's lanes then come from a few consecutive cache lines instead of one
// line per lane of the strided table (a 4096-point pass would otherwise
// touch about 1500 lines, more than the L1 left beside the shared memory).
constexpr int TW_COMPACT = 32768 + 2 * 12288;
__host__ __device__ constexpr bool tw_is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
__host__ __device__ constexpr int tw_compact_off(int M) {
  return (tw_is_pow2(M) && M <= 16384) ? M
                                       : ((M % 3 == 0 && tw_is_pow2(M / 3) && M <= 12288) ? 32768 + M : -1);
}

__host__ __device__ __forceinline__ constexpr int pidx(int i) { return i + (i >> 4); }
// Row pitch of one sequence: the padded length rounded so that pitch = 4
// (mod 16) float2s; then 4 sequences x 4 consecutive elements (the tile the
// row/column passes move per half-warp) fall on 32 distinct banks.
__host__ __device__ __forceinline__ constexpr int ld_of(int L) {
  return (((L + (L >> 4)) + 15) & ~15) + 4;
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

// 16-point DFT as 4 x 4: length-4 DFTs over n1 (n = 4 n1 + n2), the twiddles
// W16^(n2 k1), length-4 DFTs over n2; output k = k1 + 4 k2.
template <int DIR>
__device__ __forceinline__ void dft16(float2* x) {
  const float c1 = 0.92387953251128675613f;  // cos(pi/8)
  const float s1 = 0.38268343236508977173f;  // sin(pi/8)
  const float h = 0.70710678118654752440f;
#pragma unroll
  for (int n2 = 0; n2 < 4; n2++) dft4<DIR>(x[n2], x[4 + n2], x[8 + n2], x[12 + n2]);
  // x[4 k1 + n2] now holds Y_{n2}[k1]; multiply by W16^(DIR' n2 k1), where
  // W16^m = exp(DIR * 2 pi i m / 16)
  auto tw = [&](float2 v, float cr, float si) {  // v * (cr + DIR*i*si)
    return make_float2(v.x * cr - DIR * v.y * si, v.y * cr + DIR * v.x * si);
  };
  x[5] = tw(x[5], c1, s1);     // m = 1
  x[6] = tw(x[6], h, h);       // m = 2
  x[7] = tw(x[7], s1, c1);     // m = 3
  x[9] = tw(x[9], h, h);       // m = 2
  x[10] = mul_si<DIR>(x[10]);  // m = 4
  x[11] = tw(x[11], -h, h);    // m = 6
  x[13] = tw(x[13], s1, c1);   // m = 3
  x[14] = tw(x[14], -h, h);    // m = 6
  x[15] = tw(x[15], -c1, -s1); // m = 9
  float2 y[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    float2 a = x[4 * k1], b = x[4 * k1 + 1], c = x[4 * k1 + 2], d = x[4 * k1 + 3];
    dft4<DIR>(a, b, c, d);
    y[k1] = a; y[k1 + 4] = b; y[k1 + 8] = c; y[k1 + 12] = d;
  }
#pragma unroll
  for (int k = 0; k < 16; k++) x[k] = y[k];
}
template <>
__device__ __forceinline__ void dft<16, -1>(float2* x) { dft16<-1>(x); }
template <>
__device__ __forceinline__ void dft<16, 1>(float2* x) { dft16<1>(x); }

// 3-point DFT: X1,2 = a - (b + c)/2 +/- DIR i sin(2 pi/3) (b - c)
template <int DIR>
__device__ __forceinline__ void dft3(float2* x) {
  const float s = 0.86602540378443864676f;
  const float2 a = x[0], b = x[1], c = x[2];
  const float2 bc = cadd(b, c);
  const float2 t = make_float2(a.x - 0.5f * bc.x, a.y - 0.5f * bc.y);
  const float2 d = csub(b, c);
  const float2 u = mul_si<DIR>(make_float2(s * d.x, s * d.y));
  x[0] = cadd(a, bc);
  x[1] = cadd(t, u);
  x[2] = csub(t, u);
}
template <>
__device__ __forceinline__ void dft<3, -1>(float2* x) { dft3<-1>(x); }
template <>
__device__ __forceinline__ void dft<3, 1>(float2* x) { dft3<1>(x); }

// 5-point DFT with the pairs (1,4) and (2,3): cos/sin of 2 pi/5 and 4 pi/5
template <int DIR>
__device__ __forceinline__ void dft5(float2* x) {
  const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
  const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
  const float2 b1 = cadd(x[1], x[4]), b2 = cadd(x[2], x[3]);
  const float2 d1 = csub(x[1], x[4]), d2 = csub(x[2], x[3]);
  const float2 a = x[0];
  const float2 t1 = make_float2(a.x + c1 * b1.x + c2 * b2.x, a.y + c1 * b1.y + c2 * b2.y);
  const float2 t2 = make_float2(a.x + c2 * b1.x + c1 * b2.x, a.y + c2 * b1.y + c1 * b2.y);
  const float2 u1 = mul_si<DIR>(make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y));
  const float2 u2 = mul_si<DIR>(make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y));
  x[0] = make_float2(a.x + b1.x + b2.x, a.y + b1.y + b2.y);
  x[1] = cadd(t1, u1);
  x[4] = csub(t1, u1);
  x[2] = cadd(t2, u2);
  x[3] = csub(t2, u2);
}
template <>
__device__ __forceinline__ void dft<5, -1>(float2* x) { dft5<-1>(x); }
template <>
__device__ __forceinline__ void dft<5, 1>(float2* x) { dft5<1>(x); }

// Radix of the pass that starts after NS: 16 while it divides what is left,
// then 8, 4, 2, then the odd factors 3 and 5.
constexpr int fft_radix(int rem) {
  return rem % 16 == 0 ? 16 : (rem % 8 == 0 ? 8 : (rem % 4 == 0 ? 4 : (rem % 2 == 0 ? 2 : (rem % 3 == 0 ? 3 : 5))));
}

// v[r] *= W^(k r) for r = 1 .. R-1 (W = exp(DIR 2 pi i / (TWN / TWS))): a
// few powers from the table, the others as products of two table values (one
// extra rounding), which keeps the load/store pipe for the data.
template <int R, int DIR, int TWS>
__device__ __forceinline__ void apply_twiddles(float2* v, int k, const float2* __restrict__ twtab) {
  auto twiddle = [&](int r, float2 ww) {
    if (DIR > 0) ww.y = -ww.y;
    v[r] = cmul(v[r], ww);
  };
  // W_M^(r k), M = TWN / TWS: from the contiguous copy when there is one
  constexpr int OFF = tw_compact_off(TWN / TWS);
  const float2* __restrict__ tw = OFF >= 0 ? twtab + TWN + OFF : twtab;
  constexpr int ST = OFF >= 0 ? 1 : TWS;
  const float2 w1 = __ldg(tw + k * ST);
  if constexpr (R == 2) {
    twiddle(1, w1);
  } else if constexpr (R == 3 || R == 5) {
    twiddle(1, w1);
#pragma unroll
    for (int r = 2; r < R; r++) twiddle(r, __ldg(tw + r * k * ST));
  } else {
    const float2 w2 = __ldg(tw + 2 * k * ST);
    const float2 w3 = (R == 16) ? __ldg(tw + 3 * k * ST) : cmul(w1, w2);
    twiddle(1, w1);
    twiddle(2, w2);
    twiddle(3, w3);
#pragma unroll
    for (int a = 4; a < R; a += 4) {
      const float2 wa = __ldg(tw + a * k * ST);
      twiddle(a, wa);
      twiddle(a + 1, cmul(R == 16 ? wa : w1, R == 16 ? w1 : wa));
      twiddle(a + 2, cmul(w2, wa));
      twiddle(a + 3, cmul(w3, wa));
    }
  }
}

// Where the last pass puts its outputs: by default back in shared memory
// (natural order).  An output functor ``out`` instead receives them in
// registers: ``out.need(b, k)`` says whether any output k + r L/R (r < R) of
// sequence b is kept (the butterflies of the others are skipped) and
// ``out(b, i, r, v)`` is called for every output i = k + r L/R of a needed
// butterfly, so the kept elements go straight to global memory (or into the
// caller's registers) without another store, barrier and load in shared
// memory.
struct SmemOut {};

// An output functor that keeps every butterfly, around a callable f(b, i, r, v).
template <typename F>
struct AllOut {
  F f;
  __device__ __forceinline__ bool need(int, int) const { return true; }
  __device__ __forceinline__ void operator()(int b, int i, int r, float2 v) const { f(b, i, r, v); }
};
template <typename F>
__device__ __forceinline__ AllOut<F> all_out(F f) { return AllOut<F>{f}; }

// Radix of the last pass of a length-L transform.
constexpr int last_radix(int L) {
  int rem = L;
  int r = fft_radix(rem);
  while (rem > r) {
    rem /= r;
    r = fft_radix(rem);
  }
  return r;
}

// One Stockham pass (radix R, NS = product of the radices already applied),
// then the remaining passes up to the one that would start at NS = STOP
// (STOP = L: all of them).
template <int L, int NB, int T, int DIR, int NS, typename Out = SmemOut, int STOP = L>
__device__ __forceinline__ void fft_pass(float2* s, const float2* __restrict__ tw, const Out& out = Out()) {
  constexpr int R = fft_radix(L / NS);
  constexpr int LR = L / R;
  constexpr int NBF = NB * LR;
  constexpr int K = (NBF + T - 1) / T;
  constexpr int LD = ld_of(L);
  constexpr int TWS = TWN / (NS * R);
  constexpr bool DIRECT = NS * R == L && !std::is_same<Out, SmemOut>::value;
  float2 v[K][R];
#pragma unroll
  for (int i = 0; i < K; i++) {
    const int bf = threadIdx.x + i * T;
    if ((NBF % T) == 0 || bf < NBF) {
      const int b = bf / LR, j = bf - (bf / LR) * LR;
      if constexpr (DIRECT) {
        if (!out.need(b, j)) continue;
      }
      const float2* src = s + b * LD;
      const int k = j % NS;
#pragma unroll
      for (int r = 0; r < R; r++) v[i][r] = src[pidx(j + r * LR)];
      if (NS > 1) apply_twiddles<R, DIR, TWS>(v[i], k, tw);
      dft<R, DIR>(v[i]);
    }
  }
  if constexpr (DIRECT) {
    // last pass: j < NS, so output r of butterfly j is element j + r NS
#pragma unroll
    for (int i = 0; i < K; i++) {
      const int bf = threadIdx.x + i * T;
      if ((NBF % T) == 0 || bf < NBF) {
        const int b = bf / LR, j = bf - (bf / LR) * LR;
        if (!out.need(b, j)) continue;
#pragma unroll
        for (int r = 0; r < R; r++) out(b, j + r * NS, r, v[i][r]);
      }
    }
  } else {
    __syncthreads();
#pragma unroll
    for (int i = 0; i < K; i++) {
      const int bf = threadIdx.x + i * T;
      if ((NBF % T) == 0 || bf < NBF) {
        const int b = bf / LR, j = bf - (bf / LR) * LR;
        float2* dst = s + b * LD;
        const int k = j % NS;
        const int base = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) dst[pidx(base + r * NS)] = v[i][r];
      }
    }
    __syncthreads();
    if constexpr (NS * R < L && NS * R < STOP) fft_pass<L, NB, T, DIR, NS * R, Out, STOP>(s, tw, out);
  }
}

// block_fft of NB sequences whose elements come from ``load(b, i)`` (element
// i of sequence b) instead of shared memory: the first pass reads its
// butterflies straight from the loader, all of a thread's loads before any
// arithmetic, and writes its outputs to ``s``; the other passes run in shared
// memory.  Saves one store and one load of every element in shared memory.
template <int L, int NB, int T, int DIR, int STOP = L, typename Load, typename Out = SmemOut>
__device__ __forceinline__ void block_fft_from(float2* s, const float2* __restrict__ tw, Load load,
                                               const Out& out = Out()) {
  static_assert(L >= 2 && TWN % L == 0, "L must divide the twiddle table length 2^14 * 3^2 * 5");
  constexpr int R = fft_radix(L);
  constexpr int LR = L / R;
  constexpr int NBF = NB * LR;
  constexpr int K = (NBF + T - 1) / T;
  constexpr int LD = ld_of(L);
  float2 v[K][R];
#pragma unroll
  for (int i = 0; i < K; i++) {
    const int bf = threadIdx.x + i * T;
    if ((NBF % T) == 0 || bf < NBF) {
      const int b = bf / LR, j = bf - (bf / LR) * LR;
#pragma unroll
      for (int r = 0; r < R; r++) v[i][r] = load(b, j + r * LR);
    }
  }
#pragma unroll
  for (int i = 0; i < K; i++) {
    const int bf = threadIdx.x + i * T;
    if ((NBF % T) == 0 || bf < NBF) {
      const int b = bf / LR, j = bf - (bf / LR) * LR;
      dft<R, DIR>(v[i]);
#pragma unroll
      for (int r = 0; r < R; r++) s[b * LD + pidx(j * R + r)] = v[i][r];
    }
  }
  __syncthreads();
  if constexpr (R < L && R < STOP) fft_pass<L, NB, T, DIR, R, Out, STOP>(s, tw, out);
}

// The last pass of a length-L transform (radix R = last_radix(L), NS = L/R,
// after every other pass has run in shared memory) with the butterflies k
// and NS - k of one sequence in the same thread (k = 0 with NS/2), so that
// each output X[m] meets X[L - m] in registers: output r of butterfly k is
// X[k + r NS], and X[L - k - r NS] is output R-1-r of butterfly NS - k (for
// k = 0: output (R - r) mod R of butterfly 0).  For every unit (sequence b,
// k) ``pair(b, k0, X0, k1, X1)`` receives the two butterflies' outputs.
template <int L, int NB, int T, int DIR, typename Pair>
__device__ __forceinline__ void fft_last_paired(const float2* s, const float2* __restrict__ tw, Pair pair) {
  constexpr int R = last_radix(L);
  constexpr int NS = L / R;
  constexpr int LD = ld_of(L);
  constexpr int TWS = TWN / L;
  constexpr int NU = NB * (NS / 2);
  static_assert(NS % 2 == 0, "paired last pass needs an even number of butterflies");
  for (int t = threadIdx.x; t < NU; t += T) {
    const int u = t / NB, b = t - (t / NB) * NB;  // neighbouring threads: the same k of the next sequence
    const int k0 = u, k1 = u == 0 ? NS / 2 : NS - u;
    const float2* src = s + b * LD;
    float2 x0[R], x1[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      x0[r] = src[pidx(k0 + r * NS)];
      x1[r] = src[pidx(k1 + r * NS)];
    }
    if (NS > 1) {
      apply_twiddles<R, DIR, TWS>(x0, k0, tw);
      apply_twiddles<R, DIR, TWS>(x1, k1, tw);
    }
    dft<R, DIR>(x0);
    dft<R, DIR>(x1);
    pair(b, k0, x0, k1, x1);
  }
}

// Transform NB sequences of length L in shared memory (natural order in and
// out).  Must be called by all T threads of the CTA; the caller synchronises
// before (after filling ``s``); the function ends with a barrier.
template <int L, int NB, int T, int DIR>
__device__ __forceinline__ void block_fft(float2* s, const float2* __restrict__ tw) {
  static_assert(L >= 2 && TWN % L == 0, "L must divide the twiddle table length 2^14 * 3^2 * 5");
  fft_pass<L, NB, T, DIR, 1>(s, tw);
}

}  // namespace zr
