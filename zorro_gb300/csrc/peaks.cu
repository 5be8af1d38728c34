// Peak search on the correlation windows (locatePeak, zorro.py:1099-1231).
//
// One CTA per pair keeps the w x w window in shared memory and runs, with all
// threads in lock step:
//   * suppressOrigin (zorro.py:1078-1083, literal stencil);
//   * Bmode 'opti': a bounded Brent minimisation over sigma in [0, 7] of
//     std(G_sigma*C) / (max - mean) (zorro.py:1108-1121).  The minimiser is
//     Brent's golden-section/parabolic method as published by Forsythe,
//     Malcolm and Moler (FMIN, 1977), the method behind scipy's
//     minimize_scalar(method='bounded'); each function value is a full
//     separable Gaussian filter of the window with 'reflect' borders and
//     radius int(4 sigma + 0.5), the filter scipy.ndimage.gaussian_filter
//     applies (axis 0, then axis 1);
//   * the maxShift circular mask, the argmax (first index on ties) and the
//     peak significance (zorro.py:1165-1168);
//   * the sub-pixel step: the 16 x 16 patch around the peak, its DFT,
//     zero-padded to 16*subPixReg and inverted, |.| and its argmax
//     (zorro.py:1180-1216), or the integer fallback at the window edge.
// Filtered values are recomputed on the fly in blocks of rows, so the CTA
// needs only the window and one row block of shared memory.
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace zr {

// Threads of a peak-search CTA, and rows per thread of the vectorised filter
// pass (register blocking of its vertical taps: the R rows of a thread share
// each 16-byte row load).
#ifndef ZR_PK_T
#define ZR_PK_T 1024
#endif
#ifndef ZR_PK_VR
#define ZR_PK_VR 2
#endif

constexpr int PK_T = ZR_PK_T;
constexpr int PK_NW = PK_T / 32;  // warps
constexpr int PK_RB = PK_T / 64;  // rows per block of the scalar filter pass
constexpr int PK_MAXR = 64;    // largest filter radius
constexpr int PK_SUBR = 8;     // +/- patch half-size (zorro.py:619)

// The bounded Brent search's state.  It lives in shared memory and only
// thread 0 touches it, so none of it stays in registers across the filter
// passes of the other threads.
struct BrentState {
  double a, b, fulc, nfc, xf, rat, e, x, fx, ffulc, fnfc, xm, tol1, tol2;
  int num;
};

struct PkShared {
  double gw[2 * PK_MAXR + 1];
  alignas(16) float wy[2 * PK_MAXR + 4];  // 16-byte aligned: read four taps at a time
  alignas(16) float wx[2 * PK_MAXR + 4];
  double red[PK_NW][3];
  float redf[PK_NW];
  int redi[PK_NW];
  float ws1[PK_NW], ws2[PK_NW], wmx[PK_NW];  // per-warp partials of the filter statistics
  int wcnt[PK_NW];
  double bc[4];
  int bi[2];
  double st_s1, st_s2;  // block totals of the filter statistics
  float st_mx;
  int st_n;
  double x;             // the Brent search's next abscissa (thread 0 -> all)
  int go;               // 1 while the search continues
  BrentState bs;        // the search's state (thread 0 only)
};

__device__ __forceinline__ int reflect_idx(int i, int n) {
  while (i < 0 || i >= n) {
    if (i < 0) i = -i - 1;
    if (i >= n) i = 2 * n - i - 1;
  }
  return i;
}

// Gaussian weights exp(-0.5 k^2 / sigma^2), normalised (double, then float).
// Every thread computes some of the exponentials; thread 0 sums them in
// order.  All threads must call (with the same sigma).
__device__ int gauss_weights(double sigma, float* w, PkShared& sh) {
  if (!(sigma > 1e-15)) {
    if (threadIdx.x == 0) w[0] = 1.0f;
    return 0;
  }
  int r = (int)(4.0 * sigma + 0.5);
  if (r > PK_MAXR) r = PK_MAXR;
  const double c = -0.5 / (sigma * sigma);
  __syncthreads();  // a previous call may still be reading sh.gw
  for (int i = threadIdx.x; i <= 2 * r; i += blockDim.x) {
    const int k = i - r;
    sh.gw[i] = exp(c * (double)k * (double)k);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i <= 2 * r; i++) s += sh.gw[i];
    sh.bc[0] = s;
  }
  __syncthreads();
  const double s = sh.bc[0];
  for (int i = threadIdx.x; i <= 2 * r; i += blockDim.x) w[i] = (float)(sh.gw[i] / s);
  return r;
}

// Block reductions (all threads must call).
__device__ double3 block_sum3(PkShared& sh, double a, double b, double c) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sh.red[wid][0] = a; sh.red[wid][1] = b; sh.red[wid][2] = c; }
  __syncthreads();
  if (wid == 0) {
    a = lane < PK_NW ? sh.red[lane][0] : 0.0;
    b = lane < PK_NW ? sh.red[lane][1] : 0.0;
    c = lane < PK_NW ? sh.red[lane][2] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (lane == 0) { sh.bc[0] = a; sh.bc[1] = b; sh.bc[2] = c; }
  }
  __syncthreads();
  double3 r = make_double3(sh.bc[0], sh.bc[1], sh.bc[2]);
  __syncthreads();
  return r;
}

// max value with the smallest index among equal values
__device__ void block_argmax(PkShared& sh, float& v, int& idx) {
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_down_sync(0xffffffffu, v, o);
    const int oi = __shfl_down_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sh.redf[wid] = v; sh.redi[wid] = idx; }
  __syncthreads();
  if (wid == 0) {
    v = lane < PK_NW ? sh.redf[lane] : -INFINITY;
    idx = lane < PK_NW ? sh.redi[lane] : 0x7fffffff;
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_down_sync(0xffffffffu, v, o);
      const int oi = __shfl_down_sync(0xffffffffu, idx, o);
      if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    if (lane == 0) { sh.bc[3] = v; sh.bi[0] = idx; }
  }
  __syncthreads();
  v = (float)sh.bc[3];
  idx = sh.bi[0];
  __syncthreads();
}

struct FiltStats {
  double s1, s2;   // sum (f - c), sum (f - c)^2
  float mx;        // max f
  int n;
};

// Block totals of the per-thread filter statistics: float sums within each
// warp (a shuffle tree), the warps' partials summed in double by warp 0 in a
// fixed order; the count exactly, the maximum.  All threads must call; every
// thread receives the totals.  (The float64 pipe only sees one warp's worth
// of additions.)
__device__ void block_stats(PkShared& sh, float s1, float s2, int cnt, float mx, FiltStats& st) {
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
    cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sh.ws1[wid] = s1; sh.ws2[wid] = s2; sh.wcnt[wid] = cnt; sh.wmx[wid] = mx; }
  __syncthreads();
  if (wid == 0) {
    double a = lane < PK_NW ? (double)sh.ws1[lane] : 0.0;
    double b = lane < PK_NW ? (double)sh.ws2[lane] : 0.0;
    int n = lane < PK_NW ? sh.wcnt[lane] : 0;
    float m = lane < PK_NW ? sh.wmx[lane] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      n += __shfl_down_sync(0xffffffffu, n, o);
      m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    }
    if (lane == 0) { sh.st_s1 = a; sh.st_s2 = b; sh.st_n = n; sh.st_mx = m; }
  }
  __syncthreads();
  st.s1 = sh.st_s1;
  st.s2 = sh.st_s2;
  st.n = sh.st_n;
  st.mx = sh.st_mx;
  __syncthreads();  // the totals are read before any later call writes them
}

constexpr int PK_TX = 64;            // column lanes of the filter passes
constexpr int PK_TY = PK_T / PK_TX;  // rows per block (== PK_RB)
static_assert(PK_TY == PK_RB, "row block must match the thread layout");

// Visit every filtered value of the window.  MODE 0: statistics of all
// values.  MODE 1: masked statistics plus argmax of (mask ? f : 0).  rtab[i +
// PK_MAXR] is the 'reflect' index of i for i in [-PK_MAXR, w + PK_MAXR).
template <int MODE>
__device__ void filter_pass(const float* C, float* V, const int* rtab, int w, int mS, int ry, int rx,
                            const float* wy, const float* wx, float c, PkShared& sh, bool use_mask, FiltStats& st,
                            float& amax, int& aidx) {
  const int tx = threadIdx.x & (PK_TX - 1), ty = threadIdx.x / PK_TX;
  float s1 = 0.0f, s2 = 0.0f, mx = -INFINITY;
  float bv = -INFINITY;
  int bi = 0x7fffffff;
  int cnt = 0;
  for (int y0 = 0; y0 < w; y0 += PK_RB) {
    const int y = y0 + ty;
    if (y < w) {
      for (int x = tx; x < w; x += PK_TX) {
        float acc = 0.0f;
        if (ry == 0) {
          acc = C[y * w + x];
        } else if (y >= ry && y + ry < w) {
          const float* p = C + (y - ry) * w + x;
          for (int k = 0; k <= 2 * ry; k++) acc = fmaf(wy[k], p[k * w], acc);
        } else {
          const int* rt = rtab + PK_MAXR + y - ry;
          for (int k = 0; k <= 2 * ry; k++) acc = fmaf(wy[k], C[rt[k] * w + x], acc);
        }
        V[ty * w + x] = acc;
      }
    }
    __syncthreads();
    if (y < w) {
      const float* vr = V + ty * w;
      for (int x = tx; x < w; x += PK_TX) {
        float f = 0.0f;
        if (rx == 0) {
          f = vr[x];
        } else if (x >= rx && x + rx < w) {
          const float* p = vr + x - rx;
          for (int k = 0; k <= 2 * rx; k++) f = fmaf(wx[k], p[k], f);
        } else {
          const int* rt = rtab + PK_MAXR + x - rx;
          for (int k = 0; k <= 2 * rx; k++) f = fmaf(wx[k], vr[rt[k]], f);
        }
        bool in = true;
        if (MODE == 1) {
          const int dy = y - mS, dx = x - mS;
          in = !use_mask || (dy * dy + dx * dx < mS * mS);
          const float mv = in ? f : 0.0f;
          const int idx = y * w + x;
          if (mv > bv || (mv == bv && idx < bi)) { bv = mv; bi = idx; }
        }
        if (in) {
          const float d = f - c;
          s1 += d;
          s2 = fmaf(d, d, s2);
          mx = fmaxf(mx, f);
          cnt++;
        }
      }
    }
    __syncthreads();
  }
  block_stats(sh, s1, s2, cnt, mx, st);
  if (MODE == 1) {
    block_argmax(sh, bv, bi);
    amax = bv;
    aidx = bi;
  }
}

// The same visit for w % 4 == 0 with the work vectorised: each thread
// filters 4 consecutive columns; the vertical taps are float4 loads, the
// horizontal taps slide a 4-wide register window one column at a time.
// Rows per thread of the vectorised filter pass (register blocking of the
// vertical pass): 2 by default, which keeps a thread within the 64
// registers of a 1024-thread CTA.  The thread layout fixes the order in
// which the filter statistics are summed, so it is part of the results.
__host__ __device__ constexpr int pk_vec_rows(int) { return ZR_PK_VR; }
__host__ __device__ constexpr int pk_vec_pitch(int w) { return w + 8; }

// Horizontal pass of one row for 4 consecutive outputs x0..x0+3 away from
// the borders: 16-byte loads of the row (p = row + x0 - rx - OFF is 16-byte
// aligned), taps in order, the same fused multiply-adds as the scalar form.
// Taps k0..k0+3 of the four outputs from the 12 values s = (A, B, Cn) that
// start at tap k0's first input, weights W = wx[k0..k0+3].
template <int OFF>
__device__ __forceinline__ void taps4(const float4& A, const float4& B, const float4& Cn, const float4& W, float& f0,
                                      float& f1, float& f2, float& f3) {
  const float sv[12] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w, Cn.x, Cn.y, Cn.z, Cn.w};
  const float wv[4] = {W.x, W.y, W.z, W.w};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    f0 = fmaf(wv[q], sv[OFF + q], f0);
    f1 = fmaf(wv[q], sv[OFF + q + 1], f1);
    f2 = fmaf(wv[q], sv[OFF + q + 2], f2);
    f3 = fmaf(wv[q], sv[OFF + q + 3], f3);
  }
}

template <int OFF>
__device__ __forceinline__ void hrow4(const float* __restrict__ p, const float* __restrict__ wx, int rx, float& f0,
                                      float& f1, float& f2, float& f3) {
  const int K = 2 * rx;  // last tap
  float4 A = *reinterpret_cast<const float4*>(p), B = *reinterpret_cast<const float4*>(p + 4);
  int k0 = 0;
  // eight taps a step while they are all there: no per-tap tests, the weights
  // four at a time, the row chunks renamed rather than moved
  for (; k0 + 7 <= K; k0 += 8) {
    const float4 Cn = *reinterpret_cast<const float4*>(p + k0 + 8);
    taps4<OFF>(A, B, Cn, *reinterpret_cast<const float4*>(wx + k0), f0, f1, f2, f3);
    const float4 Dn = *reinterpret_cast<const float4*>(p + k0 + 12);
    taps4<OFF>(B, Cn, Dn, *reinterpret_cast<const float4*>(wx + k0 + 4), f0, f1, f2, f3);
    A = Cn;
    B = Dn;
  }
  for (; k0 <= K; k0 += 4) {
    const float4 Cn = *reinterpret_cast<const float4*>(p + k0 + 8);
    const float sv[12] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w, Cn.x, Cn.y, Cn.z, Cn.w};
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (k0 + q <= K) {
        const float wk = wx[k0 + q];
        f0 = fmaf(wk, sv[OFF + q], f0);
        f1 = fmaf(wk, sv[OFF + q + 1], f1);
        f2 = fmaf(wk, sv[OFF + q + 2], f2);
        f3 = fmaf(wk, sv[OFF + q + 3], f3);
      }
    }
    A = B;
    B = Cn;
  }
}

__device__ __forceinline__ float4 fma4(float w, const float4& v, float4 a) {
  a.x = fmaf(w, v.x, a.x);
  a.y = fmaf(w, v.y, a.y);
  a.z = fmaf(w, v.z, a.z);
  a.w = fmaf(w, v.w, a.w);
  return a;
}

// Vectorised form for w % 4 == 0: w/4 column lanes of 4 columns, RB lanes of
// R rows each per block of RB*R rows.  The vertical pass slides over the
// input rows once per thread (R outputs share each 16-byte row load), the
// horizontal pass reads 16-byte chunks of the filtered rows; every output
// still accumulates its taps in order with fmaf, as the scalar form does.
template <int MODE, int R>
__device__ void filter_pass4(const float* C, float* V, const int* rtab, int w, int mS, int ry, int rx,
                             const float* wy, const float* wx, float c, PkShared& sh, bool use_mask, FiltStats& st,
                             float& amax, int& aidx) {
  const int w4 = w >> 2;
  const int RB = PK_T / w4;
  const int VP = pk_vec_pitch(w);
  const int tx = threadIdx.x % w4, ty = threadIdx.x / w4;
  const int x0 = tx << 2;
  float s1 = 0.0f, s2 = 0.0f, mx = -INFINITY;
  float bv = -INFINITY;
  int bi = 0x7fffffff;
  int cnt = 0;
  const int OFF = (-rx) & 3;
  const bool xin = (x0 >= rx && x0 + 3 + rx < w);
  for (int yb = 0; yb < w; yb += RB * R) {
    const int y = yb + ty * R;  // first of this thread's R rows
    const bool act = ty < RB && y < w;
    if (act) {
      float4 acc[R];
#pragma unroll
      for (int j = 0; j < R; j++) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
      const bool yin = (y >= ry && y + R - 1 + ry < w);
      const int* rt = rtab + PK_MAXR + y - ry;
      float wr[R];
#pragma unroll
      for (int j = 0; j < R; j++) wr[j] = 0.0f;
      if (R == 2 && yin) {
        // rows y and y + 1 away from the borders: input row y - ry + t adds
        // wy[t] to row y and wy[t - 1] to row y + 1, taps in order (as below),
        // two input rows a step with no per-tap tests
        const float* pr = C + (y - ry) * w + x0;
        const int K = 2 * ry;
        float4 a0 = acc[0], a1 = acc[R - 1];
        float wp = wy[0];
        a0 = fma4(wp, *reinterpret_cast<const float4*>(pr), a0);
        int t = 1;
        for (; t + 1 <= K; t += 2) {
          const float4 va = *reinterpret_cast<const float4*>(pr + t * w);
          const float4 vb = *reinterpret_cast<const float4*>(pr + (t + 1) * w);
          const float wa = wy[t], wb = wy[t + 1];
          a0 = fma4(wa, va, a0);
          a1 = fma4(wp, va, a1);
          a0 = fma4(wb, vb, a0);
          a1 = fma4(wa, vb, a1);
          wp = wb;
        }
        if (t <= K) {
          const float4 va = *reinterpret_cast<const float4*>(pr + t * w);
          const float wa = wy[t];
          a0 = fma4(wa, va, a0);
          a1 = fma4(wp, va, a1);
          wp = wa;
        }
        a1 = fma4(wp, *reinterpret_cast<const float4*>(pr + (K + 1) * w), a1);
        acc[0] = a0;
        acc[R - 1] = a1;
      } else
      for (int t = 0; t <= 2 * ry + R - 1; t++) {
        // wr[j] = wy[t - j]
#pragma unroll
        for (int j = R - 1; j > 0; j--) wr[j] = wr[j - 1];
        wr[0] = t <= 2 * ry ? wy[t] : 0.0f;
        const int row = yin ? (y - ry + t) : rt[t];
        const float4 v = *reinterpret_cast<const float4*>(C + row * w + x0);
#pragma unroll
        for (int j = 0; j < R; j++) {
          if (t - j >= 0 && t - j <= 2 * ry) {
            const float wk = wr[j];
            acc[j].x = fmaf(wk, v.x, acc[j].x); acc[j].y = fmaf(wk, v.y, acc[j].y);
            acc[j].z = fmaf(wk, v.z, acc[j].z); acc[j].w = fmaf(wk, v.w, acc[j].w);
          }
        }
      }
#pragma unroll
      for (int j = 0; j < R; j++)
        if (y + j < w) *reinterpret_cast<float4*>(V + (ty * R + j) * VP + x0) = acc[j];
    }
    __syncthreads();
    if (act) {
      // the horizontal taps of the thread's R rows, then their statistics
      float fr[R][4];
#pragma unroll
      for (int j = 0; j < R; j++) {
        fr[j][0] = fr[j][1] = fr[j][2] = fr[j][3] = 0.f;
        if (y + j >= w) break;
        const float* vr = V + (ty * R + j) * VP;
        float& f0 = fr[j][0];
        float& f1 = fr[j][1];
        float& f2 = fr[j][2];
        float& f3 = fr[j][3];
        if (xin) {
          const float* pp = vr + x0 - rx - OFF;
          switch (OFF) {
            case 0: hrow4<0>(pp, wx, rx, f0, f1, f2, f3); break;
            case 1: hrow4<1>(pp, wx, rx, f0, f1, f2, f3); break;
            case 2: hrow4<2>(pp, wx, rx, f0, f1, f2, f3); break;
            default: hrow4<3>(pp, wx, rx, f0, f1, f2, f3); break;
          }
        } else {
          const int* rt = rtab + PK_MAXR + x0 - rx;
          float a0 = vr[rt[0]], a1 = vr[rt[1]], a2 = vr[rt[2]];
          for (int k = 0; k <= 2 * rx; k++) {
            const float a3 = vr[rt[k + 3]];
            const float wk = wx[k];
            f0 = fmaf(wk, a0, f0); f1 = fmaf(wk, a1, f1); f2 = fmaf(wk, a2, f2); f3 = fmaf(wk, a3, f3);
            a0 = a1; a1 = a2; a2 = a3;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < R; j++) {
        const int yy = y + j;
        if (yy >= w) break;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const float f = fr[j][q];
          const int x = x0 + q;
          bool in = true;
          if (MODE == 1) {
            const int dy = yy - mS, dx = x - mS;
            in = !use_mask || (dy * dy + dx * dx < mS * mS);
            const float mv = in ? f : 0.0f;
            const int idx = yy * w + x;
            if (mv > bv || (mv == bv && idx < bi)) { bv = mv; bi = idx; }
          }
          if (in) {
            const float d = f - c;
            s1 += d;
            s2 = fmaf(d, d, s2);
            mx = fmaxf(mx, f);
            cnt++;
          }
        }
      }
    }
    __syncthreads();
  }
  block_stats(sh, s1, s2, cnt, mx, st);
  if (MODE == 1) {
    block_argmax(sh, bv, bi);
    amax = bv;
    aidx = bi;
  }
}

template <int MODE>
__device__ void filter_any(const float* C, float* V, const int* rtab, int w, int mS, int ry, int rx, const float* wy,
                           const float* wx, float c, PkShared& sh, bool use_mask, FiltStats& st, float& amax,
                           int& aidx) {
  if ((w & 3) == 0 && w >= 16 && w <= 4 * PK_TX)
    filter_pass4<MODE, pk_vec_rows(0)>(C, V, rtab, w, mS, ry, rx, wy, wx, c, sh, use_mask, st, amax, aidx);
  else
    filter_pass<MODE>(C, V, rtab, w, mS, ry, rx, wy, wx, c, sh, use_mask, st, amax, aidx);
}

// std(G_sigma * C) / (max - mean) of the filtered window (zorro.py:1108-
// 1121).  All threads filter; the value is formed by thread 0 only (the
// others return 0).
__device__ double objective(const float* C, float* V, const int* rtab, int w, int mS, double sigma, float c,
                            PkShared& sh) {
  const int r = gauss_weights(sigma, sh.wy, sh);
  __syncthreads();
  FiltStats st;
  float am;
  int ai;
  filter_any<0>(C, V, rtab, w, mS, r, r, sh.wy, sh.wy, c, sh, false, st, am, ai);
  if (threadIdx.x != 0) return 0.0;
  const double n = (double)st.n;
  const double m1 = st.s1 / n;
  const double var = st.s2 / n - m1 * m1;
  const double mean = (double)c + m1;
  return sqrt(var > 0.0 ? var : 0.0) / ((double)st.mx - mean);
}

__device__ __forceinline__ double sgn1(double v) { return v > 0.0 ? 1.0 : (v < 0.0 ? -1.0 : 1.0); }

// Bounded Brent minimisation (FMM FMIN).  Returns the abscissa of the best
// value (to every thread); *nfev receives the number of function values.
// The search's scalar state lives in thread 0, which decides each next
// abscissa and whether to go on and hands them to the CTA through shared
// memory; all threads evaluate the objective.
// Thread 0: the next abscissa of the search (sh.x, sh.go = 1), or its end
// (sh.go = 0).
__device__ void brent_next(BrentState& S, PkShared& sh) {
  const double golden = 0.5 * (3.0 - sqrt(5.0));
  if (!(fabs(S.xf - S.xm) > (S.tol2 - 0.5 * (S.b - S.a)))) {
    sh.go = 0;
    return;
  }
  bool gstep = true;
  if (fabs(S.e) > S.tol1) {
    gstep = false;
    double r = (S.xf - S.nfc) * (S.fx - S.ffulc);
    double q = (S.xf - S.fulc) * (S.fx - S.fnfc);
    double p = (S.xf - S.fulc) * q - (S.xf - S.nfc) * r;
    q = 2.0 * (q - r);
    if (q > 0.0) p = -p;
    q = fabs(q);
    r = S.e;
    S.e = S.rat;
    if ((fabs(p) < fabs(0.5 * q * r)) && (p > q * (S.a - S.xf)) && (p < q * (S.b - S.xf))) {
      S.rat = (p + 0.0) / q;
      S.x = S.xf + S.rat;
      if (((S.x - S.a) < S.tol2) || ((S.b - S.x) < S.tol2)) S.rat = S.tol1 * sgn1(S.xm - S.xf);
    } else {
      gstep = true;
    }
  }
  if (gstep) {
    S.e = (S.xf >= S.xm) ? (S.a - S.xf) : (S.b - S.xf);
    S.rat = golden * S.e;
  }
  S.x = S.xf + sgn1(S.rat) * fmax(fabs(S.rat), S.tol1);
  sh.x = S.x;
  sh.go = 1;
}

// Bounded Brent minimisation (FMM FMIN).  Returns the abscissa of the best
// value (to every thread); *nfev receives the number of function values.
// Thread 0 runs the search (its state in shared memory), decides each next
// abscissa and whether to go on and hands them to the CTA through shared
// memory; all threads evaluate the objective.
__device__ double fmin_bounded(const float* C, float* V, const int* rtab, int w, int mS, float c, PkShared& sh,
                               double lo, double hi, double xatol, int maxfun, int* nfev) {
  const bool lead = threadIdx.x == 0;
  const double sqrt_eps = sqrt(2.2e-16);
  const double golden = 0.5 * (3.0 - sqrt(5.0));
  const double x0 = lo + golden * (hi - lo);
  const double f0 = objective(C, V, rtab, w, mS, x0, c, sh);
  if (lead) {
    BrentState S;
    S.a = lo;
    S.b = hi;
    S.fulc = x0;
    S.nfc = x0;
    S.xf = x0;
    S.rat = 0.0;
    S.e = 0.0;
    S.x = x0;
    S.fx = f0;
    S.num = 1;
    S.ffulc = f0;
    S.fnfc = f0;
    S.xm = 0.5 * (lo + hi);
    S.tol1 = sqrt_eps * fabs(x0) + xatol / 3.0;
    S.tol2 = 2.0 * S.tol1;
    brent_next(S, sh);
    if (!sh.go) {  // the search ended before its first step
      sh.x = S.xf;
      sh.bi[1] = S.num;
    }
    sh.bs = S;
  }
  __syncthreads();
  while (sh.go) {
    const double xe = sh.x;
    const double fu = objective(C, V, rtab, w, mS, xe, c, sh);  // barriers: every thread has read sh.x, sh.go
    if (lead) {
      BrentState S = sh.bs;
      S.num += 1;
      if (fu <= S.fx) {
        if (S.x >= S.xf) S.a = S.xf; else S.b = S.xf;
        S.fulc = S.nfc; S.ffulc = S.fnfc;
        S.nfc = S.xf; S.fnfc = S.fx;
        S.xf = S.x; S.fx = fu;
      } else {
        if (S.x < S.xf) S.a = S.x; else S.b = S.x;
        if ((fu <= S.fnfc) || (S.nfc == S.xf)) {
          S.fulc = S.nfc; S.ffulc = S.fnfc;
          S.nfc = S.x; S.fnfc = fu;
        } else if ((fu <= S.ffulc) || (S.fulc == S.xf) || (S.fulc == S.nfc)) {
          S.fulc = S.x; S.ffulc = fu;
        }
      }
      S.xm = 0.5 * (S.a + S.b);
      S.tol1 = sqrt_eps * fabs(S.xf) + xatol / 3.0;
      S.tol2 = 2.0 * S.tol1;
      if (S.num >= maxfun) sh.go = 0;
      else brent_next(S, sh);
      if (!sh.go) {
        sh.x = S.xf;
        sh.bi[1] = S.num;
      }
      sh.bs = S;
    }
    __syncthreads();
  }
  const double best = sh.x;
  *nfev = sh.bi[1];
  __syncthreads();
  return best;
}

// The sub-pixel step on a 16 x 16 filtered patch (zorro.py:1180-1216): its
// forward DFT (rows, then columns), the inverse DFT upsampled to an L x L
// grid (L = 16*sp, frequencies -8..7, unscaled like the reference's
// subIFFT2.execute()), |.| and its argmax (first index on ties).  ``scratch``
// holds 17*L float2 of shared memory.  All threads call.
__device__ void subpix_search(const float* patch, int sp, const float2* __restrict__ tw, float2* scratch,
                              float2* patchF, PkShared& sh, float& bv, int& bi) {
  __shared__ float2 rowF[16 * 16];
  for (int e = threadIdx.x; e < 256; e += PK_T) {
    const int i = e >> 4, v = e & 15;
    float2 acc = make_float2(0.0f, 0.0f);
    for (int j = 0; j < 16; j++) {
      const float2 t = __ldg(tw + ((v * j) & 15) * (TWN / 16));
      acc.x = fmaf(patch[i * 16 + j], t.x, acc.x);
      acc.y = fmaf(patch[i * 16 + j], t.y, acc.y);
    }
    rowF[e] = acc;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 256; e += PK_T) {
    const int u = e >> 4, v = e & 15;
    float2 acc = make_float2(0.0f, 0.0f);
    for (int i = 0; i < 16; i++) acc = cadd(acc, cmul(rowF[i * 16 + v], __ldg(tw + ((u * i) & 15) * (TWN / 16))));
    patchF[e] = acc;
  }
  __syncthreads();
  // exp(+2 pi i m / L) for m in [0, L), after the L x 16 intermediate
  const int L = 16 * sp;
  const int tws = TWN / L;
  float2* Tx = scratch;
  float2* Wl = Tx + 16 * L;
  for (int m = threadIdx.x; m < L; m += PK_T) {
    float2 t = __ldg(tw + m * tws);
    t.y = -t.y;
    Wl[m] = t;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 16 * L; e += PK_T) {
    const int fyi = e / L, nx = e - fyi * L;
    float2 acc = make_float2(0.0f, 0.0f);
    for (int fxi = 0; fxi < 16; fxi++) {
      const int fx = fxi - 8;
      const float2 t = Wl[(fx * nx) & (L - 1)];
      acc = cadd(acc, cmul(patchF[((fyi - 8) & 15) * 16 + (fx & 15)], t));
    }
    Tx[fyi * L + nx] = acc;
  }
  __syncthreads();
  bv = -INFINITY;
  bi = 0x7fffffff;
  for (int e = threadIdx.x; e < L * L; e += PK_T) {
    const int ny = e / L, nx = e - ny * L;
    float2 acc = make_float2(0.0f, 0.0f);
    for (int fyi = 0; fyi < 16; fyi++) {
      const int fy = fyi - 8;
      const float2 t = Wl[(fy * ny) & (L - 1)];
      acc = cadd(acc, cmul(Tx[fyi * L + nx], t));
    }
    const float mag = sqrtf(acc.x * acc.x + acc.y * acc.y);
    if (mag > bv || (mag == bv && e < bi)) { bv = mag; bi = e; }
  }
  block_argmax(sh, bv, bi);
}

__global__ void __launch_bounds__(PK_T, 1) k_peaks(const float* __restrict__ cwin, int mS, zr_peak_params_t p,
                                               zr_peak_result_t* __restrict__ res, const float2* __restrict__ tw) {
  extern __shared__ float smf[];
  __shared__ PkShared sh;
  __shared__ float2 patchF[16 * 16];
  __shared__ int rtab[2 * PK_MAXR + 2 * 112];
  const int w = 2 * mS;
  const int w2 = w * w;
  float* C = smf;
  float* V = smf + w2;
  const float* src = cwin + (size_t)blockIdx.x * w2;
  for (int e = threadIdx.x; e < w2; e += PK_T) C[e] = src[e];
  for (int i = threadIdx.x; i < w + 2 * PK_MAXR; i += PK_T) rtab[i] = reflect_idx(i - PK_MAXR, w);
  __syncthreads();
  const float origin = C[mS * w + mS];
  if (p.suppress_origin) {
    __syncthreads();
    if (threadIdx.x == 0) {
      const int o = mS * w + mS;
      float s = C[o + w] + C[o + 1];
      s = s + C[o - w];
      s = s + C[o - w];
      s = s + C[o + w + 1];
      s = s + C[o - w + 1];
      s = s + C[o - w + 1];
      s = s + C[o - w - 1];
      C[o] = 0.125f * s;
    }
    __syncthreads();
  }
  // mean of the window: the centring constant of the one-pass variances
  // (any value near the mean serves; the statistics are exact sums around it)
  float ls = 0.0f;
  for (int e = threadIdx.x; e < w2; e += PK_T) ls += C[e];
  FiltStats tot;
  block_stats(sh, ls, 0.0f, 0, 0.0f, tot);
  const float c = (float)(tot.s1 / (double)w2);

  double sigy = 0.0, sigx = 0.0, sig_opt = nan("");
  int nfev = 0;
  if (p.bmode == 1) {
    sig_opt = fmin_bounded(C, V, rtab, w, mS, c, sh, p.opti_lo, p.opti_hi, p.opti_xatol, p.opti_maxiter, &nfev);
    sigy = sigx = sig_opt;
  } else if (p.bmode == 2) {
    sigy = p.conv_sigma_y;
    sigx = p.conv_sigma_x;
  }
  const int ry = gauss_weights(sigy, sh.wy, sh);
  const int rx = gauss_weights(sigx, sh.wx, sh);
  __syncthreads();
  FiltStats st;
  float amax = 0.0f;
  int aidx = 0;
  filter_any<1>(C, V, rtab, w, mS, ry, rx, sh.wy, sh.wx, c, sh, p.use_mask != 0, st, amax, aidx);
  const int cy = aidx / w, cx = aidx - (aidx / w) * w;
  const float cval = C[cy * w + cx];
  float corr = cval;
  int flags = 0;
  int sy = -1, sx = -1;  // sub-pixel argmax on the upsampled grid
  float bv = 0.0f;
  const int sp = p.sub_pix_reg;
  const int L = 16 * sp;
  if (sp > 1) {
    if (cy - PK_SUBR >= 0 && cy + PK_SUBR <= w && cx - PK_SUBR >= 0 && cx + PK_SUBR <= w) {
      // the 16 x 16 filtered patch around the peak, separably: the vertical
      // pass for its 16 rows over the 16 + 2 rx columns the horizontal taps
      // reach (reflected), then the horizontal pass; the same multiply-adds
      // in the same order as the full filter pass, so the same values
      __shared__ float patch[16 * 16];
      const int pw = 16 + 2 * rx;
      for (int e = threadIdx.x; e < 16 * pw; e += PK_T) {
        const int i = e / pw, j = e - (e / pw) * pw;
        const int y = cy - PK_SUBR + i;
        const int xx = reflect_idx(cx - PK_SUBR - rx + j, w);
        float acc = 0.0f;
        if (ry == 0) acc = C[y * w + xx];
        else
          for (int k = 0; k <= 2 * ry; k++) acc = fmaf(sh.wy[k], C[rtab[PK_MAXR + y - ry + k] * w + xx], acc);
        V[e] = acc;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < 256; e += PK_T) {
        const int i = e >> 4, j = e & 15;
        float f = 0.0f;
        if (rx == 0) f = V[i * pw + j];
        else
          for (int k = 0; k <= 2 * rx; k++) f = fmaf(sh.wx[k], V[i * pw + j + k], f);
        patch[e] = f;
      }
      __syncthreads();
      int bi;
      subpix_search(patch, sp, tw, (float2*)C, patchF, sh, bv, bi);  // the window is no longer needed
      sy = bi / L;
      sx = bi - (bi / L) * L;
    } else {
      flags |= 1;
    }
  }
  if (threadIdx.x == 0) {
    const double n = (double)st.n;
    const double m1 = st.s1 / n;
    const double var = st.s2 / n - m1 * m1;
    const double mean = (double)c + m1;
    const double peaksig = ((double)amax - mean) / sqrt(var > 0.0 ? var : 0.0);
    double shy = (double)cy - w / 2.0, shx = (double)cx - w / 2.0;
    if (sy >= 0) {
      const double ry0 = (double)cy - w / 2.0, rx0 = (double)cx - w / 2.0;
      shy = ry0 + ((double)sy - L / 2.0 + (ry0 > 0 ? 1.0 : (ry0 < 0 ? -1.0 : 0.0))) / sp;
      shx = rx0 + ((double)sx - L / 2.0 + (rx0 > 0 ? 1.0 : (rx0 < 0 ? -1.0 : 0.0))) / sp;
      corr = (float)((double)bv / 256.0);
    }
    zr_peak_result_t r;
    r.shift_y = shy;
    r.shift_x = shx;
    r.sigma = sig_opt;
    r.corr = corr;
    r.peaksig = (float)peaksig;
    r.origin = origin;
    r.cy = cy;
    r.cx = cx;
    r.flags = flags;
    r.nfev = nfev;
    res[blockIdx.x] = r;
  }
}

// ---------------------------------------------------------------------------
// Peak search on uncropped correlation planes (preShift, zorro.py:1089-1092
// and 1148-1168): each plane is the whole C x C correlation, ifftshifted.  The
// planes are too large for one CTA, so the steps are separate launches over a
// batch of planes, driven by the bounded Brent search that the host runs for
// every plane of the batch in lock step:
//   k_full_prepare   origin value, the suppressOrigin stencil, plane mean;
//   k_full_vert      axis-0 Gaussian pass (reflect), into a scratch plane;
//   k_full_horz      axis-1 pass, its value kept or not, per-CTA partial
//                    (sum (f - c), sum (f - c)^2, max f) of the statistic;
//   k_full_reduce    the partials in a fixed order (repeatable sums);
//   k_full_masked    the maxShift disc rolled by the plane's offset: masked
//                    argmax (first index on ties) and the partial sums over
//                    the disc for the peak significance;
//   k_full_finish    the reduction of those and the sub-pixel step.
// ``sel`` lists the planes a launch works on (grid z).

constexpr int FP_T = 256;   // threads of the filter and masked passes
constexpr int FP_TX = 32;   // columns per filter CTA
constexpr int FP_RY = 64;   // rows per filter CTA

__global__ void __launch_bounds__(1024) k_full_prepare(float* __restrict__ planes, int C, int suppress,
                                                       float* __restrict__ origin, float* __restrict__ mean) {
  __shared__ double red[32];
  float* P = planes + (size_t)blockIdx.x * C * C;
  const int o = (C / 2) * C + C / 2;
  if (threadIdx.x == 0) {
    origin[blockIdx.x] = P[o];
    if (suppress) {  // literal stencil of zorro.py:1082-1083 at the shifted origin
      float sm = P[o + C] + P[o + 1];
      sm = sm + P[o - C];
      sm = sm + P[o - C];
      sm = sm + P[o + C + 1];
      sm = sm + P[o - C + 1];
      sm = sm + P[o - C + 1];
      sm = sm + P[o - C - 1];
      P[o] = 0.125f * sm;
    }
  }
  __syncthreads();
  float ls = 0.0f;
  double ds = 0.0;
  int cnt = 0;
  for (long long e = threadIdx.x; e < (long long)C * C; e += blockDim.x) {
    ls += P[e];
    if (++cnt == 64) { ds += ls; ls = 0.0f; cnt = 0; }
  }
  ds += ls;
  for (int off = 16; off > 0; off >>= 1) ds += __shfl_down_sync(0xffffffffu, ds, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ds;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
    mean[blockIdx.x] = (float)(t / ((double)C * C));
  }
}

// T[y][x] = sum_k wy[k] P[reflect(y + k - r)][x], the taps in order
__global__ void __launch_bounds__(FP_T) k_full_vert(const float* __restrict__ planes, int C, const int* __restrict__ sel,
                                                  const float* __restrict__ wts, const int* __restrict__ rad,
                                                  float* __restrict__ tmp) {
  const int j = blockIdx.z, p = sel[j];
  const int r = rad[2 * p];
  const float* w = wts + (size_t)p * 2 * (2 * PK_MAXR + 1);
  const float* P = planes + (size_t)p * C * C;
  float* T = tmp + (size_t)j * C * C;
  const int x = blockIdx.x * FP_TX + (threadIdx.x & (FP_TX - 1));
  if (x >= C) return;
  for (int y = blockIdx.y * FP_RY + threadIdx.x / FP_TX; y < min(C, (int)(blockIdx.y + 1) * FP_RY);
       y += FP_T / FP_TX) {
    float acc;
    if (r == 0) {
      acc = P[(size_t)y * C + x] * w[0];
    } else {
      acc = 0.0f;
      for (int k = 0; k <= 2 * r; k++) acc = fmaf(w[k], __ldg(P + (size_t)reflect_idx(y + k - r, C) * C + x), acc);
    }
    T[(size_t)y * C + x] = acc;
  }
}

// F[y][x] = sum_k wx[k] T[y][reflect(x + k - r)]; F kept when ``out`` is set;
// per-CTA partials of sum (F - c), sum (F - c)^2 and max F
__global__ void __launch_bounds__(FP_T) k_full_horz(const float* __restrict__ tmp, int C, const int* __restrict__ sel,
                                                  const float* __restrict__ wts, const int* __restrict__ rad,
                                                  const float* __restrict__ mean, float* __restrict__ out,
                                                  double* __restrict__ part) {
  __shared__ double red[FP_T / 32][3];
  const int j = blockIdx.z, p = sel[j];
  const int r = rad[2 * p + 1];
  const float* w = wts + (size_t)p * 2 * (2 * PK_MAXR + 1) + (2 * PK_MAXR + 1);
  const float* T = tmp + (size_t)j * C * C;
  const float c = mean[p];
  const int x = blockIdx.x * FP_TX + (threadIdx.x & (FP_TX - 1));
  float s1 = 0.0f, s2 = 0.0f, mx = -INFINITY;
  if (x < C) {
    for (int y = blockIdx.y * FP_RY + threadIdx.x / FP_TX; y < min(C, (int)(blockIdx.y + 1) * FP_RY);
         y += FP_T / FP_TX) {
      const float* row = T + (size_t)y * C;
      float f;
      if (r == 0) {
        f = row[x] * w[0];
      } else {
        f = 0.0f;
        for (int k = 0; k <= 2 * r; k++) f = fmaf(w[k], __ldg(row + reflect_idx(x + k - r, C)), f);
      }
      if (out) out[(size_t)p * C * C + (size_t)y * C + x] = f;
      const float d = f - c;
      s1 += d;
      s2 = fmaf(d, d, s2);
      mx = fmaxf(mx, f);
    }
  }
  double a = s1, b = s2, m = mx;
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, off);
    b += __shfl_down_sync(0xffffffffu, b, off);
    m = fmax(m, __shfl_down_sync(0xffffffffu, m, off));
  }
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5][0] = a;
    red[threadIdx.x >> 5][1] = b;
    red[threadIdx.x >> 5][2] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0, tm = -INFINITY;
    for (int i = 0; i < FP_T / 32; i++) {
      ta += red[i][0];
      tb += red[i][1];
      tm = fmax(tm, red[i][2]);
    }
    double* q = part + ((size_t)p * gridDim.y * gridDim.x + (size_t)blockIdx.y * gridDim.x + blockIdx.x) * 3;
    q[0] = ta;
    q[1] = tb;
    q[2] = tm;
  }
}

// stats[p] = (sum, sum of squares, max) over the partials of plane p, in order
__global__ void k_full_reduce(const double* __restrict__ part, int nblk, const int* __restrict__ sel,
                              double* __restrict__ stats) {
  const int p = sel[blockIdx.x];
  if (threadIdx.x != 0) return;
  double a = 0.0, b = 0.0, m = -INFINITY;
  const double* q = part + (size_t)p * nblk * 3;
  for (int i = 0; i < nblk; i++) {
    a += q[3 * i];
    b += q[3 * i + 1];
    m = fmax(m, q[3 * i + 2]);
  }
  stats[3 * p] = a;
  stats[3 * p + 1] = b;
  stats[3 * p + 2] = m;
}

constexpr int FP_MBLK = 128;  // CTAs per plane of the masked pass

// The disc of radius mS about the plane centre, np.roll-ed by (ry, rx)
// (zorro.py:1150-1153): pixel (y, x) is in it when the unrolled pixel
// ((y - ry) mod C, (x - rx) mod C) lies within mS of (C/2, C/2).
__device__ __forceinline__ bool in_rolled_disc(int y, int x, int C, int mS, int ry, int rx) {
  int yy = (y - ry) % C, xx = (x - rx) % C;
  if (yy < 0) yy += C;
  if (xx < 0) xx += C;
  const long long dy = yy - C / 2, dx = xx - C / 2;
  return dy * dy + dx * dx < (long long)mS * mS;
}

// Per-CTA partials over its share of plane p: the argmax of F * disc (zeros
// outside the disc compete, first index on ties) and sum (F - c),
// sum (F - c)^2 and the count over the disc.
__global__ void __launch_bounds__(FP_T) k_full_masked(const float* __restrict__ filt, int C, const int* __restrict__ sel,
                                                    int mS, const int* __restrict__ rolls,
                                                    const float* __restrict__ mean, double* __restrict__ part) {
  __shared__ float rv[FP_T / 32];
  __shared__ int ri[FP_T / 32];
  __shared__ double rs[FP_T / 32][3];
  const int p = sel[blockIdx.z];
  const float* F = filt + (size_t)p * C * C;
  const float c = mean[p];
  const int ry = rolls[2 * p], rx = rolls[2 * p + 1];
  float bv = -INFINITY, s1 = 0.0f, s2 = 0.0f;
  int bi = 0x7fffffff, cnt = 0;
  const long long n = (long long)C * C;
  for (long long e = (long long)blockIdx.x * FP_T + threadIdx.x; e < n; e += (long long)gridDim.x * FP_T) {
    const int y = (int)(e / C), x = (int)(e - (long long)y * C);
    const float f = F[e];
    const bool in = in_rolled_disc(y, x, C, mS, ry, rx);
    const float mv = in ? f : 0.0f;
    if (mv > bv || (mv == bv && (int)e < bi)) { bv = mv; bi = (int)e; }
    if (in) {
      const float d = f - c;
      s1 += d;
      s2 = fmaf(d, d, s2);
      cnt++;
    }
  }
  double a = s1, b = s2, k = cnt;
  for (int off = 16; off > 0; off >>= 1) {
    const float ov = __shfl_down_sync(0xffffffffu, bv, off);
    const int oi = __shfl_down_sync(0xffffffffu, bi, off);
    if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    a += __shfl_down_sync(0xffffffffu, a, off);
    b += __shfl_down_sync(0xffffffffu, b, off);
    k += __shfl_down_sync(0xffffffffu, k, off);
  }
  const int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    rv[wid] = bv;
    ri[wid] = bi;
    rs[wid][0] = a;
    rs[wid][1] = b;
    rs[wid][2] = k;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < FP_T / 32; i++) {
      if (rv[i] > rv[0] || (rv[i] == rv[0] && ri[i] < ri[0])) { rv[0] = rv[i]; ri[0] = ri[i]; }
      rs[0][0] += rs[i][0];
      rs[0][1] += rs[i][1];
      rs[0][2] += rs[i][2];
    }
    double* q = part + ((size_t)p * gridDim.x + blockIdx.x) * 5;
    q[0] = rv[0];
    q[1] = ri[0];
    q[2] = rs[0][0];
    q[3] = rs[0][1];
    q[4] = rs[0][2];
  }
}

// One CTA per plane: the masked partials in order, the peak significance,
// then the sub-pixel step on the filtered plane (or the integer fallback at
// the plane's edge) as k_peaks does it.
__global__ void __launch_bounds__(PK_T, 1) k_full_finish(const float* __restrict__ planes,
                                                       const float* __restrict__ filt, int C,
                                                       const int* __restrict__ sel, const double* __restrict__ part,
                                                       const float* __restrict__ mean, const float* __restrict__ origin,
                                                       const double* __restrict__ sigma, const int* __restrict__ nfev,
                                                       int sp, zr_peak_result_t* __restrict__ res,
                                                       const float2* __restrict__ tw) {
  extern __shared__ float2 scratch[];
  __shared__ PkShared sh;
  __shared__ float2 patchF[16 * 16];
  __shared__ float patch[16 * 16];
  __shared__ double fin[4];
  __shared__ int fidx;
  const int p = sel[blockIdx.x];
  if (threadIdx.x == 0) {
    const double* q = part + (size_t)p * FP_MBLK * 5;
    double bv = q[0], s1 = q[2], s2 = q[3], cnt = q[4];
    int bi = (int)q[1];
    for (int i = 1; i < FP_MBLK; i++) {
      const double* r = q + 5 * i;
      if (r[0] > bv || (r[0] == bv && (int)r[1] < bi)) { bv = r[0]; bi = (int)r[1]; }
      s1 += r[2];
      s2 += r[3];
      cnt += r[4];
    }
    const double m1 = s1 / cnt;
    const double var = s2 / cnt - m1 * m1;
    fin[0] = ((double)(float)bv - ((double)mean[p] + m1)) / sqrt(var > 0.0 ? var : 0.0);
    fin[1] = bv;
    fidx = bi;
  }
  __syncthreads();
  const int cy = fidx / C, cx = fidx - (fidx / C) * C;
  const float* P = planes + (size_t)p * C * C;
  const float* F = filt + (size_t)p * C * C;
  double shy = (double)cy - C / 2.0, shx = (double)cx - C / 2.0;
  float corr = P[(size_t)cy * C + cx];
  int flags = 0;
  if (sp > 1) {
    if (cy - PK_SUBR >= 0 && cy + PK_SUBR <= C && cx - PK_SUBR >= 0 && cx + PK_SUBR <= C) {
      for (int e = threadIdx.x; e < 256; e += PK_T)
        patch[e] = F[(size_t)(cy - PK_SUBR + (e >> 4)) * C + cx - PK_SUBR + (e & 15)];
      __syncthreads();
      const int L = 16 * sp;
      float bv;
      int bi;
      subpix_search(patch, sp, tw, scratch, patchF, sh, bv, bi);
      const int sy = bi / L, sx = bi - (bi / L) * L;
      const double ry0 = (double)cy - C / 2.0, rx0 = (double)cx - C / 2.0;
      shy = ry0 + ((double)sy - L / 2.0 + (ry0 > 0 ? 1.0 : (ry0 < 0 ? -1.0 : 0.0))) / sp;
      shx = rx0 + ((double)sx - L / 2.0 + (rx0 > 0 ? 1.0 : (rx0 < 0 ? -1.0 : 0.0))) / sp;
      corr = (float)((double)bv / 256.0);
    } else {
      flags |= 1;
    }
  }
  if (threadIdx.x == 0) {
    zr_peak_result_t r;
    r.shift_y = shy;
    r.shift_x = shx;
    r.sigma = sigma[p];
    r.corr = corr;
    r.peaksig = (float)fin[0];
    r.origin = origin[p];
    r.cy = cy;
    r.cx = cx;
    r.flags = flags;
    r.nfev = nfev[p];
    res[p] = r;
  }
}

static int full_blocks(int C) { return ((C + FP_TX - 1) / FP_TX) * ((C + FP_RY - 1) / FP_RY); }

}  // namespace zr

using namespace zr;

extern "C" int zr_locate_peaks(const float* cwin, int M, int max_shift, const zr_peak_params_t* params,
                               zr_peak_result_t* results, void* stream) {
  if (!cwin || !params || !results) return set_error(ZR_EINVAL, "zr_locate_peaks: null argument");
  if (M <= 0) return ZR_OK;
  const int w = 2 * max_shift;
  if (max_shift < 8 || max_shift > 112)
    return set_error(ZR_ESIZE, "zr_locate_peaks: maxShift %d outside [8, 112]", max_shift);
  if (params->sub_pix_reg > 1 && (TWN % (16 * params->sub_pix_reg) != 0 || 16 * params->sub_pix_reg > 512))
    return set_error(ZR_ESIZE, "zr_locate_peaks: subPixReg %d must be a power of two <= 32", params->sub_pix_reg);
  if (params->bmode == 2 && (4.0 * params->conv_sigma_y + 0.5 > PK_MAXR || 4.0 * params->conv_sigma_x + 0.5 > PK_MAXR))
    return set_error(ZR_ESIZE, "zr_locate_peaks: conv sigma too large");
  if (params->bmode == 1 && 4.0 * params->opti_hi + 0.5 > PK_MAXR)
    return set_error(ZR_ESIZE, "zr_locate_peaks: opti sigma bound too large");
  const float2* tw = twiddles();
  if (!tw) return ZR_ECUDA;
  // window + one block of filtered rows (RB lanes x pk_vec_rows rows at pitch
  // w + 8 for the vectorised layout, PK_RB rows otherwise)
  const bool vec = (w & 3) == 0 && w >= 16 && w <= 4 * PK_TX;
  const size_t vrows = vec ? (size_t)(PK_T / (w / 4)) * pk_vec_rows(w) : (size_t)PK_RB;
  size_t vbuf = vrows * (vec ? pk_vec_pitch(w) : w) * sizeof(float);
  // the row block also holds the vertical pass of the 16 x 16 sub-pixel patch
  const size_t pbuf = (size_t)16 * (16 + 2 * PK_MAXR) * sizeof(float);
  if (vbuf < pbuf) vbuf = pbuf;
  size_t smem = (size_t)w * w * sizeof(float) + vbuf;
  const size_t sub = (size_t)17 * 16 * params->sub_pix_reg * sizeof(float2);
  if (params->sub_pix_reg > 1 && (size_t)w * w * sizeof(float) < sub) smem = sub + vbuf;
  ZR_TRY(cuda_check(cudaFuncSetAttribute(k_peaks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "k_peaks attr"));
  k_peaks<<<M, PK_T, smem, (cudaStream_t)stream>>>(cwin, max_shift, *params, results, tw);
  return launched("k_peaks");
}

extern "C" int zr_full_prepare(float* planes, int n, int C, int suppress_origin, float* origin, float* mean,
                               void* stream) {
  if (!planes || !origin || !mean) return set_error(ZR_EINVAL, "zr_full_prepare: null argument");
  if (n <= 0) return ZR_OK;
  if (C < 32 || C > 8192 || (C & 1)) return set_error(ZR_ESIZE, "zr_full_prepare: plane side %d", C);
  k_full_prepare<<<n, 1024, 0, (cudaStream_t)stream>>>(planes, C, suppress_origin, origin, mean);
  return launched("k_full_prepare");
}

extern "C" size_t zr_full_work_bytes(int n_planes, int C) {
  const size_t filt_part = (size_t)n_planes * full_blocks(C) * 3 * sizeof(double);
  const size_t mask_part = (size_t)n_planes * FP_MBLK * 5 * sizeof(double);
  return (size_t)n_planes * C * C * sizeof(float) + (filt_part > mask_part ? filt_part : mask_part);
}

extern "C" int zr_full_filter(const float* planes, int n_planes, int C, const int* sel, int n_sel,
                              const float* weights, const int* radius, const float* mean, float* filtered,
                              double* stats, void* work, size_t work_bytes, void* stream) {
  if (!planes || !sel || !weights || !radius || !mean || !stats || !work)
    return set_error(ZR_EINVAL, "zr_full_filter: null argument");
  if (n_sel <= 0) return ZR_OK;
  if (n_sel > n_planes || C < 32 || C > 8192) return set_error(ZR_EINVAL, "zr_full_filter: bad sizes");
  if (work_bytes < zr_full_work_bytes(n_planes, C))
    return set_error(ZR_EWORK, "zr_full_filter: work buffer %zu < %zu", work_bytes, zr_full_work_bytes(n_planes, C));
  cudaStream_t st = (cudaStream_t)stream;
  float* tmp = (float*)work;
  double* part = (double*)((char*)work + (size_t)n_planes * C * C * sizeof(float));
  const dim3 grid((C + FP_TX - 1) / FP_TX, (C + FP_RY - 1) / FP_RY, n_sel);
  k_full_vert<<<grid, FP_T, 0, st>>>(planes, C, sel, weights, radius, tmp);
  ZR_TRY(launched("k_full_vert"));
  k_full_horz<<<grid, FP_T, 0, st>>>(tmp, C, sel, weights, radius, mean, filtered, part);
  ZR_TRY(launched("k_full_horz"));
  k_full_reduce<<<n_sel, 32, 0, st>>>(part, full_blocks(C), sel, stats);
  return launched("k_full_reduce");
}

extern "C" int zr_full_peaks(const float* planes, const float* filtered, int n_planes, int C, const int* sel,
                             int n_sel, int max_shift, const int* rolls, const float* mean, const float* origin,
                             const double* sigma, const int* nfev, int sub_pix_reg, zr_peak_result_t* results,
                             void* work, size_t work_bytes, void* stream) {
  if (!planes || !filtered || !sel || !rolls || !mean || !origin || !sigma || !nfev || !results || !work)
    return set_error(ZR_EINVAL, "zr_full_peaks: null argument");
  if (n_sel <= 0) return ZR_OK;
  if (n_sel > n_planes || C < 32 || C > 8192 || max_shift <= 0) return set_error(ZR_EINVAL, "zr_full_peaks: bad sizes");
  if (sub_pix_reg > 1 && (TWN % (16 * sub_pix_reg) != 0 || 16 * sub_pix_reg > 512))
    return set_error(ZR_ESIZE, "zr_full_peaks: subPixReg %d must be a power of two <= 32", sub_pix_reg);
  if (work_bytes < zr_full_work_bytes(n_planes, C))
    return set_error(ZR_EWORK, "zr_full_peaks: work buffer %zu < %zu", work_bytes, zr_full_work_bytes(n_planes, C));
  const float2* tw = twiddles();
  if (!tw) return ZR_ECUDA;
  cudaStream_t st = (cudaStream_t)stream;
  double* part = (double*)((char*)work + (size_t)n_planes * C * C * sizeof(float));
  k_full_masked<<<dim3(FP_MBLK, 1, n_sel), FP_T, 0, st>>>(filtered, C, sel, max_shift, rolls, mean, part);
  ZR_TRY(launched("k_full_masked"));
  const size_t smem = sub_pix_reg > 1 ? (size_t)17 * 16 * sub_pix_reg * sizeof(float2) : 16;
  ZR_TRY(cuda_check(cudaFuncSetAttribute(k_full_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "k_full_finish attr"));
  k_full_finish<<<n_sel, PK_T, smem, st>>>(planes, filtered, C, sel, part, mean, origin, sigma, nfev, sub_pix_reg,
                                           results, tw);
  return launched("k_full_finish");
}
