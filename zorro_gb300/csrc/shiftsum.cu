// Shift every frame and sum (applyShifts, zorro.py:1734-1808, with
// lanczosIndexedShift, zorro_util.py:341-379), plus the even/odd half sums of
// lazyFouRingCorr (zorro.py:2237-2238), in one pass over the raw frames.
//
// Frame n is rolled by (roll_y, roll_x) (np.roll: out[i] = in[i - shift],
// circular; the offsets are given reduced to [0, H) and [0, W)), then convolved with the separable 3x3 kernel ky (x) kx
// (scipy.ndimage.convolve: out[i] = sum_k w[k] in[i - k + 1], 'reflect'
// borders of the rolled frame).  Sums run over frames in order in float32,
// as np.sum(images, axis=0) does for a float32 stack.
#include "common.cuh"
#include "internal.h"

namespace zr {

constexpr int SS_TX = 64, SS_TY = 16, SS_THR = 256;
#ifndef ZR_SS_MINB
#define ZR_SS_MINB 8
#endif

__device__ __forceinline__ int refl1(int i, int n) { return i < 0 ? -i - 1 : (i >= n ? 2 * n - i - 1 : i); }

// One raw value of the compile-time type TYPE, as float.
template <int TYPE>
__device__ __forceinline__ float raw_at(const void* raw, long long idx) {
  if constexpr (TYPE == ZR_U8) return (float)__ldg((const uint8_t*)raw + idx);
  if constexpr (TYPE == ZR_U16) return (float)__ldg((const uint16_t*)raw + idx);
  if constexpr (TYPE == ZR_F16) return __half2float(__ldg((const __half*)raw + idx));
  return __ldg((const float*)raw + idx);
}

// A CTA owns a 64 x 16 output tile and walks the frames in order.  The halo
// tile of frame n+1 (the corrected values at the rolled, reflected source
// pixels) is loaded into registers while frame n is filtered; the three
// running sums live in shared memory, which leaves the registers for the
// loads in flight at eight resident CTAs per SM.
//
// Each thread filters four rows of one column: the six horizontal 3-tap
// results it needs are computed once and slid down its rows for the vertical
// taps (the same products and sums as tap by tap).  The even and odd sums are
// kept only with HALVES (the lazy FRC reads them).
//
// With VEC (arrays aligned for vector loads), a frame whose 66 source columns
// of this tile are one contiguous run (the tile away from the left and right
// edges and the roll not wrapping inside it: nearly every tile) is read in
// 4-pixel chunks: each of the 18 halo rows is 18 aligned chunks of the raw
// frame, the gain and the hot-pixel maps, corrected in registers and written
// to the tile columns they cover.  Other frames read pixel by pixel.  Both
// paths apply the same operations to every pixel.
constexpr int SS_TW = SS_TX + 2, SS_TH = SS_TY + 2;
constexpr int SS_NCH = 18;                                    // chunks per halo row
constexpr int SS_VT = SS_TH * SS_NCH;                         // chunk tasks per tile
constexpr int SS_VPT = (SS_VT + SS_THR - 1) / SS_THR;         // chunk tasks per thread
constexpr int SS_LPT = (SS_TH * SS_TW + SS_THR - 1) / SS_THR;  // pixel tasks per thread
constexpr int SS_PRE = SS_LPT > 4 * SS_VPT ? SS_LPT : 4 * SS_VPT;

template <int TYPE>
__device__ __forceinline__ float corrected_at(const FrameSrc& f, long long fo, long long p) {
  float v = raw_at<TYPE>(f.raw, fo + p);
  if (f.gain) v = __fmul_rn(__ldg(f.gain + p), v);
  if (f.gdiv != 0.0f) v = __fdiv_rn(v, f.gdiv);
  if (f.ha) v = __fmaf_rn(__ldg(f.ha + p), v, __ldg(f.hb + p));
  return v;
}

template <int TYPE, bool VEC, bool HALVES>
__global__ void __launch_bounds__(SS_THR, ZR_SS_MINB)
    k_shift_sum(FrameSrc f, const zr_shift_t* __restrict__ sh, float* __restrict__ sum,
                float* __restrict__ even, float* __restrict__ odd, float* __restrict__ aligned) {
  __shared__ float tile[SS_TH][SS_TW];
  __shared__ float acc[HALVES ? 3 : 1][SS_TY][SS_TX];  // all frames (, even frames, odd frames)
  const int x0 = blockIdx.x * SS_TX, y0 = blockIdx.y * SS_TY;
  const int tx = threadIdx.x & (SS_TX - 1), ty = threadIdx.x / SS_TX;  // ty in [0,4)
  constexpr int RPT = SS_TY / (SS_THR / SS_TX);                            // rows per thread (4)
#pragma unroll
  for (int i = 0; i < RPT; i++) {
    acc[0][ty * RPT + i][tx] = 0.0f;
    if (HALVES) acc[1][ty * RPT + i][tx] = acc[2][ty * RPT + i][tx] = 0.0f;
  }
  const int H = f.H, W = f.W;
  constexpr int TE = SS_TH * SS_TW;
  const bool x_inside = x0 >= 1 && x0 + SS_TX + 1 <= W;  // halo columns x0-1 .. x0+64 all in [0, W)
  float pre[SS_PRE];
  int jb[SS_VPT];  // vector path: tile column of each chunk's first pixel
  bool vec_next = false;
  // roll offsets arrive reduced to [0, H) and [0, W)
  auto fetch = [&](int n) {
    const zr_shift_t t = sh[n];
    const long long fo = (long long)n * f.fstride;
    int c0 = x0 - 1 - t.roll_x;
    if (c0 < 0) c0 += W;
    vec_next = VEC && x_inside && c0 + SS_TW <= W;
    if (VEC && vec_next) {
      const long long HW = (long long)H * W;
#pragma unroll
      for (int v = 0; v < SS_VPT; v++) {
        const int task = threadIdx.x + v * SS_THR;
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        int j0 = 0;
        if (task < SS_VT) {
          const int i = task / SS_NCH, k = task - (task / SS_NCH) * SS_NCH;
          j0 = 4 * k;
          const int gy = y0 - 1 + i;
          if (gy < H + 1) {
            int sy = refl1(gy, H) - t.roll_y;
            if (sy < 0) sy += H;
            const long long p0 = (long long)sy * W + c0;  // source of tile column 0
            const long long a = (p0 & ~3LL) + 4 * k;      // this chunk's first pixel
            j0 = (int)(a - p0);
            if (a < p0 + SS_TW) {
              if (a + 4 <= HW) {
                float4 r = quad_value<TYPE>(raw_quad<TYPE>(f.raw, fo + a));
                if (f.gain) {
                  const float4 g = __ldg(reinterpret_cast<const float4*>(f.gain + a));
                  r = make_float4(__fmul_rn(g.x, r.x), __fmul_rn(g.y, r.y), __fmul_rn(g.z, r.z), __fmul_rn(g.w, r.w));
                }
                if (f.gdiv != 0.0f)
                  r = make_float4(__fdiv_rn(r.x, f.gdiv), __fdiv_rn(r.y, f.gdiv), __fdiv_rn(r.z, f.gdiv),
                                  __fdiv_rn(r.w, f.gdiv));
                if (f.ha) {
                  const float4 A = __ldg(reinterpret_cast<const float4*>(f.ha + a));
                  const float4 B = __ldg(reinterpret_cast<const float4*>(f.hb + a));
                  r = make_float4(__fmaf_rn(A.x, r.x, B.x), __fmaf_rn(A.y, r.y, B.y), __fmaf_rn(A.z, r.z, B.z),
                                  __fmaf_rn(A.w, r.w, B.w));
                }
                q = r;
              } else {
                // the chunk runs past the end of the frame: its pixels of the run only
                if (a >= p0) q.x = corrected_at<TYPE>(f, fo, a);
                if (a + 1 >= p0 && a + 1 < p0 + SS_TW) q.y = corrected_at<TYPE>(f, fo, a + 1);
                if (a + 2 >= p0 && a + 2 < p0 + SS_TW) q.z = corrected_at<TYPE>(f, fo, a + 2);
                if (a + 3 >= p0 && a + 3 < p0 + SS_TW) q.w = corrected_at<TYPE>(f, fo, a + 3);
              }
            }
          }
        }
        pre[4 * v] = q.x;
        pre[4 * v + 1] = q.y;
        pre[4 * v + 2] = q.z;
        pre[4 * v + 3] = q.w;
        jb[v] = j0;
      }
      return;
    }
#pragma unroll
    for (int l = 0; l < SS_LPT; l++) {
      const int e = threadIdx.x + l * SS_THR;
      pre[l] = 0.0f;
      if (e < TE) {
        const int i = e / SS_TW, j = e - i * SS_TW;
        if (y0 - 1 + i < H + 1 && x0 - 1 + j < W + 1) {
          const int Y = refl1(y0 - 1 + i, H), X = refl1(x0 - 1 + j, W);
          int sy = Y - t.roll_y;
          if (sy < 0) sy += H;
          int sx = X - t.roll_x;
          if (sx < 0) sx += W;
          pre[l] = corrected_at<TYPE>(f, fo, (long long)sy * W + sx);
        }
      }
    }
  };
  fetch(0);
  for (int n = 0; n < f.N; n++) {
    const zr_shift_t t = sh[n];
    __syncthreads();
    if (VEC && vec_next) {
#pragma unroll
      for (int v = 0; v < SS_VPT; v++) {
        const int task = threadIdx.x + v * SS_THR;
        if (task < SS_VT) {
          const int i = task / SS_NCH;
#pragma unroll
          for (int e = 0; e < 4; e++) {
            const int j = jb[v] + e;
            if (j >= 0 && j < SS_TW) tile[i][j] = pre[4 * v + e];
          }
        }
      }
    } else {
#pragma unroll
      for (int l = 0; l < SS_LPT; l++) {
        const int e = threadIdx.x + l * SS_THR;
        if (e < TE) tile[e / SS_TW][e % SS_TW] = pre[l];
      }
    }
    __syncthreads();
    if (n + 1 < f.N) fetch(n + 1);
    const int x = x0 + tx, ly0 = ty * RPT;
    float* const arow = aligned ? aligned + (size_t)n * H * W : nullptr;
    auto emit = [&](int i, float a) {
      const int y = y0 + ly0 + i;
      acc[0][ly0 + i][tx] += a;
      if (HALVES) acc[1 + (n & 1)][ly0 + i][tx] += a;
      if (arow && y < H && x < W) arow[(size_t)y * W + x] = a;
    };
    if (t.apply) {
      auto hrow = [&](int r) {
        return fmaf(t.kx[0], tile[r][tx + 2], fmaf(t.kx[1], tile[r][tx + 1], t.kx[2] * tile[r][tx]));
      };
      float h0 = hrow(ly0), h1 = hrow(ly0 + 1);
#pragma unroll
      for (int i = 0; i < RPT; i++) {
        const float h2 = hrow(ly0 + i + 2);
        emit(i, fmaf(t.ky[0], h2, fmaf(t.ky[1], h1, t.ky[2] * h0)));
        h0 = h1;
        h1 = h2;
      }
    } else {
#pragma unroll
      for (int i = 0; i < RPT; i++) emit(i, tile[ly0 + i + 1][tx + 1]);
    }
  }
  const int x = x0 + tx;
#pragma unroll
  for (int i = 0; i < RPT; i++) {
    const int y = y0 + ty * RPT + i;
    if (y < H && x < W) {
      const size_t p = (size_t)y * W + x;
      sum[p] = acc[0][ty * RPT + i][tx];
      if (HALVES) {
        if (even) even[p] = acc[1][ty * RPT + i][tx];
        if (odd) odd[p] = acc[2][ty * RPT + i][tx];
      }
    }
  }
}

}  // namespace zr

using namespace zr;

extern "C" int zr_shift_sum(const zr_frames_t* frames, const zr_shift_t* shifts, float* image_sum, float* even_sum,
                            float* odd_sum, float* aligned, void* stream) {
  if (frames && frames->frame_movie)
    return set_error(ZR_EINVAL, "zr_shift_sum: one movie at a time (frame_movie must be NULL)");
  if (!frames || !frames->raw || !shifts || !image_sum) return set_error(ZR_EINVAL, "zr_shift_sum: null argument");
  FrameSrc f = make_src(frames);
  if (f.N <= 0 || f.H < 2 || f.W < 2) return set_error(ZR_EINVAL, "zr_shift_sum: empty movie");
  dim3 grid((f.W + SS_TX - 1) / SS_TX, (f.H + SS_TY - 1) / SS_TY);
  cudaStream_t st = (cudaStream_t)stream;
  // chunked reads: every array aligned for its 4-pixel vector load at any
  // pixel index that is a multiple of 4
  const int qbytes = f.type == ZR_U8 ? 4 : (f.type == ZR_F32 ? 16 : 8);
  const bool vec = f.fstride % 4 == 0 && ((uintptr_t)f.raw % qbytes) == 0 && ((uintptr_t)f.gain & 15) == 0 &&
                   ((uintptr_t)f.ha & 15) == 0 && ((uintptr_t)f.hb & 15) == 0;
  const bool halves = even_sum || odd_sum;
#define ZR_SS_LAUNCH(T)                                                                                             \
  (vec ? (halves ? k_shift_sum<T, true, true><<<grid, SS_THR, 0, st>>>(f, shifts, image_sum, even_sum, odd_sum, aligned)   \
                 : k_shift_sum<T, true, false><<<grid, SS_THR, 0, st>>>(f, shifts, image_sum, even_sum, odd_sum, aligned)) \
       : (halves ? k_shift_sum<T, false, true><<<grid, SS_THR, 0, st>>>(f, shifts, image_sum, even_sum, odd_sum, aligned)  \
                 : k_shift_sum<T, false, false><<<grid, SS_THR, 0, st>>>(f, shifts, image_sum, even_sum, odd_sum, aligned)))
  switch (f.type) {
    case ZR_U8: ZR_SS_LAUNCH(ZR_U8); break;
    case ZR_U16: ZR_SS_LAUNCH(ZR_U16); break;
    case ZR_F16: ZR_SS_LAUNCH(ZR_F16); break;
    case ZR_F32: ZR_SS_LAUNCH(ZR_F32); break;
    default: return set_error(ZR_EINVAL, "zr_shift_sum: raw type %d", f.type);
  }
#undef ZR_SS_LAUNCH
  return launched("k_shift_sum");
}
