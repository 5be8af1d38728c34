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
template <int TYPE>
__global__ void __launch_bounds__(SS_THR, ZR_SS_MINB)
    k_shift_sum(FrameSrc f, const zr_shift_t* __restrict__ sh, float* __restrict__ sum,
                float* __restrict__ even, float* __restrict__ odd, float* __restrict__ aligned) {
  __shared__ float tile[SS_TY + 2][SS_TX + 2];
  __shared__ float acc[3][SS_TY][SS_TX];  // all frames, even frames, odd frames
  const int x0 = blockIdx.x * SS_TX, y0 = blockIdx.y * SS_TY;
  const int tx = threadIdx.x & (SS_TX - 1), ty = threadIdx.x / SS_TX;  // ty in [0,4)
  constexpr int RPT = SS_TY / (SS_THR / SS_TX);                            // rows per thread (4)
#pragma unroll
  for (int i = 0; i < RPT; i++) acc[0][ty * RPT + i][tx] = acc[1][ty * RPT + i][tx] = acc[2][ty * RPT + i][tx] = 0.0f;
  const int H = f.H, W = f.W;
  constexpr int TE = (SS_TY + 2) * (SS_TX + 2);
  constexpr int LPT = (TE + SS_THR - 1) / SS_THR;
  float pre[LPT];
  auto fetch = [&](int n) {
    const zr_shift_t t = sh[n];
    const long long fo = (long long)n * f.fstride;
#pragma unroll
    for (int l = 0; l < LPT; l++) {
      const int e = threadIdx.x + l * SS_THR;
      pre[l] = 0.0f;
      if (e < TE) {
        const int i = e / (SS_TX + 2), j = e - i * (SS_TX + 2);
        if (y0 - 1 + i < H + 1 && x0 - 1 + j < W + 1) {
          const int Y = refl1(y0 - 1 + i, H), X = refl1(x0 - 1 + j, W);
          // roll offsets arrive reduced to [0, H) and [0, W)
          int sy = Y - t.roll_y;
          if (sy < 0) sy += H;
          int sx = X - t.roll_x;
          if (sx < 0) sx += W;
          // the corrected value, in the order of load_corrected
          const long long p = (long long)sy * W + sx;
          float v = raw_at<TYPE>(f.raw, fo + p);
          if (f.gain) v = __fmul_rn(__ldg(f.gain + p), v);
          if (f.gdiv != 0.0f) v = __fdiv_rn(v, f.gdiv);
          if (f.ha) v = __fmaf_rn(__ldg(f.ha + p), v, __ldg(f.hb + p));
          pre[l] = v;
        }
      }
    }
  };
  fetch(0);
  for (int n = 0; n < f.N; n++) {
    const zr_shift_t t = sh[n];
    __syncthreads();
#pragma unroll
    for (int l = 0; l < LPT; l++) {
      const int e = threadIdx.x + l * SS_THR;
      if (e < TE) tile[e / (SS_TX + 2)][e % (SS_TX + 2)] = pre[l];
    }
    __syncthreads();
    if (n + 1 < f.N) fetch(n + 1);
    const int x = x0 + tx;
    float* const half_acc = acc[1 + (n & 1)][0];
#pragma unroll
    for (int i = 0; i < RPT; i++) {
      const int y = y0 + ty * RPT + i;
      float a;
      const int ly = ty * RPT + i + 1, lx = tx + 1;
      if (t.apply) {
        // sum_a ky[a] sum_b kx[b] R(y - a + 1, x - b + 1)
        float r0 = fmaf(t.kx[0], tile[ly + 1][lx + 1], fmaf(t.kx[1], tile[ly + 1][lx], t.kx[2] * tile[ly + 1][lx - 1]));
        float r1 = fmaf(t.kx[0], tile[ly][lx + 1], fmaf(t.kx[1], tile[ly][lx], t.kx[2] * tile[ly][lx - 1]));
        float r2 = fmaf(t.kx[0], tile[ly - 1][lx + 1], fmaf(t.kx[1], tile[ly - 1][lx], t.kx[2] * tile[ly - 1][lx - 1]));
        a = fmaf(t.ky[0], r0, fmaf(t.ky[1], r1, t.ky[2] * r2));
      } else {
        a = tile[ly][lx];
      }
      acc[0][ly - 1][tx] += a;
      half_acc[(ly - 1) * SS_TX + tx] += a;
      if (aligned && y < H && x < W) aligned[(size_t)n * H * W + (size_t)y * W + x] = a;
    }
  }
  const int x = x0 + tx;
#pragma unroll
  for (int i = 0; i < RPT; i++) {
    const int y = y0 + ty * RPT + i;
    if (y < H && x < W) {
      const size_t p = (size_t)y * W + x;
      sum[p] = acc[0][ty * RPT + i][tx];
      if (even) even[p] = acc[1][ty * RPT + i][tx];
      if (odd) odd[p] = acc[2][ty * RPT + i][tx];
    }
  }
}

}  // namespace zr

using namespace zr;

extern "C" int zr_shift_sum(const zr_frames_t* frames, const zr_shift_t* shifts, float* image_sum, float* even_sum,
                            float* odd_sum, float* aligned, void* stream) {
  if (!frames || !frames->raw || !shifts || !image_sum) return set_error(ZR_EINVAL, "zr_shift_sum: null argument");
  FrameSrc f = make_src(frames);
  if (f.N <= 0 || f.H < 2 || f.W < 2) return set_error(ZR_EINVAL, "zr_shift_sum: empty movie");
  dim3 grid((f.W + SS_TX - 1) / SS_TX, (f.H + SS_TY - 1) / SS_TY);
  cudaStream_t st = (cudaStream_t)stream;
  switch (f.type) {
    case ZR_U8: k_shift_sum<ZR_U8><<<grid, SS_THR, 0, st>>>(f, shifts, image_sum, even_sum, odd_sum, aligned); break;
    case ZR_U16: k_shift_sum<ZR_U16><<<grid, SS_THR, 0, st>>>(f, shifts, image_sum, even_sum, odd_sum, aligned); break;
    case ZR_F16: k_shift_sum<ZR_F16><<<grid, SS_THR, 0, st>>>(f, shifts, image_sum, even_sum, odd_sum, aligned); break;
    case ZR_F32: k_shift_sum<ZR_F32><<<grid, SS_THR, 0, st>>>(f, shifts, image_sum, even_sum, odd_sum, aligned); break;
    default: return set_error(ZR_EINVAL, "zr_shift_sum: raw type %d", f.type);
  }
  return launched("k_shift_sum");
}
