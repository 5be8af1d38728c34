// Shared device-side helpers for the Zorro movie-registration kernels.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/zorro_gb300.h"
#include "fft_core.cuh"

namespace zr {

// One movie's frames as the kernels read them.  The corrected value of
// pixel (y, x) of frame n is
//     v = float32(gain[y,x] * raw[n,y,x])          (loadData, zorro.py:3466)
//     v = v / gdiv                                  (zorro.py:3477-3478, if gdiv != 0)
//     v = ha[y,x] * v + hb[y,x]                     (hotpixFilter, zorro.py:2649)
// with each step skipped when its pointer (or gdiv) is null/zero.
struct FrameSrc {
  const void* raw;
  int type;  // ZR_F32, ZR_U8, ZR_U16, ZR_F16
  const float* gain;
  const float* ha;
  const float* hb;
  float gdiv;
  int N, H, W;
  long long fstride;  // elements between consecutive frames
  const int* fmap;    // frame -> movie whose maps it reads (null: one map set)
  long long mstride;  // elements between the maps of consecutive movies
};

__host__ inline FrameSrc make_src(const zr_frames_t* f) {
  FrameSrc s;
  s.raw = f->raw;
  s.type = f->raw_type;
  s.gain = f->gain;
  s.ha = f->hot_a;
  s.hb = f->hot_b;
  s.gdiv = f->gain_divisor;
  s.N = f->n_frames;
  s.H = f->height;
  s.W = f->width;
  s.fstride = f->frame_stride ? f->frame_stride : (long long)f->height * f->width;
  s.fmap = f->frame_movie;
  s.mstride = f->frame_movie ? f->map_stride : 0;
  return s;
}

// Offset of frame n's gain and hot-pixel maps (the batched path's frames
// read the maps of their own movie).
__device__ __forceinline__ long long map_off(const FrameSrc& f, int n) {
  return f.fmap ? (long long)__ldg(f.fmap + n) * f.mstride : 0;
}

__device__ __forceinline__ float load_raw(const FrameSrc& f, long long idx) {
  switch (f.type) {
    case ZR_U8: return (float)__ldg((const uint8_t*)f.raw + idx);
    case ZR_U16: return (float)__ldg((const uint16_t*)f.raw + idx);
    case ZR_F16: return __half2float(__ldg((const __half*)f.raw + idx));
    default: return __ldg((const float*)f.raw + idx);
  }
}

__device__ __forceinline__ float load_corrected(const FrameSrc& f, int n, int y, int x) {
  const long long q = (long long)y * f.W + x;
  float v = load_raw(f, (long long)n * f.fstride + q);
  const long long p = q + map_off(f, n);
  if (f.gain) v = __fmul_rn(__ldg(f.gain + p), v);
  if (f.gdiv != 0.0f) v = __fdiv_rn(v, f.gdiv);
  if (f.ha) v = __fmaf_rn(__ldg(f.ha + p), v, __ldg(f.hb + p));
  return v;
}

// Corrected values of the four consecutive pixels p..p+3 (flattened within
// the frame) of frame n.  Needs p % 4 == 0 and fstride % 4 == 0 (aligned
// vector loads of every array).
__device__ __forceinline__ float4 load4_corrected(const FrameSrc& f, int n, long long p) {
  const long long i = (long long)n * f.fstride + p;
  const long long pm = p + map_off(f, n);
  float4 v;
  switch (f.type) {
    case ZR_U8: {
      const uchar4 r = __ldg(reinterpret_cast<const uchar4*>((const uint8_t*)f.raw + i));
      v = make_float4(r.x, r.y, r.z, r.w);
      break;
    }
    case ZR_U16: {
      const ushort4 r = __ldg(reinterpret_cast<const ushort4*>((const uint16_t*)f.raw + i));
      v = make_float4(r.x, r.y, r.z, r.w);
      break;
    }
    case ZR_F16: {
      const __half* h = (const __half*)f.raw + i;
      const __half2 a = __ldg(reinterpret_cast<const __half2*>(h)), b = __ldg(reinterpret_cast<const __half2*>(h + 2));
      v = make_float4(__low2float(a), __high2float(a), __low2float(b), __high2float(b));
      break;
    }
    default: v = __ldg(reinterpret_cast<const float4*>((const float*)f.raw + i));
  }
  if (f.gain) {
    const float4 g = __ldg(reinterpret_cast<const float4*>(f.gain + pm));
    v = make_float4(__fmul_rn(g.x, v.x), __fmul_rn(g.y, v.y), __fmul_rn(g.z, v.z), __fmul_rn(g.w, v.w));
  }
  if (f.gdiv != 0.0f)
    v = make_float4(__fdiv_rn(v.x, f.gdiv), __fdiv_rn(v.y, f.gdiv), __fdiv_rn(v.z, f.gdiv), __fdiv_rn(v.w, f.gdiv));
  if (f.ha) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(f.ha + pm)), b = __ldg(reinterpret_cast<const float4*>(f.hb + pm));
    v = make_float4(__fmaf_rn(a.x, v.x, b.x), __fmaf_rn(a.y, v.y, b.y), __fmaf_rn(a.z, v.z, b.z),
                    __fmaf_rn(a.w, v.w, b.w));
  }
  return v;
}

// Raw bits of the four consecutive pixels at element i of the compile-time
// type TYPE (u8 in .x, u16/f16 in .x/.y, f32 in .x-.w; i a multiple of 4 and
// the array aligned for the vector load) and their values.
template <int TYPE>
__device__ __forceinline__ uint4 raw_quad(const void* raw, long long i) {
  uint4 r = make_uint4(0u, 0u, 0u, 0u);
  if (TYPE == ZR_U8) {
    r.x = __ldg(reinterpret_cast<const unsigned int*>((const uint8_t*)raw + i));
  } else if (TYPE == ZR_U16 || TYPE == ZR_F16) {
    const uint2 v = __ldg(reinterpret_cast<const uint2*>((const uint16_t*)raw + i));
    r.x = v.x;
    r.y = v.y;
  } else {
    r = __ldg(reinterpret_cast<const uint4*>((const float*)raw + i));
  }
  return r;
}

template <int TYPE>
__device__ __forceinline__ float4 quad_value(const uint4 r) {
  if (TYPE == ZR_U8)
    return make_float4((float)(r.x & 0xffu), (float)((r.x >> 8) & 0xffu), (float)((r.x >> 16) & 0xffu),
                       (float)(r.x >> 24));
  if (TYPE == ZR_U16)
    return make_float4((float)(r.x & 0xffffu), (float)(r.x >> 16), (float)(r.y & 0xffffu), (float)(r.y >> 16));
  if (TYPE == ZR_F16)
    return make_float4(__half2float(__ushort_as_half((unsigned short)(r.x & 0xffffu))),
                       __half2float(__ushort_as_half((unsigned short)(r.x >> 16))),
                       __half2float(__ushort_as_half((unsigned short)(r.y & 0xffffu))),
                       __half2float(__ushort_as_half((unsigned short)(r.y >> 16))));
  return make_float4(__uint_as_float(r.x), __uint_as_float(r.y), __uint_as_float(r.z), __uint_as_float(r.w));
}

// load4_corrected split in two, so that a thread can issue the loads of
// several pixel quads before it uses any: Px4 holds the raw bits and the map
// values of one quad; finish4 applies the same operations in the same order.
struct Px4 {
  uint4 raw;  // the quad's raw bits: u8 in .x, u16/f16 in .x/.y, f32 in .x-.w
  float4 g, a, b;
};

__device__ __forceinline__ void fetch4(const FrameSrc& f, int n, long long p, Px4& q) {
  const long long i = (long long)n * f.fstride + p;
  switch (f.type) {
    case ZR_U8: q.raw.x = __ldg(reinterpret_cast<const unsigned int*>((const uint8_t*)f.raw + i)); break;
    case ZR_U16:
    case ZR_F16: {
      const uint2 r = __ldg(reinterpret_cast<const uint2*>((const uint16_t*)f.raw + i));
      q.raw.x = r.x;
      q.raw.y = r.y;
      break;
    }
    default: q.raw = __ldg(reinterpret_cast<const uint4*>((const float*)f.raw + i));
  }
  const long long pm = p + map_off(f, n);
  if (f.gain) q.g = __ldg(reinterpret_cast<const float4*>(f.gain + pm));
  if (f.ha) {
    q.a = __ldg(reinterpret_cast<const float4*>(f.ha + pm));
    q.b = __ldg(reinterpret_cast<const float4*>(f.hb + pm));
  }
}

__device__ __forceinline__ float4 finish4(const FrameSrc& f, const Px4& q) {
  float4 v;
  switch (f.type) {
    case ZR_U8: {
      const unsigned int r = q.raw.x;
      v = make_float4((float)(r & 0xffu), (float)((r >> 8) & 0xffu), (float)((r >> 16) & 0xffu), (float)(r >> 24));
      break;
    }
    case ZR_U16:
      v = make_float4((float)(q.raw.x & 0xffffu), (float)(q.raw.x >> 16), (float)(q.raw.y & 0xffffu),
                      (float)(q.raw.y >> 16));
      break;
    case ZR_F16:
      v = make_float4(__half2float(__ushort_as_half((unsigned short)(q.raw.x & 0xffffu))),
                      __half2float(__ushort_as_half((unsigned short)(q.raw.x >> 16))),
                      __half2float(__ushort_as_half((unsigned short)(q.raw.y & 0xffffu))),
                      __half2float(__ushort_as_half((unsigned short)(q.raw.y >> 16))));
      break;
    default:
      v = make_float4(__uint_as_float(q.raw.x), __uint_as_float(q.raw.y), __uint_as_float(q.raw.z),
                      __uint_as_float(q.raw.w));
  }
  if (f.gain)
    v = make_float4(__fmul_rn(q.g.x, v.x), __fmul_rn(q.g.y, v.y), __fmul_rn(q.g.z, v.z), __fmul_rn(q.g.w, v.w));
  if (f.gdiv != 0.0f)
    v = make_float4(__fdiv_rn(v.x, f.gdiv), __fdiv_rn(v.y, f.gdiv), __fdiv_rn(v.z, f.gdiv), __fdiv_rn(v.w, f.gdiv));
  if (f.ha)
    v = make_float4(__fmaf_rn(q.a.x, v.x, q.b.x), __fmaf_rn(q.a.y, v.y, q.b.y), __fmaf_rn(q.a.z, v.z, q.b.z),
                    __fmaf_rn(q.a.w, v.w, q.b.w));
  return v;
}

__device__ __forceinline__ int ilog2c(int v) { return 31 - __clz(v); }

// Element i of the length-L complex sequence whose inverse FFT holds two real
// rows (row a in the real part, row b in the imaginary part), from the rows'
// half-plane spectra ``ra``/``rb`` (elements 0..L/2; null: a zero row):
// ga + i gb up to L/2, the Hermitian mirror conj(ga) + i conj(gb) above.
template <int L>
__device__ __forceinline__ float2 packed_rows(const float2* __restrict__ ra, const float2* __restrict__ rb, int i) {
  constexpr int half = L / 2;
  const int k = i <= half ? i : L - i;
  const float2 ga = ra ? __ldg(ra + k) : make_float2(0.0f, 0.0f);
  const float2 gb = rb ? __ldg(rb + k) : make_float2(0.0f, 0.0f);
  if (i == 0 || i == half) return make_float2(ga.x, gb.x);
  if (i < half) return make_float2(ga.x - gb.y, ga.y + gb.x);
  return make_float2(ga.x + gb.y, -ga.y + gb.x);
}

}  // namespace zr
