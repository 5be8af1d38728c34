// Unpacking of 4-bit movies (MRC mode 101, the packed counting frames that
// SerialEM writes and mrcz reads for zorro.loadData, zorro.py:3414-3425):
// two pixels per byte, the first in the low 4 bits, each row padded to a
// whole byte.  The packed bytes cross the host link (half the bytes of the
// uint8 frames) and are expanded here, in HBM, into the uint8 frames every
// other kernel reads.
#include "common.cuh"
#include "internal.h"

namespace zr {

// One thread per packed byte: its two pixels (the second dropped past the
// end of an odd-width row).  Rows are (W + 1) / 2 bytes.
__global__ void k_unpack_u4(const uint8_t* __restrict__ in, long long nbytes, int W, int RB,
                            uint8_t* __restrict__ out) {
  for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < nbytes;
       b += (long long)gridDim.x * blockDim.x) {
    const long long row = b / RB;
    const int x = 2 * (int)(b - row * RB);
    const uint8_t v = __ldg(in + b);
    uint8_t* o = out + row * W + x;
    o[0] = v & 0x0f;
    if (x + 1 < W) o[1] = v >> 4;
  }
}

// Even widths have no row padding: packed byte b holds pixels 2b and 2b+1
// of the whole stack.  16 packed bytes in, 32 pixels out per thread (16-byte
// loads and stores); the last (nbytes % 16) bytes by the scalar rule.
__device__ __forceinline__ unsigned int spread_nibbles(unsigned int x) {
  // bytes b1 b0 (low half of x) -> b1.hi b1.lo b0.hi b0.lo, one nibble a byte
  return (x & 0xFu) | ((x & 0xF0u) << 4) | ((x & 0xF00u) << 8) | ((x & 0xF000u) << 12);
}

__global__ void k_unpack_u4_flat(const uint4* __restrict__ in, long long n16, const uint8_t* __restrict__ tail_in,
                                 int ntail, uint4* __restrict__ out, uint8_t* __restrict__ tail_out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) {
    const uint4 v = __ldg(in + i);
    out[2 * i] = make_uint4(spread_nibbles(v.x), spread_nibbles(v.x >> 16), spread_nibbles(v.y),
                            spread_nibbles(v.y >> 16));
    out[2 * i + 1] = make_uint4(spread_nibbles(v.z), spread_nibbles(v.z >> 16), spread_nibbles(v.w),
                                spread_nibbles(v.w >> 16));
  }
  if (blockIdx.x == 0 && (int)threadIdx.x < ntail) {
    const uint8_t b = tail_in[threadIdx.x];
    tail_out[2 * threadIdx.x] = b & 0x0f;
    tail_out[2 * threadIdx.x + 1] = b >> 4;
  }
}

}  // namespace zr

using namespace zr;

extern "C" int zr_unpack_u4(const void* packed, int n_frames, int height, int width, void* frames, void* stream) {
  if (!packed || !frames) return set_error(ZR_EINVAL, "zr_unpack_u4: null argument");
  if (n_frames <= 0 || height <= 0 || width <= 0) return set_error(ZR_EINVAL, "zr_unpack_u4: empty movie");
  const int RB = (width + 1) / 2;
  const long long nbytes = (long long)n_frames * height * RB;
  const bool aligned16 = ((uintptr_t)packed % 16 == 0) && ((uintptr_t)frames % 16 == 0);
  if (width % 2 == 0 && aligned16) {
    const long long n16 = nbytes / 16;
    const int ntail = (int)(nbytes - 16 * n16);
    long long blocks = (n16 + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    k_unpack_u4_flat<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
        (const uint4*)packed, n16, (const uint8_t*)packed + 16 * n16, ntail, (uint4*)frames,
        (uint8_t*)frames + 32 * n16);
    return launched("k_unpack_u4_flat");
  }
  long long blocks = (nbytes + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  k_unpack_u4<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>((const uint8_t*)packed, nbytes, width, RB,
                                                                 (uint8_t*)frames);
  return launched("k_unpack_u4");
}
