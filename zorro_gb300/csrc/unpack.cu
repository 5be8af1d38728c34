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

}  // namespace zr

using namespace zr;

extern "C" int zr_unpack_u4(const void* packed, int n_frames, int height, int width, void* frames, void* stream) {
  if (!packed || !frames) return set_error(ZR_EINVAL, "zr_unpack_u4: null argument");
  if (n_frames <= 0 || height <= 0 || width <= 0) return set_error(ZR_EINVAL, "zr_unpack_u4: empty movie");
  const int RB = (width + 1) / 2;
  const long long nbytes = (long long)n_frames * height * RB;
  long long blocks = (nbytes + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  k_unpack_u4<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>((const uint8_t*)packed, nbytes, width, RB,
                                                                 (uint8_t*)frames);
  return launched("k_unpack_u4");
}
