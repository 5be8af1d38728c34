// zr_xcorr_pairs_noalloc: the all-pairs correlation of zr_xcorr_pairs with
// its scratch taken from a fixed device array compiled into the library, for
// callers that may not allocate device memory at call time.
//
// The scratch is a file-scope __device__ array of ZR_XCORR_STATIC_SCRATCH
// bytes.  Its address is looked up once per device with cudaGetSymbolAddress
// (with that device current) and cached; the pairs are then processed in
// waves of floor(ZR_XCORR_STATIC_SCRATCH / per-pair bytes) by the same kernels
// as zr_xcorr_pairs.  No element of the scratch needs to start at zero: the
// column pass writes every element the row pass reads.  All calls on one
// device share the one array, so calls that overlap in time (different
// streams or threads without ordering between them) race on it.
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace zr {

static __device__ __align__(256) unsigned char g_xcorr_static_scratch[ZR_XCORR_STATIC_SCRATCH];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[64];

// Address of this device's copy of the scratch array (the current device).
static int static_scratch(void** out) {
  int dev = 0;
  ZR_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  if (dev < 0 || dev >= 64) return set_error(ZR_EINVAL, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    ZR_TRY(cuda_check(cudaGetSymbolAddress(&p, g_xcorr_static_scratch), "cudaGetSymbolAddress(static scratch)"));
    if (!p) return set_error(ZR_ECUDA, "cudaGetSymbolAddress returned no address for the static scratch");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return ZR_OK;
}

}  // namespace zr

using namespace zr;

extern "C" int zr_xcorr_pairs_noalloc(const void* G, const float* terms, const int* pairs, int M, int N, int C0,
                                      int C1, int max_shift, float* cwin, void* stream) {
  if (!G || !terms || !pairs || !cwin || N <= 0) return set_error(ZR_EINVAL, "zr_xcorr_pairs_noalloc: null argument");
  if (M <= 0) return ZR_OK;
  // sizes outside the kernels' range (crop, maxShift < 2) get zr_xcorr_pairs'
  // own ZR_ESIZE below; only a pair too large for the array is refused here
  const size_t per_pair =
      (C1 > 0 && max_shift > 0) ? (size_t)2 * max_shift * zr_spectrum_pitch(C1) * sizeof(float2) : 0;
  if (per_pair > (size_t)ZR_XCORR_STATIC_SCRATCH)
    return set_error(ZR_ESIZE,
                     "zr_xcorr_pairs_noalloc: one pair needs %zu bytes of scratch (crop %d, maxShift %d), more than "
                     "the %zu-byte static scratch; use zr_xcorr_pairs with a work buffer",
                     per_pair, C1, max_shift, (size_t)ZR_XCORR_STATIC_SCRATCH);
  void* scratch = nullptr;
  ZR_TRY(static_scratch(&scratch));
  return zr_xcorr_pairs(G, terms, pairs, M, N, C0, C1, max_shift, cwin, scratch, (size_t)ZR_XCORR_STATIC_SCRATCH,
                        stream);
}
