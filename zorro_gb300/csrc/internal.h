// Internal helpers shared by the translation units of libzorrogb.
#pragma once
#include <cuda_runtime.h>

namespace zr {

// Record an error message for zr_last_error() and return ``code``.
int set_error(int code, const char* fmt, ...);
// Check a CUDA runtime result; on failure record it and return ZR_ECUDA.
int cuda_check(cudaError_t e, const char* what);
// Count one kernel launch and check it was accepted.
int launched(const char* what);
// Twiddle table of the current device (initialises it on first use).
const float2* twiddles();

inline bool is_pow2(long long v) { return v > 0 && (v & (v - 1)) == 0; }
// Transform lengths the library is built for: powers of two and 3 x 2^k
// (the reference's default Fourier crop is 3072).
inline bool fft_len_ok(long long v) { return is_pow2(v) || v == 384 || v == 768 || v == 1536 || v == 3072; }
inline int ilog2(long long v) {
  int l = 0;
  while ((1LL << l) < v) ++l;
  return l;
}

// Threads for a batched shared-memory FFT of NB sequences of length L:
// ZR_FFT_EPT elements per thread and pass (radix-8 butterflies of 8).
#ifndef ZR_FFT_EPT
#define ZR_FFT_EPT 32
#endif
#ifndef ZR_FFT_MINB
#define ZR_FFT_MINB 2
#endif
constexpr int fft_threads(int L, int NB, int ept = ZR_FFT_EPT) {
  return (NB * L / ept < 64) ? 64 : ((NB * L / ept > 512) ? 512 : NB * L / ept);
}
// Resident CTAs per SM to ask the register allocator for (short transforms).
constexpr int fft_minblocks(int L) { return L <= 2048 ? ZR_FFT_MINB : 1; }

}  // namespace zr

#define ZR_TRY(expr)            \
  do {                          \
    int _zr_rc = (expr);        \
    if (_zr_rc != 0) return _zr_rc; \
  } while (0)
