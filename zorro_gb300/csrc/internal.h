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
// (the reference's default Fourier crop is 3072; 6144 pads the 5760-pixel
// side of binned K3 super-resolution frames).
inline bool fft_len_ok(long long v) {
  return is_pow2(v) || v == 384 || v == 768 || v == 1536 || v == 3072 || v == 6144;
}
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
// CTAs of T threads per SM to ask the register allocator for, so that
// ZR_SM_THREADS threads fit an SM (512: up to 128 registers a thread).
#ifndef ZR_SM_THREADS
#define ZR_SM_THREADS 512
#endif
__host__ __device__ constexpr int sm_minb(int T) { return T >= ZR_SM_THREADS ? 1 : ZR_SM_THREADS / T; }

// Launch variants of the transform kernels, chosen per transform length by
// the planner (zr_plan) or set from saved choices (zr_plan_set): sequences
// per CTA of the forward row and column passes and of the correlation column
// and row passes.  A variant changes only how the work is split between
// CTAs, never the arithmetic of a transform.  0 in the table means the
// built-in default.
enum TuneStage { TUNE_FWD_ROWS = 0, TUNE_FWD_COLS = 1, TUNE_XC_COLS = 2, TUNE_XC_ROWS = 3, TUNE_STAGES = 4 };
int tune_get(int stage, int length);
int tune_set(int stage, int length, int value);

}  // namespace zr

#define ZR_TRY(expr)            \
  do {                          \
    int _zr_rc = (expr);        \
    if (_zr_rc != 0) return _zr_rc; \
  } while (0)
