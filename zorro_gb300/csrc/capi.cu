// Library-wide C ABI pieces: error reporting, per-device initialisation and
// the twiddle table.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include "common.cuh"
#include "internal.h"

#define ZR_VERSION 100

namespace zr {

static thread_local char g_err[512] = "";

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return ZR_OK;
  return set_error(ZR_ECUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

static std::atomic<unsigned long long> g_launches{0};

int launched(const char* what) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cuda_check(cudaGetLastError(), what);
}

// W_TWN^k = exp(-2 pi i k / TWN), then its contiguous copies per
// sub-transform length (tw_compact_off), one table per device.
static __device__ float2 d_twiddle[TWN + TW_COMPACT];

static std::mutex g_init_mu;
static bool g_init_done[64];
static const float2* g_tw_ptr[64];

static int init_device(int dev) {
  std::lock_guard<std::mutex> lk(g_init_mu);
  if (dev < 0 || dev >= 64) return set_error(ZR_EINVAL, "device %d out of range", dev);
  if (g_init_done[dev]) return ZR_OK;
  int prev = 0;
  ZR_TRY(cuda_check(cudaGetDevice(&prev), "cudaGetDevice"));
  if (prev != dev) ZR_TRY(cuda_check(cudaSetDevice(dev), "cudaSetDevice"));
  static float2 host[TWN + TW_COMPACT];
  for (int k = 0; k < TWN; k++) {
    const double a = -2.0 * M_PI * (double)k / (double)TWN;
    host[k] = make_float2((float)cos(a), (float)sin(a));
  }
  for (int k = 0; k < TW_COMPACT; k++) host[TWN + k] = make_float2(0.0f, 0.0f);
  for (int M = 1; M <= 16384; M *= 2) {
    for (int j = 0; j < M; j++) host[TWN + tw_compact_off(M) + j] = host[(size_t)j * (TWN / M)];
    if (3 * M <= 12288)
      for (int j = 0; j < 3 * M; j++) host[TWN + tw_compact_off(3 * M) + j] = host[(size_t)j * (TWN / (3 * M))];
  }
  int rc = cuda_check(cudaMemcpyToSymbol(d_twiddle, host, sizeof(host)), "twiddle upload");
  void* p = nullptr;
  if (rc == ZR_OK) rc = cuda_check(cudaGetSymbolAddress(&p, d_twiddle), "twiddle address");
  if (prev != dev) cudaSetDevice(prev);
  if (rc != ZR_OK) return rc;
  g_tw_ptr[dev] = (const float2*)p;
  g_init_done[dev] = true;
  return ZR_OK;
}

// The planner's choices: per device, stage and transform length (a slot per
// supported length), the chosen sequences per CTA (0: the default).
static const int k_tune_lengths[] = {64, 128, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096, 6144};
constexpr int k_tune_nlen = sizeof(k_tune_lengths) / sizeof(k_tune_lengths[0]);
static int g_tune[64][TUNE_STAGES][k_tune_nlen];

static int tune_slot(int length) {
  for (int i = 0; i < k_tune_nlen; i++)
    if (k_tune_lengths[i] == length) return i;
  return -1;
}

int tune_get(int stage, int length) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || stage < 0 || stage >= TUNE_STAGES) return 0;
  const int k = tune_slot(length);
  return k < 0 ? 0 : g_tune[dev][stage][k];
}

int tune_set(int stage, int length, int value) {
  int dev = 0;
  ZR_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  if (dev < 0 || dev >= 64 || stage < 0 || stage >= TUNE_STAGES) return set_error(ZR_EINVAL, "tune_set: bad stage");
  const int k = tune_slot(length);
  if (k < 0) return set_error(ZR_ESIZE, "tune_set: transform length %d has no variants", length);
  if (value != 0 && value != 1 && value != 2 && value != 4)
    return set_error(ZR_EINVAL, "tune_set: %d sequences per CTA (1, 2 or 4; 0 for the default)", value);
  g_tune[dev][stage][k] = value;
  return ZR_OK;
}

const float2* twiddles() {
  int dev = 0;
  if (cuda_check(cudaGetDevice(&dev), "cudaGetDevice") != ZR_OK) return nullptr;
  if (dev < 0 || dev >= 64) return nullptr;
  if (!g_init_done[dev] && init_device(dev) != ZR_OK) return nullptr;
  return g_tw_ptr[dev];
}

}  // namespace zr

extern "C" int zr_version(void) { return ZR_VERSION; }

extern "C" int zr_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return (int)strlen(zr::g_err);
  strncpy(buf, zr::g_err, len - 1);
  buf[len - 1] = 0;
  return (int)strlen(buf);
}

extern "C" int zr_init(int device) { return zr::init_device(device); }

extern "C" unsigned long long zr_launch_count(void) { return zr::g_launches.load(); }
