// Shared host/device utilities of libpadenti_gb300: error reporting, exact
// float helpers (one IEEE operation each, never contracted into an FMA), and a
// grow-only device buffer.
#pragma once

#if defined(__CUDACC_RTC__)
// compiled at run time by NVRTC (user feature plugins): device code only
typedef signed char int8_t;
typedef unsigned char uint8_t;
typedef short int16_t;
typedef unsigned short uint16_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
#else
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#endif

#include "padenti_gb300.h"

#if defined(__CUDACC__)
#define PD_HD __host__ __device__ __forceinline__
#define PD_D __device__ __forceinline__
#else
#define PD_HD inline
#define PD_D inline
#endif

namespace pd {

#if !defined(__CUDACC_RTC__)
// ---------------------------------------------------------------- errors ----
int set_error(int code, const char *fmt, ...);
const char *last_error();

#define PD_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t pd_err_ = (call);                                                  \
    if (pd_err_ != cudaSuccess)                                                    \
      return ::pd::set_error(PD_ERR_CUDA, "%s failed: %s (%s:%d)", #call,           \
                             cudaGetErrorString(pd_err_), __FILE__, __LINE__);      \
  } while (0)

#define PD_CHECK(cond, code, ...)                                                  \
  do {                                                                             \
    if (!(cond)) return ::pd::set_error((code), __VA_ARGS__);                      \
  } while (0)

#define PD_TRY(expr)                                                               \
  do {                                                                             \
    int pd_rc_ = (expr);                                                           \
    if (pd_rc_ != PD_OK) return pd_rc_;                                            \
  } while (0)
#endif

// ---------------------------------------------- exact scalar arithmetic ----
// Host code is compiled with -ffp-contract=off; device code uses the _rn
// intrinsics, so each helper is exactly one correctly rounded IEEE operation on
// both sides.
PD_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
PD_HD float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
PD_HD double dadd(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
PD_HD double dsub(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
PD_HD double dmul(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
PD_HD double ddiv(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
PD_HD float u2f(uint32_t v) {
#if defined(__CUDA_ARCH__)
  return __uint2float_rn(v);
#else
  return (float)v;
#endif
}

#if !defined(__CUDACC_RTC__)
// ------------------------------------------------------- device buffers ----
// Grow-only device allocation owned by a context.  Contents are not preserved
// across growth.
struct DevBuf {
  void *ptr = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return PD_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
      ptr = nullptr;
      cudaGetLastError();
      return set_error(PD_ERR_NOMEM, "cudaMalloc(%zu bytes) failed: %s", want, cudaGetErrorString(e));
    }
    cap = want;
    return PD_OK;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

// Grow-only page-locked host buffer (staging for host -> device copies).
struct HostBuf {
  void *ptr = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return PD_OK;
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    cap = 0;
    cudaError_t e = cudaMallocHost(&ptr, bytes);
    if (e != cudaSuccess) {
      ptr = nullptr;
      cudaGetLastError();
      return set_error(PD_ERR_NOMEM, "cudaMallocHost(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
    }
    cap = bytes;
    return PD_OK;
  }
  void release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

inline size_t feat_size(int feat_type) { return feat_type == PD_FEAT_I16 ? 2 : 4; }
inline size_t img_size(int img_type) {
  return img_type == PD_IMG_U8 ? 1 : (img_type == PD_IMG_U16 || img_type == PD_IMG_I16 ? 2 : 4);
}

#endif

}  // namespace pd
