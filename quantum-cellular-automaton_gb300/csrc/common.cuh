// Shared helpers for the qca_gb300 CUDA library: complex arithmetic, status
// codes, error capture and launch checking.  sm_103a only.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/qca_gb300.h"

namespace qca {

// ----------------------------------------------------------------------------------
// error capture: every C-ABI entry point returns an int status; the message of the
// last failure on this host thread is kept for qca_last_error().
// ----------------------------------------------------------------------------------
void set_error(const char* fmt, ...);
const char* last_error();

// Kernels launched by the TDVP engine's launch functions (process-wide): the
// engine's per-class statistics count kernels, not grouped-launch regions.
void count_launches(int k);
long long launches_so_far();

#define QCA_CUDA(call)                                                                    \
  do {                                                                                    \
    cudaError_t _e = (call);                                                              \
    if (_e != cudaSuccess) {                                                              \
      ::qca::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
      return QCA_ERR_CUDA;                                                                \
    }                                                                                     \
  } while (0)

#define QCA_LAUNCH_CHECK()                                                                 \
  do {                                                                                     \
    cudaError_t _e = cudaGetLastError();                                                   \
    if (_e != cudaSuccess) {                                                               \
      ::qca::set_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
      return QCA_ERR_CUDA;                                                                 \
    }                                                                                      \
  } while (0)

#define QCA_TRY(expr)          \
  do {                         \
    int _s = (expr);           \
    if (_s != QCA_OK) return _s; \
  } while (0)

// ----------------------------------------------------------------------------------
// complex numbers as plain structs (interleaved re, im: the layout of numpy complex)
// ----------------------------------------------------------------------------------
template <typename T>
struct alignas(2 * sizeof(T)) cplx {
  T re, im;
};
using c64 = cplx<float>;
using c128 = cplx<double>;

template <typename T>
__host__ __device__ __forceinline__ cplx<T> mk(T r, T i) {
  cplx<T> z;
  z.re = r;
  z.im = i;
  return z;
}
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator*(T s, cplx<T> a) { return mk(s * a.re, s * a.im); }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> conj(cplx<T> a) { return mk(a.re, -a.im); }
template <typename T>
__host__ __device__ __forceinline__ T norm2(cplx<T> a) { return a.re * a.re + a.im * a.im; }
// acc += a * b  (complex fused multiply-add)
template <typename T>
__host__ __device__ __forceinline__ void cfma(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(-a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im);
  acc.im = fma(a.im, b.re, acc.im);
}
// acc += conj(a) * b
template <typename T>
__host__ __device__ __forceinline__ void cfma_conj(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im);
  acc.im = fma(-a.im, b.re, acc.im);
}

// ----------------------------------------------------------------------------------
// Slot of the current device in per-device caches of one-time launch set-up
// (function attributes are per device); -1 when it cannot be used, and the caller
// then sets up on every launch.
constexpr int kMaxDevices = 64;
inline int device_slot() {
  int d = -1;
  if (cudaGetDevice(&d) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return d >= 0 && d < kMaxDevices ? d : -1;
}

// warp / block reductions in double precision
// ----------------------------------------------------------------------------------
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block; the result is valid in every thread.  `sh` needs 33 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double t = lane < nw ? sh[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace qca
