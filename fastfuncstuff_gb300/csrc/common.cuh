// Shared helpers of libffs_reml: status/error plumbing, warp reductions and the
// bf16 hi/lo split used by the tensor-core projection.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stdio.h>

#include <map>
#include <mutex>
#include <utility>

#include "../../include/ffs_reml.h"

namespace ffsk {

// Row stride of every K x T matrix the library stores (U, G, Q0, Xt): T
// rounded up to a multiple of 4, so each row starts on a 16-byte boundary;
// the padding samples are zero.
__host__ __device__ inline int ld_t(int T) { return (T + 3) & ~3; }

// Records a message for ffs_last_error() on the calling host thread.
void set_error(const char* fmt, ...);
void clear_error();

// Returns FFS_ERR_CUDA (with the CUDA message recorded) if a launch failed.
int check_launch(const char* what);

#define FFS_REQUIRE(cond, ...)                 \
  do {                                         \
    if (!(cond)) {                             \
      ::ffsk::set_error(__VA_ARGS__);           \
      return FFS_ERR_INVALID;                  \
    }                                          \
  } while (0)

#define FFS_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t _e = (call);                                                  \
    if (_e != cudaSuccess) {                                                  \
      ::ffsk::set_error("%s: %s", #call, cudaGetErrorString(_e));              \
      return FFS_ERR_CUDA;                                                    \
    }                                                                         \
  } while (0)

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// warp_sum of N values at once: the same butterfly per value (so the same
// sums), the N shuffle chains interleaved
template <int N>
__device__ __forceinline__ void warp_sum_n(float (&v)[N]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float t[N];
#pragma unroll
    for (int k = 0; k < N; ++k) t[k] = __shfl_xor_sync(0xffffffffu, v[k], o);
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] += t[k];
  }
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// x ~ hi + lo with hi = bf16(x), lo = bf16(x - hi): about 16 significant bits.
__device__ __forceinline__ void split_bf16(float x, uint16_t& hi, uint16_t& lo) {
  __nv_bfloat16 h = __float2bfloat16_rn(x);
  float r = __fsub_rn(x, __bfloat162float(h));
  __nv_bfloat16 l = __float2bfloat16_rn(r);
  hi = __bfloat16_as_ushort(h);
  lo = __bfloat16_as_ushort(l);
}

// x ~ hi + lo with hi = fp16(x), lo = fp16(x - hi): about 22 significant bits
// while |x| stays in fp16's normal range (the callers scale by a power of two).
__device__ __forceinline__ void split_fp16(float x, uint16_t& hi, uint16_t& lo) {
  __half h = __float2half_rn(x);
  float r = __fsub_rn(x, __half2float(h));
  __half l = __float2half_rn(r);
  hi = __half_as_ushort(h);
  lo = __half_as_ushort(l);
}

// Power of two that brings amax into [128, 256) (0 for amax == 0).
__device__ __forceinline__ int scale_exp(float amax) {
  if (!(amax > 0.f) || !isfinite(amax)) return 0;
  int e;
  frexpf(amax, &e);  // amax = f * 2^e, f in [0.5, 1)
  return 8 - e;
}

// float32 lambda in the reference's operation order, no contraction:
// (a+b)*(1+a*b) / ((1+b*b) + (2*a)*b)
__device__ __forceinline__ float lambda_f32(float a, float b) {
  float num = __fmul_rn(__fadd_rn(a, b), __fadd_rn(1.0f, __fmul_rn(a, b)));
  float den = __fadd_rn(__fadd_rn(1.0f, __fmul_rn(b, b)), __fmul_rn(__fmul_rn(2.0f, a), b));
  return __fdiv_rn(num, den);
}

__device__ __forceinline__ double lambda_f64(double a, double b) {
  double num = __dmul_rn(__dadd_rn(a, b), __dadd_rn(1.0, __dmul_rn(a, b)));
  double den = __dadd_rn(__dadd_rn(1.0, __dmul_rn(b, b)), __dmul_rn(__dmul_rn(2.0, a), b));
  return __ddiv_rn(num, den);
}

// The per-voxel output lambda: (b+a)*(1+a*b) / (((1+(2a)b) + b*b) + 1e-10), float32.
__device__ __forceinline__ float lambda_out_f32(float a, float b) {
  float num = __fmul_rn(__fadd_rn(b, a), __fadd_rn(1.0f, __fmul_rn(a, b)));
  float den = __fadd_rn(__fadd_rn(__fadd_rn(1.0f, __fmul_rn(__fmul_rn(2.0f, a), b)), __fmul_rn(b, b)),
                        1e-10f);
  return __fdiv_rn(num, den);
}

// Two floats in one 64-bit register and the packed f32x2 arithmetic on them
// (two independent round-to-nearest operations per instruction).
__device__ __forceinline__ uint64_t pack2(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void unpack2(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) only when a kernel needs
// more than it was last given on this device: launches then make no other
// runtime call than the launch itself (also while a stream is being captured).
inline cudaError_t ensure_dyn_smem(const void* fn, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t& have = done[{fn, dev}];
  if (bytes <= have) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) have = bytes;
  return e;
}

// SM count of the current device, looked up once per device
inline cudaError_t sm_count(int* n) {
  static std::mutex mu;
  static std::map<int, int> known;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  auto it = known.find(dev);
  if (it != known.end()) {
    *n = it->second;
    return cudaSuccess;
  }
  e = cudaDeviceGetAttribute(n, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) known[dev] = *n;
  return e;
}

}  // namespace ffsk
