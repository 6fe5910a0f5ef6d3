// letkf_common.cuh -- shared device helpers for the GB300 LETKF kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/letkf_gpu.h"

namespace letkf {

// launch bookkeeping shared by every translation unit (defined in abi.cu)
void note_launch();
int cuda_status(cudaError_t e);

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per kernel and device:
// later launches (including those recorded into a CUDA graph) skip the call.
template <typename K>
inline cudaError_t set_smem_once(K kern, size_t bytes, std::atomic<uint32_t>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint32_t bit = 1u << (dev & 31);
  if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
  return e;
}

// x*x + y*y with each operation rounded on its own (no FMA contraction), as
// the reference computes it without FMA and the oracle does with
// -ffp-contract=off: a distance exactly at a cut-off then tests the same way
__device__ __forceinline__ double sumsq_rn(double x, double y) {
  return __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
}

constexpr double kSigmaB = 0.04;  // common/common_letkf.f90:75 error stdev of parm_infl

// Newton-Schulz map of one eigenvalue of ZY, x (3 - x)^2 / 4
__device__ __forceinline__ float f_ns(float x) {
  const float t = 3.f - x;
  return 0.25f * x * t * t;
}

// Newton-Schulz step scale a >= 1 for a spectrum of ZY in [lo, 1 + d], d = 0.02:
// the a with f(a lo) = f(a (1 + d)), a = 3 (1 - sqrt(l)) / (1 - l^1.5) / (1 + d),
// l = lo / (1 + d); S <- sqrt(a) S (3I - aZY) / 2 maps eigenvalue x to f(a x)
__device__ __forceinline__ float ns_scale(float lo) {
  const float d1 = 1.02f;
  const float l = fminf(fmaxf(lo / d1, 0.f), 0.999f);
  const float r = sqrtf(l);
  const float al = 3.f * (1.f - r) / ((1.f - l * r) * d1);
  return fmaxf(al, 1.f);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Block-wide sum; `red` holds >= 32 elements of scratch.  All threads get the result.
template <typename T, int NT>
__device__ __forceinline__ T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  T s = T(0);
  if (w == 0) {
    s = lane < NT / 32 ? red[lane] : T(0);
    s = warp_sum(s);
    if (lane == 0) red[0] = s;
  }
  __syncthreads();
  s = red[0];
  return s;
}

// Block-wide sums of K values at once (two barriers instead of three per
// value); `red` holds >= K * NT / 32 elements.  Every thread gets the sums.
template <typename T, int NT, int K>
__device__ __forceinline__ void block_sum_k(T (&v)[K], T* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < K; i++) v[i] = warp_sum(v[i]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < K; i++) red[w * K + i] = v[i];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < K; i++) {
    T s = T(0);
#pragma unroll
    for (int q = 0; q < NT / 32; q++) s += red[q * K + i];
    v[i] = s;
  }
}

// Fortran SIGN(a,b)
__device__ __forceinline__ double fsign(double a, double b) { return copysign(fabs(a), b); }
__device__ __forceinline__ float fsignf(float a, float b) { return copysignf(fabsf(a), b); }

}  // namespace letkf
