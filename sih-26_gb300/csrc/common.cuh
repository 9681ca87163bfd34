// common.cuh -- device helpers shared by every kernel of the GB300 PDHG engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace sgb {

constexpr int kWarp = 32;

// Absent bound: +-inf or any magnitude at or above 1e30, exactly as is_finite_bound in the
// reference (include/sankhya/types.hpp:88-96).
__host__ __device__ __forceinline__ bool finite_bound(double v) {
  return !(isinf(v) || fabs(v) >= 1e30);
}
__host__ __device__ __forceinline__ bool finite_bound(float v) {
  return !(isinf(v) || fabsf(v) >= 1e30f);
}

// Projection onto [lo, hi] tolerant of infinite sides (src/pdhg/pdhg.cpp:68-72).
template <typename T>
__host__ __device__ __forceinline__ T project(T v, T lo, T hi) {
  if (finite_bound(lo) && v < lo) return lo;
  if (finite_bound(hi) && v > hi) return hi;
  return v;
}

// Projection onto [lo, hi] when an absent side is an IEEE infinity (lo <= hi): the same
// value as project() for every non-NaN input, in two min/max instructions.
// Programmatic dependent launch: a kernel launched with programmatic stream serialization
// (launch_after, below) may have its blocks placed while the previous kernel in the stream is
// still finishing. Before it reads anything that kernel wrote, it waits here for that kernel's
// completion and the visibility of its memory. In a kernel launched the ordinary way the wait
// returns at once.
__device__ __forceinline__ void grid_dependency_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Launches kernel<<<grid, threads, smem, s>>>(args...) with programmatic stream
// serialization: its blocks are placed on the SMs as the previous kernel's blocks leave them,
// instead of after the whole kernel and its launch; the kernel must call
// grid_dependency_wait() before its first read of the previous kernel's results. Returns the
// launch's error.
template <typename... Params, typename... Args>
inline cudaError_t launch_after(void (*kernel)(Params...), int grid, int threads, int smem,
                                cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(static_cast<unsigned>(grid));
  cfg.blockDim = dim3(static_cast<unsigned>(threads));
  cfg.dynamicSmemBytes = static_cast<size_t>(smem);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

__device__ __forceinline__ double clamp_box(double v, double lo, double hi) {
  return fmin(fmax(v, lo), hi);
}
__device__ __forceinline__ float clamp_box(float v, float lo, float hi) {
  return fminf(fmaxf(v, lo), hi);
}

// std::max / std::min semantics (comparison order matters for NaN).
__host__ __device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }
__host__ __device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }

// ---- Deterministic reductions ------------------------------------------------------------
// Every sum in the engine goes through these: a fixed xor-butterfly inside a warp, then the
// warps of a block in index order. With a fixed grid the result is bit-identical from run to
// run, so the step-size and restart decisions are reproducible.

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = dmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Sum of `v` over a group of G consecutive lanes (G a power of two <= 32); every lane of the
// group receives the total.
template <int G, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of NV values per thread. `scratch` holds NV * (blockDim/32) doubles. Thread 0
// receives the totals in out[]. All threads must call it.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* scratch, double (&out)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = warp_sum(v[q]);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) scratch[q * nwarps + warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double s = lane < nwarps ? scratch[q * nwarps + lane] : 0.0;
      s = warp_sum(s);
      out[q] = s;
    }
  }
  __syncthreads();
}

template <int NV>
__device__ __forceinline__ void block_max(double (&v)[NV], double* scratch, double (&out)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = warp_max(v[q]);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) scratch[q * nwarps + warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double s = lane < nwarps ? scratch[q * nwarps + lane] : 0.0;
      s = warp_max(s);
      out[q] = s;
    }
  }
  __syncthreads();
}

}  // namespace sgb
