/*
 * devcommon.cuh — device helpers shared by the kernels: the reference's cell
 * index clamps, type packing in float4.w, and block reductions.
 */
#ifndef FLIP_DEVCOMMON_CUH
#define FLIP_DEVCOMMON_CUH

#include "flipgpu_impl.h"
#include "refmath.h"
#include "../../include/flip_rng.h"

/* int i = fmax(0, fmin(gn-1, gn*p)) (src/sorter.cpp:35-37): the double
 * clamp of a float product is exact in float. */
__device__ __forceinline__ int cell_clamp(float p, float fn, int n) {
  return (int)fmaxf(0.0f, fminf((float)(n - 1), fn * p));
}

/* int i = fmin(N-1, fmax(0, p*N)) (src/flip3D.cpp:903-905, 944). */
__device__ __forceinline__ int cell_clamp_minmax(float p, float fn, int n) {
  return (int)fminf((float)(n - 1), fmaxf(0.0f, p * fn));
}

/* FLOAT x = max(0, min(cs, cs*p)) with the macros of src/utility.h:16-17
 * (src/corrector.cpp:59-61), truncated by the int parameter: range [0, n]. */
__device__ __forceinline__ int cell_clamp_macro(float p, float fn) {
  float v = fn * p;
  float mn = (fn > v) ? v : fn;
  float mx = (0.0f > mn) ? 0.0f : mn;
  return (int)mx;
}

/* (i, j, k) of linear index c over extents (., e1, e2), k fastest, in 32-bit
 * arithmetic (grids are at most 1024^3 cells or 1025 x 1024^2 faces, so
 * every index fits; 64-bit division costs several times more) */
__device__ __forceinline__ void decode_index(size_t c, int e1, int e2, int &i, int &j, int &k) {
  const unsigned c32 = (unsigned)c, u1 = (unsigned)e1, u2 = (unsigned)e2;
  const unsigned row = c32 / u2;
  k = (int)(c32 - row * u2);
  i = (int)(row / u1);
  j = (int)(row - (unsigned)i * u1);
}

__device__ __forceinline__ size_t cell_id(int n, int i, int j, int k) {
  return ((size_t)i * n + j) * n + k;
}

__device__ __forceinline__ float pack_type(uint8_t t) {
  return __int_as_float((int)t);
}
__device__ __forceinline__ int unpack_type(float w) { return __float_as_int(w); }

/* Deterministic block sum of doubles: fixed shuffle tree, then warp 0. */
template <int BLOCK>
__device__ __forceinline__ double block_sum_double(double v) {
  __shared__ double warp_part[BLOCK / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_part[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = (lane < BLOCK / 32) ? warp_part[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r; /* valid in thread 0 */
}

template <int BLOCK>
__device__ __forceinline__ uint32_t block_sum_u32(uint32_t v) {
  __shared__ uint32_t warp_part[BLOCK / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_part[wid] = v;
  __syncthreads();
  uint32_t r = 0;
  if (wid == 0) {
    r = (lane < BLOCK / 32) ? warp_part[lane] : 0u;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;
}

/* Double-float accumulator: hi + lo carries about 44+ significant bits with
 * FP32 instructions only (Knuth TwoSum; products split exactly by FMA). Used
 * for dot products, where per-element FP64 is GB300's bottleneck. */
struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff_zero() { return FF{0.0f, 0.0f}; }

/* acc += b (b a float) */
__device__ __forceinline__ void ff_add(FF &a, float b) {
  float s, e;
  refmath::two_sum(a.hi, b, s, e);
  a.hi = s;
  a.lo += e;
}

/* acc += x*y with the product kept exact */
__device__ __forceinline__ void ff_add_prod(FF &a, float x, float y) {
  float p = x * y;
  float pe = fmaf(x, y, -p);
  ff_add(a, p);
  a.lo += pe;
}

__device__ __forceinline__ FF ff_merge(FF a, FF b) {
  float s, e;
  refmath::two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  float hi = s + e;
  float lo = e - (hi - s);
  return FF{hi, lo};
}

__device__ __forceinline__ FF ff_shfl_down(FF v, int o) {
  return FF{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

/* Block sum in a fixed tree; the result is valid in every thread. */
template <int BLOCK> __device__ __forceinline__ FF block_sum_ff(FF v) {
  __shared__ FF warp_part[BLOCK / 32];
  __shared__ FF total;
  for (int o = 16; o > 0; o >>= 1) v = ff_merge(v, ff_shfl_down(v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_part[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    FF t = warp_part[0];
    for (int i = 1; i < BLOCK / 32; i++) t = ff_merge(t, warp_part[i]);
    total = t;
  }
  __syncthreads();
  FF r = total;
  __syncthreads();
  return r;
}

__device__ __forceinline__ double ff_to_double(FF v) { return (double)v.hi + (double)v.lo; }

#endif
