// Shared definitions for the fricc_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>

// Status codes (FRICC_OK, FRICC_ERR_*) are those of the public C ABI.
#include "../../include/fricc_gb300.h"

// Device error word bits (written by kernels, read by the host after a sync).
#define FRICC_DEV_P_GT_ONE 1u
#define FRICC_DEV_TIMEOUT 2u
#define FRICC_DEV_INDEX 4u
#define FRICC_DEV_PIVOTAL 8u

// ---------------------------------------------------------------------------
// Split an FP64 value into a float pair hi + lo (|d - hi - lo| < 2^-47 |d|)
// with integer operations only.  GB300's FP64 unit (which also runs the
// double<->float conversions) issues 1/64 as fast as the FP32 lanes, so a
// conversion-based split (RN(d), RN(d - RN(d))) staged for every operand
// tile can cost as much as the FP32-pair arithmetic it feeds.  For
// 2^-74 <= |d| < 2^128 the pair is read off the bit pattern: hi keeps the
// top 24 significand bits (truncated), lo is the remaining 29-bit field
// rounded (half up) to 24 bits; both are then normal floats.  Zeros map to
// (d, 0); anything else (tiny, huge, inf, NaN) takes the conversion path.
// kept out of line: if-converted into the fast path, its FP64 instructions
// would issue (predicated off) for every element
static __device__ __noinline__ float2 split_f2_conv(double d) {
  const float h = __double2float_rn(d);
  return make_float2(h, __double2float_rn(d - (double)h));
}

__device__ __forceinline__ float2 split_f2_bits(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const int E = (int)((u >> 52) & 0x7ffu);
  const unsigned sgn = (unsigned)(u >> 32) & 0x80000000u;
  if (E >= 1023 - 74 && E <= 1023 + 127) {
    const unsigned long long M = u & 0xfffffffffffffull;
    const unsigned hib = sgn | ((unsigned)(E - 1023 + 127) << 23) | (unsigned)(M >> 29);
    const unsigned rest = (unsigned)(M & 0x1fffffffu);
    unsigned lob = sgn;  // +-0 when the low field is empty
    if (rest) {
      const int p = 31 - __clz((int)rest);  // leading bit, 0..28
      const int sh = p - 23;
      unsigned m;                           // 24-bit significand incl. the leading 1, or 2^24 after a carry
      if (sh <= 0) m = rest << (-sh);
      else m = (rest >> sh) + ((rest >> (sh - 1)) & 1u);
      const int ef = E - 1023 - 52 + p + 127;  // 1..230 on this path
      lob = sgn | (((unsigned)(ef - 1) << 23) + m);
    }
    return make_float2(__uint_as_float(hib), __uint_as_float(lob));
  }
  if ((u << 1) == 0ull) return make_float2(__uint_as_float(sgn), 0.0f);
  return split_f2_conv(d);
}

// float -> double, exactly, with integer operations (the conversion
// instruction runs on the slow FP64 unit); zeros, subnormals, inf and NaN
// take the conversion path.
static __device__ __noinline__ double f2d_conv(float f) { return (double)f; }

__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned long long sgn = (unsigned long long)(b & 0x80000000u) << 32;
  if (e != 0u && e != 255u)
    return __longlong_as_double((long long)(sgn | ((unsigned long long)(e + 896u) << 52) |
                                            ((unsigned long long)(b & 0x7fffffu) << 29)));
  if ((b & 0x7fffffffu) == 0u) return __longlong_as_double((long long)sgn);
  return f2d_conv(f);
}

// hi + lo of a float pair, rounded once to FP64
__device__ __forceinline__ double pair_to_f64(float hi, float lo) { return f2d_bits(hi) + f2d_bits(lo); }

// The second output of a paired systematic compression: the same tensor
// compressed with another draw (host value rn, or the double at rn_dev).
struct CompressPairOut {
  int64_t* flat;
  double* vals;
  unsigned long long* meta;
  double rn;
  const double* rn_dev;
};

void fricc_set_error(const char* fmt, ...);
int fricc_cuda_fail(cudaError_t e, const char* what, const char* file, int line);
int fricc_cuda_check(cudaError_t e, const char* what);  // FRICC_OK on success

#define FRICC_CUDA(call)                                                         \
  do {                                                                           \
    cudaError_t _e = (call);                                                     \
    if (_e != cudaSuccess) return fricc_cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define FRICC_LAUNCH_CHECK() FRICC_CUDA(cudaGetLastError())

// Stream-ordered scratch allocation (memory comes from the device's default
// pool, whose release threshold is raised once so freed blocks are reused).
int fricc_alloc(void** p, size_t bytes, cudaStream_t s);
void fricc_free(void* p, cudaStream_t s);

// Instrumentation: a count of every kernel this library launches, and CUDA
// event timing of the sparse contraction kernel (off unless enabled).
void fricc_note_launch(int n = 1);

// Launch-configuration overrides set by an autotuner (thread-local, so a
// tuning solver does not change other threads' launches); -1 = the built-in
// choice.  Knobs: FRICC_TUNE_SPMM_PPT (output pairs per thread of the
// float-pair sparse kernel: 1, 2 or 4), FRICC_TUNE_GEMM_TILE (the FP32-pair
// GEMM's tile: 0 = 64x64, 1 = 128x32, 2 = 32x128, 3 = 32x160),
// FRICC_TUNE_GEMM_COVER (CTAs per SM the GEMM's split K aims for, 1..16).
#define FRICC_TUNE_SPMM_PPT 0
#define FRICC_TUNE_GEMM_TILE 1
#define FRICC_TUNE_GEMM_COVER 2
// test only: before its look-back, tile 1 of a compression's compaction
// polls a word nothing sets this many times, then reports FRICC_DEV_TIMEOUT
// (the compaction itself then runs as usual, so every result stays valid)
#define FRICC_TUNE_TEST_WAIT 3
// the width in bits (10..13) of a compression's first select digit, which
// decides how many candidates the exact sort takes (never which are kept)
#define FRICC_TUNE_SELECT_BITS 4
// the float-pair sparse kernel as a persistent, q-tile-major launch of this
// many CTAs per SM (1..8; unset: one CTA per (bucket, q tile) item)
#define FRICC_TUNE_SPMM_PERSIST 5
#define FRICC_TUNE_KNOBS 6
int fricc_tune_get(int knob);
bool fricc_prof_on();
void fricc_prof_record(cudaStream_t st, bool start, double flops, int channel = 0);

template <class T>
inline int fricc_alloc_t(T** p, size_t n, cudaStream_t s) {
  return fricc_alloc(reinterpret_cast<void**>(p), n * sizeof(T) + 16, s);
}

__host__ __device__ inline int64_t fricc_cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------- warp/block
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned warp_id() { return threadIdx.x >> 5; }

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <class T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// Block-wide minimum; every thread gets the result.  smem: >= 32 T.
template <class T>
__device__ __forceinline__ T block_min(T v, T* smem) {
  v = warp_min(v);
  const int nw = blockDim.x >> 5;
  __syncthreads();
  if (lane_id() == 0) smem[warp_id()] = v;
  __syncthreads();
  T r = smem[0];
  for (int w = 1; w < nw; ++w) r = smem[w] < r ? smem[w] : r;
  __syncthreads();
  return r;
}

// Block-wide exclusive sum of int64 (thread order); returns the exclusive
// prefix and writes the block total into *total.  smem: >= 33 int64.
__device__ __forceinline__ int64_t block_excl_sum(int64_t v, int64_t* smem, int64_t* total) {
  int64_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t w = __shfl_up_sync(0xffffffffu, incl, o);
    if ((int)lane_id() >= o) incl += w;
  }
  const int nw = blockDim.x >> 5;
  __syncthreads();
  if (lane_id() == 31) smem[warp_id()] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (int w = 0; w < nw; ++w) {
      int64_t t = smem[w];
      smem[w] = run;
      run += t;
    }
    smem[32] = run;
  }
  __syncthreads();
  int64_t r = smem[warp_id()] + incl - v;
  *total = smem[32];
  __syncthreads();
  return r;
}

// Deterministic block sum of doubles (fixed tree for a fixed blockDim).
__device__ __forceinline__ double block_sum_det(double v, double* smem) {
  v = warp_sum(v);
  const int nw = blockDim.x >> 5;
  __syncthreads();
  if (lane_id() == 0) smem[warp_id()] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < nw; ++w) r += smem[w];
    smem[0] = r;
  }
  __syncthreads();
  r = smem[0];
  __syncthreads();
  return r;
}
