// Fused symmetrised accumulation of the T2 residual:
//   out[i,j,a,b] += coef * (X[i,j,a,b] + X[j,i,b,a])
// for X any strided 4-index view (fricc/friccsd.py:245-267 builds these as
// "tmp + tmp.transpose(1,0,3,2)" and adds them to t2new).  One pass over the
// output: a CTA takes one (i,j) pair and a 32 x 32 tile of (a,b); each of
// the two reads of X runs along whichever of its (a,b) indices is
// contiguous, through a shared-memory transpose when that index is a, so
// both stay coalesced; the output (C order) is read and written along b.
#include <cstdlib>

#include "common.cuh"

namespace {

constexpr int TD = 32, TR = 8;  // 32 x 32 tile, 32 x 8 threads

// tile[a'][b'] = x(a0 + a', b0 + b') for the plane (p, q) of X, read along b
// (rows of 32 b) or along a (then stored transposed)
__device__ __forceinline__ void load_tile(double (*tile)[TD + 1], const double* __restrict__ X, int64_t base,
                                          int64_t sa, int64_t sb, int64_t a0, int64_t b0, int64_t v_a, int64_t v_b,
                                          bool along_b) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < TD; r += TR) {
    if (along_b) {  // thread tx walks b
      const int64_t a = a0 + r, b = b0 + tx;
      tile[r][tx] = (a < v_a && b < v_b) ? X[base + a * sa + b * sb] : 0.0;
    } else {        // thread tx walks a
      const int64_t a = a0 + tx, b = b0 + r;
      tile[tx][r] = (a < v_a && b < v_b) ? X[base + a * sa + b * sb] : 0.0;
    }
  }
}

__global__ void __launch_bounds__(TD* TR) k_symadd(double* __restrict__ out, const double* __restrict__ X, int64_t o,
                                                    int64_t v, int64_t s0, int64_t s1, int64_t s2, int64_t s3,
                                                    double coef, int first_along_b, int second_along_b,
                                                    int64_t xr = 0) {
  __shared__ double t1[TD][TD + 1], t2[TD][TD + 1];
  // replica batches: blockIdx.z = r o^2 + ij; replica r's X starts xr
  // elements after the previous one's, its output o^2 v^2 after
  const unsigned oo = (unsigned)(o * o);  // blockIdx.z < 65536: 32-bit divisions
  const unsigned rep = blockIdx.z / oo;
  const int64_t ij = blockIdx.z - rep * oo;
  X += rep * xr;
  out += rep * o * o * v * v;
  const int64_t i = (unsigned)ij / (unsigned)o, j = ij - i * o;
  const int64_t a0 = (int64_t)blockIdx.y * TD, b0 = (int64_t)blockIdx.x * TD;
  // X[i,j,a,b] over (a,b): strides (s2, s3); X[j,i,b,a] over (a,b): strides (s3, s2)
  load_tile(t1, X, i * s0 + j * s1, s2, s3, a0, b0, v, v, first_along_b != 0);
  load_tile(t2, X, j * s0 + i * s1, s3, s2, a0, b0, v, v, second_along_b != 0);
  __syncthreads();
  const int tx = threadIdx.x, ty = threadIdx.y;
  double* orow = out + (ij * v) * v;
  for (int r = ty; r < TD; r += TR) {
    const int64_t a = a0 + r, b = b0 + tx;
    if (a < v && b < v) orow[a * v + b] += coef * (t1[r][tx] + t2[r][tx]);
  }
}

}  // namespace

extern "C" int fricc_symadd(double* out, const double* X, int64_t nocc, int64_t nvir, const int64_t strides[4],
                            double coef, void* stream) {
  if (!out || !X || !strides || nocc <= 0 || nvir <= 0) {
    fricc_set_error("symadd: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (nocc * nocc > 65535) {
    fricc_set_error("symadd: nocc^2 above the grid limit");
    return FRICC_ERR_ARG;
  }
  const int64_t s0 = strides[0], s1 = strides[1], s2 = strides[2], s3 = strides[3];
  // the first read walks (a,b) with strides (s2, s3), the second with (s3, s2)
  const int first_along_b = std::llabs(s3) <= std::llabs(s2) ? 1 : 0;
  const int second_along_b = std::llabs(s2) <= std::llabs(s3) ? 1 : 0;
  const dim3 grid((unsigned)fricc_cdiv(nvir, TD), (unsigned)fricc_cdiv(nvir, TD), (unsigned)(nocc * nocc));
  k_symadd<<<grid, dim3(TD, TR), 0, (cudaStream_t)stream>>>(out, X, nocc, nvir, s0, s1, s2, s3, coef, first_along_b,
                                                           second_along_b);
  fricc_note_launch();
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "symadd", __FILE__, __LINE__);
}

// R replicas: out [R][o][o][v][v] (C order), X replica r at X + r xr with
// the per-replica strides of fricc_symadd.
extern "C" int fricc_symadd_b(double* out, const double* X, int64_t R, int64_t nocc, int64_t nvir,
                              const int64_t strides[5], double coef, void* stream) {
  if (!out || !X || !strides || nocc <= 0 || nvir <= 0 || R < 1) {
    fricc_set_error("symadd_b: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (R * nocc * nocc > 65535) {
    fricc_set_error("symadd_b: replicas x nocc^2 above the grid limit");
    return FRICC_ERR_ARG;
  }
  const int64_t s0 = strides[1], s1 = strides[2], s2 = strides[3], s3 = strides[4];
  const int first_along_b = std::llabs(s3) <= std::llabs(s2) ? 1 : 0;
  const int second_along_b = std::llabs(s2) <= std::llabs(s3) ? 1 : 0;
  const dim3 grid((unsigned)fricc_cdiv(nvir, TD), (unsigned)fricc_cdiv(nvir, TD), (unsigned)(R * nocc * nocc));
  k_symadd<<<grid, dim3(TD, TR), 0, (cudaStream_t)stream>>>(out, X, nocc, nvir, s0, s1, s2, s3, coef, first_along_b,
                                                           second_along_b, strides[0]);
  fricc_note_launch();
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "symadd_b", __FILE__, __LINE__);
}
