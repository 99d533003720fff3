// The reference's random stream, generated on the device.
//
// fri-cc draws its uniforms as rand() / RAND_MAX from glibc (src/fri_utils.cpp:47
// for systematic sampling, :73 once per element for pivotal sampling).  glibc's
// default generator (TYPE_3) is an additive lagged-Fibonacci recurrence on
// 32-bit words,
//     r_k = r_{k-31} + r_{k-3}  (mod 2^32),   rand() = r_k >> 1,
// so its whole state is the history h = (r_{k-31}, ..., r_{k-1}) before the
// next draw.  Advancing the history by one draw is a fixed 31x31 linear map M
// over Z/2^32; by C draws it is J = M^C, built on the host by repeated
// squaring.  One block walks the chunk starts h_{cC} = J h_{(c-1)C}, then one
// thread per chunk produces its C uniforms from its start, the ring of 31
// words held in registers (the loop is unrolled 31 deep so every ring index
// is static).  The history after the last draw goes back to the caller, so a
// host-side copy of the stream continues exactly where the device stopped.
#include <vector>

#include "common.cuh"

namespace {

constexpr int RDEG = 31;
constexpr int RSEP = 3;
constexpr int64_t GCH = 31 * 64;  // draws per chunk (a multiple of the ring length)

// out[c * 31 + t] = history at the start of chunk c (oldest first)
__global__ void k_glibc_starts(const unsigned* __restrict__ J, const unsigned* __restrict__ h0, int64_t nch,
                               unsigned* __restrict__ starts) {
  __shared__ unsigned h[RDEG];
  __shared__ unsigned Js[RDEG * RDEG];
  const int t = threadIdx.x;
  for (int i = t; i < RDEG * RDEG; i += blockDim.x) Js[i] = J[i];
  if (t < RDEG) h[t] = h0[t];
  __syncthreads();
  for (int64_t c = 0; c < nch; ++c) {
    unsigned nx = 0;
    if (t < RDEG) {
      starts[c * RDEG + t] = h[t];
      for (int s = 0; s < RDEG; ++s) nx += Js[t * RDEG + s] * h[s];  // wraps mod 2^32
    }
    __syncthreads();
    if (t < RDEG) h[t] = nx;
    __syncthreads();
  }
}

// chunk c: draws [c*GCH, min((c+1)*GCH, k)); the thread holding the last draw
// writes the history that follows it
__global__ void k_glibc_gen(const unsigned* __restrict__ starts, int64_t nch, int64_t k, double* __restrict__ out,
                            unsigned* __restrict__ hist_out) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nch) return;
  unsigned r[RDEG];
#pragma unroll
  for (int t = 0; t < RDEG; ++t) r[t] = starts[c * RDEG + t];
  const int64_t base = c * GCH;
  const int64_t cnt = k - base < GCH ? k - base : GCH;  // > 0
  int64_t done = 0;
  // ring: after d draws of a round the oldest word sits at index d
  while (done < cnt) {
#pragma unroll
    for (int d = 0; d < RDEG; ++d) {
      if (done + d < cnt) {
        const unsigned w = r[d] + r[(d + RDEG - RSEP) % RDEG];
        r[d] = w;
        out[base + done + d] = (double)(int)(w >> 1) / 2147483647.0;
      }
    }
    done += RDEG;
  }
  if (base + cnt == k) {
    // cnt draws leave the oldest word at ring index cnt % 31
    const int off = (int)(cnt % RDEG);
#pragma unroll
    for (int t = 0; t < RDEG; ++t) hist_out[t] = r[(off + t) % RDEG];
  }
}

using Mat = std::vector<unsigned>;

Mat mat_mul(const Mat& A, const Mat& B) {
  Mat C(RDEG * RDEG, 0u);
  for (int i = 0; i < RDEG; ++i)
    for (int k = 0; k < RDEG; ++k) {
      const unsigned a = A[i * RDEG + k];
      if (!a) continue;
      for (int j = 0; j < RDEG; ++j) C[i * RDEG + j] += a * B[k * RDEG + j];
    }
  return C;
}

// M^e: M maps (h_0..h_30) to (h_1, ..., h_30, h_0 + h_28)
Mat step_power(int64_t e) {
  Mat M(RDEG * RDEG, 0u), R(RDEG * RDEG, 0u);
  for (int t = 0; t + 1 < RDEG; ++t) M[t * RDEG + t + 1] = 1u;
  M[(RDEG - 1) * RDEG + 0] = 1u;
  M[(RDEG - 1) * RDEG + (RDEG - RSEP)] = 1u;
  for (int t = 0; t < RDEG; ++t) R[t * RDEG + t] = 1u;
  while (e > 0) {
    if (e & 1) R = mat_mul(R, M);
    M = mat_mul(M, M);
    e >>= 1;
  }
  return R;
}

}  // namespace

// k uniforms rand()/RAND_MAX of the glibc stream whose history is hist[31]
// (host, oldest first) into out (device); hist is advanced past them.
// Synchronises the stream (the new history is read back).
int fricc_glibc_uniforms_device(unsigned* hist, int64_t k, double* out, cudaStream_t st) {
  if (!hist || k < 0 || (k > 0 && !out)) {
    fricc_set_error("glibc_uniforms: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (k == 0) return FRICC_OK;
  const int64_t nch = fricc_cdiv(k, GCH);
  static const Mat J = step_power(GCH);
  unsigned *dJ = nullptr, *dh = nullptr, *starts = nullptr;
  int rc = fricc_alloc_t(&dJ, RDEG * RDEG + 2 * RDEG, st);
  if (!rc) rc = fricc_alloc_t(&starts, nch * RDEG, st);
  if (rc) {
    fricc_free(dJ, st);
    return rc;
  }
  dh = dJ + RDEG * RDEG;
  unsigned* dout = dh + RDEG;
  // pageable sources: the copies complete before cudaMemcpyAsync returns
  cudaError_t e = cudaMemcpyAsync(dJ, J.data(), sizeof(unsigned) * RDEG * RDEG, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dh, hist, sizeof(unsigned) * RDEG, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_glibc_starts<<<1, 32, 0, st>>>(dJ, dh, nch, starts);
    k_glibc_gen<<<(unsigned)fricc_cdiv(nch, 128), 128, 0, st>>>(starts, nch, k, out, dout);
    fricc_note_launch(2);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(hist, dout, sizeof(unsigned) * RDEG, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  fricc_free(starts, st);
  fricc_free(dJ, st);
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "glibc_uniforms", __FILE__, __LINE__);
}
