// Strided batched GEMM with FP64 operands computed in FP32-pair arithmetic:
//   C[b] = alpha * A[b] @ B[b] + beta * C[b]
// A[b] is M x K with element strides (sAm, sAk), B[b] is K x N (sBk, sBn),
// C[b] is M x N (sCm, sCn); batch strides sAb, sBb, sCb (0 = shared).
//
// The dense O^2V^3 contractions of an FRI-CCSD iteration run here instead
// of in FP64 (GB300 issues 2 FP64 FMAs per SM per clock against 128 FP32
// lanes).  Operands are split on the fly into (hi, lo) float pairs as they
// are staged in shared memory; products are formed exactly to ~48 bits
// (one FMA recovers the rounding error of hi*hi) and accumulated with an
// error-free two-sum, renormalised every K tile.  Relative error of each
// output ~1e-14.  A long K is split over blockIdx.z; the partial tiles are
// summed afterwards in a fixed order, so results are deterministic.
#include "common.cuh"

namespace {

constexpr int BK = 16, NT = 256;

__device__ __forceinline__ float2 split(double d) {
  const float h = __double2float_rn(d);
  return make_float2(h, __double2float_rn(d - (double)h));
}

struct GemmArgs {
  const double* A;
  const double* B;
  double* C;      // final output (splits == 1) or nullptr
  double* part;   // [batch][splits][M][N] partials (splits > 1)
  int64_t M, N, K;
  int64_t sAm, sAk, sAb, sBk, sBn, sBb, sCm, sCn, sCb;
  double alpha, beta;
  int splits;
  int64_t kchunk;  // K per split (multiple of BK)
};

// 256 threads as 16 x 16; each owns a TM x TN block of C (rows ty + 16 i,
// columns tx + 16 j), so a CTA tile is (16 TM) x (16 TN): 64x64 for square
// problems, 128x32 / 32x128 when one side is as small as nocc.
template <int TM, int TN>
__global__ void __launch_bounds__(NT) k_gemm_df(GemmArgs g) {
  constexpr int BM = 16 * TM, BN = 16 * TN;
  __shared__ float2 As[BK][BM + 1];
  __shared__ float2 Bs[BK][BN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  const int64_t bz = blockIdx.z / g.splits;
  const int sp = blockIdx.z % g.splits;
  const int64_t k_begin = (int64_t)sp * g.kchunk;
  const int64_t k_end = k_begin + g.kchunk < g.K ? k_begin + g.kchunk : g.K;
  const double* A = g.A + bz * g.sAb;
  const double* B = g.B + bz * g.sBb;

  float ah[TM][TN], al[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) ah[i][j] = al[i][j] = 0.f;

  const bool a_kfast = g.sAk == 1;
  const bool b_nfast = g.sBn == 1;
  for (int64_t k0 = k_begin; k0 < k_end; k0 += BK) {
    __syncthreads();
#pragma unroll
    for (int r = 0; r < (BM * BK) / NT; ++r) {
      const int idx = r * NT + threadIdx.x;
      int mm, kk;
      if (a_kfast) { mm = idx / BK; kk = idx % BK; } else { kk = idx / BM; mm = idx % BM; }
      const int64_t m = m0 + mm, k = k0 + kk;
      As[kk][mm] = split((m < g.M && k < k_end) ? A[m * g.sAm + k * g.sAk] : 0.0);
    }
#pragma unroll
    for (int r = 0; r < (BN * BK) / NT; ++r) {
      const int idx = r * NT + threadIdx.x;
      int nn, kk;
      if (b_nfast) { kk = idx / BN; nn = idx % BN; } else { nn = idx / BK; kk = idx % BK; }
      const int64_t n = n0 + nn, k = k0 + kk;
      Bs[kk][nn] = split((n < g.N && k < k_end) ? B[k * g.sBk + n * g.sBn] : 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      float2 a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          // error-free transforms with explicit rounding (no compiler FMA contraction)
          const float ph = __fmul_rn(a[i].x, b[j].x);
          float pl = __fmaf_rn(a[i].x, b[j].x, -ph);
          pl = __fmaf_rn(a[i].x, b[j].y, pl);
          pl = __fmaf_rn(a[i].y, b[j].x, pl);
          const float s = __fadd_rn(ah[i][j], ph);
          const float z = __fsub_rn(s, ah[i][j]);
          const float e = __fadd_rn(__fsub_rn(ah[i][j], __fsub_rn(s, z)), __fsub_rn(ph, z));
          al[i][j] = __fadd_rn(al[i][j], __fadd_rn(e, pl));
          ah[i][j] = s;
        }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const float s = __fadd_rn(ah[i][j], al[i][j]);
        al[i][j] = __fsub_rn(al[i][j], __fsub_rn(s, ah[i][j]));
        ah[i][j] = s;
      }
  }
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
      if (m < g.M && n < g.N) {
        const double acc = (double)ah[i][j] + (double)al[i][j];
        if (g.splits == 1) {
          double* c = g.C + bz * g.sCb + m * g.sCm + n * g.sCn;
          *c = g.beta == 0.0 ? g.alpha * acc : fma(g.alpha, acc, g.beta * *c);
        } else {
          g.part[((bz * g.splits + sp) * g.M + m) * g.N + n] = acc;
        }
      }
    }
}

// C = alpha * sum_s part[s] + beta * C, splits summed in order
__global__ void k_gemm_reduce(GemmArgs g, int64_t batch) {
  const int64_t MN = g.M * g.N;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < batch * MN;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / MN, r = t % MN, m = r / g.N, n = r % g.N;
    double acc = 0.0;
    for (int s = 0; s < g.splits; ++s) acc += g.part[(b * g.splits + s) * MN + r];
    double* c = g.C + b * g.sCb + m * g.sCm + n * g.sCn;
    *c = g.beta == 0.0 ? g.alpha * acc : fma(g.alpha, acc, g.beta * *c);
  }
}

}  // namespace

int fricc_gemm_df_device(const double* A, const double* B, double* C, int64_t batch, int64_t M, int64_t N, int64_t K,
                         const int64_t sA[3], const int64_t sB[3], const int64_t sC[3], double alpha, double beta,
                         cudaStream_t st) {
  if (!A || !B || !C || batch <= 0 || M <= 0 || N <= 0 || K < 0) {
    fricc_set_error("gemm_df: bad arguments");
    return FRICC_ERR_ARG;
  }
  GemmArgs g{};
  g.A = A;
  g.B = B;
  g.C = C;
  g.M = M;
  g.N = N;
  g.K = K;
  g.sAm = sA[0]; g.sAk = sA[1]; g.sAb = sA[2];
  g.sBk = sB[0]; g.sBn = sB[1]; g.sBb = sB[2];
  g.sCm = sC[0]; g.sCn = sC[1]; g.sCb = sC[2];
  g.alpha = alpha;
  g.beta = beta;
  // tile shape: the one of 64x64, 128x32, 32x128 that pads C least (a side
  // as short as nocc would waste half of a 64-wide tile)
  int tm = 4, tn = 4;
  {
    const int cand[3][2] = {{4, 4}, {8, 2}, {2, 8}};
    int64_t best = -1;
    for (const auto& c : cand) {
      const int64_t pad = fricc_cdiv(M, 16 * c[0]) * 16 * c[0] * fricc_cdiv(N, 16 * c[1]) * 16 * c[1];
      if (best < 0 || pad < best) { best = pad; tm = c[0]; tn = c[1]; }
    }
  }
  const int64_t BM = 16 * tm, BN = 16 * tn;
  const int64_t tiles = fricc_cdiv(M, BM) * fricc_cdiv(N, BN) * batch;
  // split K until the grid covers the GPU about four times over
  int splits = 1;
  while (splits < 1024 && tiles * splits < 152 * 4 && K / (2 * splits) >= 8 * BK) splits *= 2;
  g.splits = splits;
  g.kchunk = fricc_cdiv(fricc_cdiv(K, splits), BK) * BK;
  if (fricc_cdiv(M, BM) > 65535 || batch * splits > 65535) {
    fricc_set_error("gemm_df: grid too large (M=%lld, batch=%lld)", (long long)M, (long long)batch);
    return FRICC_ERR_ARG;
  }
  double* part = nullptr;
  if (splits > 1) {
    int rc = fricc_alloc_t(&part, (size_t)(batch * splits * M * N), st);
    if (rc) return rc;
    g.part = part;
  }
  dim3 grid((unsigned)fricc_cdiv(N, BN), (unsigned)fricc_cdiv(M, BM), (unsigned)(batch * splits));
  if (tm == 8) k_gemm_df<8, 2><<<grid, NT, 0, st>>>(g);
  else if (tm == 2) k_gemm_df<2, 8><<<grid, NT, 0, st>>>(g);
  else k_gemm_df<4, 4><<<grid, NT, 0, st>>>(g);
  fricc_note_launch();
  if (splits > 1) {
    int64_t n = batch * M * N;
    int64_t gr = fricc_cdiv(n, 256);
    if (gr > 152 * 32) gr = 152 * 32;
    k_gemm_reduce<<<(unsigned)gr, 256, 0, st>>>(g, batch);
    fricc_note_launch();
  }
  cudaError_t e = cudaGetLastError();
  fricc_free(part, st);
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "gemm_df", __FILE__, __LINE__);
}
