// Strided batched FP64 GEMM on the FP64 FMA pipe:
//   C[b] = alpha * A[b] @ B[b] + beta * C[b]
// A[b] is M x K with element strides (sAm, sAk), B[b] is K x N (sBk, sBn),
// C[b] is M x N (sCm, sCn); batch strides sAb, sBb, sCb (0 = shared).
//
// The dense O^2V^3 / O^3V^2 contractions of the FP64 FRI-CCSD iteration (the
// PySCF einsums of fricc/friccsd.py:144-192,211,238-241).  GB300 runs FP64
// FMA at 2 per SM per clock (1.26 TFLOP/s), and its FP64 mma.sync at less
// (1.05 TFLOP/s), so every output is a plain DFMA chain: the FP64 pipe, not
// memory, bounds any tile that keeps a few accumulators per thread, and a
// tile only has to keep enough warps on every SM.  Each output is summed in
// k order (deterministic); a long K with few output tiles is split over
// blockIdx.x (beside the N tiles; blockIdx.z is the batch) and the partial
// tiles summed afterwards in slice order.
#include "common.cuh"

namespace {

constexpr int BK = 16, NT = 256;

struct GemmArgs {
  const double* A;
  const double* B;
  double* C;      // final output (splits == 1)
  double* part;   // [batch][splits][M][N] partials (splits > 1)
  int64_t M, N, K;
  int64_t sAm, sAk, sAb, sBk, sBn, sBb, sCm, sCn, sCb;
  // a second batch level (replicas): batch index bz = b2 * nb1 + b
  int64_t nb1, sAb2, sBb2, sCb2;
  double alpha, beta;
  // the epilogue's case, from alpha and beta on the host (GB300's FP64 unit
  // is too slow for per-output FP64 comparisons): 0 C = acc, 1 C = -acc,
  // 2 C = alpha acc, 3 C += acc, 4 C -= acc, 5 C = alpha acc + beta C
  int emode;
  int splits;
  int64_t ntn;     // N tiles: blockIdx.x = split * ntn + N tile
  int64_t kchunk;  // K per split (multiple of BK)
};

__device__ __forceinline__ int64_t boffA(const GemmArgs& g, int64_t bz) {
  return (bz % g.nb1) * g.sAb + (bz / g.nb1) * g.sAb2;
}
__device__ __forceinline__ int64_t boffB(const GemmArgs& g, int64_t bz) {
  return (bz % g.nb1) * g.sBb + (bz / g.nb1) * g.sBb2;
}
__device__ __forceinline__ int64_t boffC(const GemmArgs& g, int64_t bz) {
  return (bz % g.nb1) * g.sCb + (bz / g.nb1) * g.sCb2;
}

__device__ __forceinline__ void store_out(const GemmArgs& g, int64_t bz, int sp, int64_t m, int64_t n, double acc) {
  if (g.splits == 1) {
    double* cp = g.C + boffC(g, bz) + m * g.sCm + n * g.sCn;
    switch (g.emode) {
      case 0: *cp = acc; break;
      case 1: *cp = -acc; break;
      case 2: *cp = g.alpha * acc; break;
      case 3: *cp = *cp + acc; break;
      case 4: *cp = *cp - acc; break;
      default: *cp = fma(g.alpha, acc, g.beta * *cp);
    }
  } else {
    g.part[((bz * g.splits + sp) * g.M + m) * g.N + n] = acc;
  }
}

// 256 threads as 16 x 16: thread (tx, ty) owns rows ty + 16 i (i < TM) and
// columns tx + 16 j (j < TN) of a (16 TM) x (16 TN) tile of C.  Operand
// tiles go global -> registers -> shared; the loads of tile k+1 are issued
// before tile k is computed, and a partial last K tile runs only its valid k.
template <int TM, int TN>
__global__ void __launch_bounds__(NT, 2) k_gemm_f64(GemmArgs g) {
  constexpr int BM = 16 * TM, BN = 16 * TN;
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)(blockIdx.x % g.ntn) * BN;
  const int64_t bz = blockIdx.z;
  const int sp = (int)(blockIdx.x / g.ntn);
  const int64_t k_begin = (int64_t)sp * g.kchunk;
  const int64_t k_end = k_begin + g.kchunk < g.K ? k_begin + g.kchunk : g.K;
  const double* A = g.A + boffA(g, bz);
  const double* B = g.B + boffB(g, bz);

  double acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;

  const bool a_kfast = g.sAk == 1;
  const bool b_nfast = g.sBn == 1;
  constexpr int RA = (BM * BK) / NT, RB = (BN * BK) / NT;
  static_assert((BM * BK) % NT == 0 && (BN * BK) % NT == 0, "tile not a multiple of the block");
  double ra[RA], rb[RB];
  auto a_coord = [&](int r, int& mm, int& kk) {
    const int idx = r * NT + threadIdx.x;
    if (a_kfast) { mm = idx / BK; kk = idx % BK; } else { kk = idx / BM; mm = idx % BM; }
  };
  auto b_coord = [&](int r, int& nn, int& kk) {
    const int idx = r * NT + threadIdx.x;
    if (b_nfast) { kk = idx / BN; nn = idx % BN; } else { nn = idx / BK; kk = idx % BK; }
  };
  auto gload = [&](int64_t k0) {
#pragma unroll
    for (int r = 0; r < RA; ++r) {
      int mm, kk;
      a_coord(r, mm, kk);
      const int64_t m = m0 + mm, k = k0 + kk;
      ra[r] = (m < g.M && k < k_end) ? A[m * g.sAm + k * g.sAk] : 0.0;
    }
#pragma unroll
    for (int r = 0; r < RB; ++r) {
      int nn, kk;
      b_coord(r, nn, kk);
      const int64_t n = n0 + nn, k = k0 + kk;
      rb[r] = (n < g.N && k < k_end) ? B[k * g.sBk + n * g.sBn] : 0.0;
    }
  };
  auto kstep = [&](int kk) {
    double a[TM], b[TN];
#pragma unroll
    for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
    for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
  };
  gload(k_begin);
  for (int64_t k0 = k_begin; k0 < k_end; k0 += BK) {
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RA; ++r) {
      int mm, kk;
      a_coord(r, mm, kk);
      As[kk][mm] = ra[r];
    }
#pragma unroll
    for (int r = 0; r < RB; ++r) {
      int nn, kk;
      b_coord(r, nn, kk);
      Bs[kk][nn] = rb[r];
    }
    __syncthreads();
    if (k0 + BK < k_end) gload(k0 + BK);
    const int kn = k_end - k0 < BK ? (int)(k_end - k0) : BK;
    if (kn == BK) {
#pragma unroll 4
      for (int kk = 0; kk < BK; ++kk) kstep(kk);
    } else {
#pragma unroll 1
      for (int kk = 0; kk < kn; ++kk) kstep(kk);
    }
  }
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
      if (m < g.M && n < g.N) store_out(g, bz, sp, m, n, acc[i][j]);
    }
}

// C = alpha * sum_s part[s] + beta * C, splits summed in order
__global__ void k_gemm_f64_reduce(GemmArgs g, int64_t batch) {
  const int64_t MN = g.M * g.N;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < batch * MN;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / MN, r = t % MN, m = r / g.N, n = r % g.N;
    double acc = 0.0;
    for (int s = 0; s < g.splits; ++s) acc += g.part[(b * g.splits + s) * MN + r];
    double* c = g.C + boffC(g, b) + m * g.sCm + n * g.sCn;
    *c = g.emode <= 2 ? g.alpha * acc : fma(g.alpha, acc, g.beta * *c);
  }
}

// Skinny shapes (a GEMV, or an output a few rows or columns wide) waste a
// 32-wide tile on padding; they take one of two dot-product kernels.
//
// One warp per output (b, m, n): the lanes stride over k (coalesced when A
// is k-contiguous), and a fixed shuffle tree sums their partials.
__global__ void __launch_bounds__(256) k_gemv_warp(GemmArgs g, int64_t batch) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= batch * g.M * g.N) return;
  const int64_t n = w % g.N, m = (w / g.N) % g.M, b = w / (g.N * g.M);
  const double* A = g.A + boffA(g, b) + m * g.sAm;
  const double* B = g.B + boffB(g, b) + n * g.sBn;
  double acc = 0.0;
  for (int64_t k = lane; k < g.K; k += 32) acc = fma(__ldg(A + k * g.sAk), __ldg(B + k * g.sBk), acc);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if (lane == 0) {
    GemmArgs one = g;
    one.splits = 1;
    store_out(one, b, 0, m, n, acc);
  }
}

// One thread per output (b, m, n) over a K slice (blockIdx.y of g.splits):
// for few rows and an n-contiguous B, a warp reads 32 consecutive columns.
__global__ void __launch_bounds__(256) k_gemv_cols(GemmArgs g) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.N) return;
  const int sp = blockIdx.y;
  const int64_t bm = blockIdx.z, m = bm % g.M, b = bm / g.M;
  const int64_t k0 = (int64_t)sp * g.kchunk;
  const int64_t k1 = k0 + g.kchunk < g.K ? k0 + g.kchunk : g.K;
  const double* A = g.A + boffA(g, b) + m * g.sAm;
  const double* B = g.B + boffB(g, b) + n * g.sBn;
  double acc = 0.0;
  for (int64_t k = k0; k < k1; ++k) acc = fma(__ldg(A + k * g.sAk), __ldg(B + k * g.sBk), acc);
  store_out(g, b, sp, m, n, acc);
}

}  // namespace

int fricc_gemm_f64_device(const double* A, const double* B, double* C, int64_t batch, int64_t M, int64_t N, int64_t K,
                          const int64_t sA[3], const int64_t sB[3], const int64_t sC[3], double alpha, double beta,
                          cudaStream_t st, int64_t batch2, const int64_t* s2) {
  if (((!A || !B) && K > 0) || !C || batch <= 0 || M <= 0 || N <= 0 || K < 0 || !sA || !sB || !sC) {
    fricc_set_error("gemm_f64: bad arguments");
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
  g.emode = beta == 0.0 ? (alpha == 1.0 ? 0 : (alpha == -1.0 ? 1 : 2))
                        : (beta == 1.0 && alpha == 1.0 ? 3 : (beta == 1.0 && alpha == -1.0 ? 4 : 5));
  // a second batch level: batch2 groups of `batch` products, group strides
  // s2 = {A, B, C}; from here on `batch` counts every product
  if (batch2 < 1 || batch2 > 65535) {
    fricc_set_error("gemm: bad second batch count");
    return FRICC_ERR_ARG;
  }
  g.nb1 = batch;
  g.sAb2 = s2 ? s2[0] : 0;
  g.sBb2 = s2 ? s2[1] : 0;
  g.sCb2 = s2 ? s2[2] : 0;
  batch *= batch2;
  const bool prof = fricc_prof_on();
  const double flops = 2.0 * (double)batch * (double)M * (double)N * (double)K;
  if (K > 0 && ((N <= 4 && (g.sAk == 1 || M <= 4)) || (M <= 4 && g.sBn != 1 && N <= 64))) {
    // a few outputs per row or column with a k-contiguous A (or few outputs
    // altogether): one warp per output
    const int64_t outs = batch * M * N;
    if (fricc_cdiv(outs, 8) > 0x7fffffff) {
      fricc_set_error("gemm_f64: too many outputs for the dot-product kernel");
      return FRICC_ERR_ARG;
    }
    if (prof) fricc_prof_record(st, true, 0.0, 2);
    k_gemv_warp<<<(unsigned)fricc_cdiv(outs, 8), 256, 0, st>>>(g, batch);
    fricc_note_launch();
    if (prof) fricc_prof_record(st, false, flops, 2);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "gemm_f64", __FILE__, __LINE__);
  }
  if (K > 0 && M <= 4) {
    // a few rows: one thread per output column, K split until the grid
    // covers the GPU about four times over (slices of at least 64)
    const int64_t cols = fricc_cdiv(N, 256) * M;  // per product, as the tiled path
    if (batch * M > 65535) {
      fricc_set_error("gemm_f64: batch x rows too large for the column kernel");
      return FRICC_ERR_ARG;
    }
    int splits = 1;
    while (splits < 1024 && cols * splits < 152 * 4 && K / (2 * splits) >= 64) splits *= 2;
    g.splits = splits;
    g.kchunk = fricc_cdiv(K, splits);
    double* part = nullptr;
    if (splits > 1) {
      int rc = fricc_alloc_t(&part, (size_t)(batch * splits * M * N), st);
      if (rc) return rc;
      g.part = part;
    }
    if (prof) fricc_prof_record(st, true, 0.0, 2);
    k_gemv_cols<<<dim3((unsigned)fricc_cdiv(N, 256), (unsigned)splits, (unsigned)(batch * M)), 256, 0, st>>>(g);
    fricc_note_launch();
    if (splits > 1) {
      int64_t n = batch * M * N;
      int64_t gr = fricc_cdiv(n, 256);
      if (gr > 152 * 32) gr = 152 * 32;
      k_gemm_f64_reduce<<<(unsigned)gr, 256, 0, st>>>(g, batch);
      fricc_note_launch();
    }
    if (prof) fricc_prof_record(st, false, flops, 2);
    cudaError_t e = cudaGetLastError();
    fricc_free(part, st);
    return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "gemm_f64", __FILE__, __LINE__);
  }
  // tile shape: the one of 64x64, 128x32, 32x128, 32x160, 32x32 that pads C
  // least
  int tm = 4, tn = 4;
  {
    // the small 32x32 tile counts 1.3 times its area (two rows and two
    // columns per thread reuse each operand load less): it wins only for
    // outputs of a few tens of rows and columns, such as cc_Foo's o x o
    const int cand[5][2] = {{4, 4}, {8, 2}, {2, 8}, {2, 10}, {2, 2}};
    const int weight10[5] = {10, 10, 10, 10, 13};
    const int forced = fricc_tune_get(FRICC_TUNE_GEMM_TILE);
    if (forced >= 0) {
      tm = cand[forced][0];
      tn = cand[forced][1];
    } else {
      int64_t best = -1;
      for (int c = 0; c < 5; ++c) {
        const int64_t pad = fricc_cdiv(M, 16 * cand[c][0]) * 16 * cand[c][0] * fricc_cdiv(N, 16 * cand[c][1]) * 16 *
                            cand[c][1] * weight10[c];
        if (best < 0 || pad < best) { best = pad; tm = cand[c][0]; tn = cand[c][1]; }
      }
    }
  }
  const int64_t BM = 16 * tm, BN = 16 * tn;
  // split K as for a single product, so that each product's sums are the
  // same whatever batch it runs in (a long K comes with few output tiles;
  // the batched products of an iteration have short K and never split)
  const int64_t tiles = fricc_cdiv(M, BM) * fricc_cdiv(N, BN);
  // split K until the grid covers the GPU about four (or the tuned number
  // of) times over
  const int cover = fricc_tune_get(FRICC_TUNE_GEMM_COVER) > 0 ? fricc_tune_get(FRICC_TUNE_GEMM_COVER) : 4;
  int splits = 1;
  while (splits < 1024 && tiles * splits < 152 * cover && K / (2 * splits) >= 8 * BK) splits *= 2;
  g.splits = splits;
  g.kchunk = fricc_cdiv(fricc_cdiv(K, splits), BK) * BK;
  g.ntn = fricc_cdiv(N, BN);
  if (fricc_cdiv(M, BM) > 65535 || batch > 65535 || g.ntn * splits > 0x7fffffff) {
    fricc_set_error("gemm_f64: grid too large (M=%lld, batch=%lld)", (long long)M, (long long)batch);
    return FRICC_ERR_ARG;
  }
  double* part = nullptr;
  if (splits > 1) {
    int rc = fricc_alloc_t(&part, (size_t)(batch * splits * M * N), st);
    if (rc) return rc;
    g.part = part;
  }
  if (prof) fricc_prof_record(st, true, 0.0, 2);
  dim3 grid((unsigned)(g.ntn * splits), (unsigned)fricc_cdiv(M, BM), (unsigned)batch);
  if (tm == 8) k_gemm_f64<8, 2><<<grid, NT, 0, st>>>(g);
  else if (tn == 8) k_gemm_f64<2, 8><<<grid, NT, 0, st>>>(g);
  else if (tn == 10) k_gemm_f64<2, 10><<<grid, NT, 0, st>>>(g);
  else if (tm == 2 && tn == 2) k_gemm_f64<2, 2><<<grid, NT, 0, st>>>(g);
  else k_gemm_f64<4, 4><<<grid, NT, 0, st>>>(g);
  fricc_note_launch();
  if (splits > 1) {
    int64_t n = batch * M * N;
    int64_t gr = fricc_cdiv(n, 256);
    if (gr > 152 * 32) gr = 152 * 32;
    k_gemm_f64_reduce<<<(unsigned)gr, 256, 0, st>>>(g, batch);
    fricc_note_launch();
  }
  if (prof) fricc_prof_record(st, false, flops, 2);
  cudaError_t e = cudaGetLastError();
  fricc_free(part, st);
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "gemm_f64", __FILE__, __LINE__);
}
