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
// error-free two-sum, renormalised every K tile, two adjacent outputs per
// packed f32x2 instruction.  Relative error of each
// output ~1e-14.  A long K is split over blockIdx.x (beside the N tiles;
// blockIdx.z is the batch); the partial tiles are
// summed afterwards in a fixed order, so results are deterministic.
#include "common.cuh"

namespace {

constexpr int BK = 16, NT = 256;

__device__ __forceinline__ float2 split(double d) { return split_f2_bits(d); }

// two floats in one 64-bit register pair, and the packed f32x2 arithmetic
// (one issue slot per two lanes of FP32 work)
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float2 upk2(f32x2 r) {
  float2 f;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(f.x), "=f"(f.y) : "l"(r));
  return f;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

struct GemmArgs {
  const double* A;
  const double* B;
  double* C;      // final output (splits == 1) or nullptr
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

// 256 threads as 16 x 16.  Thread (tx, ty) owns rows ty + 16 i (i < TM) and
// the column pairs 2 (tx + 16 j) + {0, 1} (j < TN / 2) of a (16 TM) x (16 TN)
// tile of C; each pair is accumulated with packed f32x2 instructions.  The
// shared tiles hold the operands already split: A as (h, h, l, l) per
// element (broadcast to both lanes of a pair), B per column pair as
// (h0, h1, l0, l1) plus (-h0, -h1) (the negated high part gives the exact
// product error with one fma).  Rows are padded by one element so that the
// staging stores do not conflict on banks.
template <int TM, int TN>
__global__ void __launch_bounds__(NT, 2) k_gemm_df(GemmArgs g) {
  constexpr int BM = 16 * TM, BN = 16 * TN, NP = BN / 2, JP = TN / 2;
  __shared__ ulonglong2 As[BK][BM + 1];
  __shared__ ulonglong2 Bs[BK][NP + 1];
  __shared__ f32x2 Bn[BK][NP + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)(blockIdx.x % g.ntn) * BN;
  const int64_t bz = blockIdx.z;
  const int sp = (int)(blockIdx.x / g.ntn);
  const int64_t k_begin = (int64_t)sp * g.kchunk;
  const int64_t k_end = k_begin + g.kchunk < g.K ? k_begin + g.kchunk : g.K;
  const double* A = g.A + boffA(g, bz);
  const double* B = g.B + boffB(g, bz);

  f32x2 ah[TM][JP], al[TM][JP];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < JP; ++j) ah[i][j] = al[i][j] = 0ull;  // +0.0f in both lanes

  const bool a_kfast = g.sAk == 1;
  const bool b_nfast = g.sBn == 1;
  // Operand tiles go global -> registers (raw FP64) -> shared (split): the
  // loads of tile k+1 are issued before tile k is computed, so their latency
  // hides behind the arithmetic; the split happens once per element per CTA.
  constexpr int RA = (BM * BK) / NT, RB = (NP * BK + NT - 1) / NT;
  double ra[RA], rb0[RB], rb1[RB];
  auto a_coord = [&](int r, int& mm, int& kk) {
    const int idx = r * NT + threadIdx.x;
    if (a_kfast) { mm = idx / BK; kk = idx % BK; } else { kk = idx / BM; mm = idx % BM; }
  };
  auto b_coord = [&](int r, int& pp, int& kk) {
    const int idx = r * NT + threadIdx.x;
    if (b_nfast) { kk = idx / NP; pp = idx % NP; } else { pp = idx / BK; kk = idx % BK; }
    return (NP * BK) % NT == 0 || idx < NP * BK;
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
      int pp, kk;
      const bool on = b_coord(r, pp, kk);
      const int64_t n = n0 + 2 * pp, k = k0 + kk;
      const bool kin = on && k < k_end;
      rb0[r] = (n < g.N && kin) ? B[k * g.sBk + n * g.sBn] : 0.0;
      rb1[r] = (n + 1 < g.N && kin) ? B[k * g.sBk + (n + 1) * g.sBn] : 0.0;
    }
  };
  gload(k_begin);
  for (int64_t k0 = k_begin; k0 < k_end; k0 += BK) {
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RA; ++r) {
      int mm, kk;
      a_coord(r, mm, kk);
      const float2 a = split(ra[r]);
      As[kk][mm] = make_ulonglong2(pk2(a.x, a.x), pk2(a.y, a.y));
    }
#pragma unroll
    for (int r = 0; r < RB; ++r) {
      int pp, kk;
      if (b_coord(r, pp, kk)) {
        const float2 b0 = split(rb0[r]);
        const float2 b1 = split(rb1[r]);
        Bs[kk][pp] = make_ulonglong2(pk2(b0.x, b1.x), pk2(b0.y, b1.y));
        Bn[kk][pp] = pk2(-b0.x, -b1.x);
      }
    }
    __syncthreads();
    if (k0 + BK < k_end) gload(k0 + BK);
#pragma unroll 2
    for (int kk = 0; kk < BK; ++kk) {
      ulonglong2 a[TM], b[JP];
      f32x2 nb[JP];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < JP; ++j) {
        b[j] = Bs[kk][tx + 16 * j];
        nb[j] = Bn[kk][tx + 16 * j];
      }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < JP; ++j) {
          const f32x2 nph = mul2(a[i].x, nb[j]);      // -RN(ah bh)
          f32x2 pl = fma2(a[i].x, b[j].x, nph);       // ah bh - ph, exact
          pl = fma2(a[i].x, b[j].y, pl);
          pl = fma2(a[i].y, b[j].x, pl);
          const f32x2 s = sub2(ah[i][j], nph);        // two-sum (acc, ph), written with -ph
          const f32x2 z = sub2(s, ah[i][j]);
          const f32x2 e = sub2(sub2(ah[i][j], sub2(s, z)), add2(nph, z));
          al[i][j] = add2(al[i][j], add2(e, pl));
          ah[i][j] = s;
        }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < JP; ++j) {
        const f32x2 s = add2(ah[i][j], al[i][j]);
        al[i][j] = sub2(al[i][j], sub2(s, ah[i][j]));
        ah[i][j] = s;
      }
  }
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < JP; ++j) {
      const int64_t m = m0 + ty + 16 * i, n = n0 + 2 * (tx + 16 * j);
      const float2 h = upk2(ah[i][j]), l = upk2(al[i][j]);
      const double acc[2] = {pair_to_f64(h.x, l.x), pair_to_f64(h.y, l.y)};
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        if (m < g.M && n + c < g.N) {
          if (g.splits == 1) {
            double* cp = g.C + boffC(g, bz) + m * g.sCm + (n + c) * g.sCn;
            // FP64 work per output kept to one operation in the common cases
            switch (g.emode) {
              case 0: *cp = acc[c]; break;
              case 1: *cp = -acc[c]; break;
              case 2: *cp = g.alpha * acc[c]; break;
              case 3: *cp = *cp + acc[c]; break;
              case 4: *cp = *cp - acc[c]; break;
              default: *cp = fma(g.alpha, acc[c], g.beta * *cp);
            }
          } else {
            g.part[((bz * g.splits + sp) * g.M + m) * g.N + n + c] = acc[c];
          }
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
    double* c = g.C + boffC(g, b) + m * g.sCm + n * g.sCn;
    *c = g.emode <= 2 ? g.alpha * acc : fma(g.alpha, acc, g.beta * *c);
  }
}

}  // namespace

int fricc_gemm_df_device(const double* A, const double* B, double* C, int64_t batch, int64_t M, int64_t N, int64_t K,
                         const int64_t sA[3], const int64_t sB[3], const int64_t sC[3], double alpha, double beta,
                         cudaStream_t st, int64_t batch2, const int64_t* s2) {
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
  // tile shape: the one of 64x64, 128x32, 32x128, 32x160, 32x32 that pads C
  // least
  // (a side as short as nocc would waste half of a 64-wide tile)
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
    fricc_set_error("gemm_df: grid too large (M=%lld, batch=%lld)", (long long)M, (long long)batch);
    return FRICC_ERR_ARG;
  }
  double* part = nullptr;
  if (splits > 1) {
    int rc = fricc_alloc_t(&part, (size_t)(batch * splits * M * N), st);
    if (rc) return rc;
    g.part = part;
  }
  dim3 grid((unsigned)(g.ntn * splits), (unsigned)fricc_cdiv(M, BM), (unsigned)batch);
  if (tm == 8) k_gemm_df<8, 2><<<grid, NT, 0, st>>>(g);
  else if (tn == 8) k_gemm_df<2, 8><<<grid, NT, 0, st>>>(g);
  else if (tn == 10) k_gemm_df<2, 10><<<grid, NT, 0, st>>>(g);
  else if (tm == 2 && tn == 2) k_gemm_df<2, 2><<<grid, NT, 0, st>>>(g);
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
