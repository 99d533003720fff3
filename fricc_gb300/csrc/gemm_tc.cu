// BF16 tensor-core GEMM on the 5th-generation tensor cores (tcgen05), and the
// split-BF16x3 rebuild of integral blocks from a Cholesky factor.
//
// C[M][N] = A[M][K] B[N][K]^T, A and B BF16 and K-major, FP32 accumulation in
// tensor memory (TMEM).  A persistent kernel: one CTA per SM walks 128 x BN
// output tiles (BN = 256, or 64 for outputs as narrow as nocc), or split-K
// slices of them, with warp-specialised roles:
//   warp 0, one lane  -- TMA producer: 128 x 64 and BN x 64 operand boxes
//                        (128-byte swizzle) into a 4-stage (BN = 256) or
//                        8-stage (BN = 64) shared-memory ring, each stage
//                        guarded by a "full" and an "empty" mbarrier;
//   warp 1, one lane  -- MMA issuer: four tcgen05.mma (M=128, N=BN, K=16) per
//                        stage into one of two TMEM accumulators of BN
//                        columns, tcgen05.commit to the stage's "empty"
//                        barrier, and at the end of a tile to the
//                        accumulator's "full" barrier (warp 1 also allocates
//                        and frees the 2 BN TMEM columns);
//   warps 2-9         -- epilogue: tcgen05.ld of their 32 TMEM lanes (one
//                        output row per thread, 16 columns per load; two
//                        warps per lane quadrant, each with half the
//                        columns) into the epilogue functor, then an arrive
//                        on the accumulator's "empty" barrier -- overlapping
//                        the MMAs of the next tile in the other accumulator.
// Every mbarrier wait is bounded (2 s of global time); a wait that gives up
// sets a device error word, the roles stop issuing, the producer waits
// (bounded) for its copies in flight, and the CTA frees its TMEM and exits.
//
// Split-BF16x3: x = hi + lo with hi = bf16(x), lo = bf16(x - hi), and
// A B^T ~ Ahi Bhi^T + Ahi Blo^T + Alo Bhi^T (the lo*lo term is below FP32
// accumulation error).  The three products are one GEMM over a K-concatenated
// operand pair A' = [Ahi | Ahi | Alo], B' = [Bhi | Blo | Bhi] (K' = 3K).
#include <atomic>
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "common.cuh"

namespace tc {

constexpr int BM = 128, BK = 64;
constexpr int A_BYTES = BM * BK * 2;  // 16 KB
constexpr int EPI_WARPS = 8;  // two per TMEM lane quadrant, each draining half the columns
constexpr int NT = 32 * (2 + EPI_WARPS);  // producer warp, MMA warp, epilogue warps

// Tile width BN (the MMA's N: 256 for wide outputs, 64 for outputs as
// narrow as nocc, whose 256-wide tiles would be mostly padding), with the
// stage count that fills ~192 KB of shared memory.
// Instruction descriptor (kind::f16): D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
template <int BN_>
struct Tile {
  static constexpr int BN = BN_;
  static constexpr int STAGES = BN_ >= 256 ? 4 : 8;
  static constexpr int B_BYTES = BN_ * BK * 2;
  static constexpr int SMEM_BYTES = STAGES * (A_BYTES + B_BYTES) + 1024;  // + alignment slack
  static constexpr uint32_t TMEM_COLS = 2 * BN_;                          // two accumulators, a power of 2
  static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN_ >> 3) << 17) |
                                    ((uint32_t)(BM >> 4) << 24);
  static_assert(BN_ % 16 == 0 && BN_ >= 16 && BN_ <= 256, "MMA N for M = 128");
  static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
};

// Shared-memory matrix descriptor of a K-major operand tile written by TMA
// with the 128-byte swizzle: rows of 128 bytes, 8-row atoms 1024 bytes apart
// (stride byte offset), start address >> 4 in bits 0-13, leading byte offset
// (unused for this layout) 16 bytes, descriptor version 1 at bit 46, swizzle
// mode 2 (128 B) at bits 61-63.  Stepping K by 16 elements inside the
// 128-byte row adds 32 bytes to the start address.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t gtime() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(a),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase of parity `parity` to complete; false after ~2 s.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity) {
  if (mbar_try(a, parity)) return true;
  const uint64_t t0 = gtime();
  for (;;) {
    for (int i = 0; i < 256; ++i)
      if (mbar_try(a, parity)) return true;
    if (gtime() - t0 > 2000000000ull) return false;
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

// arrive on the mbarrier once every tcgen05 op issued so far by this thread completes
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// C row-major FP32 [M][ldc]
struct EpiRowMajor {
  static constexpr int kStageBytes = 0;
  float* C;
  int64_t M, N, ldc;
  __device__ __forceinline__ void operator()(int64_t row, int64_t col0, const float* v, int, int) const {
    if (row >= M) return;
    float* c = C + row * ldc + col0;
    if (col0 + 16 <= N && (ldc & 3) == 0) {
#pragma unroll
      for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(c + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i)
        if (col0 + i < N) c[i] = v[i];
    }
  }
};

// C row-major FP64 [M][ldc] (the FP32 accumulators widened exactly)
struct EpiRowMajorF64 {
  static constexpr int kStageBytes = 0;
  double* C;
  int64_t M, N, ldc;
  __device__ __forceinline__ void operator()(int64_t row, int64_t col0, const float* v, int, int) const {
    if (row >= M) return;
    double* c = C + row * ldc + col0;
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (col0 + i < N) c[i] = f2d_bits(v[i]);
  }
};

// C (FP64, strided) = alpha acc + beta C, for GEMMs whose rows or columns
// flatten a (batch, index) pair: element (r, c) sits at
// (r / mi) sro + (r % mi) sri + (c / ni) sco + (c % ni) sci.
struct EpiStridedF64 {
  static constexpr int kStageBytes = 0;
  double* C;
  int64_t M, N, mi, ni, sro, sri, sco, sci;
  double alpha, beta;
  int64_t srep;  // C offset of replica r: r * srep
  int beta0;     // beta == 0 (decided on the host: no per-element FP64 compare)
  // The cases of alpha and beta, decided on the host: GB300's FP64 unit runs
  // 2 operations per SM per clock, so a tile's 32K outputs cost ~16 us of
  // FP64 work at one multiply and one FMA each, far above the MMA time of
  // a GEMM with a short K.  amode 0: alpha = 1, 1: alpha = -1 (a sign-bit
  // flip), 2: alpha x.  bmode 0: beta = 0, 1: beta = 1 (one add), 2: beta C
  // (one FMA).  Each case gives the bits of alpha * x + beta * C.
  int amode = 2, bmode = 2;
  __device__ __forceinline__ void operator()(int64_t r, int64_t c0, const float* v, int, int rep) const {
    if (r >= M) return;
    const int64_t ro = r / mi;
    const int64_t rbase = rep * srep + ro * sro + (r - ro * mi) * sri;
    int64_t co = c0 / ni, ci = c0 - co * ni;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      if (c0 + i < N) {
        double* p = C + rbase + co * sco + ci * sci;
        double x = f2d_bits(v[i]);
        if (amode == 1) x = __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
        else if (amode == 2) x = alpha * x;
        if (bmode == 0) *p = x;
        else if (bmode == 1) *p = x + *p;
        else *p = fma(beta, *p, x);
      }
      if (++ci == ni) {
        ci = 0;
        ++co;
      }
    }
  }
};

// split K: slice s of replica rep's sum into the FP32 partial
// P[rep][s][N][M], column-major, so that a warp's 32 lanes (32 consecutive
// rows) store 128 contiguous bytes per column
struct EpiPartial {
  static constexpr int kStageBytes = 0;
  float* P;
  int64_t M, N;
  int ks;
  __device__ __forceinline__ void operator()(int64_t r, int64_t c0, const float* v, int s, int rep) const {
    if (r >= M) return;
    float* p = P + (((int64_t)rep * ks + s) * N + c0) * M + r;
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (c0 + i < N) p[(int64_t)i * M] = v[i];
  }
};

// C (the EpiStridedF64 mapping) = alpha sum_s P[s] + beta C, for each of
// `reps` replicas.  The FP32 slices are summed in slice order in FP32-pair
// arithmetic on the FP32 pipe (an error-free two-sum per slice, Knuth's
// TwoSum; the running pair carries ~48 bits) and rounded once to FP64:
// GB300's FP64 unit, not memory, bounded the FP64 sum of the slices.
// MODE 0: C = sum, 1: C = sum + C, 2: C = alpha sum + beta C (the host
// picks it, so no FP64 work is spent deciding per element).
// 32 x 32 tiles of (row, column): the partials are read with the lanes
// along rows (their contiguous index), the sums pass through shared memory,
// and C is written with the lanes along whichever of its rows or columns is
// contiguous.  Block 32 x 8 threads.
template <int MODE>
__global__ void __launch_bounds__(256) k_reduce_partials(const float* __restrict__ P, int ks, int64_t M, int64_t N,
                                                         EpiStridedF64 o, int reps, int rows_fast) {
  __shared__ double t[32][33];  // [column][row] of the tile
  const int lane = threadIdx.x, wy = threadIdx.y;
  const int64_t tm = (M + 31) / 32, tn = (N + 31) / 32, per = tm * tn, NM = N * M;
  for (int64_t b = blockIdx.x; b < reps * per; b += gridDim.x) {
    const int64_t rep = b / per, rem = b - rep * per;
    const int64_t r0 = (rem / tn) * 32, c0 = (rem % tn) * 32;
    // a thread's four elements (columns wy + 8 jj), eight slices' loads in
    // flight at a time, each sum in slice order
    float hs[4] = {0.0f, 0.0f, 0.0f, 0.0f}, ls[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const float* q[4];
    bool in[4];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int64_t r = r0 + lane, c = c0 + wy + 8 * jj;
      in[jj] = r < M && c < N;
      q[jj] = in[jj] ? P + (rep * ks * N + c) * M + r : P;
    }
    for (int s0 = 0; s0 < ks; s0 += 8) {
      const int cnt = ks - s0 < 8 ? ks - s0 : 8;
      float v[4][8];
#pragma unroll
      for (int jj = 0; jj < 4; ++jj)
#pragma unroll
        for (int u = 0; u < 8; ++u) v[jj][u] = (in[jj] && u < cnt) ? q[jj][(int64_t)(s0 + u) * NM] : 0.0f;
#pragma unroll
      for (int jj = 0; jj < 4; ++jj)
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (u < cnt) {
            const float x = v[jj][u];
            const float sh = __fadd_rn(hs[jj], x);
            const float bp = __fsub_rn(sh, hs[jj]);
            const float e = __fadd_rn(__fsub_rn(hs[jj], __fsub_rn(sh, bp)), __fsub_rn(x, bp));
            hs[jj] = sh;
            ls[jj] = __fadd_rn(ls[jj], e);
          }
    }
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) t[wy + 8 * jj][lane] = pair_to_f64(hs[jj], ls[jj]);
    __syncthreads();
    for (int j = wy; j < 32; j += 8) {
      const int64_t r = r0 + (rows_fast ? lane : j), c = c0 + (rows_fast ? j : lane);
      if (r < M && c < N) {
        const double acc = rows_fast ? t[j][lane] : t[lane][j];
        const int64_t ro = r / o.mi, co = c / o.ni;
        double* p = o.C + rep * o.srep + ro * o.sro + (r - ro * o.mi) * o.sri + co * o.sco + (c - co * o.ni) * o.sci;
        if (MODE == 0) *p = acc;
        else if (MODE == 1) *p = acc + *p;
        else *p = o.beta0 ? o.alpha * acc : o.alpha * acc + o.beta * *p;
      }
    }
    __syncthreads();
  }
}

// The (vv|vv) block for the O^2V^4 contraction.  The factor is symmetric
// (L[P,a,c] = L[P,c,a]), so row r of L_vv^T serves both operands and the
// GEMM value at (r1, r2) = (d v + b, c v + a) is (bd|ac) = (ac|bd); it is
// stored at W[(c v + d) * ldw + a v + b] (rows (c,d), columns (a,b): the
// layout the FP32 sparse kernel streams).  A warp's 32 lanes are 32
// consecutive r1, i.e. consecutive b: each of its stores writes one
// contiguous 128-byte run (two where the warp crosses a d boundary).
struct EpiVvvv {
  static constexpr int kStageBytes = 0;
  float* W;
  int64_t v, ldw;
  __device__ __forceinline__ void operator()(int64_t r1, int64_t r2, const float* x, int, int) const {
    if (r1 >= v * v) return;
    const int64_t d = r1 / v, b = r1 - d * v;
    int64_t c = r2 / v, a = r2 - c * v;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      if (c < v) W[(c * v + d) * ldw + a * v + b] = x[i];
      if (++a == v) {
        a = 0;
        ++c;
      }
    }
  }
};

__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(a)
      : "memory");
}

// linear tile index -> (m tile, n tile): groups of 16 M tiles sweep all N
// tiles, so the CTAs working at once share a few operand panels in L2
__host__ __device__ __forceinline__ void tile_coords(int id, int tiles_m, int tiles_n, int& mt, int& nt) {
  constexpr int GROUP = 16;
  const int per_group = GROUP * tiles_n;
  const int g = id / per_group, rem = id - g * per_group;
  const int gm = min(GROUP, tiles_m - g * GROUP);
  mt = g * GROUP + rem % gm;
  nt = rem / gm;
}

// Persistent: each CTA walks tiles blockIdx.x, +gridDim.x, ...  The TMEM
// accumulator is double-buffered (2 x 256 columns), so the epilogue warps
// drain tile i while the MMA warp accumulates tile i+1.
// The (vv|vv) block straight into the B' operand of the dense O^2V^4 GEMM:
// B'[q][k] for q = (a,b), k = (c,d) holds (ac|bd) as [hi | lo | hi] at
// k, R + k, 2R + k (R = v^2, rows of kpo elements).  GEMM row r1 = b v + d
// (L[:, b, d]) and column r2 = a v + c give (bd|ac) = (ac|bd); a warp's 32
// lanes are 32 consecutive d, so each store is one contiguous run.
struct EpiVvvvSplitB {
  // each epilogue warp stages a 32 x 16 block (rows padded to 17 floats)
  static constexpr int kStageBytes = EPI_WARPS * 32 * 17 * 4;
  __nv_bfloat16* B;
  int64_t v, kpo;
  int tri;  // only the tiles of the upper triangle run (RepTC::tri): write (r1, r2) and its mirror (r2, r1)
  __device__ __forceinline__ void put(int64_t a, int64_t b, int64_t c, int64_t d, float x) const {
    const int64_t R = v * v;
    const __nv_bfloat16 hi = __float2bfloat16(x);
    const __nv_bfloat16 lo = __float2bfloat16(x - __bfloat162float(hi));
    __nv_bfloat16* row = B + (a * v + b) * kpo + c * v + d;
    row[0] = hi;
    row[R] = lo;
    row[2 * R] = hi;
  }
  __device__ __forceinline__ void operator()(int64_t r1, int64_t r2, const float* x, int, int) const {
    const int64_t R = v * v;
    if (r1 >= R) return;
    const int64_t b = r1 / v, d = r1 - b * v;
    int64_t a = r2 / v, c = r2 - a * v;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      if (a < v) put(a, b, c, d, x[i]);
      if (++c == v) {
        c = 0;
        ++a;
      }
    }
  }
  // Triangle: the GEMM is symmetric (value (r1, r2) = (bd|ac) = (ac|bd) =
  // value (r2, r1)), so only tiles touching r1 <= r2 run, and each element
  // with r1 <= r2 is written at (r1, r2) and, for r1 < r2, at its mirror
  // (r2, r1); elements with r1 > r2 in a diagonal tile are written by their
  // mirror only, so every element is written once.  The direct stores are
  // contiguous along the lanes' rows (consecutive d); the mirror's
  // contiguous index is the column, so the warp's 32 x 16 block goes
  // through shared memory and each half-warp stores one mirrored row of 16.
  __device__ __forceinline__ void staged(int64_t r1, int64_t r2, const float* x, float* stg, int lane) const {
    if (!tri) {
      (*this)(r1, r2, x, 0, 0);
      return;
    }
    const int64_t R = v * v;
    if (r1 < R) {
      const int64_t b = r1 / v, d = r1 - b * v;
      int64_t a = r2 / v, c = r2 - a * v;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        if (a < v && r1 <= r2 + i) put(a, b, c, d, x[i]);
        if (++c == v) {
          c = 0;
          ++a;
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 16; ++i) stg[lane * 17 + i] = x[i];
    __syncwarp();
    // lane -> column i = lane & 15 of the block, rows j = 2 s + (lane >> 4)
    const int i = lane & 15;
    const int64_t q2 = r2 + i;  // (a, c) of the mirror's row and column
    if (q2 < R) {
      const int64_t a = q2 / v, c = q2 - a * v;
      const int64_t q1 = r1 - lane + (lane >> 4);  // the warp's first row, plus this lane's half
      int64_t b = q1 / v, d = q1 - b * v;
#pragma unroll 4
      for (int s = 0; s < 16; ++s) {
        const int64_t rr1 = q1 + 2 * s;
        if (rr1 < q2 && rr1 < R) put(b, a, d, c, stg[(2 * s + (lane >> 4)) * 17 + i]);
        d += 2;
        while (d >= v) {
          d -= v;
          ++b;
        }
      }
    }
    __syncwarp();
  }
};

// Upper-triangle tile enumeration of a symmetric GEMM with BN = 2 BM: tile
// (mt, nt) holds an element with row <= column iff mt <= 2 nt + 1.  The
// order is tile_coords' (groups of 16 M tiles, each sweeping its N tiles,
// M fastest) with the tiles below the diagonal left out; group g's needed
// tiles start at column 8 g, whose k-th column (k = nt - 8 g) holds
// min(2 k + 2, gm) of them.
__host__ __device__ __forceinline__ int tri_group_count(int g, int tiles_m, int tiles_n) {
  const int gm = min(16, tiles_m - 16 * g);
  const int kcols = tiles_n - 8 * g;  // columns from 8 g on
  if (gm <= 0 || kcols <= 0) return 0;
  const int kf = (gm - 1) / 2;        // first column holding all gm
  const int kp = min(kcols, kf);      // partial columns present
  return kp * (kp + 1) + max(0, kcols - kf) * gm;
}

__host__ __device__ __forceinline__ int tri_count(int tiles_m, int tiles_n) {
  int n = 0;
  for (int g = 0; 16 * g < tiles_m; ++g) n += tri_group_count(g, tiles_m, tiles_n);
  return n;
}

__host__ __device__ __forceinline__ void tri_coords(int id, int tiles_m, int tiles_n, int& mt, int& nt) {
  int g = 0;
  for (;; ++g) {
    const int cnt = tri_group_count(g, tiles_m, tiles_n);
    if (id < cnt || 16 * (g + 1) >= tiles_m) break;
    id -= cnt;
  }
  const int gm = min(16, tiles_m - 16 * g);
  const int kcols = tiles_n - 8 * g;
  const int kp = min(kcols, (gm - 1) / 2);
  const int P = kp * (kp + 1);
  int k;
  if (id < P) {  // column k holds 2 k + 2 tiles: k (k + 1) <= id < (k + 1)(k + 2)
    k = (int)((sqrtf(4.0f * (float)id + 1.0f) - 1.0f) * 0.5f);
    while ((k + 1) * (k + 2) <= id) ++k;
    while (k * (k + 1) > id) --k;
    mt = 16 * g + (id - k * (k + 1));
  } else {
    id -= P;
    k = kp + id / gm;
    mt = 16 * g + id % gm;
  }
  nt = 8 * g + k;
}

// Replicas: `reps` GEMMs of one shape in one launch (work units replica-
// major); replica r reads A' rows from r * a_rep (0: one A' for all) and B'
// rows from r * b_rep, and its epilogue gets r.  Each replica's tiles, K
// slices and accumulation order are those of a launch of its GEMM alone.
struct RepTC {
  int reps = 1;
  int a_rep = 0, b_rep = 0;
  int tri = 0;  // symmetric output, BN = 2 BM, M = N: only the upper-triangle tiles (tri_coords)
};

template <class TC, class Epi>
__global__ void __launch_bounds__(NT, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap tma, const __grid_constant__ CUtensorMap tmb, int K, int tiles_m,
              int tiles_n, int ksplit, Epi epi, unsigned* err, RepTC rt) {
  constexpr int BN = TC::BN, STAGES = TC::STAGES, B_BYTES = TC::B_BYTES;
  constexpr uint32_t IDESC = TC::IDESC;
  extern __shared__ uint8_t dsm[];
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], tfull[2], tempty[2];
  __shared__ uint32_t tbase;
  __shared__ int failed;
  const uint32_t base = (smem_u32(dsm) + 1023u) & ~1023u;
  const uint32_t sA = base, sB = base + STAGES * A_BYTES;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = rt.tri ? tri_count(tiles_m, tiles_n) : tiles_m * tiles_n;
  const int nk = (K + BK - 1) / BK;
  // split K: work unit u = (tile u % ntiles, K slice u / ntiles), each slice
  // nkc k blocks (the last one shorter, never empty)
  const int nkc = (nk + ksplit - 1) / ksplit;
  const int per_rep = ntiles * ksplit;
  const int nunits = per_rep * rt.reps;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&tfull[b]), 1);
      mbar_init(smem_u32(&tempty[b]), EPI_WARPS);
    }
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tbase)),
                 "r"(TC::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tbase;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      int g = 0;      // k blocks issued over all tiles
      for (int u = blockIdx.x; u < nunits && !*(volatile int*)&failed; u += gridDim.x) {
        const int rep = u / per_rep, w = u - rep * per_rep;
        int mt, nt;
        if (rt.tri) tri_coords(w % ntiles, tiles_m, tiles_n, mt, nt);
        else tile_coords(w % ntiles, tiles_m, tiles_n, mt, nt);
        const int kb1 = min(nk, (w / ntiles + 1) * nkc);
        for (int kb = (w / ntiles) * nkc; kb < kb1; ++kb, ++g) {
          const int s = g % STAGES;
          const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
          if (g >= STAGES && !mbar_wait(smem_u32(&empty[s]), ph ^ 1u)) {
            atomicOr(err, FRICC_DEV_TIMEOUT);
            failed = 1;
            break;
          }
          mbar_expect_tx(smem_u32(&full[s]), A_BYTES + B_BYTES);
          tma_load_2d(sA + s * A_BYTES, &tma, kb * BK, rep * rt.a_rep + mt * BM, smem_u32(&full[s]));
          tma_load_2d(sB + s * B_BYTES, &tmb, kb * BK, rep * rt.b_rep + nt * BN, smem_u32(&full[s]));
        }
      }
      if (*(volatile int*)&failed) {
        // let the copies in flight land before the CTA's shared memory goes away
        for (int q = g - STAGES < 0 ? 0 : g - STAGES; q < g; ++q)
          mbar_wait(smem_u32(&full[q % STAGES]), (uint32_t)(q / STAGES) & 1u);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      int g = 0, i = 0;
      for (int uu = blockIdx.x; uu < nunits; uu += gridDim.x, ++i) {
        const int w = uu % per_rep;
        const int b = i & 1;
        const uint32_t u = (uint32_t)(i >> 1);
        const int kb0 = (w / ntiles) * nkc, kb1 = min(nk, kb0 + nkc);
        // the epilogue must have drained this accumulator's previous tile
        if (i >= 2 && !mbar_wait(smem_u32(&tempty[b]), (u & 1u) ^ 1u)) {
          atomicOr(err, FRICC_DEV_TIMEOUT);
          failed = 1;
        }
        if (*(volatile int*)&failed) break;
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * BN);
        for (int kb = kb0; kb < kb1; ++kb, ++g) {
          const int s = g % STAGES;
          const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
          if (!mbar_wait(smem_u32(&full[s]), ph)) {
            atomicOr(err, FRICC_DEV_TIMEOUT);
            failed = 1;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = sA + s * A_BYTES, b0 = sB + s * B_BYTES;
#pragma unroll
          for (int k = 0; k < BK / 16; ++k)
            tc_mma(acc, sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), IDESC, ((kb - kb0) | k) != 0);
          tc_commit(smem_u32(&empty[s]));
        }
        tc_commit(smem_u32(&tfull[b]));  // arrives when this tile's MMAs have completed
        if (*(volatile int*)&failed) break;
      }
    }
  } else {  // epilogue warps 2..9: TMEM lanes 32 (warp % 4) ..., column half (warp - 2) / 4
    const int quad = warp & 3;
    const int half = (warp - 2) >> 2;
    int i = 0;
    for (int uu = blockIdx.x; uu < nunits; uu += gridDim.x, ++i) {
      const int rep = uu / per_rep, w = uu - rep * per_rep;
      const int b = i & 1;
      const uint32_t u = (uint32_t)(i >> 1);
      bool ok = mbar_wait(smem_u32(&tfull[b]), u & 1u);
      ok = __all_sync(0xffffffffu, ok && !*(volatile int*)&failed);
      if (!ok) {
        if (lane == 0) {
          atomicOr(err, FRICC_DEV_TIMEOUT);
          failed = 1;
        }
        break;
      }
      tc_fence_after();
      int mt, nt;
      if (rt.tri) tri_coords(w % ntiles, tiles_m, tiles_n, mt, nt);
        else tile_coords(w % ntiles, tiles_m, tiles_n, mt, nt);
      const int64_t row = (int64_t)mt * BM + quad * 32 + lane;
      const uint32_t lane_base = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * BN);
#pragma unroll 1
      for (int c = half * (BN / 32); c < (half + 1) * (BN / 32); ++c) {
        float v[16];
        tc_ld16(lane_base + (uint32_t)(c * 16), v);
        if constexpr (Epi::kStageBytes > 0) {
          float* stg = reinterpret_cast<float*>(dsm + (base - smem_u32(dsm)) + STAGES * (A_BYTES + B_BYTES)) +
                       (warp - 2) * 32 * 17;
          epi.staged(row, (int64_t)nt * BN + c * 16, v, stg, lane);
        } else {
          epi(row, (int64_t)nt * BN + c * 16, v, w / ntiles, rep);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&tempty[b]));
    }
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC::TMEM_COLS)
                 : "memory");
}

// x (FP64, strided) -> A' [rows][kp] = [hi | hi | lo] and B' [rows][kp] =
// [hi | lo | hi] (either may be null), kp >= 3k, padding columns zero.
// Row r = (r / ri, r % ri) and column j < k of x sit at
// (r / ri) sro + (r % ri) sri + j sk: a transposed or batch-flattened view
// becomes a K-major operand in the same pass.
__device__ __forceinline__ void split_put(double xv, int64_t k, __nv_bfloat16* ar, __nv_bfloat16* br) {
  const __nv_bfloat16 hi = __double2bfloat16(xv);
  const __nv_bfloat16 lo = __double2bfloat16(xv - (double)__bfloat162float(hi));
  if (ar) {
    ar[0] = hi;
    ar[k] = hi;
    ar[2 * k] = lo;
  }
  if (br) {
    br[0] = hi;
    br[k] = lo;
    br[2 * k] = hi;
  }
}

// columns contiguous (or any layout): work items of (row, 1024 columns), a
// block's threads over the columns, so a few very long rows spread as well
__global__ void k_split_rows(const double* __restrict__ x, int64_t rows, int64_t k, int64_t ri, int64_t sro,
                             int64_t sri, int64_t sk, int64_t kp, __nv_bfloat16* __restrict__ Ap,
                             __nv_bfloat16* __restrict__ Bp) {
  constexpr int64_t CH = 1024;
  const int64_t nch = fricc_cdiv(kp - 2 * k, CH);  // chunks over j < k, then the padding j >= 3k
  for (int64_t w = blockIdx.x; w < rows * nch; w += gridDim.x) {
    const int64_t r = w / nch, c = w - r * nch;
    const int64_t ro = r / ri;
    const double* xr = x + ro * sro + (r - ro * ri) * sri;
    __nv_bfloat16* ar = Ap ? Ap + r * kp : nullptr;
    __nv_bfloat16* br = Bp ? Bp + r * kp : nullptr;
    const int64_t j1 = (c + 1) * CH < k ? (c + 1) * CH : k;
    for (int64_t j = c * CH + threadIdx.x; j < j1; j += blockDim.x)
      split_put(xr[j * sk], k, ar ? ar + j : nullptr, br ? br + j : nullptr);
    // padding: chunk c also zeroes columns 3k + [c*CH - k, ...) that fall in [3k, kp)
    for (int64_t j = 3 * k + c * CH - k + threadIdx.x; j < kp && j < 3 * k + (c + 1) * CH - k; j += blockDim.x)
      if (j >= 3 * k) {
        if (ar) ar[j] = __float2bfloat16(0.0f);
        if (br) br[j] = __float2bfloat16(0.0f);
      }
  }
}

// rows contiguous (sri == 1, within runs of ri rows): 32 x 32 tiles read
// along r and written along j through shared memory
__global__ void k_split_tr(const double* __restrict__ x, int64_t rows, int64_t k, int64_t ri, int64_t sro, int64_t sk,
                           int64_t kp, __nv_bfloat16* __restrict__ Ap, __nv_bfloat16* __restrict__ Bp) {
  __shared__ double tile[32][33];
  const int64_t tiles_r = fricc_cdiv(rows, 32), tiles_k = fricc_cdiv(k, 32);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int64_t t = blockIdx.x; t < tiles_r * tiles_k; t += gridDim.x) {
    const int64_t r0 = (t / tiles_k) * 32, j0 = (t % tiles_k) * 32;
    __syncthreads();
    for (int yy = ty; yy < 32; yy += 8) {  // tile[j][r]: read x(r0 + tx, j0 + yy)
      const int64_t r = r0 + tx, j = j0 + yy;
      double v = 0.0;
      if (r < rows && j < k) {
        const int64_t ro = r / ri;
        v = x[ro * sro + (r - ro * ri) + j * sk];
      }
      tile[yy][tx] = v;
    }
    __syncthreads();
    for (int yy = ty; yy < 32; yy += 8) {  // write row r0 + yy, columns j0 + tx
      const int64_t r = r0 + yy, j = j0 + tx;
      if (r < rows && j < k)
        split_put(tile[tx][yy], k, Ap ? Ap + r * kp + j : nullptr, Bp ? Bp + r * kp + j : nullptr);
    }
  }
  // padding columns
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < rows * (kp - 3 * k);
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / (kp - 3 * k), j = 3 * k + (t - r * (kp - 3 * k));
    if (Ap) Ap[r * kp + j] = __float2bfloat16(0.0f);
    if (Bp) Bp[r * kp + j] = __float2bfloat16(0.0f);
  }
}

// looked up once; a function-local static is initialised exactly once even
// when several host threads (a request server's workers) arrive together
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return nullptr;
  }();
  return fn;
}

// 2-D map of a K-major BF16 matrix [rows][ld] (K = k columns used), box
// (64 K elements = 128 bytes) x box_rows, 128-byte swizzle, zero fill.
int make_map(CUtensorMap* map, const void* ptr, int64_t rows, int64_t k, int64_t ld, int box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    fricc_set_error("gemm_tc: cuTensorMapEncodeTiled is unavailable");
    return FRICC_ERR_CUDA;
  }
  cuuint64_t gdim[2] = {(cuuint64_t)k, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), gdim, gstride, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    fricc_set_error("gemm_tc: cuTensorMapEncodeTiled failed (%d)", (int)r);
    return FRICC_ERR_ARG;
  }
  return FRICC_OK;
}

// status == nullptr: synchronous, a gave-up wait returns FRICC_ERR_TIMEOUT;
// otherwise stream-ordered (capturable): the kernel ORs FRICC_DEV_TIMEOUT into
// *status and the caller reads it later.
int sm_count(int* out) {
  static std::atomic<int> cached{0};  // shared by the host threads; every writer stores the same value
  int nsm = cached.load(std::memory_order_relaxed);
  if (!nsm) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || nsm <= 0)
      return fricc_cuda_fail(e != cudaSuccess ? e : cudaErrorUnknown, "gemm_tc SM count", __FILE__, __LINE__);
    cached.store(nsm, std::memory_order_relaxed);
  }
  *out = nsm;
  return FRICC_OK;
}

template <class TC, class Epi>
int launch_tile(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N, int64_t K,
                const Epi& epi, cudaStream_t st, unsigned* status, int ksplit, RepTC rt) {
  constexpr int BN = TC::BN, SMEM_BYTES = TC::SMEM_BYTES + Epi::kStageBytes;
  static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
  if (!A || !B || M <= 0 || N <= 0 || K <= 0 || lda < K || ldb < K || (lda % 8) || (ldb % 8) ||
      (reinterpret_cast<uintptr_t>(A) % 16) || (reinterpret_cast<uintptr_t>(B) % 16)) {
    fricc_set_error("gemm_tc: bad arguments (K-major BF16 operands: 16-byte aligned, ld >= K, ld %% 8 == 0)");
    return FRICC_ERR_ARG;
  }
  // a replica's operand rows must not overlap the next replica's
  if (rt.reps < 1 || (rt.a_rep != 0 && rt.a_rep < M) || (rt.b_rep != 0 && rt.b_rep < N) || rt.a_rep < 0 ||
      rt.b_rep < 0) {
    fricc_set_error("gemm_tc: bad replica layout");
    return FRICC_ERR_ARG;
  }
  if (rt.tri && (BN != 2 * BM || M != N || rt.reps != 1)) {
    fricc_set_error("gemm_tc: the triangle schedule needs BN = 2 BM, M = N and one replica");
    return FRICC_ERR_ARG;
  }
  // the rows of A' and B' over all replicas (TMA coordinates are 32-bit)
  const int64_t rows_a = rt.a_rep ? (int64_t)rt.reps * rt.a_rep : M;
  const int64_t rows_b = rt.b_rep ? (int64_t)rt.reps * rt.b_rep : N;
  const int64_t tm = fricc_cdiv(M, BM), tn = fricc_cdiv(N, BN);
  if (tm * tn * ksplit * rt.reps > 0x7fffffffLL || K > 0x7fffffffLL || rows_a + BM > 0x7fffffffLL ||
      rows_b + BN > 0x7fffffffLL) {
    fricc_set_error("gemm_tc: problem too large for one launch");
    return FRICC_ERR_ARG;
  }
  CUtensorMap ma, mb;
  int rc = make_map(&ma, A, rows_a, K, lda, BM);
  if (!rc) rc = make_map(&mb, B, rows_b, K, ldb, BN);
  if (rc) return rc;
  // per instantiation; threads that race here all set the same attribute
  static std::atomic<bool> attr{false};
  cudaError_t e = cudaSuccess;
  if (!attr.load(std::memory_order_acquire)) {
    e = cudaFuncSetAttribute(k_gemm_tc<TC, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return fricc_cuda_fail(e, "gemm_tc attribute", __FILE__, __LINE__);
    attr.store(true, std::memory_order_release);
  }
  int nsm = 0;
  rc = sm_count(&nsm);
  if (rc) return rc;
  const int64_t nk = fricc_cdiv(K, BK);
  if (ksplit < 1 || ksplit > nk) {
    fricc_set_error("gemm_tc: split K must be between 1 and the number of 64-wide K blocks");
    return FRICC_ERR_ARG;
  }
  const int64_t nkc = fricc_cdiv(nk, ksplit);
  ksplit = (int)fricc_cdiv(nk, nkc);  // every slice non-empty
  const int64_t tiles = rt.tri ? tri_count((int)tm, (int)tn) : tm * tn;
  const int64_t units = tiles * ksplit * rt.reps;
  // flops the tensor cores run: the triangle's share of M N
  const double mn = (double)M * (double)N * (double)tiles / (double)(tm * tn);
  const unsigned grid = (unsigned)(units < nsm ? units : nsm);  // persistent: one CTA per SM
  const bool prof = fricc_prof_on();
  if (status) {
    if (prof) fricc_prof_record(st, true, 0.0, 1);
    k_gemm_tc<TC, Epi><<<grid, NT, SMEM_BYTES, st>>>(ma, mb, (int)K, (int)tm, (int)tn, ksplit, epi, status, rt);
    if (prof) fricc_prof_record(st, false, 2.0 * rt.reps * mn * (double)K, 1);
    fricc_note_launch();
    e = cudaGetLastError();
    return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "gemm_tc", __FILE__, __LINE__);
  }
  unsigned* err = nullptr;
  rc = fricc_alloc_t(&err, 1, st);
  if (rc) return rc;
  e = cudaMemsetAsync(err, 0, sizeof(unsigned), st);
  if (e == cudaSuccess) {
    if (prof) fricc_prof_record(st, true, 0.0, 1);
    k_gemm_tc<TC, Epi><<<grid, NT, SMEM_BYTES, st>>>(ma, mb, (int)K, (int)tm, (int)tn, ksplit, epi, err, rt);
    if (prof) fricc_prof_record(st, false, 2.0 * rt.reps * mn * (double)K, 1);
    fricc_note_launch();
    e = cudaGetLastError();
  }
  unsigned herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  fricc_free(err, st);
  if (e != cudaSuccess) return fricc_cuda_fail(e, "gemm_tc", __FILE__, __LINE__);
  if (herr) {
    fricc_set_error("gemm_tc: a bounded pipeline wait gave up (device error 0x%x)", herr);
    return FRICC_ERR_TIMEOUT;
  }
  return FRICC_OK;
}

// tile width by the output's N: 64 when N <= 64 (nocc-wide outputs), else 256
template <class Epi>
int launch(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N, int64_t K, const Epi& epi,
           cudaStream_t st, unsigned* status = nullptr, int ksplit = 1, RepTC rt = RepTC{}) {
  if (N <= 64) return launch_tile<Tile<64>>(A, lda, B, ldb, M, N, K, epi, st, status, ksplit, rt);
  return launch_tile<Tile<256>>(A, lda, B, ldb, M, N, K, epi, st, status, ksplit, rt);
}

}  // namespace tc

extern "C" {

int fricc_gemm_bf16_tn(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N, int64_t K,
                       float* C, int64_t ldc, void* stream) {
  if (!C || ldc < N) {
    fricc_set_error("gemm_bf16_tn: bad output");
    return FRICC_ERR_ARG;
  }
  return tc::launch(A, lda, B, ldb, M, N, K, tc::EpiRowMajor{C, M, N, ldc}, (cudaStream_t)stream);
}

int fricc_gemm_bf16_tn_f64(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N, int64_t K,
                           double* C, int64_t ldc, void* stream) {
  if (!C || ldc < N) {
    fricc_set_error("gemm_bf16_tn_f64: bad output");
    return FRICC_ERR_ARG;
  }
  return tc::launch(A, lda, B, ldb, M, N, K, tc::EpiRowMajorF64{C, M, N, ldc}, (cudaStream_t)stream);
}

int fricc_split_bf16x3_strided(const double* x, int64_t rows, int64_t k, int64_t ri, int64_t sro, int64_t sri,
                               int64_t sk, int64_t kp, void* Ap, void* Bp, void* stream) {
  if (rows < 0 || k <= 0 || ri <= 0 || kp < 3 * k || (kp % 8) || (rows > 0 && (!x || (!Ap && !Bp)))) {
    fricc_set_error("split_bf16x3: bad arguments");
    return FRICC_ERR_ARG;
  }
  const int64_t n = rows * kp;
  if (n == 0) return FRICC_OK;
  auto* a = static_cast<__nv_bfloat16*>(Ap);
  auto* b = static_cast<__nv_bfloat16*>(Bp);
  if (sri == 1 && sk != 1 && ri >= 32) {
    int64_t g = fricc_cdiv(rows, 32) * fricc_cdiv(k, 32);
    if (g > 152 * 16) g = 152 * 16;
    tc::k_split_tr<<<(unsigned)g, 256, 0, (cudaStream_t)stream>>>(x, rows, k, ri, sro, sk, kp, a, b);
  } else {
    const int64_t items = rows * fricc_cdiv(kp - 2 * k, 1024);
    const int64_t g = items < 152 * 16 ? items : 152 * 16;
    tc::k_split_rows<<<(unsigned)g, 128, 0, (cudaStream_t)stream>>>(x, rows, k, ri, sro, sri, sk, kp, a, b);
  }
  fricc_note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "split_bf16x3", __FILE__, __LINE__);
}

int fricc_split_bf16x3(const double* x, int64_t rows, int64_t k, int64_t ld, int64_t kp, void* Ap, void* Bp,
                       void* stream) {
  if (ld < k || !Ap || !Bp) {
    fricc_set_error("split_bf16x3: bad arguments");
    return FRICC_ERR_ARG;
  }
  return fricc_split_bf16x3_strided(x, rows, k, 1, ld, ld, 1, kp, Ap, Bp, stream);
}

int fricc_gemm_bf16_tn_strided_b(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N,
                                 int64_t K, double* C, int64_t mi, int64_t ni, int64_t sro, int64_t sri, int64_t sco,
                                 int64_t sci, double alpha, double beta, int ksplit, int reps, int64_t a_rep,
                                 int64_t b_rep, int64_t c_rep, unsigned* status, void* stream) {
  if (!C || mi <= 0 || ni <= 0 || ksplit < 1 || reps < 1 || reps > 65535 || a_rep < 0 || b_rep < 0 ||
      a_rep > 0x7fffffffLL || b_rep > 0x7fffffffLL) {
    fricc_set_error("gemm_bf16_tn_strided: bad output, split or replica layout");
    return FRICC_ERR_ARG;
  }
  tc::EpiStridedF64 out{C, M, N, mi, ni, sro, sri, sco, sci, alpha, beta, c_rep, beta == 0.0 ? 1 : 0};
  out.amode = alpha == 1.0 ? 0 : (alpha == -1.0 ? 1 : 2);
  out.bmode = beta == 0.0 ? 0 : (beta == 1.0 ? 1 : 2);
  tc::RepTC rt;
  rt.reps = reps;
  rt.a_rep = (int)a_rep;
  rt.b_rep = (int)b_rep;
  cudaStream_t st = (cudaStream_t)stream;
  if (ksplit == 1) return tc::launch(A, lda, B, ldb, M, N, K, out, st, status, 1, rt);
  // split K: FP32 partials per slice, then one ordered reduction into C
  const int64_t nk = fricc_cdiv(K, tc::BK);
  if (ksplit > nk) ksplit = (int)nk;
  const int ks = (int)fricc_cdiv(nk, fricc_cdiv(nk, ksplit));
  float* P = nullptr;
  int rc = fricc_alloc_t(&P, (size_t)reps * ks * M * N, st);
  if (rc) return rc;
  rc = tc::launch(A, lda, B, ldb, M, N, K, tc::EpiPartial{P, M, N, ks}, st, status, ks, rt);
  if (!rc) {
    int64_t g = reps * fricc_cdiv(M, 32) * fricc_cdiv(N, 32);
    if (g > 152 * 16) g = 152 * 16;
    // write C along its rows when they are the contiguous index
    const int rows_fast = (sri == 1 && sci != 1) ? 1 : 0;
    const dim3 blk(32, 8);
    if (alpha == 1.0 && beta == 0.0) tc::k_reduce_partials<0><<<(unsigned)g, blk, 0, st>>>(P, ks, M, N, out, reps, rows_fast);
    else if (alpha == 1.0 && beta == 1.0)
      tc::k_reduce_partials<1><<<(unsigned)g, blk, 0, st>>>(P, ks, M, N, out, reps, rows_fast);
    else tc::k_reduce_partials<2><<<(unsigned)g, blk, 0, st>>>(P, ks, M, N, out, reps, rows_fast);
    fricc_note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = fricc_cuda_fail(e, "gemm_tc reduce", __FILE__, __LINE__);
  }
  fricc_free(P, st);
  return rc;
}

int fricc_gemm_bf16_tn_strided(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N,
                               int64_t K, double* C, int64_t mi, int64_t ni, int64_t sro, int64_t sri, int64_t sco,
                               int64_t sci, double alpha, double beta, int ksplit, unsigned* status, void* stream) {
  return fricc_gemm_bf16_tn_strided_b(A, lda, B, ldb, M, N, K, C, mi, ni, sro, sri, sco, sci, alpha, beta, ksplit, 1,
                                      0, 0, 0, status, stream);
}

int fricc_vvvv_rebuild_bf16x3(const void* Ap, const void* Bp, int64_t v, int64_t kp, float* W, int64_t ldw,
                              unsigned* status, void* stream) {
  if (!W || v <= 0 || ldw < v * v) {
    fricc_set_error("vvvv_rebuild_bf16x3: bad arguments");
    return FRICC_ERR_ARG;
  }
  return tc::launch(Ap, kp, Bp, kp, v * v, v * v, kp, tc::EpiVvvv{W, v, ldw}, (cudaStream_t)stream, status);
}

int fricc_vvvv_rebuild_split_b(const void* Ap, const void* Bp, int64_t v, int64_t kp, void* Bout, int64_t kpo,
                               unsigned* status, void* stream) {
  if (!Bout || v <= 0 || kpo < 3 * v * v || (kpo % 8)) {
    fricc_set_error("vvvv_rebuild_split_b: bad arguments");
    return FRICC_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  // the padding columns past 3 v^2 must be zero
  if (kpo > 3 * v * v) {
    cudaError_t e = cudaMemset2DAsync(static_cast<__nv_bfloat16*>(Bout) + 3 * v * v, sizeof(__nv_bfloat16) * kpo, 0,
                                      sizeof(__nv_bfloat16) * (kpo - 3 * v * v), v * v, st);
    if (e != cudaSuccess) return fricc_cuda_fail(e, "vvvv_rebuild_split_b padding", __FILE__, __LINE__);
  }
  // the GEMM is symmetric: above 64 columns (the 256-wide tile) only its
  // upper-triangle tiles run, each writing its elements and their mirrors
  if (v * v > 64) {
    tc::RepTC rt;
    rt.tri = 1;
    return tc::launch_tile<tc::Tile<256>>(Ap, kp, Bp, kp, v * v, v * v, kp,
                                          tc::EpiVvvvSplitB{static_cast<__nv_bfloat16*>(Bout), v, kpo, 1}, st,
                                          status, 1, rt);
  }
  return tc::launch(Ap, kp, Bp, kp, v * v, v * v, kp,
                    tc::EpiVvvvSplitB{static_cast<__nv_bfloat16*>(Bout), v, kpo, 0}, st, status);
}

}  // extern "C"
