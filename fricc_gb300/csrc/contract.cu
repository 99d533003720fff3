// The eleven sparse-T2 x dense-W contraction terms of fri-cc
// (src/sparse_tensor.cpp:12-346, dispatcher :349-382) as one bucketed
// SpMM kernel driven by a term table.
//
// Every term has the form
//     out'[P, q] += coef * sum_{e in bucket P} W'[key_e, q] * value_e
// where P is the pair of index slots the reference filters on, key_e the
// pair of slots that indexes W, and q the two dense indices of the inner
// loops.  W' and out' are W and out with their axes permuted so that q is
// the contiguous innermost pair; a W or out that already has that layout
// (any strides that say so) is used in place, anything else is gathered
// into a permuted copy first (and scattered back for out).
//
// The reference visits the nonzeros of each output element in slot order;
// the bucketing is a stable sort, so each output element here receives its
// contributions in the same order (fused multiply-add, one rounding per
// term instead of two).
#include <cmath>
#include <cstring>

#include <cuda_bf16.h>

#include "radix.cuh"
#include "sparse.cuh"

namespace {

struct TermSpec {
  const char* name;
  int pa, pb;     // bucket slots (outer pair of the reference loop)
  int ka, kb;     // slots that index W
  int permW[4];   // W' axis j = W axis permW[j]
  int permO[4];   // out' axis j = out axis permO[j]
  double coef;
};

// Index algebra per term, from the loops of src/sparse_tensor.cpp.
const TermSpec kTerms[] = {
    // out(i,j,a,b) += W(k,l,i,j) T(k,l,a,b)                     :12-37
    {"0101", 2, 3, 0, 1, {0, 1, 2, 3}, {2, 3, 0, 1}, 1.0},
    // out(i,j,a,b) += W(a,b,c,d) T(i,j,c,d)                     :40-86
    {"2323", 0, 1, 2, 3, {2, 3, 0, 1}, {0, 1, 2, 3}, 1.0},
    // out(i,j,a,b) += 2 W(a,k,i,c) T(k,j,c,b)                   :89-115
    {"1302", 1, 3, 0, 2, {1, 3, 2, 0}, {1, 3, 0, 2}, 2.0},
    // out(i,j,a,b) -= W(a,k,c,i) T(k,j,c,b)                     :118-144
    {"1202", 1, 3, 0, 2, {1, 2, 3, 0}, {1, 3, 0, 2}, -1.0},
    // out(i,j,a,b) += W(a,k,i,c) T(k,j,b,c)                     :147-173
    {"1303", 1, 2, 0, 3, {1, 3, 2, 0}, {1, 3, 0, 2}, 1.0},
    // out(i,j,a,b) += W(b,k,c,i) T(k,j,a,c)                     :176-202
    {"1203", 1, 2, 0, 3, {1, 2, 3, 0}, {1, 2, 0, 3}, 1.0},
    // out(k,l,i,j) += ovov(k,c,l,d) T(i,j,c,d)                  :205-230
    {"1323", 0, 1, 2, 3, {1, 3, 0, 2}, {2, 3, 0, 1}, 1.0},
    // out(a,k,i,c) -= 0.5 ovov(l,d,k,c) T(i,l,d,a)              :233-259
    {"0112", 3, 0, 1, 2, {0, 1, 2, 3}, {0, 2, 1, 3}, -0.5},
    // out(a,k,i,c) += ovov(l,d,k,c) T(i,l,a,d)                  :292-317
    {"0113", 2, 0, 1, 3, {0, 1, 2, 3}, {0, 2, 1, 3}, 1.0},
    // out(a,k,i,c) -= 0.5 ovov(l,c,k,d) T(i,l,a,d)              :262-289
    {"0313", 2, 0, 1, 3, {0, 3, 2, 1}, {0, 2, 1, 3}, -0.5},
    // out(a,k,c,i) -= 0.5 ovov(l,c,k,d) T(i,l,d,a)              :320-346
    {"0312", 3, 0, 1, 2, {0, 3, 2, 1}, {0, 3, 1, 2}, -0.5},
};

const TermSpec* find_term(const char* name) {
  if (!name) return nullptr;
  for (const auto& t : kTerms)
    if (std::strcmp(t.name, name) == 0) return &t;
  return nullptr;
}

// Replica batches: per-replica strides (elements) of the m-sized arrays
// (slots count 4 per entry), of bptr, of W' and of the output; the replica
// is blockIdx.y (blockIdx.z in the contraction kernels).  Zero outside a
// batch.
struct RepC {
  int64_t m = 0, b = 0, w = 0, o = 0;
};

__global__ void k_pair_keys(const int* __restrict__ slots, int64_t m, int pa, int pb, int64_t dpb,
                            unsigned long long* __restrict__ keys, unsigned* __restrict__ idx, RepC rp = RepC{}) {
  slots += 4 * blockIdx.y * rp.m;
  keys += blockIdx.y * rp.m;
  idx += blockIdx.y * rp.m;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m; s += (int64_t)gridDim.x * blockDim.x) {
    keys[s] = (unsigned long long)slots[4 * s + pa] * (unsigned long long)dpb + (unsigned long long)slots[4 * s + pb];
    idx[s] = (unsigned)s;
  }
}

// bptr[P] = first position whose key >= P (keys sorted ascending)
__global__ void k_bptr(const unsigned long long* __restrict__ keys, int64_t m, int64_t nb, int* __restrict__ bptr,
                       RepC rp = RepC{}) {
  keys += blockIdx.y * rp.m;
  bptr += blockIdx.y * rp.b;
  for (int64_t P = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; P <= nb; P += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = m;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (keys[mid] < (unsigned long long)P) lo = mid + 1;
      else hi = mid;
    }
    bptr[P] = (int)lo;
  }
}

// per-term entry list in bucket order: W' row and coef * value
__global__ void k_entries(const int* __restrict__ slots, const double* __restrict__ vals,
                          const unsigned* __restrict__ order, int64_t m, int ka, int kb, int64_t dkb, double coef,
                          int* __restrict__ erow, double* __restrict__ eval, RepC rp = RepC{}) {
  slots += 4 * blockIdx.y * rp.m;
  vals += blockIdx.y * rp.m;
  order += blockIdx.y * rp.m;
  erow += blockIdx.y * rp.m;
  eval += blockIdx.y * rp.m;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
    const unsigned s = order[e];
    erow[e] = (int)((int64_t)slots[4 * s + ka] * dkb + slots[4 * s + kb]);
    eval[e] = coef * vals[s];  // coef is +-1, 2 or -1/2: exact
  }
}

constexpr int SP_NT = 128;
constexpr int SP_QPT = 2;

__global__ void __launch_bounds__(SP_NT) k_spmm(const int* __restrict__ bptr, const int* __restrict__ erow,
                                                const double* __restrict__ eval, const double* __restrict__ Wp,
                                                double* __restrict__ Op, int64_t QS, RepC rp = RepC{}) {
  {
    const int64_t r = blockIdx.z;
    bptr += r * rp.b;
    erow += r * rp.m;
    eval += r * rp.m;
    Wp += r * rp.w;
    Op += r * rp.o;
  }
  __shared__ int srow[SP_NT];
  __shared__ double sval[SP_NT];
  const int64_t P = blockIdx.x;
  const int e0 = bptr[P], e1 = bptr[P + 1];
  if (e0 == e1) return;
  const int64_t q0 = (int64_t)blockIdx.y * (SP_NT * SP_QPT) + threadIdx.x;
  double* orow = Op + P * QS;
  double acc[SP_QPT];
#pragma unroll
  for (int k = 0; k < SP_QPT; ++k) {
    const int64_t q = q0 + k * SP_NT;
    acc[k] = q < QS ? orow[q] : 0.0;
  }
  for (int eb = e0; eb < e1; eb += SP_NT) {
    const int cnt = e1 - eb < SP_NT ? e1 - eb : SP_NT;
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      srow[threadIdx.x] = erow[eb + threadIdx.x];
      sval[threadIdx.x] = eval[eb + threadIdx.x];
    }
    __syncthreads();
    for (int j = 0; j < cnt; ++j) {
      const double* w = Wp + (int64_t)srow[j] * QS;
      const double v = sval[j];
#pragma unroll
      for (int k = 0; k < SP_QPT; ++k) {
        const int64_t q = q0 + k * SP_NT;
        if (q < QS) acc[k] = fma(w[q], v, acc[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < SP_QPT; ++k) {
    const int64_t q = q0 + k * SP_NT;
    if (q < QS) orow[q] = acc[k];
  }
}

// ---------------------------------------------------------------------------
// FP32-pair ("double-float") variant.  GB300 issues 128 FP32 lanes per SM per
// clock but only 2 FP64 FMAs, so each product-accumulate is done on pairs of
// floats carrying ~48 significand bits:
//   W = Wh + Wl, v = vh + vl (split once from FP64 by bit manipulation,
//   split_f2_bits: |W - Wh - Wl| < 2^-47 |W|, |Wl| < 2^-23 |Wh|),
//   p = Wh*vh exactly as ph + e (one FMA recovers the rounding error),
//   pl = e + Wh*vl + Wl*vh (Wl*vl, ~2^-48 relative, is dropped),
//   (ah, al) += (ph, pl) with an error-free two-sum on the high parts,
// renormalised once per staged chunk of terms; the FP64 result is
// (double)ah + (double)al.  Relative error per output ~1e-14, against
// FP64's ~1e-16.
//
// Each thread owns pairs of adjacent outputs (q, q+1) and runs both through
// the packed f32x2 instructions (add/sub/mul/fma.rn.f32x2): one issue slot
// per two lanes of arithmetic.  W' is stored to match ("q-pair layout"):
// row r, pair t holds the float4 (Wh[r][2t], Wh[r][2t+1], Wl[r][2t],
// Wl[r][2t+1]); rows have ceil(QS/2) pairs, an odd QS padded with zero.
__device__ __forceinline__ float2 split_f2(double d) { return split_f2_bits(d); }

typedef unsigned long long f32x2;  // two floats in one 64-bit register pair

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

constexpr int DF_NT = 128;  // threads per CTA; PPT q-pairs per thread, so a CTA covers 256 PPT outputs of a row

// one staged chunk of terms into the thread's PPT accumulator pairs
template <int DF_PPT, bool FULL>
__device__ __forceinline__ void df_tile(const int* __restrict__ srow, const ulonglong2* __restrict__ sv,
                                        const f32x2* __restrict__ snv, int cnt, const ulonglong2* __restrict__ wq,
                                        int64_t QS2, int64_t trem, f32x2* ah, f32x2* al) {
  for (int j = 0; j < cnt; ++j) {
    const ulonglong2* w = wq + (int64_t)srow[j] * QS2;
    const ulonglong2 v = sv[j];  // (vh, vh), (vl, vl)
    const f32x2 nvh = snv[j];    // (-vh, -vh)
#pragma unroll
    for (int k = 0; k < DF_PPT; ++k) {
      if (FULL || k * DF_NT < trem) {
        const ulonglong2 x = w[k * DF_NT];           // (Wh, Wh'), (Wl, Wl')
        const f32x2 nph = mul2(x.x, nvh);            // -ph = -RN(Wh vh)
        f32x2 pl = fma2(x.x, v.x, nph);              // Wh vh - ph, exact
        pl = fma2(x.x, v.y, pl);
        pl = fma2(x.y, v.x, pl);
        // two-sum (ah, ph) -> (s, err), written with -ph
        const f32x2 s = sub2(ah[k], nph);
        const f32x2 z = sub2(s, ah[k]);
        const f32x2 err = sub2(sub2(ah[k], sub2(s, z)), add2(nph, z));
        al[k] = add2(al[k], add2(err, pl));
        ah[k] = s;
      }
    }
  }
}

// One (bucket P, q tile qt) work item of the float-pair sparse kernel:
// out'[P][q tile] += sum over the bucket's entries, staged DF_NT at a time.
template <int DF_PPT>
__device__ __forceinline__ void spmm_df_item(int64_t P, int64_t qt, const int* __restrict__ bptr,
                                             const int* __restrict__ erow, const float2* __restrict__ eval,
                                             const float4* __restrict__ Wp4, double* __restrict__ Op, int64_t QS,
                                             int* srow, ulonglong2* sv, f32x2* snv) {
  const int e0 = bptr[P], e1 = bptr[P + 1];
  if (e0 == e1) return;
  const int64_t QS2 = (QS + 1) >> 1;
  const int64_t t0 = qt * (DF_NT * DF_PPT) + threadIdx.x;
  const int64_t trem = QS2 - t0;  // this thread's pairs are t0 + k*DF_NT < QS2  <=>  k*DF_NT < trem
  const bool full = (qt + 1) * (DF_NT * DF_PPT) <= QS2;  // uniform per block
  double* orow = Op + P * QS;
  const ulonglong2* wq = reinterpret_cast<const ulonglong2*>(Wp4) + t0;
  f32x2 ah[DF_PPT], al[DF_PPT];
#pragma unroll
  for (int k = 0; k < DF_PPT; ++k) {
    const int64_t q = 2 * (t0 + k * DF_NT);
    const float2 a = split_f2(q < QS ? orow[q] : 0.0);
    const float2 b = split_f2(q + 1 < QS ? orow[q + 1] : 0.0);
    ah[k] = pk2(a.x, b.x);
    al[k] = pk2(a.y, b.y);
  }
  for (int eb = e0; eb < e1; eb += DF_NT) {
    const int cnt = e1 - eb < DF_NT ? e1 - eb : DF_NT;
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      const float2 v = eval[eb + threadIdx.x];
      srow[threadIdx.x] = erow[eb + threadIdx.x];
      sv[threadIdx.x] = make_ulonglong2(pk2(v.x, v.x), pk2(v.y, v.y));
      snv[threadIdx.x] = pk2(-v.x, -v.x);
    }
    __syncthreads();
    if (full) df_tile<DF_PPT, true>(srow, sv, snv, cnt, wq, QS2, trem, ah, al);
    else df_tile<DF_PPT, false>(srow, sv, snv, cnt, wq, QS2, trem, ah, al);
    // renormalise once per staged chunk (<= DF_NT terms): keeps |al| ~ ulp(ah)
#pragma unroll
    for (int k = 0; k < DF_PPT; ++k) {
      const f32x2 s = add2(ah[k], al[k]);
      al[k] = sub2(al[k], sub2(s, ah[k]));
      ah[k] = s;
    }
  }
#pragma unroll
  for (int k = 0; k < DF_PPT; ++k) {
    const int64_t q = 2 * (t0 + k * DF_NT);
    const float2 h = upk2(ah[k]), l = upk2(al[k]);
    if (q < QS) orow[q] = pair_to_f64(h.x, l.x);
    if (q + 1 < QS) orow[q + 1] = pair_to_f64(h.y, l.y);
  }
}

// At least 8 CTAs per SM (a 64-register cap): measured 6% less time in
// this kernel over the o30v150 terms than the compiler's own register choice
// (62), which left the same occupancy but scheduled the loads worse.
template <int DF_PPT>
__global__ void __launch_bounds__(DF_NT, 8) k_spmm_df(const int* __restrict__ bptr, const int* __restrict__ erow,
                                                   const float2* __restrict__ eval, const float4* __restrict__ Wp4,
                                                   double* __restrict__ Op, int64_t QS, int qtile0,
                                                   RepC rp = RepC{}) {
  {
    const int64_t r = blockIdx.z;
    bptr += r * rp.b;
    erow += r * rp.m;
    eval += r * rp.m;
    Wp4 += r * rp.w;
    Op += r * rp.o;
  }
  __shared__ int srow[DF_NT];
  __shared__ ulonglong2 sv[DF_NT];
  __shared__ f32x2 snv[DF_NT];
  spmm_df_item<DF_PPT>(blockIdx.x, (int64_t)blockIdx.y + qtile0, bptr, erow, eval, Wp4, Op, QS, srow, sv, snv);
}

// Persistent form: gridDim.x CTAs take (bucket, q tile) items from a
// counter in q-tile-major order (all buckets of q tile 0, then q tile 1,
// ...), so the W' columns in use at once are those of the items the
// resident CTAs hold -- a window set by the grid size rather than by the
// hardware's occupancy.  Same arithmetic and order per output as k_spmm_df.
template <int DF_PPT>
__global__ void __launch_bounds__(DF_NT, 8) k_spmm_df_persist(const int* __restrict__ bptr,
                                                           const int* __restrict__ erow,
                                                           const float2* __restrict__ eval,
                                                           const float4* __restrict__ Wp4, double* __restrict__ Op,
                                                           int64_t QS, int64_t nb, int64_t nitems,
                                                           unsigned long long* __restrict__ counter) {
  __shared__ int srow[DF_NT];
  __shared__ ulonglong2 sv[DF_NT];
  __shared__ f32x2 snv[DF_NT];
  __shared__ long long item;
  for (;;) {
    __syncthreads();  // the previous item's staged entries are no longer read
    if (threadIdx.x == 0) item = (long long)atomicAdd(counter, 1ull);
    __syncthreads();
    const long long w = item;
    if (w >= nitems) return;
    const int64_t qt = w / nb;
    spmm_df_item<DF_PPT>(w - qt * nb, qt, bptr, erow, eval, Wp4, Op, QS, srow, sv, snv);
  }
}

// The compressed T viewed as a dense [nP][R] matrix (rows P = (pa,pb) pair,
// columns r = (ka,kb) pair), coef * value split into BF16 hi + lo and
// scattered into the K-concatenated tensor-core operand A' = [hi | hi | lo]
// (rows of kp elements, zeroed beforehand): the split-precision form runs
// every sparse term as a dense GEMM on the tensor cores.  (P, r) is unique
// per nonzero, so the scatter has no collisions.
// (A batch of replicas: replica blockIdx.y reads its m entries at
// blockIdx.y * m and writes its own nP rows of A' at blockIdx.y * a_rep.)
__global__ void k_densify_bf16x3(const int* __restrict__ slots, const double* __restrict__ vals, int64_t m, int pa,
                                 int pb, int64_t dpb, int ka, int kb, int64_t dkb, double coef, int64_t R, int64_t kp,
                                 __nv_bfloat16* __restrict__ Ap, int64_t a_rep = 0) {
  slots += 4 * (int64_t)blockIdx.y * m;
  vals += (int64_t)blockIdx.y * m;
  Ap += (int64_t)blockIdx.y * a_rep;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t P = (int64_t)slots[4 * s + pa] * dpb + slots[4 * s + pb];
    const int64_t r = (int64_t)slots[4 * s + ka] * dkb + slots[4 * s + kb];
    const double x = coef * vals[s];
    const __nv_bfloat16 hi = __double2bfloat16(x);
    const __nv_bfloat16 lo = __double2bfloat16(x - (double)__bfloat162float(hi));
    __nv_bfloat16* row = Ap + P * kp;
    row[r] = hi;
    row[R + r] = hi;
    row[2 * R + r] = lo;
  }
}

// The same contraction against an FP32 W (the split-precision (vv|vv) block
// rebuilt on the tensor cores): row r of W holds ldw floats, read as pairs
// (W[r][2t], W[r][2t+1]); the compressed T values stay float pairs, so
//   ph + e = W vh exactly, pl = e + W vl, and the same two-sum accumulation.
// Half the bytes of the q-pair layout per term and one FMA fewer.
template <int PPT, bool FULL>
__device__ __forceinline__ void f1_tile(const int* __restrict__ srow, const ulonglong2* __restrict__ sv,
                                        const f32x2* __restrict__ snv, int cnt, const f32x2* __restrict__ wq,
                                        int64_t ldw2, int64_t trem, f32x2* ah, f32x2* al) {
  for (int j = 0; j < cnt; ++j) {
    const f32x2* w = wq + (int64_t)srow[j] * ldw2;
    const ulonglong2 v = sv[j];  // (vh, vh), (vl, vl)
    const f32x2 nvh = snv[j];    // (-vh, -vh)
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      if (FULL || k * DF_NT < trem) {
        const f32x2 x = w[k * DF_NT];       // (W, W')
        const f32x2 nph = mul2(x, nvh);     // -ph
        f32x2 pl = fma2(x, v.x, nph);       // W vh - ph, exact
        pl = fma2(x, v.y, pl);
        const f32x2 s = sub2(ah[k], nph);
        const f32x2 z = sub2(s, ah[k]);
        const f32x2 err = sub2(sub2(ah[k], sub2(s, z)), add2(nph, z));
        al[k] = add2(al[k], add2(err, pl));
        ah[k] = s;
      }
    }
  }
}

template <int PPT>
__global__ void __launch_bounds__(DF_NT) k_spmm_f1(const int* __restrict__ bptr, const int* __restrict__ erow,
                                                   const float2* __restrict__ eval, const float2* __restrict__ W2,
                                                   int64_t ldw2, double* __restrict__ Op, int64_t QS) {
  __shared__ int srow[DF_NT];
  __shared__ ulonglong2 sv[DF_NT];
  __shared__ f32x2 snv[DF_NT];
  const int64_t P = blockIdx.x;
  const int e0 = bptr[P], e1 = bptr[P + 1];
  if (e0 == e1) return;
  const int64_t QS2 = (QS + 1) >> 1;
  const int64_t qt = blockIdx.y;
  const int64_t t0 = qt * (DF_NT * PPT) + threadIdx.x;
  const int64_t trem = QS2 - t0;
  const bool full = (qt + 1) * (DF_NT * PPT) <= QS2;
  double* orow = Op + P * QS;
  const f32x2* wq = reinterpret_cast<const f32x2*>(W2) + t0;
  f32x2 ah[PPT], al[PPT];
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int64_t q = 2 * (t0 + k * DF_NT);
    const float2 a = split_f2(q < QS ? orow[q] : 0.0);
    const float2 b = split_f2(q + 1 < QS ? orow[q + 1] : 0.0);
    ah[k] = pk2(a.x, b.x);
    al[k] = pk2(a.y, b.y);
  }
  for (int eb = e0; eb < e1; eb += DF_NT) {
    const int cnt = e1 - eb < DF_NT ? e1 - eb : DF_NT;
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      const float2 v = eval[eb + threadIdx.x];
      srow[threadIdx.x] = erow[eb + threadIdx.x];
      sv[threadIdx.x] = make_ulonglong2(pk2(v.x, v.x), pk2(v.y, v.y));
      snv[threadIdx.x] = pk2(-v.x, -v.x);
    }
    __syncthreads();
    if (full) f1_tile<PPT, true>(srow, sv, snv, cnt, wq, ldw2, trem, ah, al);
    else f1_tile<PPT, false>(srow, sv, snv, cnt, wq, ldw2, trem, ah, al);
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      const f32x2 s = add2(ah[k], al[k]);
      al[k] = sub2(al[k], sub2(s, ah[k]));
      ah[k] = s;
    }
  }
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int64_t q = 2 * (t0 + k * DF_NT);
    const float2 h = upk2(ah[k]), l = upk2(al[k]);
    if (q < QS) orow[q] = pair_to_f64(h.x, l.x);
    if (q + 1 < QS) orow[q + 1] = pair_to_f64(h.y, l.y);
  }
}

// FP32 throughout (the split-precision form, whose integrals carry ~2^-16
// relative error anyway): W rows of ldw floats read as pairs, T values as
// floats, one packed FMA per output pair per term, the FP32 sum added to the
// FP64 output once at the end.  PPT q-pairs per thread.
template <int PPT, bool FULL>
__device__ __forceinline__ void f32_tile(const int* __restrict__ srow, const f32x2* __restrict__ sv, int cnt,
                                         const f32x2* __restrict__ wq, int64_t ldw2, int64_t trem, f32x2* acc) {
#pragma unroll 4
  for (int j = 0; j < cnt; ++j) {
    const f32x2* w = wq + (int64_t)srow[j] * ldw2;
    const f32x2 v = sv[j];  // (t, t)
#pragma unroll
    for (int k = 0; k < PPT; ++k)
      if (FULL || k * DF_NT < trem) acc[k] = fma2(w[k * DF_NT], v, acc[k]);
  }
}

template <int PPT>
__global__ void __launch_bounds__(DF_NT) k_spmm_f32(const int* __restrict__ bptr, const int* __restrict__ erow,
                                                    const float2* __restrict__ eval, const float2* __restrict__ W2,
                                                    int64_t ldw2, double* __restrict__ Op, int64_t QS) {
  __shared__ int srow[DF_NT];
  __shared__ f32x2 sv[DF_NT];
  const int64_t P = blockIdx.x;
  const int e0 = bptr[P], e1 = bptr[P + 1];
  if (e0 == e1) return;
  const int64_t QS2 = (QS + 1) >> 1;
  const int64_t qt = blockIdx.y;
  const int64_t t0 = qt * (DF_NT * PPT) + threadIdx.x;
  const int64_t trem = QS2 - t0;
  const bool full = (qt + 1) * (DF_NT * PPT) <= QS2;
  const f32x2* wq = reinterpret_cast<const f32x2*>(W2) + t0;
  f32x2 acc[PPT];
#pragma unroll
  for (int k = 0; k < PPT; ++k) acc[k] = 0ull;
  for (int eb = e0; eb < e1; eb += DF_NT) {
    const int cnt = e1 - eb < DF_NT ? e1 - eb : DF_NT;
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      const float2 v = eval[eb + threadIdx.x];
      const float t = v.x + v.y;
      srow[threadIdx.x] = erow[eb + threadIdx.x];
      sv[threadIdx.x] = pk2(t, t);
    }
    __syncthreads();
    if (full) f32_tile<PPT, true>(srow, sv, cnt, wq, ldw2, trem, acc);
    else f32_tile<PPT, false>(srow, sv, cnt, wq, ldw2, trem, acc);
  }
  double* orow = Op + P * QS;
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int64_t q = 2 * (t0 + k * DF_NT);
    const float2 a = upk2(acc[k]);
    if (q < QS) orow[q] += f2d_bits(a.x);
    if (q + 1 < QS) orow[q + 1] += f2d_bits(a.y);
  }
}

__global__ void k_entries_df(const int* __restrict__ slots, const double* __restrict__ vals,
                             const unsigned* __restrict__ order, int64_t m, int ka, int kb, int64_t dkb, double coef,
                             int* __restrict__ erow, float2* __restrict__ eval, RepC rp = RepC{}) {
  slots += 4 * blockIdx.y * rp.m;
  vals += blockIdx.y * rp.m;
  order += blockIdx.y * rp.m;
  erow += blockIdx.y * rp.m;
  eval += blockIdx.y * rp.m;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
    const unsigned s = order[e];
    erow[e] = (int)((int64_t)slots[4 * s + ka] * dkb + slots[4 * s + kb]);
    eval[e] = split_f2(coef * vals[s]);
  }
}

// x [rows][QS] (FP64) -> the q-pair layout of k_spmm_df
__global__ void k_split_f2(const double* __restrict__ x, int64_t rows, int64_t QS, float4* __restrict__ out) {
  const int64_t QS2 = (QS + 1) >> 1, n = rows * QS2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / QS2, q = 2 * (i - r * QS2);
    const float2 a = split_f2(x[r * QS + q]);
    const float2 b = split_f2(q + 1 < QS ? x[r * QS + q + 1] : 0.0);
    out[i] = make_float4(a.x, b.x, a.y, b.y);
  }
}

// dst (contiguous, extents e0..e3) = src viewed with strides s0..s3
__global__ void k_gather4(const double* __restrict__ src, int64_t s0, int64_t s1, int64_t s2, int64_t s3, int64_t e0,
                          int64_t e1, int64_t e2, int64_t e3, double* __restrict__ dst) {
  const int64_t n = e0 * e1 * e2 * e3;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t;
    const int64_t i3 = r % e3; r /= e3;
    const int64_t i2 = r % e2; r /= e2;
    const int64_t i1 = r % e1;
    const int64_t i0 = r / e1;
    dst[t] = src[i0 * s0 + i1 * s1 + i2 * s2 + i3 * s3];
  }
}

__global__ void k_scatter4(const double* __restrict__ src, int64_t s0, int64_t s1, int64_t s2, int64_t s3, int64_t e0,
                           int64_t e1, int64_t e2, int64_t e3, double* __restrict__ dst) {
  const int64_t n = e0 * e1 * e2 * e3;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t;
    const int64_t i3 = r % e3; r /= e3;
    const int64_t i2 = r % e2; r /= e2;
    const int64_t i1 = r % e1;
    const int64_t i0 = r / e1;
    dst[i0 * s0 + i1 * s1 + i2 * s2 + i3 * s3] = src[t];
  }
}

inline unsigned grid_for(int64_t n, int nt) {
  int64_t g = fricc_cdiv(n, nt);
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

bool is_contig_perm(const int64_t dims[4], const int64_t strides[4], const int perm[4]) {
  int64_t expect = 1;
  for (int j = 3; j >= 0; --j) {
    if (dims[perm[j]] > 1 && strides[perm[j]] != expect) return false;
    expect *= dims[perm[j]];
  }
  return true;
}

}  // namespace

double fricc_contract_flops_impl(const char* term, const FriccSparse* T);

// A re-compression keeps every bucketing's arrays (m and dims do not change)
// and only marks it stale; it is rebuilt in place on first use, so a steady
// iteration allocates nothing that outlives it (which also keeps it
// capturable in a CUDA graph).
int fricc_sparse_bucketing(FriccSparse* T, int pa, int pb, cudaStream_t st, Bucketing** out) {
  Bucketing* slot = nullptr;
  for (auto& b : T->buck)
    if (b.pa == pa && b.pb == pb && b.bptr) {
      if (b.valid) {
        *out = &b;
        return FRICC_OK;
      }
      slot = &b;
      break;
    }
  if (!slot)
    for (auto& b : T->buck)
      if (!b.bptr) {
        slot = &b;
        break;
      }
  if (!slot) return FRICC_ERR_ARG;
  const bool fresh = slot->bptr == nullptr;
  const int64_t m = T->m;
  const int64_t nb = T->dims[pa] * T->dims[pb];
  int bits = 8;
  while (bits < 64 && (1ll << bits) < nb) bits += 8;
  unsigned long long *keys = nullptr, *ktmp = nullptr;
  unsigned *vtmp = nullptr, *hist = nullptr;
  int rc = fricc_alloc_t(&keys, m, st);
  if (!rc) rc = fricc_alloc_t(&ktmp, m, st);
  if (!rc) rc = fricc_alloc_t(&vtmp, m, st);
  if (!rc) rc = fricc_alloc_t(&hist, radix::hist_words(m), st);
  if (!rc && fresh) rc = fricc_alloc_t(&slot->order, m, st);
  if (!rc && fresh) rc = fricc_alloc_t(&slot->bptr, nb + 1, st);
  if (!rc) {
    k_pair_keys<<<grid_for(m, 256), 256, 0, st>>>(T->slots, m, pa, pb, T->dims[pb], keys, slot->order);
    rc = radix::sort_pairs(keys, slot->order, ktmp, vtmp, m, bits, false, hist, st);
    fricc_note_launch(1);
  }
  if (!rc) {
    k_bptr<<<grid_for(nb + 1, 256), 256, 0, st>>>(keys, m, nb, slot->bptr);
    fricc_note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = fricc_cuda_fail(e, "bucketing", __FILE__, __LINE__);
  }
  fricc_free(keys, st);
  fricc_free(ktmp, st);
  fricc_free(vtmp, st);
  fricc_free(hist, st);
  if (rc) {
    fricc_free(slot->order, st);
    fricc_free(slot->bptr, st);
    slot->order = nullptr;
    slot->bptr = nullptr;
    return rc;
  }
  slot->pa = pa;
  slot->pb = pb;
  slot->nbuckets = nb;
  slot->valid = true;
  *out = slot;
  return FRICC_OK;
}

int fricc_contract_device(const char* term, const double* W, const int64_t Wd[4], const int64_t Ws[4], FriccSparse* T,
                          double* out, const int64_t Od[4], const int64_t Os[4], cudaStream_t st) {
  const TermSpec* ts = find_term(term);
  if (!ts) {
    fricc_set_error("CASE NOT IMPLEMENTED: contraction term '%s'", term ? term : "(null)");
    return FRICC_ERR_TERM;
  }
  if (!W || !out || !T) {
    fricc_set_error("contract: null argument");
    return FRICC_ERR_ARG;
  }
  const int64_t* td = T->dims;
  // W' = (key0, key1, q0, q1), out' = (p0, p1, q0, q1)
  int64_t we[4], oe[4], wsp[4], osp[4];
  for (int j = 0; j < 4; ++j) {
    we[j] = Wd[ts->permW[j]];
    wsp[j] = Ws[ts->permW[j]];
    oe[j] = Od[ts->permO[j]];
    osp[j] = Os[ts->permO[j]];
  }
  if (we[0] != td[ts->ka] || we[1] != td[ts->kb] || oe[0] != td[ts->pa] || oe[1] != td[ts->pb] || we[2] != oe[2] ||
      we[3] != oe[3]) {
    fricc_set_error(
        "contract %s: shapes do not match the sparse tensor dims (W %lldx%lldx%lldx%lld, out %lldx%lldx%lldx%lld, "
        "T %lldx%lldx%lldx%lld)",
        ts->name, (long long)Wd[0], (long long)Wd[1], (long long)Wd[2], (long long)Wd[3], (long long)Od[0],
        (long long)Od[1], (long long)Od[2], (long long)Od[3], (long long)td[0], (long long)td[1], (long long)td[2],
        (long long)td[3]);
    return FRICC_ERR_ARG;
  }
  const int64_t QS = we[2] * we[3];
  const int64_t nW = we[0] * we[1] * QS;
  const int64_t nO = oe[0] * oe[1] * QS;
  if (T->m == 0 || nO == 0) return FRICC_OK;

  Bucketing* bk = nullptr;
  int rc = fricc_sparse_bucketing(T, ts->pa, ts->pb, st, &bk);
  if (rc) return rc;

  const bool w_direct = is_contig_perm(Wd, Ws, ts->permW);
  const bool o_direct = is_contig_perm(Od, Os, ts->permO);
  double* Wp = nullptr;
  double* Op = nullptr;
  int* erow = nullptr;
  double* eval = nullptr;
  rc = fricc_alloc_t(&erow, T->m, st);
  if (!rc) rc = fricc_alloc_t(&eval, T->m, st);
  if (!rc && !w_direct) rc = fricc_alloc_t(&Wp, nW, st);
  if (!rc && !o_direct) rc = fricc_alloc_t(&Op, nO, st);
  if (!rc) {
    k_entries<<<grid_for(T->m, 256), 256, 0, st>>>(T->slots, T->vals, bk->order, T->m, ts->ka, ts->kb, td[ts->kb],
                                                   ts->coef, erow, eval);
    if (!w_direct)
      k_gather4<<<grid_for(nW, 256), 256, 0, st>>>(W, wsp[0], wsp[1], wsp[2], wsp[3], we[0], we[1], we[2], we[3], Wp);
    if (!o_direct)
      k_gather4<<<grid_for(nO, 256), 256, 0, st>>>(out, osp[0], osp[1], osp[2], osp[3], oe[0], oe[1], oe[2], oe[3],
                                                   Op);
    const double* Wuse = w_direct ? W : Wp;
    double* Ouse = o_direct ? out : Op;
    const int64_t ntq = fricc_cdiv(QS, SP_NT * SP_QPT);
    if (ntq > 65535 || bk->nbuckets > 0x7fffffffLL) {
      fricc_set_error("contract %s: problem too large for one launch", ts->name);
      rc = FRICC_ERR_ARG;
    } else {
      dim3 grid((unsigned)bk->nbuckets, (unsigned)ntq);
      const bool prof = fricc_prof_on();
      if (prof) fricc_prof_record(st, true, 0.0);
      k_spmm<<<grid, SP_NT, 0, st>>>(bk->bptr, erow, eval, Wuse, Ouse, QS);
      if (prof) fricc_prof_record(st, false, fricc_contract_flops_impl(term, T));
      fricc_note_launch(2 + (w_direct ? 0 : 1) + (o_direct ? 0 : 2));
      if (!o_direct)
        k_scatter4<<<grid_for(nO, 256), 256, 0, st>>>(Op, osp[0], osp[1], osp[2], osp[3], oe[0], oe[1], oe[2], oe[3],
                                                      out);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) rc = fricc_cuda_fail(e, "contract", __FILE__, __LINE__);
    }
  }
  fricc_free(erow, st);
  fricc_free(eval, st);
  fricc_free(Wp, st);
  fricc_free(Op, st);
  return rc;
}

// Generic form: out'[P, q] += coef * sum_{e in bucket P} W'[key_e, q] * value_e
// with P = slot[pa]*dims[pb] + slot[pb], key = slot[ka]*dims[kb] + slot[kb],
// W' contiguous [dims[ka]*dims[kb]][QS] and out' contiguous [dims[pa]*dims[pb]][QS].
int fricc_spmm_device(FriccSparse* T, int pa, int pb, int ka, int kb, double coef, const double* Wp, int64_t QS,
                      double* Op, cudaStream_t st) {
  if (!T || !Wp || !Op || QS <= 0 || pa < 0 || pa > 3 || pb < 0 || pb > 3 || ka < 0 || ka > 3 || kb < 0 || kb > 3 ||
      pa == pb || ka == kb) {
    fricc_set_error("spmm: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (T->m == 0) return FRICC_OK;
  Bucketing* bk = nullptr;
  int rc = fricc_sparse_bucketing(T, pa, pb, st, &bk);
  if (rc) return rc;
  int* erow = nullptr;
  double* eval = nullptr;
  rc = fricc_alloc_t(&erow, T->m, st);
  if (!rc) rc = fricc_alloc_t(&eval, T->m, st);
  const int64_t ntq = fricc_cdiv(QS, SP_NT * SP_QPT);
  if (!rc && (ntq > 65535 || bk->nbuckets > 0x7fffffffLL)) {
    fricc_set_error("spmm: problem too large for one launch");
    rc = FRICC_ERR_ARG;
  }
  if (!rc) {
    k_entries<<<grid_for(T->m, 256), 256, 0, st>>>(T->slots, T->vals, bk->order, T->m, ka, kb, T->dims[kb], coef,
                                                   erow, eval);
    const bool prof = fricc_prof_on();
    if (prof) fricc_prof_record(st, true, 0.0);
    k_spmm<<<dim3((unsigned)bk->nbuckets, (unsigned)ntq), SP_NT, 0, st>>>(bk->bptr, erow, eval, Wp, Op, QS);
    if (prof) fricc_prof_record(st, false, 2.0 * (double)T->m * (double)QS);
    fricc_note_launch(2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = fricc_cuda_fail(e, "spmm", __FILE__, __LINE__);
  }
  fricc_free(erow, st);
  fricc_free(eval, st);
  return rc;
}

// As fricc_spmm_device with W' pre-split into float pairs (fricc_split_f2);
// the products and sums run on the FP32 pipe in pair arithmetic.
int fricc_spmm_f2_device(FriccSparse* T, int pa, int pb, int ka, int kb, double coef, const float4* Wp, int64_t QS,
                         double* Op, cudaStream_t st) {
  if (!T || !Wp || !Op || QS <= 0 || pa < 0 || pa > 3 || pb < 0 || pb > 3 || ka < 0 || ka > 3 || kb < 0 || kb > 3 ||
      pa == pb || ka == kb) {
    fricc_set_error("spmm_f2: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (reinterpret_cast<uintptr_t>(Wp) % 16 != 0) {
    fricc_set_error("spmm_f2: W' (q-pair layout) must be 16-byte aligned");
    return FRICC_ERR_ARG;
  }
  if (T->m == 0) return FRICC_OK;
  Bucketing* bk = nullptr;
  int rc = fricc_sparse_bucketing(T, pa, pb, st, &bk);
  if (rc) return rc;
  int* erow = nullptr;
  float2* eval = nullptr;
  rc = fricc_alloc_t(&erow, T->m, st);
  if (!rc) rc = fricc_alloc_t(&eval, T->m, st);
  // 2 q-pairs per thread unless tuned: measured against 1 and 4 over the
  // o30v150 terms (fewer leaves loads too few per thread, more costs
  // occupancy); a term's best can differ (an autotuner sets the knob)
  const int64_t QS2 = (QS + 1) / 2;
  const int ppt = fricc_tune_get(FRICC_TUNE_SPMM_PPT) > 0 ? fricc_tune_get(FRICC_TUNE_SPMM_PPT) : 2;
  const int64_t ntq = fricc_cdiv(QS2, DF_NT * ppt);
  if (!rc && (ntq > 65535 || bk->nbuckets > 0x7fffffffLL)) {
    fricc_set_error("spmm_f2: problem too large for one launch");
    rc = FRICC_ERR_ARG;
  }
  if (!rc) {
    k_entries_df<<<grid_for(T->m, 256), 256, 0, st>>>(T->slots, T->vals, bk->order, T->m, ka, kb, T->dims[kb], coef,
                                                      erow, eval);
    const bool prof = fricc_prof_on();
    if (prof) fricc_prof_record(st, true, 0.0);
    // One launch over all (bucket, q tile) pairs, buckets fastest.  For the
    // wide-row terms (2323, X/Y) the W' rows of the ~1.4 q tiles resident at
    // once exceed L2 and DRAM sees ~9x the W' bytes, yet only 1.6 TB/s;
    // launching one q tile at a time cut that traffic 6x but ran 50% longer
    // (900-CTA launches leave SMs idle at each tail), so it is not done.
    const int persist = fricc_tune_get(FRICC_TUNE_SPMM_PERSIST);
    if (persist > 0) {
      // persistent, q-tile-major: `persist` CTAs per SM
      unsigned long long* ctr = nullptr;
      rc = fricc_alloc_t(&ctr, 1, st);
      int nsm = 0;
      if (!rc) rc = fricc_cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, T->device), "sm count");
      if (!rc) rc = fricc_cuda_check(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), st), "counter");
      if (!rc) {
        const int64_t nitems = bk->nbuckets * ntq;
        const int64_t g64 = (int64_t)nsm * (persist > 8 ? 8 : persist);
        const unsigned g = (unsigned)(g64 < nitems ? g64 : nitems);
        if (ppt == 1) k_spmm_df_persist<1><<<g, DF_NT, 0, st>>>(bk->bptr, erow, eval, Wp, Op, QS, bk->nbuckets, nitems, ctr);
        else if (ppt == 4) k_spmm_df_persist<4><<<g, DF_NT, 0, st>>>(bk->bptr, erow, eval, Wp, Op, QS, bk->nbuckets, nitems, ctr);
        else k_spmm_df_persist<2><<<g, DF_NT, 0, st>>>(bk->bptr, erow, eval, Wp, Op, QS, bk->nbuckets, nitems, ctr);
      }
      fricc_free(ctr, st);
    } else {
      const dim3 grid((unsigned)bk->nbuckets, (unsigned)ntq);
      if (ppt == 1) k_spmm_df<1><<<grid, DF_NT, 0, st>>>(bk->bptr, erow, eval, Wp, Op, QS, 0);
      else if (ppt == 4) k_spmm_df<4><<<grid, DF_NT, 0, st>>>(bk->bptr, erow, eval, Wp, Op, QS, 0);
      else k_spmm_df<2><<<grid, DF_NT, 0, st>>>(bk->bptr, erow, eval, Wp, Op, QS, 0);
    }
    fricc_note_launch();
    if (prof) fricc_prof_record(st, false, 2.0 * (double)T->m * (double)QS);
    fricc_note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = fricc_cuda_fail(e, "spmm_f2", __FILE__, __LINE__);
  }
  fricc_free(erow, st);
  fricc_free(eval, st);
  return rc;
}

int fricc_spmm_f1_device(FriccSparse* T, int pa, int pb, int ka, int kb, double coef, const float* W, int64_t QS,
                         int64_t ldw, double* Op, cudaStream_t st, bool fp32) {
  if (!T || !W || !Op || QS <= 0 || ldw < QS || (ldw & 1) || pa < 0 || pa > 3 || pb < 0 || pb > 3 || ka < 0 ||
      ka > 3 || kb < 0 || kb > 3 || pa == pb || ka == kb) {
    fricc_set_error("spmm_f1: bad arguments (W rows of ldw >= QS floats, ldw even)");
    return FRICC_ERR_ARG;
  }
  if (reinterpret_cast<uintptr_t>(W) % 8 != 0) {
    fricc_set_error("spmm_f1: W must be 8-byte aligned");
    return FRICC_ERR_ARG;
  }
  if (T->m == 0) return FRICC_OK;
  Bucketing* bk = nullptr;
  int rc = fricc_sparse_bucketing(T, pa, pb, st, &bk);
  if (rc) return rc;
  int* erow = nullptr;
  float2* eval = nullptr;
  rc = fricc_alloc_t(&erow, T->m, st);
  if (!rc) rc = fricc_alloc_t(&eval, T->m, st);
  constexpr int ppt = 2;
  const int64_t QS2 = (QS + 1) / 2;
  const int64_t ntq = fricc_cdiv(QS2, DF_NT * ppt);
  if (!rc && (ntq > 65535 || bk->nbuckets > 0x7fffffffLL)) {
    fricc_set_error("spmm_f1: problem too large for one launch");
    rc = FRICC_ERR_ARG;
  }
  if (!rc) {
    k_entries_df<<<grid_for(T->m, 256), 256, 0, st>>>(T->slots, T->vals, bk->order, T->m, ka, kb, T->dims[kb], coef,
                                                      erow, eval);
    const bool prof = fricc_prof_on();
    if (prof) fricc_prof_record(st, true, 0.0);
    const dim3 grid((unsigned)bk->nbuckets, (unsigned)ntq);
    if (fp32)
      k_spmm_f32<ppt><<<grid, DF_NT, 0, st>>>(bk->bptr, erow, eval, reinterpret_cast<const float2*>(W), ldw / 2, Op,
                                             QS);
    else
      k_spmm_f1<ppt><<<grid, DF_NT, 0, st>>>(bk->bptr, erow, eval, reinterpret_cast<const float2*>(W), ldw / 2, Op,
                                            QS);
    if (prof) fricc_prof_record(st, false, 2.0 * (double)T->m * (double)QS);
    fricc_note_launch(2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = fricc_cuda_fail(e, "spmm_f1", __FILE__, __LINE__);
  }
  fricc_free(erow, st);
  fricc_free(eval, st);
  return rc;
}

int fricc_densify_bf16x3_device(FriccSparse* T, int pa, int pb, int ka, int kb, double coef, void* Ap, int64_t kp,
                                cudaStream_t st) {
  if (!T || !Ap || pa < 0 || pa > 3 || pb < 0 || pb > 3 || ka < 0 || ka > 3 || kb < 0 || kb > 3 || pa == pb ||
      ka == kb) {
    fricc_set_error("densify_bf16x3: bad arguments");
    return FRICC_ERR_ARG;
  }
  const int64_t nP = T->dims[pa] * T->dims[pb], R = T->dims[ka] * T->dims[kb];
  if (kp < 3 * R) {
    fricc_set_error("densify_bf16x3: kp must be >= 3 * dims[ka] * dims[kb]");
    return FRICC_ERR_ARG;
  }
  cudaError_t e = cudaMemsetAsync(Ap, 0, sizeof(__nv_bfloat16) * (size_t)(nP * kp), st);
  if (e == cudaSuccess && T->m > 0) {
    k_densify_bf16x3<<<grid_for(T->m, 256), 256, 0, st>>>(T->slots, T->vals, T->m, pa, pb, T->dims[pb], ka, kb,
                                                          T->dims[kb], coef, R, kp,
                                                          static_cast<__nv_bfloat16*>(Ap));
    fricc_note_launch();
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "densify_bf16x3", __FILE__, __LINE__);
}

// The batch form: every replica's compression `which` into its own nP rows
// of A' ([R][nP][kp], zeroed here), one launch.
int fricc_batch_densify_device(FriccSparseBatch* B, int which, int pa, int pb, int ka, int kb, double coef, void* Ap,
                               int64_t kp, cudaStream_t st) {
  if (!B || !Ap || which < 0 || which > 1 || pa < 0 || pa > 3 || pb < 0 || pb > 3 || ka < 0 || ka > 3 || kb < 0 ||
      kb > 3 || pa == pb || ka == kb) {
    fricc_set_error("batch densify_bf16x3: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (!B->compressed) {
    fricc_set_error("batch densify_bf16x3: the batch has not been compressed yet");
    return FRICC_ERR_ARG;
  }
  const int64_t nP = B->dims[pa] * B->dims[pb], R = B->dims[ka] * B->dims[kb];
  if (kp < 3 * R) {
    fricc_set_error("batch densify_bf16x3: kp must be >= 3 * dims[ka] * dims[kb]");
    return FRICC_ERR_ARG;
  }
  cudaError_t e = cudaMemsetAsync(Ap, 0, sizeof(__nv_bfloat16) * (size_t)(B->R * nP * kp), st);
  if (e == cudaSuccess) {
    k_densify_bf16x3<<<dim3(grid_for(B->m, 256), B->R), 256, 0, st>>>(
        B->slots[which], B->vals[which], B->m, pa, pb, B->dims[pb], ka, kb, B->dims[kb], coef, R, kp,
        static_cast<__nv_bfloat16*>(Ap), nP * kp);
    fricc_note_launch();
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "batch densify_bf16x3", __FILE__, __LINE__);
}

int fricc_split_f2_device(const double* x, int64_t rows, int64_t qs, float4* out, cudaStream_t st) {
  if (rows < 0 || qs < 0 || (rows > 0 && qs > 0 && (!x || !out))) {
    fricc_set_error("split_f2: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (reinterpret_cast<uintptr_t>(out) % 16 != 0) {
    fricc_set_error("split_f2: output must be 16-byte aligned");
    return FRICC_ERR_ARG;
  }
  const int64_t n = rows * ((qs + 1) / 2);
  if (n == 0) return FRICC_OK;
  k_split_f2<<<grid_for(n, 256), 256, 0, st>>>(x, rows, qs, out);
  fricc_note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "split_f2", __FILE__, __LINE__);
}

// Flop count of one term (2 per multiply-add), for roofline accounting.
double fricc_contract_flops_impl(const char* term, const FriccSparse* T) {
  const TermSpec* ts = find_term(term);
  if (!ts || !T) return 0.0;
  const double o = (double)T->dims[0], v = (double)T->dims[2];
  double q = o * v;                                                // the O^3V^3 terms
  if (std::strcmp(ts->name, "2323") == 0) q = v * v;               // O^2V^4
  else if (std::strcmp(ts->name, "0101") == 0 || std::strcmp(ts->name, "1323") == 0) q = o * o;  // O^4V^2
  return 2.0 * (double)T->m * q;
}

// ---------------------------------------------------------------------------
// Replica batches: the bucketing and the sparse terms of R compressed tensors
// of one shape in one set of launches, each replica's arithmetic (entry
// order, accumulation order) that of its own single call.
int fricc_batch_bucketing(FriccSparseBatch* B, int which, int pa, int pb, cudaStream_t st, BatchBucketing** out) {
  BatchBucketing* slot = nullptr;
  for (auto& b : B->buck[which])
    if (b.pa == pa && b.pb == pb && b.bptr) {
      if (b.valid) {
        *out = &b;
        return FRICC_OK;
      }
      slot = &b;
      break;
    }
  if (!slot)
    for (auto& b : B->buck[which])
      if (!b.bptr) {
        slot = &b;
        break;
      }
  if (!slot) return FRICC_ERR_ARG;
  const bool fresh = slot->bptr == nullptr;
  const int R = B->R;
  const int64_t m = B->m;
  const int64_t nb = B->dims[pa] * B->dims[pb];
  int bits = 8;
  while (bits < 64 && (1ll << bits) < nb) bits += 8;
  unsigned long long *keys = nullptr, *ktmp = nullptr;
  unsigned *vtmp = nullptr, *hist = nullptr;
  const int64_t hw = radix::hist_words(m);
  int rc = fricc_alloc_t(&keys, (size_t)R * m, st);
  if (!rc) rc = fricc_alloc_t(&ktmp, (size_t)R * m, st);
  if (!rc) rc = fricc_alloc_t(&vtmp, (size_t)R * m, st);
  if (!rc) rc = fricc_alloc_t(&hist, (size_t)R * hw, st);
  if (!rc && fresh) rc = fricc_alloc_t(&slot->order, (size_t)R * m, st);
  if (!rc && fresh) rc = fricc_alloc_t(&slot->bptr, (size_t)R * (nb + 1), st);
  if (!rc) {
    RepC rp;
    rp.m = m;
    rp.b = nb + 1;
    k_pair_keys<<<dim3(grid_for(m, 256), R), 256, 0, st>>>(B->slots[which], m, pa, pb, B->dims[pb], keys,
                                                          slot->order, rp);
    radix::Batch bt;
    bt.kv_stride = m;
    bt.hist_stride = hw;
    rc = radix::sort_pairs(keys, slot->order, ktmp, vtmp, m, bits, false, hist, st, nullptr, R, bt);
    fricc_note_launch(1);
    if (!rc) {
      k_bptr<<<dim3(grid_for(nb + 1, 256), R), 256, 0, st>>>(keys, m, nb, slot->bptr, rp);
      fricc_note_launch();
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) rc = fricc_cuda_fail(e, "batch bucketing", __FILE__, __LINE__);
    }
  }
  fricc_free(keys, st);
  fricc_free(ktmp, st);
  fricc_free(vtmp, st);
  fricc_free(hist, st);
  if (rc) {
    fricc_free(slot->order, st);
    fricc_free(slot->bptr, st);
    slot->order = nullptr;
    slot->bptr = nullptr;
    return rc;
  }
  slot->pa = pa;
  slot->pb = pb;
  slot->nbuckets = nb;
  slot->valid = true;
  *out = slot;
  return FRICC_OK;
}

// Op_r[P][q] += coef * sum_e W'_r[key_e][q] value_e for every replica r:
// W'_r = Wp + r w_stride (w_stride 0: one W' for all), Op_r = Op + r o_stride.
// f2: W' in the q-pair float layout of fricc_spmm_f2 (w_stride in float4s).
int fricc_batch_spmm_device(FriccSparseBatch* B, int which, int pa, int pb, int ka, int kb, double coef,
                            const void* Wp, int64_t w_stride, int64_t QS, double* Op, int64_t o_stride, bool f2,
                            cudaStream_t st) {
  if (!B || !Wp || !Op || which < 0 || which > 1 || QS <= 0 || pa < 0 || pa > 3 || pb < 0 || pb > 3 || ka < 0 ||
      ka > 3 || kb < 0 || kb > 3 || pa == pb || ka == kb || w_stride < 0 || o_stride < 0) {
    fricc_set_error("batch spmm: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (!B->compressed) {
    fricc_set_error("batch spmm: the batch has not been compressed yet");
    return FRICC_ERR_ARG;
  }
  if (f2 && reinterpret_cast<uintptr_t>(Wp) % 16 != 0) {
    fricc_set_error("batch spmm: W' (q-pair layout) must be 16-byte aligned");
    return FRICC_ERR_ARG;
  }
  const int R = B->R;
  const int64_t m = B->m;
  BatchBucketing* bk = nullptr;
  int rc = fricc_batch_bucketing(B, which, pa, pb, st, &bk);
  if (rc) return rc;
  int* erow = nullptr;
  void* eval = nullptr;
  rc = fricc_alloc_t(&erow, (size_t)R * m, st);
  if (!rc) rc = fricc_alloc(&eval, (size_t)R * m * (f2 ? sizeof(float2) : sizeof(double)), st);
  const int64_t QS2 = (QS + 1) / 2;
  const int ppt = f2 ? (fricc_tune_get(FRICC_TUNE_SPMM_PPT) > 0 ? fricc_tune_get(FRICC_TUNE_SPMM_PPT) : 2) : 0;
  const int64_t ntq = f2 ? fricc_cdiv(QS2, DF_NT * ppt) : fricc_cdiv(QS, SP_NT * SP_QPT);
  if (!rc && (ntq > 65535 || bk->nbuckets > 0x7fffffffLL)) {
    fricc_set_error("batch spmm: problem too large for one launch");
    rc = FRICC_ERR_ARG;
  }
  if (!rc) {
    RepC rp;
    rp.m = m;
    rp.b = bk->nbuckets + 1;
    rp.w = w_stride;
    rp.o = o_stride;
    const int* slots = B->slots[which];
    const double* vals = B->vals[which];
    const bool prof = fricc_prof_on();
    const dim3 grid((unsigned)bk->nbuckets, (unsigned)ntq, (unsigned)R);
    if (f2) {
      k_entries_df<<<dim3(grid_for(m, 256), R), 256, 0, st>>>(slots, vals, bk->order, m, ka, kb, B->dims[kb], coef,
                                                             erow, static_cast<float2*>(eval), rp);
      if (prof) fricc_prof_record(st, true, 0.0);
      const float4* W4 = static_cast<const float4*>(Wp);
      const float2* ev = static_cast<const float2*>(eval);
      if (ppt == 1) k_spmm_df<1><<<grid, DF_NT, 0, st>>>(bk->bptr, erow, ev, W4, Op, QS, 0, rp);
      else if (ppt == 4) k_spmm_df<4><<<grid, DF_NT, 0, st>>>(bk->bptr, erow, ev, W4, Op, QS, 0, rp);
      else k_spmm_df<2><<<grid, DF_NT, 0, st>>>(bk->bptr, erow, ev, W4, Op, QS, 0, rp);
    } else {
      k_entries<<<dim3(grid_for(m, 256), R), 256, 0, st>>>(slots, vals, bk->order, m, ka, kb, B->dims[kb], coef,
                                                          erow, static_cast<double*>(eval), rp);
      if (prof) fricc_prof_record(st, true, 0.0);
      k_spmm<<<grid, SP_NT, 0, st>>>(bk->bptr, erow, static_cast<const double*>(eval),
                                     static_cast<const double*>(Wp), Op, QS, rp);
    }
    if (prof) fricc_prof_record(st, false, 2.0 * (double)R * (double)m * (double)QS);
    fricc_note_launch(2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = fricc_cuda_fail(e, "batch spmm", __FILE__, __LINE__);
  }
  fricc_free(erow, st);
  fricc_free(eval, st);
  return rc;
}
