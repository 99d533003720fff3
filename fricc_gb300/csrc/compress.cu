// FRI compression of a dense FP64 tensor on the GPU, bit for bit equal to
// the reference's single-threaded fri_compression (fri-cc
// src/fri_utils.cpp:439-522, systematic sampling) and "largest" compression
// (include/sparse_tensor.hpp:46-56).
//
// Pipeline (x resident in HBM, N elements, keep m):
//   1. histogram of the top 12 bits of |x| -> host picks the digit holding
//      the m-th largest magnitude (a few KB copied back);
//   2. stable compaction of every element at or above that digit
//      (decoupled look-back, one pass) and an LSD radix sort of the
//      candidates by descending |x|, ties by ascending index: the first m
//      are argsort(x, m) (:11-36);
//   3. one_norm (:164-171) as an exact sequential chain (exactsum.cuh);
//   4. the remaining-norm chain R -= |x_(d)| over the sorted candidates and
//      the acceptance test (m-d)|x_(d)| >= R-|x_(d)| && R > 1e-14
//      (:411-421), evaluated for every d from exact chain values;
//   5. p_i = |x_i| / R * m' (:375, this operation order), the p > 1 check
//      (:383-395), the exact partial sums of p (:142-143) and, for every
//      interval [I_j, I_{j+1}), the samples u_k = k + rn that land in it
//      (:136, :147-157); unmatched samples keep index 0, as in the reference;
//   6. output D in sorted order then S ascending, values x_D and x_S/p_S.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "exactsum.cuh"
#include "radix.cuh"
#include "sparse.cuh"

namespace {

// The first select digit: the top `bits` bits of |x| below the sign, 12 by
// default (bits [62:51]: the exponent and one mantissa bit, half an octave
// per bin), 10-13 through FRICC_TUNE_SELECT_BITS.  A wider digit leaves
// fewer candidates for the sort; every width selects the same elements.
constexpr int DIG_BITS_DEFAULT = 12, DIG_BITS_MIN = 10, DIG_BITS_MAX = 13;
constexpr int NDIG = 1 << DIG_BITS_MAX;  // histogram words per compression

int select_bits() {
  const int b = fricc_tune_get(FRICC_TUNE_SELECT_BITS);
  return b >= DIG_BITS_MIN && b <= DIG_BITS_MAX ? b : DIG_BITS_DEFAULT;
}

__device__ __forceinline__ unsigned long long abs_key(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// Replica batches (R compressions of R equal-sized tensors in one set of
// launches): per-replica strides, in elements, of the n-sized arrays, the
// m-sized arrays and the tile-state words; `one` is 1 for single words and
// structs (0, with every stride 0, outside a batch).  The replica is
// blockIdx.y, or blockIdx.x for the one-block kernels.
struct Rep {
  int64_t n = 0, m = 0, tile = 0, one = 0;
};

// histogram of the first select digit (1 << bits bins of dynamic shared memory)
__global__ void __launch_bounds__(256) k_hist_sel(const double* __restrict__ x, int64_t n, unsigned* __restrict__ hist,
                                                  int bits, Rep rp = Rep{}) {
  x += blockIdx.y * rp.n;
  hist += blockIdx.y * rp.one * NDIG;
  extern __shared__ unsigned h[];
  const int nb = 1 << bits, shift = 63 - bits;
  for (int i = threadIdx.x; i < nb; i += 256) h[i] = 0;
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * 256;
  for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += stride)
    atomicAdd(&h[abs_key(x[i]) >> shift], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += 256)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

// Values decided on the device between the phases of one compression.
struct Ctl {
  int64_t dmin;       // first select digit kept as a candidate
  int64_t ncand;      // candidates (every element at or above dmin)
  int64_t nd;         // |D|
  int64_t mp;         // m - |D|
  unsigned long long dkey;  // |x| bits of the last element of D
  int64_t didx;       // its index (-1: D is empty)
  double R;           // remaining norm
  double mprime;      // (double)(m - |D|)
  int sample;         // 1: R > 0 and finite, so samples can land in intervals
  double rn;          // the uniform draw
  // pivotal sampling
  int64_t jend;       // last element the sampler visits (it stops once m' indices are out)
  int64_t npush;      // indices emitted up to jend (chain), then in total (final)
  int64_t plast;      // the pivot after jend
  int broke;          // 1: the sampler stopped early with m' indices
};

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

constexpr unsigned long long ST_AGG = 1ull << 62, ST_INCL = 2ull << 62, ST_VAL = (1ull << 62) - 1;
constexpr long long SPIN_LIMIT = 1ll << 22;

// Stable compaction of {i : top digit of |x_i| >= dmin} into (ckey, cidx),
// in ascending i.  Tiles take tickets in launch order; each publishes its
// count and looks back over its predecessors for its output offset.
__global__ void __launch_bounds__(256) k_compact(const double* __restrict__ x, int64_t n, const Ctl* __restrict__ c,
                                                 unsigned long long* __restrict__ ckey, unsigned* __restrict__ cidx,
                                                 unsigned long long* tstate, unsigned* ticket, unsigned* err,
                                                 const unsigned long long* never_set, long long test_spins,
                                                 int shift, Rep rp = Rep{}) {
  constexpr int NT = 256, ITEMS = 16, TILE = NT * ITEMS;
  {
    const int64_t r = blockIdx.y;
    x += r * rp.n;
    c += r * rp.one;
    ckey += r * rp.n;
    cidx += r * rp.n;
    tstate += r * rp.tile;
    never_set += r * rp.tile;
    ticket += r * rp.one;
    err += r * rp.one;
  }
  const unsigned dmin = (unsigned)c->dmin;
  __shared__ int s_tile;
  __shared__ int64_t s_pre;
  __shared__ int64_t sm[33];
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(ticket, 1u);
  __syncthreads();
  const int tile = s_tile;
  const int64_t base = (int64_t)tile * TILE + threadIdx.x * ITEMS;
  unsigned long long key[ITEMS];
  int cnt = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int64_t i = base + k;
    key[k] = i < n ? abs_key(x[i]) : 0ull;
    if (i < n && (unsigned)(key[k] >> shift) >= dmin) ++cnt;
  }
  int64_t tot;
  const int64_t excl = block_excl_sum(cnt, sm, &tot);
  if (threadIdx.x == 0) {
    int64_t pre = 0;
    if (tile == 0) {
      atomicExch(&tstate[0], ST_INCL | (unsigned long long)tot);
    } else {
      atomicExch(&tstate[tile], ST_AGG | (unsigned long long)tot);
      if (test_spins > 0 && tile == 1) {
        // test only: a bounded wait on a word nothing sets runs out
        long long w = 0;
        while (ld_acquire(never_set) == 0ull) {
          if (++w > test_spins) {
            atomicOr(err, FRICC_DEV_TIMEOUT);
            break;
          }
        }
      }
      int j = tile - 1;
      long long spins = 0;
      while (j >= 0) {
        const unsigned long long v = ld_acquire(&tstate[j]);
        const unsigned long long fl = v & ~ST_VAL;
        if (fl == 0) {
          if (++spins > SPIN_LIMIT) {
            atomicOr(err, FRICC_DEV_TIMEOUT);
            break;
          }
          continue;
        }
        pre += (int64_t)(v & ST_VAL);
        if (fl == ST_INCL) break;
        --j;
      }
      atomicExch(&tstate[tile], ST_INCL | (unsigned long long)(pre + tot));
    }
    s_pre = pre;
  }
  __syncthreads();
  int64_t o = s_pre + excl;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int64_t i = base + k;
    if (i < n && (unsigned)(key[k] >> shift) >= dmin) {
      ckey[o] = key[k];
      cidx[o] = (unsigned)i;
      ++o;
    }
  }
}

struct GenAbs {
  const double* x;
  int64_t rs = 0;  // replica stride of x
  __device__ __forceinline__ double operator()(int64_t i) const { return fabs(x[i]); }
  __device__ __forceinline__ GenAbs at(int r) const { return GenAbs{x + r * rs, rs}; }
};

struct GenSorted {
  const unsigned long long* keys;
  int64_t rs = 0;
  __device__ __forceinline__ double operator()(int64_t i) const { return __longlong_as_double((long long)keys[i]); }
  __device__ __forceinline__ GenSorted at(int r) const { return GenSorted{keys + r * rs, rs}; }
};

// p_i of make_probability_vector (src/fri_utils.cpp:375,378-381); D membership
// is "at or before the last kept element in (|x| desc, index asc) order".
struct GenP {
  const double* x;
  const Ctl* c;
  int64_t rs = 0, cs = 0;  // replica strides of x and c
  __device__ __forceinline__ GenP at(int r) const { return GenP{x + r * rs, c + r * cs, rs, cs}; }
  __device__ __forceinline__ double operator()(int64_t i) const {
    const double a = fabs(x[i]);
    const unsigned long long k = abs_key(a);
    const int64_t didx = c->didx;
    if (didx >= 0 && (k > c->dkey || (k == c->dkey && i <= didx))) return 0.0;
    const double p = __dmul_rn(__ddiv_rn(a, c->R), c->mprime);
    // with R <= 0 or not finite no sample can land anywhere: feed the exact
    // chain zeros (NaN addends would only slow it down), but keep any p > 1
    // visible to the check of make_probability_vector
    return (c->sample || p > 1.0) ? p : 0.0;
  }
  __device__ __forceinline__ double value(int64_t i) const {  // the reference's p_i itself
    const double a = fabs(x[i]);
    const unsigned long long k = abs_key(a);
    const int64_t didx = c->didx;
    if (didx >= 0 && (k > c->dkey || (k == c->dkey && i <= didx))) return 0.0;
    return __dmul_rn(__ddiv_rn(a, c->R), c->mprime);
  }
};

// The probabilities once computed into P (one division per element instead
// of one per pass of the exact chain); the p > 1 check was made then.
struct GenPv {
  const double* P;
  const double* x;
  const Ctl* c;
  int64_t rs = 0, cs = 0;  // replica strides of P and x, and of c
  __device__ __forceinline__ GenPv at(int r) const { return GenPv{P + r * rs, x + r * rs, c + r * cs, rs, cs}; }
  __device__ __forceinline__ double operator()(int64_t i) const { return c->sample ? P[i] : 0.0; }
  __device__ __forceinline__ double value(int64_t i) const { return P[i]; }
};

// get_d_largest's acceptance test for every position d of the sorted list.
struct ConsAccept {
  int64_t m;
  double* Rb;                    // [m+1]: R before element d (Rb[m]: after the last)
  unsigned long long* first_fail;
  int64_t one = 0;               // 1 in a replica batch
  __device__ __forceinline__ ConsAccept at(int r) const {
    return ConsAccept{m, Rb + r * one * (m + 1), first_fail + r * one, one};
  }
  __device__ __forceinline__ void operator()(int64_t d, double before, double after, double a) const {
    Rb[d] = before;
    if (d == m - 1) Rb[m] = after;
    const bool acc = (__dmul_rn((double)(unsigned long long)(m - d), a) >= after) && (before > 1e-14);
    if (!acc) atomicMin(first_fail, (unsigned long long)d);
  }
};

// number of k in [0, mp) with fl(k + rn) < I  (u_k increases with k)
__device__ __forceinline__ int64_t count_below(double I, double rn, int64_t mp) {
  if (!(I > rn)) return 0;
  double g = floor(I - rn);
  int64_t k = g < 0.0 ? 0 : (g > (double)mp ? mp : (int64_t)g);
  for (int it = 0; it < 64 && k > 0 && __dadd_rn((double)(k - 1), rn) >= I; ++it) --k;
  for (int it = 0; it < 64 && k < mp && __dadd_rn((double)k, rn) < I; ++it) ++k;
  return k;
}

// sample_systematic's interval search: the samples of interval j.
struct ConsSample {
  const Ctl* c;
  unsigned* S;
  int64_t cs = 0, ss = 0;  // replica strides of c and S
  __device__ __forceinline__ ConsSample at(int r) const { return ConsSample{c + r * cs, S + r * ss, cs, ss}; }
  __device__ __forceinline__ void operator()(int64_t j, double lo, double hi, double p) const {
    if (!c->sample || !(p > 0.0)) return;
    const double rn = c->rn;
    const int64_t mp = c->mp;
    const int64_t k0 = count_below(lo, rn, mp);
    const int64_t k1 = count_below(hi, rn, mp);
    for (int64_t k = k0; k < k1; ++k) S[k] = (unsigned)j;
  }
};

// Two systematic samplers over one chain: the two compressions of the same
// tensor an iteration makes (different draws) share every phase up to the
// probabilities, and the partial sums too.
struct ConsSample2 {
  ConsSample a, b;
  __device__ __forceinline__ ConsSample2 at(int r) const { return ConsSample2{a.at(r), b.at(r)}; }
  __device__ __forceinline__ void operator()(int64_t j, double lo, double hi, double p) const {
    a(j, lo, hi, p);
    b(j, lo, hi, p);
  }
};

// The select digit: the largest d with count(digit >= d) >= m (one thread).
__global__ void k_select_digit(const unsigned* __restrict__ hist, int64_t m, Ctl* c, int bits, Rep rp = Rep{}) {
  hist += blockIdx.x * rp.one * NDIG;
  c += blockIdx.x * rp.one;
  int64_t cum = 0;
  int d = (1 << bits) - 1;
  for (; d >= 0; --d) {
    cum += hist[d];
    if (cum >= m) break;
  }
  c->dmin = d < 0 ? 0 : d;
  c->ncand = cum;
}

// After the remaining-norm chain: |D|, R, the D threshold, m' (one thread).
__global__ void k_finish_d(const unsigned long long* __restrict__ ffail, const double* __restrict__ Rb,
                           const unsigned long long* __restrict__ ckey, const unsigned* __restrict__ cidx, int64_t m,
                           Ctl* c, Rep rp = Rep{}) {
  {
    const int64_t r = blockIdx.x;
    ffail += r * rp.one;
    Rb += r * rp.one * (m + 1);
    ckey += r * rp.n;
    cidx += r * rp.n;
    c += r * rp.one;
  }
  const int64_t nd = (int64_t)*ffail;
  c->nd = nd;
  c->mp = m - nd;
  c->mprime = (double)(unsigned long long)(m - nd);
  c->R = Rb[nd];
  c->dkey = nd > 0 ? ckey[nd - 1] : 0ull;
  c->didx = nd > 0 ? (int64_t)cidx[nd - 1] : -1;
  c->sample = (c->R > 0.0 && isfinite(c->R)) ? 1 : 0;
}

__global__ void k_zero_u32(unsigned* p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = 0;
}

// D part of the output: flat = sorted index, value = x (src/fri_utils.cpp:494,498-500)
__global__ void k_out_d(const double* __restrict__ x, const unsigned* __restrict__ sidx, int64_t nd_max,
                        const Ctl* __restrict__ c, int64_t* __restrict__ flat, double* __restrict__ vals,
                        Rep rp = Rep{}) {
  {
    const int64_t r = blockIdx.y;
    x += r * rp.n;
    sidx += r * rp.n;
    if (c) c += r * rp.one;
    flat += r * rp.m;
    vals += r * rp.m;
  }
  const int64_t nd = c ? c->nd : nd_max;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned j = sidx[i];
    flat[i] = j;
    vals[i] = x[j];
  }
}

// S part: flat = S_k, value = x / p (src/fri_utils.cpp:495,502-504)
template <class G>
__global__ void k_out_s(G gp0, const unsigned* __restrict__ S, int64_t* __restrict__ flat,
                        double* __restrict__ vals, Rep rp = Rep{}) {
  const G gp = exact::replica_of(gp0, blockIdx.y);
  S += blockIdx.y * rp.m;
  flat += blockIdx.y * rp.m;
  vals += blockIdx.y * rp.m;
  const int64_t mp = gp.c->mp, nd = gp.c->nd;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < mp; k += (int64_t)gridDim.x * blockDim.x) {
    const unsigned j = S[k];
    flat[nd + k] = j;
    vals[nd + k] = __ddiv_rn(gp.x[j], gp.value(j));
  }
}

__global__ void k_unpack(const int64_t* __restrict__ flat, int64_t m, int64_t d0, int64_t d1, int64_t d2, int64_t d3,
                         int* __restrict__ slots, unsigned* err, Rep rp = Rep{}) {
  flat += blockIdx.y * rp.m;
  slots += 4 * blockIdx.y * rp.m;
  err += blockIdx.y * rp.one;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m; s += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long f = (unsigned long long)flat[s];
    const unsigned long long D1 = d1, D2 = d2, D3 = d3;
    if (f >= (unsigned long long)d0 * D1 * D2 * D3) {
      // an index a failed compression left behind: flagged, and unpacked as
      // (0,0,0,0) so that the contractions launched before the status is
      // read stay inside their operands
      atomicOr(err, FRICC_DEV_INDEX);
      f = 0;
    }
    const unsigned long long i0 = f / (D1 * D2 * D3);
    const unsigned long long i1 = f % (D1 * D2 * D3) / (D2 * D3);
    const unsigned long long i2 = f % (D2 * D3) / D3;
    const unsigned long long i3 = f % D3;
    slots[4 * s + 0] = (int)i0;
    slots[4 * s + 1] = (int)i1;
    slots[4 * s + 2] = (int)i2;
    slots[4 * s + 3] = (int)i3;
  }
}

// ---------------------------------------------------------------------------
// Pivotal sampling (src/fri_utils.cpp:63-127).  The sampler carries a weight
// a = p_0; for j = 1, 2, ...: a += p_j and one uniform rn_j is drawn; below 1
// the pivot i moves to j if rn_j < p_j / a; at or above 1, a -= 1 and one
// index is emitted: the pivot (which then moves to j) if
// rn_j < (1 - p_j) / (1 - a), else j; it stops once m' indices are out.
//
// Only the carried weight is a true recurrence (sequential FP64 with a
// wrap), and it does not depend on the draws, nor does which elements emit.
// So: (1) one warp walks the weight and records a_j and the wrap flag for
// every element, which fixes where the sampler stops and how many draws it
// consumes; (2) the draws arrive; (3) every decision is independent given
// a_j, p_j and rn_j; (4) the pivot an element emits is the last "take"
// before it, a max-scan; its slot in S is the count of emits before it, a
// sum-scan.  Per-element codes: bit 0 the pivot moves here, bit 1 the
// element emits, bit 2 it emits the pivot.
constexpr unsigned char PV_TAKE = 1, PV_EMIT = 2, PV_PIVOT = 4;

__global__ void k_pvec(GenP gp0, int64_t n, double* __restrict__ P, unsigned* err, Rep rp = Rep{}) {
  const GenP gp = gp0.at(blockIdx.y);
  P += blockIdx.y * rp.n;
  err += blockIdx.y * rp.one;
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double p = gp.value(i);
    P[i] = p;
    bad |= p > 1.0;
  }
  if (bad) atomicOr(err, FRICC_DEV_P_GT_ONE);
}

// One warp.  Lane t of a batch of 32 elements keeps a_j and the wrap flag
// of element j0 + t; every lane walks the same chain (the p_j come in by
// shuffle, the next batch's are loaded while this one runs).
__global__ void __launch_bounds__(32) k_piv_chain(const double* __restrict__ P, int64_t n, Ctl* c,
                                                  double* __restrict__ A, unsigned char* __restrict__ code) {
  const int lane = threadIdx.x;
  const int64_t mp = c->mp;
  double a = P[0];
  if (lane == 0) {
    A[0] = a;
    code[0] = 0;
  }
  int64_t cnt = 0, jend = n - 1;
  int broke = 0;
  double pn = 1 + lane < n ? P[1 + lane] : 0.0;
  for (int64_t j0 = 1; j0 < n; j0 += 32) {
    const double pj = pn;
    const int64_t jn = j0 + 32 + lane;
    pn = jn < n ? P[jn] : 0.0;
    double myA = 0.0;
    bool myW = false;
#pragma unroll
    for (int t = 0; t < 32; ++t) {
      const double pt = __shfl_sync(0xffffffffu, pj, t);
      const double sum = __dadd_rn(a, pt);
      const bool w = !(sum < 1.0);
      a = w ? __dsub_rn(sum, 1.0) : sum;
      if (lane == t) {
        myA = a;
        myW = w;
      }
    }
    const int64_t j = j0 + lane;
    const bool valid = j < n;
    const unsigned wm = __ballot_sync(0xffffffffu, myW && valid);
    // the first element of this batch after which exactly m' indices are out
    int stop = -1;
    if (mp == 0) {
      if (j0 == 1 && !(wm & 1u)) stop = 0;
    } else if (cnt < mp && cnt + __popc(wm) >= mp) {
      int64_t r = mp - cnt;
      for (int b = 0; b < 32; ++b)
        if (((wm >> b) & 1u) && --r == 0) {
          stop = b;
          break;
        }
    }
    if (valid && (stop < 0 || lane <= stop)) {
      A[j] = myA;
      code[j] = myW ? PV_EMIT : 0;
    }
    if (stop >= 0) {
      jend = j0 + stop;
      broke = 1;
      cnt = mp;
      break;
    }
    cnt += __popc(wm);
  }
  if (lane == 0) {
    c->jend = jend;
    c->npush = cnt;
    c->broke = broke;
  }
}

// decisions for j in [1, jend], with rn_j = R[j-1]
__global__ void k_piv_decide(const double* __restrict__ P, const double* __restrict__ A,
                             unsigned char* __restrict__ code, const double* __restrict__ R, const Ctl* c,
                             unsigned* err) {
  const int64_t jend = c->jend;
  bool bad = false;
  for (int64_t j = 1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j <= jend;
       j += (int64_t)gridDim.x * blockDim.x) {
    const double rn = R[j - 1], p = P[j], a = A[j];
    unsigned char cd = code[j];
    if (!(cd & PV_EMIT)) {
      if (rn < __ddiv_rn(p, a)) cd |= PV_TAKE;
    } else {
      const double pa = __ddiv_rn(__dsub_rn(1.0, p), __dsub_rn(1.0, a));
      bad |= pa > 1.0 || pa < 0.0;
      if (rn < pa) cd |= PV_TAKE | PV_PIVOT;
    }
    code[j] = cd;
  }
  if (bad) atomicOr(err, FRICC_DEV_PIVOTAL);
}

constexpr int PV_NT = 256, PV_IT = 16, PV_TILE = PV_NT * PV_IT;

// block-wide exclusive max of int64 (identity -1), thread order; smem >= 33
__device__ __forceinline__ int64_t block_excl_max(int64_t v, int64_t* smem, int64_t* total) {
  int64_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t w = __shfl_up_sync(0xffffffffu, incl, o);
    if ((int)lane_id() >= o && w > incl) incl = w;
  }
  const int64_t excl_w = __shfl_up_sync(0xffffffffu, incl, 1);
  const int nw = blockDim.x >> 5;
  __syncthreads();
  if (lane_id() == 31) smem[warp_id()] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = -1;
    for (int w = 0; w < nw; ++w) {
      const int64_t t = smem[w];
      smem[w] = run;
      run = t > run ? t : run;
    }
    smem[32] = run;
  }
  __syncthreads();
  int64_t r = smem[warp_id()];
  if (lane_id() > 0 && excl_w > r) r = excl_w;
  *total = smem[32];
  __syncthreads();
  return r;
}

// per tile: the last take and the number of emits among j in [1, jend]
__global__ void __launch_bounds__(PV_NT) k_piv_tiles(const unsigned char* __restrict__ code, const Ctl* c,
                                                     int64_t* __restrict__ tlast, int64_t* __restrict__ tcnt) {
  __shared__ int64_t sm[33];
  const int64_t jend = c->jend;
  const int64_t j0 = (int64_t)blockIdx.x * PV_TILE + (int64_t)threadIdx.x * PV_IT;
  int64_t last = -1, cnt = 0;
#pragma unroll
  for (int k = 0; k < PV_IT; ++k) {
    const int64_t j = j0 + k;
    if (j >= 1 && j <= jend) {
      const unsigned char cd = code[j];
      if (cd & PV_TAKE) last = j;
      cnt += (cd & PV_EMIT) ? 1 : 0;
    }
  }
  int64_t tot_last, tot_cnt;
  block_excl_max(last, sm, &tot_last);
  block_excl_sum(cnt, sm, &tot_cnt);
  if (threadIdx.x == 0) {
    tlast[blockIdx.x] = tot_last;
    tcnt[blockIdx.x] = tot_cnt;
  }
}

// exclusive scans over tiles, in place; the pivot starts at index 0
__global__ void __launch_bounds__(1024) k_piv_carry(int64_t* __restrict__ tlast, int64_t* __restrict__ tcnt,
                                                    int64_t ntile, Ctl* c) {
  __shared__ int64_t sm[33];
  int64_t run_last = 0, run_cnt = 0;
  for (int64_t b = 0; b < ntile; b += 1024) {
    const int64_t t = b + threadIdx.x;
    const int64_t l = t < ntile ? tlast[t] : -1, k = t < ntile ? tcnt[t] : 0;
    int64_t tl, tk;
    int64_t el = block_excl_max(l, sm, &tl);
    const int64_t ek = block_excl_sum(k, sm, &tk);
    el = el > run_last ? el : run_last;
    if (t < ntile) {
      tlast[t] = el;
      tcnt[t] = run_cnt + ek;
    }
    run_last = tl > run_last ? tl : run_last;
    run_cnt += tk;
  }
  if (threadIdx.x == 0) {
    c->plast = run_last;
    c->npush = run_cnt;
  }
}

// S[slot] for every emit with slot < m'
__global__ void __launch_bounds__(PV_NT) k_piv_emit(const unsigned char* __restrict__ code,
                                                    const int64_t* __restrict__ clast,
                                                    const int64_t* __restrict__ ccnt, const Ctl* c,
                                                    unsigned* __restrict__ S) {
  __shared__ int64_t sm[33];
  const int64_t jend = c->jend, mp = c->mp;
  const int64_t j0 = (int64_t)blockIdx.x * PV_TILE + (int64_t)threadIdx.x * PV_IT;
  unsigned char cd[PV_IT];
  int64_t last = -1, cnt = 0;
#pragma unroll
  for (int k = 0; k < PV_IT; ++k) {
    const int64_t j = j0 + k;
    cd[k] = (j >= 1 && j <= jend) ? code[j] : 0;
    if (cd[k] & PV_TAKE) last = j;
    cnt += (cd[k] & PV_EMIT) ? 1 : 0;
  }
  int64_t tl, tk;
  int64_t piv = block_excl_max(last, sm, &tl);
  int64_t slot = block_excl_sum(cnt, sm, &tk);
  const int64_t cl = clast[blockIdx.x];
  piv = piv > cl ? piv : cl;
  slot += ccnt[blockIdx.x];
#pragma unroll
  for (int k = 0; k < PV_IT; ++k) {
    const int64_t j = j0 + k;
    if (cd[k] & PV_EMIT) {
      if (slot < mp) S[slot] = (unsigned)((cd[k] & PV_PIVOT) ? piv : j);
      ++slot;
    }
    if (cd[k] & PV_TAKE) piv = j;
  }
}

// the end of the walk: a sampler that visited every element emits its pivot
// when |a - 1| < 1e-5; the count must come out at m'
__global__ void k_piv_final(const double* __restrict__ A, int64_t n, Ctl* c, unsigned* __restrict__ S,
                            unsigned* err) {
  int64_t np = c->npush;
  bool bad = false;
  if (!c->broke && n >= 2) {
    if (fabs(__dsub_rn(A[n - 1], 1.0)) < 1e-5) {
      if (np < c->mp) S[np] = (unsigned)c->plast;
      ++np;
    } else {
      bad = true;
    }
  }
  if (np != c->mp) bad = true;
  c->npush = np;
  if (bad) atomicOr(err, FRICC_DEV_PIVOTAL);
}

__global__ void k_set_u64(unsigned long long* p, unsigned long long v) { *p = v; }

// |D| (m for "largest") and the error word into a handle's status block
__global__ void k_put_meta(const Ctl* c, int64_t nd_fixed, const unsigned* err, unsigned long long* meta,
                           Rep rp = Rep{}) {
  if (c) c += blockIdx.x * rp.one;
  err += blockIdx.x * rp.one;
  meta += 2 * blockIdx.x * rp.one;
  meta[0] = (unsigned long long)(c ? c->nd : nd_fixed);
  meta[1] |= (unsigned long long)*err;
}
__global__ void k_set_f64(double* p, double v) { *p = v; }

inline unsigned grid_for(int64_t n, int nt) {
  int64_t g = fricc_cdiv(n, nt);
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace

// Scratch for one compression; everything comes from the stream-ordered pool.
struct CompressScratch {
  unsigned* hist = nullptr;
  unsigned* err = nullptr;
  unsigned long long* ckey = nullptr;
  unsigned* cidx = nullptr;
  unsigned long long* ktmp = nullptr;
  unsigned* vtmp = nullptr;
  unsigned* rhist = nullptr;
  unsigned long long* tstate = nullptr;
  unsigned* ticket = nullptr;
  double* dzero = nullptr;
  double* Rb = nullptr;
  unsigned long long* ffail = nullptr;
  unsigned* S = nullptr;
  double* P = nullptr;
  exact::ChainScratch chain;
};

static void free_scratch(CompressScratch& s, cudaStream_t st) {
  fricc_free(s.hist, st);
  fricc_free(s.err, st);
  fricc_free(s.ckey, st);
  fricc_free(s.cidx, st);
  fricc_free(s.ktmp, st);
  fricc_free(s.vtmp, st);
  fricc_free(s.rhist, st);
  fricc_free(s.tstate, st);
  fricc_free(s.ticket, st);
  fricc_free(s.dzero, st);
  fricc_free(s.Rb, st);
  fricc_free(s.ffail, st);
  fricc_free(s.S, st);
  fricc_free(s.P, st);
  exact::free_chain(s.chain, st);
}

static int dev_status(unsigned e) {
  if (e & FRICC_DEV_P_GT_ONE) {
    fricc_set_error("ERROR MAKING PROBABILITY VECTOR: a sampling probability exceeds 1");
    return FRICC_ERR_P_GT_ONE;
  }
  if (e & FRICC_DEV_PIVOTAL) {
    fricc_set_error("ERROR IN PIVOTAL SAMPLING: acceptance probability outside [0, 1], leftover weight "
                    "|a - 1| >= 1e-5, or a wrong number of sampled elements");
    return FRICC_ERR_PIVOTAL;
  }
  if (e & FRICC_DEV_TIMEOUT) {
    fricc_set_error("a bounded device-side wait timed out");
    return FRICC_ERR_TIMEOUT;
  }
  if (e & FRICC_DEV_INDEX) {
    fricc_set_error("Indices are out of range for given tensor");
    return FRICC_ERR_INDEX;
  }
  return FRICC_OK;
}

// Compress x (device, n doubles) keeping m entries.  mode 0: "fri"
// (systematic, one uniform draw rn), mode 1: "largest".  Writes flat[m],
// vals[m] (device).  Every decision between phases (select digit, candidate
// count, |D|, R, the D threshold) stays on the device, so the only host
// round trip is the final one: with n_largest != nullptr the call
// synchronises the stream, reads |D| and the error word and reports them;
// with n_largest == nullptr it returns at once (nothing read back).
int fricc_glibc_uniforms_device(unsigned* hist, int64_t k, double* out, cudaStream_t st);

// ---------------------------------------------------------------------------
// parallel_sample (src/fri_utils.cpp:176-362): T chunks sampled pivotally,
// each walked by its own warp.  Per chunk (one block of 32): the reference's
// adjustment of the chunk's probabilities towards its integer count g (a
// running FP64 sum with a break; the per-element y is formed by every lane
// in parallel, only the running sum is sequential), then the pivotal weight
// walk of k_piv_chain on the adjusted probabilities.
struct SegInfo {
  int64_t lo, len;   // chunk position and length in q
  double t, a, qn;   // frac(a), a, the chunk's norm
  int64_t g;         // samples the chunk must give
};

__global__ void __launch_bounds__(32) k_seg_chain(const SegInfo* __restrict__ seg, double* __restrict__ P,
                                                  double* __restrict__ A, unsigned char* __restrict__ code,
                                                  Ctl* __restrict__ ctl) {
  const SegInfo sg = seg[blockIdx.x];
  Ctl* c = ctl + blockIdx.x;
  double* p = P + sg.lo;
  const int lane = threadIdx.x;
  const double gd = (double)sg.g;
  // 1. the adjustment (fri_utils.cpp:297-328): p_i <- y_i until the running sum
  //    crosses g, the crossing element taking the remainder
  const int mode = gd > sg.a ? 1 : (gd < sg.a ? -1 : 0);
  if (mode != 0) {
    double sj = sg.qn;
    bool done = false;
    for (int64_t i0 = 0; i0 < sg.len && !done; i0 += 32) {
      const int64_t i = i0 + lane;
      const double q = i < sg.len ? p[i] : 0.0;
      double y;
      if (mode > 0) {
        const double r = __ddiv_rn(q, sg.t);
        y = r < 1.0 ? r : 1.0;            // std::min(1., r): 1 unless r < 1 (NaN -> 1)
      } else {
        const double r = __ddiv_rn(__dsub_rn(q, sg.t), __dsub_rn(1.0, sg.t));
        y = 0.0 < r ? r : 0.0;            // std::max(0., r): r if 0 < r (NaN -> 0)
      }
      const double d = __dsub_rn(y, q);
      double myv = y;
      int hit = 32;
#pragma unroll
      for (int t = 0; t < 32; ++t) {
        const double dt = __shfl_sync(0xffffffffu, d, t);
        const double yt = __shfl_sync(0xffffffffu, y, t);
        if (i0 + t < sg.len && hit == 32) {
          sj = __dadd_rn(sj, dt);
          if (mode > 0 ? sj >= gd : sj <= gd) {
            hit = t;
            if (lane == t) myv = __dsub_rn(__dadd_rn(yt, gd), sj);
          }
        }
      }
      if (i < sg.len && lane <= hit) p[i] = myv;
      if (hit < 32) done = true;
    }
  }
  __syncwarp();
  // 2. the pivotal weight walk over the adjusted chunk (as k_piv_chain)
  const int64_t n = sg.len, mp = c->mp;
  double a = n > 0 ? p[0] : 0.0;
  if (lane == 0 && n > 0) {
    A[sg.lo] = a;
    code[sg.lo] = 0;
  }
  int64_t cnt = 0, jend = n - 1;
  int broke = 0;
  double pn = 1 + lane < n ? p[1 + lane] : 0.0;
  for (int64_t j0 = 1; j0 < n; j0 += 32) {
    const double pj = pn;
    const int64_t jn = j0 + 32 + lane;
    pn = jn < n ? p[jn] : 0.0;
    double myA = 0.0;
    bool myW = false;
#pragma unroll
    for (int t = 0; t < 32; ++t) {
      const double pt = __shfl_sync(0xffffffffu, pj, t);
      const double sum = __dadd_rn(a, pt);
      const bool w = !(sum < 1.0);
      a = w ? __dsub_rn(sum, 1.0) : sum;
      if (lane == t) {
        myA = a;
        myW = w;
      }
    }
    const int64_t j = j0 + lane;
    const bool valid = j < n;
    const unsigned wm = __ballot_sync(0xffffffffu, myW && valid);
    int stop = -1;
    if (mp == 0) {
      if (j0 == 1 && !(wm & 1u)) stop = 0;
    } else if (cnt < mp && cnt + __popc(wm) >= mp) {
      int64_t r = mp - cnt;
      for (int b = 0; b < 32; ++b)
        if (((wm >> b) & 1u) && --r == 0) {
          stop = b;
          break;
        }
    }
    if (valid && (stop < 0 || lane <= stop)) {
      A[sg.lo + j] = myA;
      code[sg.lo + j] = myW ? PV_EMIT : 0;
    }
    if (stop >= 0) {
      jend = j0 + stop;
      broke = 1;
      cnt = mp;
      break;
    }
    cnt += __popc(wm);
  }
  if (lane == 0) {
    c->jend = jend < 0 ? 0 : jend;
    c->npush = cnt;
    c->broke = broke;
  }
}

__global__ void k_s_to_flat(const unsigned* __restrict__ S, int64_t n, int64_t off, int64_t* __restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    out[k] = (int64_t)S[k] + off;
}

// the reference's sample_pivotal on the host, for the T chunk fractions
template <class Draw>
static int host_pivotal(int64_t n_sample, const std::vector<double>& probs, Draw draw, std::vector<int64_t>& S,
                        int64_t* used) {
  S.clear();
  *used = 0;
  const int64_t n = (int64_t)probs.size();
  if (n == 0) return n_sample == 0 ? FRICC_OK : FRICC_ERR_PIVOTAL;
  int64_t i = 0;
  double a = probs[0];
  for (int64_t j = 1; j < n; ++j) {
    a += probs[(size_t)j];
    const double r = draw();
    ++*used;
    if (a < 1.) {
      if (r < probs[(size_t)j] / a) i = j;
    } else {
      a -= 1.;
      const double pa = (1. - probs[(size_t)j]) / (1. - a);
      if (pa > 1 || pa < 0) return FRICC_ERR_PIVOTAL;
      if (r < pa) {
        S.push_back(i);
        i = j;
      } else {
        S.push_back(j);
      }
    }
    if ((int64_t)S.size() == n_sample) break;
    if (j == n - 1) {
      if (std::fabs(a - 1.) < 1e-5) S.push_back(i);
      else return FRICC_ERR_PIVOTAL;
    }
  }
  return (int64_t)S.size() == n_sample ? FRICC_OK : FRICC_ERR_PIVOTAL;
}

// glibc's rand() recurrence on a 31-word history (oldest first), on the host
static double host_glibc_uniform(unsigned* h) {
  const unsigned w = h[0] + h[28];
  for (int t = 0; t < 30; ++t) h[t] = h[t + 1];
  h[30] = w;
  return (double)(int)(w >> 1) / 2147483647.0;
}

// Steps of pivotal sampling after D, R and m' are on the device (ctl): the
// weight walk, the draws, the decisions, the scans; leaves S (m' indices).
// Phase timing of a compression (the reference's verbose table,
// src/fri_utils.cpp:509-519): CUDA events at the phase boundaries of the
// calling thread's compressions while enabled.  Boundaries: 0 start, 1 the
// largest elements and the remaining norm (the reference's "Sorting":
// get_d_largest), 2 the probability vector, 3 the samples, 4 the outputs
// ("Wrap up").
struct PhaseTimer {
  bool on = false;
  bool recorded = false;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};
static thread_local PhaseTimer g_phase;

static void phase_mark(int k, cudaStream_t st) {
  if (!g_phase.on) return;
  if (!g_phase.ev[k] && cudaEventCreate(&g_phase.ev[k]) != cudaSuccess) {
    g_phase.ev[k] = nullptr;
    return;
  }
  cudaEventRecord(g_phase.ev[k], st);
  if (k == 4) g_phase.recorded = true;
}

extern "C" int fricc_phase_timing_set(int on) {
  g_phase.on = on != 0;
  g_phase.recorded = false;
  return FRICC_OK;
}

// Seconds of each phase of the calling thread's last timed compression:
// sorting, P vector, sampling, wrap up, total (waits for its events).
extern "C" int fricc_phase_timing_read(double sec[5]) {
  if (!sec) {
    fricc_set_error("phase_timing_read: null output");
    return FRICC_ERR_ARG;
  }
  if (!g_phase.recorded) {
    fricc_set_error("phase_timing_read: no compression was timed on this thread");
    return FRICC_ERR_ARG;
  }
  float ms[5] = {0, 0, 0, 0, 0};
  FRICC_CUDA(cudaEventSynchronize(g_phase.ev[4]));
  for (int k = 0; k < 4; ++k) FRICC_CUDA(cudaEventElapsedTime(&ms[k], g_phase.ev[k], g_phase.ev[k + 1]));
  FRICC_CUDA(cudaEventElapsedTime(&ms[4], g_phase.ev[0], g_phase.ev[4]));
  for (int k = 0; k < 5; ++k) sec[k] = ms[k] * 1e-3;
  return FRICC_OK;
}

static int pivotal(const double* x, int64_t n, int64_t m, const GenP& gp, Ctl* ctl, CompressScratch& s,
                   unsigned* glibc_hist, int64_t* n_draws, cudaStream_t st) {
  (void)x;
  double *P = nullptr, *A = nullptr, *R = nullptr;
  unsigned char* code = nullptr;
  int64_t *tlast = nullptr, *tcnt = nullptr;
  const int64_t ntile = fricc_cdiv(n, PV_TILE);
  int rc = fricc_alloc_t(&P, n, st);
  if (!rc) rc = fricc_alloc_t(&A, n, st);
  if (!rc) rc = fricc_alloc_t(&code, n, st);
  if (!rc) rc = fricc_alloc_t(&tlast, ntile, st);
  if (!rc) rc = fricc_alloc_t(&tcnt, ntile, st);
  if (!rc) rc = fricc_alloc_t(&s.S, m, st);
  int64_t jend = 0;
  unsigned e = 0;
  if (!rc) {
    k_zero_u32<<<grid_for(m, 256), 256, 0, st>>>(s.S, m);
    k_pvec<<<grid_for(n, 256), 256, 0, st>>>(gp, n, P, s.err);
    phase_mark(2, st);
    k_piv_chain<<<1, 32, 0, st>>>(P, n, ctl, A, code);
    fricc_note_launch(3);
    rc = fricc_cuda_check(cudaGetLastError(), "pivotal chain");
  }
  if (!rc) rc = fricc_cuda_check(cudaMemcpyAsync(&jend, &ctl->jend, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "jend");
  if (!rc) rc = fricc_cuda_check(cudaMemcpyAsync(&e, s.err, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "err");
  if (!rc) rc = fricc_cuda_check(cudaStreamSynchronize(st), "pivotal chain");
  if (!rc) rc = dev_status(e);  // p > 1: the reference exits before drawing
  const int64_t used = jend;   // one draw per visited element j = 1..jend
  if (!rc && used > 0) {
    rc = fricc_alloc_t(&R, used, st);
    if (!rc && glibc_hist) {
      rc = fricc_glibc_uniforms_device(glibc_hist, used, R, st);
    } else if (!rc) {
      std::vector<double> h((size_t)used);
      for (int64_t k = 0; k < used; ++k) h[(size_t)k] = (double)rand() / RAND_MAX;
      rc = fricc_cuda_check(cudaMemcpyAsync(R, h.data(), sizeof(double) * (size_t)used, cudaMemcpyHostToDevice, st),
                            "draws");
      if (!rc) rc = fricc_cuda_check(cudaStreamSynchronize(st), "draws");
    }
  }
  if (!rc) {
    if (n_draws) *n_draws = used;
    if (used > 0) k_piv_decide<<<grid_for(used, 256), 256, 0, st>>>(P, A, code, R, ctl, s.err);
    k_piv_tiles<<<(unsigned)ntile, PV_NT, 0, st>>>(code, ctl, tlast, tcnt);
    k_piv_carry<<<1, 1024, 0, st>>>(tlast, tcnt, ntile, ctl);
    k_piv_emit<<<(unsigned)ntile, PV_NT, 0, st>>>(code, tlast, tcnt, ctl, s.S);
    k_piv_final<<<1, 1, 0, st>>>(A, n, ctl, s.S, s.err);
    fricc_note_launch(used > 0 ? 5 : 4);
    rc = fricc_cuda_check(cudaGetLastError(), "pivotal");
  }
  if (!rc) rc = fricc_cuda_check(cudaMemcpyAsync(&e, s.err, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "err");
  if (!rc) rc = fricc_cuda_check(cudaStreamSynchronize(st), "pivotal");
  if (!rc) rc = dev_status(e);
  fricc_free(P, st);
  fricc_free(A, st);
  fricc_free(R, st);
  fricc_free(code, st);
  fricc_free(tlast, st);
  fricc_free(tcnt, st);
  return rc;
}

// mode 2: "fri" with pivotal sampling.  Its draws (one per visited element)
// come from the glibc stream whose history is glibc_hist[31] (host, oldest
// first; advanced past the draws on return), or with glibc_hist == nullptr
// from this process's own rand(), as the reference draws them.  *n_draws
// receives the number consumed.  Synchronises the stream twice (the number
// of draws, then the result).
// meta (device, 2 words, optional): receives |D| and ORs in the error bits,
// in stream order, so a caller that passes n_largest == nullptr never waits.
int fricc_compress_device(const double* x, int64_t n, int64_t m, int mode, double rn, cudaStream_t st,
                          int64_t* flat, double* vals, int64_t* n_largest, unsigned* glibc_hist, int64_t* n_draws,
                          unsigned long long* meta, const double* rn_dev, const CompressPairOut* pair) {
  if (pair && (mode != 0 || !meta || !pair->flat || !pair->vals || !pair->meta)) {
    fricc_set_error("compress: a paired compression is systematic FRI with status blocks");
    return FRICC_ERR_ARG;
  }
  if (n < 0 || m <= 0 || m > n) {
    fricc_set_error("Bad m_keep value: need 0 < m <= tensor size (m=%lld, size=%lld)", (long long)m,
                    (long long)n);
    return FRICC_ERR_ARG;
  }
  if (n >= 0xffffffffLL) {
    fricc_set_error("tensor too large for 32-bit indices (%lld elements)", (long long)n);
    return FRICC_ERR_ARG;
  }
  CompressScratch s;
  Ctl* ctl = nullptr;
  Ctl* ctl2 = nullptr;  // a paired compression's second state
  unsigned* S2 = nullptr;
  int rc = FRICC_OK;
#define TRY(x)                  \
  do {                          \
    rc = (x);                   \
    if (rc) goto done;          \
  } while (0)

  {
    const int64_t ntile = fricc_cdiv(n, 4096);
    TRY(fricc_alloc_t(&ctl, 1, st));
    TRY(fricc_alloc_t(&s.hist, NDIG, st));
    TRY(fricc_alloc_t(&s.err, 1, st));
    TRY(fricc_alloc_t(&s.ckey, n, st));
    TRY(fricc_alloc_t(&s.cidx, n, st));
    TRY(fricc_alloc_t(&s.ktmp, n, st));
    TRY(fricc_alloc_t(&s.vtmp, n, st));
    TRY(fricc_alloc_t(&s.tstate, ntile + 1, st));  // + a zero word no tile writes (the test-only wait)
    TRY(fricc_alloc_t(&s.ticket, 1, st));
    TRY(fricc_alloc_t(&s.rhist, radix::hist_words(n), st));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.hist, 0, NDIG * sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.err, 0, sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.tstate, 0, (ntile + 1) * sizeof(unsigned long long), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.ticket, 0, sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st), "memset"));
    if (rn_dev) {
      // the draw already in device memory (stream-ordered; capturable)
      TRY(fricc_cuda_check(cudaMemcpyAsync(&ctl->rn, rn_dev, sizeof(double), cudaMemcpyDeviceToDevice, st), "rn"));
    } else {
      // the draw goes through a device word (a pageable-source copy completes
      // before cudaMemcpyAsync returns, so a stack value is safe)
      const double rn_h = rn;
      TRY(fricc_cuda_check(cudaMemcpyAsync(&ctl->rn, &rn_h, sizeof(double), cudaMemcpyHostToDevice, st), "rn"));
    }

    // 1-2. select digit, candidates, sort (argsort, src/fri_utils.cpp:11-36)
    phase_mark(0, st);
    {
      const int bits = select_bits();
      k_hist_sel<<<grid_for(n, 256), 256, sizeof(unsigned) << bits, st>>>(x, n, s.hist, bits);
      k_select_digit<<<1, 1, 0, st>>>(s.hist, m, ctl, bits);
      k_compact<<<(unsigned)ntile, 256, 0, st>>>(x, n, ctl, s.ckey, s.cidx, s.tstate, s.ticket, s.err,
                                                 s.tstate + ntile, (long long)fricc_tune_get(FRICC_TUNE_TEST_WAIT),
                                                 63 - bits);
    }
    fricc_note_launch(3);
    TRY(radix::sort_pairs(s.ckey, s.cidx, s.ktmp, s.vtmp, n, 64, true, s.rhist, st, &ctl->ncand));

    if (mode == 1) {  // "largest": argsort(x, m) with unscaled values
      phase_mark(1, st);
      phase_mark(2, st);
      phase_mark(3, st);
      k_out_d<<<grid_for(m, 256), 256, 0, st>>>(x, s.cidx, m, nullptr, flat, vals);
      fricc_note_launch();
      phase_mark(4, st);
      if (meta) {
        k_put_meta<<<1, 1, 0, st>>>(nullptr, m, s.err, meta);
        fricc_note_launch();
      }
      TRY(fricc_cuda_check(cudaGetLastError(), "largest"));
      if (n_largest) {
        unsigned e = 0;
        TRY(fricc_cuda_check(cudaMemcpyAsync(&e, s.err, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "err"));
        TRY(fricc_cuda_check(cudaStreamSynchronize(st), "compression"));
        TRY(dev_status(e));
        *n_largest = m;
      }
      goto done;
    }

    // 3. one_norm
    TRY(fricc_alloc_t(&s.dzero, 1, st));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.dzero, 0, sizeof(double), st), "memset"));
    TRY((exact::run_chain<GenAbs, exact::ConsNull, false, false>(GenAbs{x}, n, s.dzero, false, exact::ConsNull{},
                                                                 s.chain, s.err, st)));
    const int64_t nch_n = fricc_cdiv(n, exact::CH);
    double* R0 = nullptr;
    TRY(fricc_alloc_t(&R0, 1, st));
    cudaMemcpyAsync(R0, s.chain.cstart + nch_n, sizeof(double), cudaMemcpyDeviceToDevice, st);

    // 4. remaining-norm chain over the sorted top m, acceptance test
    TRY(fricc_alloc_t(&s.Rb, m + 1, st));
    TRY(fricc_alloc_t(&s.ffail, 1, st));
    k_set_u64<<<1, 1, 0, st>>>(s.ffail, (unsigned long long)m);
    fricc_note_launch();
    ConsAccept ca{m, s.Rb, s.ffail};
    rc = exact::run_chain<GenSorted, ConsAccept, false, true>(GenSorted{s.ckey}, m, R0, true, ca, s.chain, s.err, st);
    fricc_free(R0, st);
    if (rc) goto done;
    k_finish_d<<<1, 1, 0, st>>>(s.ffail, s.Rb, s.ckey, s.cidx, m, ctl);
    fricc_note_launch();
    phase_mark(1, st);
    if (pair) {  // the second compression: the same state, its own draw
      TRY(fricc_alloc_t(&ctl2, 1, st));
      TRY(fricc_cuda_check(cudaMemcpyAsync(ctl2, ctl, sizeof(Ctl), cudaMemcpyDeviceToDevice, st), "ctl"));
      if (pair->rn_dev) {
        TRY(fricc_cuda_check(cudaMemcpyAsync(&ctl2->rn, pair->rn_dev, sizeof(double), cudaMemcpyDeviceToDevice, st),
                             "rn"));
      } else {
        const double rn_h = pair->rn;
        TRY(fricc_cuda_check(cudaMemcpyAsync(&ctl2->rn, &rn_h, sizeof(double), cudaMemcpyHostToDevice, st), "rn"));
      }
    }

    GenP gp{x, ctl};
    if (mode == 2) {
      TRY(pivotal(x, n, m, gp, ctl, s, glibc_hist, n_draws, st));
      phase_mark(3, st);
      k_out_d<<<grid_for(m, 256), 256, 0, st>>>(x, s.cidx, m, ctl, flat, vals);
      k_out_s<<<grid_for(m, 256), 256, 0, st>>>(gp, s.S, flat, vals);
      fricc_note_launch(2);
      phase_mark(4, st);
      if (meta) {
        k_put_meta<<<1, 1, 0, st>>>(ctl, 0, s.err, meta);
        fricc_note_launch();
      }
      TRY(fricc_cuda_check(cudaGetLastError(), "output"));
      if (n_largest) {
        int64_t nd = 0;
        TRY(fricc_cuda_check(cudaMemcpyAsync(&nd, &ctl->nd, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "nd"));
        TRY(fricc_cuda_check(cudaStreamSynchronize(st), "compression"));
        *n_largest = nd;
      }
      goto done;
    }

    // 5. probabilities (once, with the p > 1 check), exact partial sums,
    //    systematic samples
    TRY(fricc_alloc_t(&s.S, m, st));
    TRY(fricc_alloc_t(&s.P, n, st));
    k_zero_u32<<<grid_for(m, 256), 256, 0, st>>>(s.S, m);
    k_pvec<<<grid_for(n, 256), 256, 0, st>>>(gp, n, s.P, s.err);
    fricc_note_launch(2);
    phase_mark(2, st);
    // with m' = 0 every p is 0 (or NaN); with R <= 0 or not finite no
    // interval matches (ConsSample checks ctl->sample): in both cases all
    // samples keep index 0, as in the reference
    const GenPv gpv{s.P, x, ctl};
    ConsSample cs{ctl, s.S};
    if (pair) {
      TRY(fricc_alloc_t(&S2, m, st));
      k_zero_u32<<<grid_for(m, 256), 256, 0, st>>>(S2, m);
      fricc_note_launch();
      ConsSample2 cs2{cs, ConsSample{ctl2, S2}};
      TRY((exact::run_chain<GenPv, ConsSample2, false, true>(gpv, n, s.dzero, false, cs2, s.chain, s.err, st)));
    } else {
      TRY((exact::run_chain<GenPv, ConsSample, false, true>(gpv, n, s.dzero, false, cs, s.chain, s.err, st)));
    }

    // 6. output
    phase_mark(3, st);
    k_out_d<<<grid_for(m, 256), 256, 0, st>>>(x, s.cidx, m, ctl, flat, vals);
    k_out_s<<<grid_for(m, 256), 256, 0, st>>>(gpv, s.S, flat, vals);
    fricc_note_launch(2);
    if (!pair) phase_mark(4, st);
    if (meta) {
      k_put_meta<<<1, 1, 0, st>>>(ctl, 0, s.err, meta);
      fricc_note_launch();
    }
    if (pair) {
      const GenPv gpv2{s.P, x, ctl2};
      k_out_d<<<grid_for(m, 256), 256, 0, st>>>(x, s.cidx, m, ctl2, pair->flat, pair->vals);
      k_out_s<<<grid_for(m, 256), 256, 0, st>>>(gpv2, S2, pair->flat, pair->vals);
      k_put_meta<<<1, 1, 0, st>>>(ctl2, 0, s.err, pair->meta);
      fricc_note_launch(3);
      phase_mark(4, st);
    }
    TRY(fricc_cuda_check(cudaGetLastError(), "output"));
    if (n_largest) {
      unsigned e = 0;
      int64_t nd = 0;
      TRY(fricc_cuda_check(cudaMemcpyAsync(&e, s.err, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "err"));
      TRY(fricc_cuda_check(cudaMemcpyAsync(&nd, &ctl->nd, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "nd"));
      TRY(fricc_cuda_check(cudaStreamSynchronize(st), "compression"));
      TRY(dev_status(e));
      *n_largest = nd;
    }
  }
done:
#undef TRY
  free_scratch(s, st);
  fricc_free(ctl, st);
  fricc_free(ctl2, st);
  fricc_free(S2, st);
  return rc;
}

// ---------------------------------------------------------------------------
// Replica batches: the paired systematic compression of R tensors of one
// shape (replica r's tensor x + r n) in one set of launches -- every kernel
// of the single path with the replica on its grid's y (or x) dimension, each
// replica's arithmetic that of its own single compression, so each output is
// bit for bit the one fricc_sp_recompress_pair would give.
namespace {

__global__ void k_fill_u64_b(unsigned long long* p, unsigned long long v, int R) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < R) p[r] = v;
}

// R0[r] = the exact one_norm of replica r (the end of its chain)
__global__ void k_chain_end_b(const double* cstart, int64_t nch, double* R0, int R) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < R) R0[r] = cstart[(int64_t)r * (nch + 1) + nch];
}

// the replicas' draws into their two compression states
__global__ void k_set_rn_b(Ctl* a, Ctl* b, const double* rn, int R) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < R) {
    a[r].rn = rn[2 * r];
    b[r].rn = rn[2 * r + 1];
  }
}

__global__ void k_meta_or_b(const unsigned* err, unsigned long long* meta, int R) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < R) meta[2 * r + 1] |= (unsigned long long)err[r];
}

}  // namespace

int fricc_compress_pair_batch_device(const double* x, int64_t n, int64_t m, int R, const double* rn_dev,
                                     int64_t* flatA, double* valsA, unsigned long long* metaA, int64_t* flatB,
                                     double* valsB, unsigned long long* metaB, cudaStream_t st) {
  if (!x || !rn_dev || !flatA || !valsA || !metaA || !flatB || !valsB || !metaB || R < 1 || R > 65535) {
    fricc_set_error("compress batch: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (n <= 0 || m <= 0 || m > n || n >= 0xffffffffLL) {
    fricc_set_error("Bad m_keep value: need 0 < m <= tensor size < 2^32 (m=%lld, size=%lld)", (long long)m,
                    (long long)n);
    return FRICC_ERR_ARG;
  }
  const int64_t ntile = fricc_cdiv(n, 4096);
  const int64_t nch_n = fricc_cdiv(n, exact::CH), nch_m = fricc_cdiv(m, exact::CH);
  const int64_t rhw = radix::hist_words(n);
  Rep rp;
  rp.n = n;
  rp.m = m;
  rp.tile = ntile + 1;
  rp.one = 1;
  CompressScratch s;
  Ctl *ctl = nullptr, *ctl2 = nullptr;
  unsigned* S2 = nullptr;
  double* R0 = nullptr;
  int rc = FRICC_OK;
#define TRY(x)         \
  do {                 \
    rc = (x);          \
    if (rc) goto done; \
  } while (0)
  {
    const unsigned rb = (unsigned)fricc_cdiv(R, 256);
    TRY(fricc_alloc_t(&ctl, R, st));
    TRY(fricc_alloc_t(&ctl2, R, st));
    TRY(fricc_alloc_t(&s.hist, (size_t)R * NDIG, st));
    TRY(fricc_alloc_t(&s.err, R, st));
    TRY(fricc_alloc_t(&s.ckey, (size_t)R * n, st));
    TRY(fricc_alloc_t(&s.cidx, (size_t)R * n, st));
    TRY(fricc_alloc_t(&s.ktmp, (size_t)R * n, st));
    TRY(fricc_alloc_t(&s.vtmp, (size_t)R * n, st));
    TRY(fricc_alloc_t(&s.tstate, (size_t)R * (ntile + 1), st));
    TRY(fricc_alloc_t(&s.ticket, R, st));
    TRY(fricc_alloc_t(&s.rhist, (size_t)R * rhw, st));
    TRY(fricc_alloc_t(&s.dzero, 1, st));
    TRY(fricc_alloc_t(&R0, R, st));
    TRY(fricc_alloc_t(&s.Rb, (size_t)R * (m + 1), st));
    TRY(fricc_alloc_t(&s.ffail, R, st));
    TRY(fricc_alloc_t(&s.S, (size_t)R * m, st));
    TRY(fricc_alloc_t(&S2, (size_t)R * m, st));
    TRY(fricc_alloc_t(&s.P, (size_t)R * n, st));
    {
      const int64_t nch = nch_n > nch_m ? nch_n : nch_m;
      TRY(fricc_alloc_t(&s.chain.csum, (size_t)R * (nch + 1), st));
      TRY(fricc_alloc_t(&s.chain.cbin, (size_t)R * (nch + 1), st));
      TRY(fricc_alloc_t(&s.chain.cmap, (size_t)R * (nch + 1), st));
      TRY(fricc_alloc_t(&s.chain.cstart, (size_t)R * (nch + 1), st));
      s.chain.cap = R * (nch + 1);
    }
    TRY(fricc_cuda_check(cudaMemsetAsync(s.hist, 0, (size_t)R * NDIG * sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.err, 0, (size_t)R * sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.tstate, 0, (size_t)R * (ntile + 1) * sizeof(unsigned long long), st),
                         "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.ticket, 0, (size_t)R * sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(ctl, 0, (size_t)R * sizeof(Ctl), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.dzero, 0, sizeof(double), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.S, 0, (size_t)R * m * sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(S2, 0, (size_t)R * m * sizeof(unsigned), st), "memset"));
    const unsigned gn = grid_for(n, 256), gm = grid_for(m, 256);

    // 1-2. select digit, candidates, sort
    const int bits = select_bits();
    k_hist_sel<<<dim3(gn, R), 256, sizeof(unsigned) << bits, st>>>(x, n, s.hist, bits, rp);
    k_select_digit<<<R, 1, 0, st>>>(s.hist, m, ctl, bits, rp);
    k_compact<<<dim3((unsigned)ntile, R), 256, 0, st>>>(x, n, ctl, s.ckey, s.cidx, s.tstate, s.ticket, s.err,
                                                        s.tstate + ntile,
                                                        (long long)fricc_tune_get(FRICC_TUNE_TEST_WAIT), 63 - bits,
                                                        rp);
    fricc_note_launch(3);
    {
      radix::Batch bt;
      bt.kv_stride = n;
      bt.hist_stride = rhw;
      bt.n_stride = (int64_t)(sizeof(Ctl) / sizeof(int64_t));
      static_assert(sizeof(Ctl) % sizeof(int64_t) == 0, "Ctl must be a whole number of int64 words");
      TRY(radix::sort_pairs(s.ckey, s.cidx, s.ktmp, s.vtmp, n, 64, true, s.rhist, st, &ctl->ncand, R, bt));
    }

    // 3. one_norm
    {
      exact::ChainStride cs;
      cs.s_init = 0;
      cs.err = 1;
      TRY((exact::run_chain<GenAbs, exact::ConsNull, false, false>(GenAbs{x, n}, n, s.dzero, false,
                                                                   exact::ConsNull{}, s.chain, s.err, st, R, cs)));
      k_chain_end_b<<<rb, 256, 0, st>>>(s.chain.cstart, nch_n, R0, R);
      fricc_note_launch();
    }

    // 4. remaining-norm chain and acceptance test
    k_fill_u64_b<<<rb, 256, 0, st>>>(s.ffail, (unsigned long long)m, R);
    fricc_note_launch();
    {
      exact::ChainStride cs;
      cs.s_init = 1;
      cs.err = 1;
      ConsAccept ca{m, s.Rb, s.ffail, 1};
      TRY((exact::run_chain<GenSorted, ConsAccept, false, true>(GenSorted{s.ckey, n}, m, R0, true, ca, s.chain,
                                                                s.err, st, R, cs)));
    }
    k_finish_d<<<R, 1, 0, st>>>(s.ffail, s.Rb, s.ckey, s.cidx, m, ctl, rp);
    fricc_note_launch();
    // the second compression: the same state, its own draw
    TRY(fricc_cuda_check(cudaMemcpyAsync(ctl2, ctl, (size_t)R * sizeof(Ctl), cudaMemcpyDeviceToDevice, st), "ctl"));
    k_set_rn_b<<<rb, 256, 0, st>>>(ctl, ctl2, rn_dev, R);
    fricc_note_launch();

    // 5. probabilities, exact partial sums, both samplers
    const GenP gp{x, ctl, n, 1};
    k_pvec<<<dim3(gn, R), 256, 0, st>>>(gp, n, s.P, s.err, rp);
    fricc_note_launch();
    const GenPv gpv{s.P, x, ctl, n, 1};
    {
      exact::ChainStride cs;
      cs.s_init = 0;
      cs.err = 1;
      ConsSample2 cs2{ConsSample{ctl, s.S, 1, m}, ConsSample{ctl2, S2, 1, m}};
      TRY((exact::run_chain<GenPv, ConsSample2, false, true>(gpv, n, s.dzero, false, cs2, s.chain, s.err, st, R,
                                                             cs)));
    }

    // 6. outputs
    k_out_d<<<dim3(gm, R), 256, 0, st>>>(x, s.cidx, m, ctl, flatA, valsA, rp);
    k_out_s<<<dim3(gm, R), 256, 0, st>>>(gpv, s.S, flatA, valsA, rp);
    k_put_meta<<<R, 1, 0, st>>>(ctl, 0, s.err, metaA, rp);
    const GenPv gpv2{s.P, x, ctl2, n, 1};
    k_out_d<<<dim3(gm, R), 256, 0, st>>>(x, s.cidx, m, ctl2, flatB, valsB, rp);
    k_out_s<<<dim3(gm, R), 256, 0, st>>>(gpv2, S2, flatB, valsB, rp);
    k_put_meta<<<R, 1, 0, st>>>(ctl2, 0, s.err, metaB, rp);
    fricc_note_launch(6);
    TRY(fricc_cuda_check(cudaGetLastError(), "compress batch"));
  }
done:
#undef TRY
  free_scratch(s, st);
  fricc_free(ctl, st);
  fricc_free(ctl2, st);
  fricc_free(S2, st);
  fricc_free(R0, st);
  return rc;
}

// Unpack the flat indices of R compressions (m each, stacked) into slots;
// an out-of-range index is ORed into the replica's meta[1].
int fricc_unpack_batch_async(const int64_t* flat, int64_t m, int R, const int64_t dims[4], int* slots,
                             unsigned long long* meta, cudaStream_t st) {
  unsigned* err = nullptr;
  int rc = fricc_alloc_t(&err, R, st);
  if (rc) return rc;
  cudaMemsetAsync(err, 0, (size_t)R * sizeof(unsigned), st);
  Rep rp;
  rp.m = m;
  rp.one = 1;
  k_unpack<<<dim3(grid_for(m, 256), R), 256, 0, st>>>(flat, m, dims[0], dims[1], dims[2], dims[3], slots, err, rp);
  k_meta_or_b<<<(unsigned)fricc_cdiv(R, 256), 256, 0, st>>>(err, meta, R);
  fricc_note_launch(2);
  cudaError_t ce = cudaGetLastError();
  fricc_free(err, st);
  return ce == cudaSuccess ? FRICC_OK : fricc_cuda_fail(ce, "unpack batch", __FILE__, __LINE__);
}

// The error bits of a deferred status word, as a status code (and message).
int fricc_dev_status(unsigned e) { return dev_status(e); }

__global__ void k_meta_or(const unsigned* err, unsigned long long* meta) { meta[1] |= (unsigned long long)*err; }

// Unpack without waiting: an out-of-range index is ORed into meta[1].
int fricc_unpack_async(const int64_t* flat, int64_t m, const int64_t dims[4], int* slots, unsigned long long* meta,
                       cudaStream_t st) {
  unsigned* err = nullptr;
  int rc = fricc_alloc_t(&err, 1, st);
  if (rc) return rc;
  cudaMemsetAsync(err, 0, sizeof(unsigned), st);
  k_unpack<<<grid_for(m, 256), 256, 0, st>>>(flat, m, dims[0], dims[1], dims[2], dims[3], slots, err);
  k_meta_or<<<1, 1, 0, st>>>(err, meta);
  fricc_note_launch(2);
  cudaError_t ce = cudaGetLastError();
  fricc_free(err, st);
  return ce == cudaSuccess ? FRICC_OK : fricc_cuda_fail(ce, "unpack", __FILE__, __LINE__);
}

int fricc_unpack_device(const int64_t* flat, int64_t m, const int64_t dims[4], int* slots, cudaStream_t st) {
  unsigned* err = nullptr;
  int rc = fricc_alloc_t(&err, 1, st);
  if (rc) return rc;
  cudaMemsetAsync(err, 0, sizeof(unsigned), st);
  k_unpack<<<grid_for(m, 256), 256, 0, st>>>(flat, m, dims[0], dims[1], dims[2], dims[3], slots, err);
  fricc_note_launch();
  unsigned e = 0;
  cudaMemcpyAsync(&e, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  cudaError_t ce = cudaStreamSynchronize(st);
  fricc_free(err, st);
  if (ce != cudaSuccess) return fricc_cuda_fail(ce, "unpack", __FILE__, __LINE__);
  return dev_status(e);
}

namespace {
struct ConsWrite {
  double* out;
  __device__ __forceinline__ void operator()(int64_t i, double, double after, double) const { out[i] = after; }
};
}  // namespace

// out[i] = fl(out[i-1] + |x_i|), out[-1] = 0: the running sums of one_norm
// (src/fri_utils.cpp:164-171) / std::partial_sum (:142-143), bit for bit.
int fricc_seq_cumsum_device(const double* x, int64_t n, double* out, cudaStream_t st) {
  if (n < 0 || (n > 0 && (!x || !out))) {
    fricc_set_error("seq_cumsum: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (n == 0) return FRICC_OK;
  exact::ChainScratch sc;
  double* dzero = nullptr;
  unsigned* err = nullptr;
  int rc = fricc_alloc_t(&dzero, 1, st);
  if (!rc) rc = fricc_alloc_t(&err, 1, st);
  if (!rc) {
    cudaMemsetAsync(dzero, 0, sizeof(double), st);
    cudaMemsetAsync(err, 0, sizeof(unsigned), st);
    rc = exact::run_chain<GenAbs, ConsWrite, false, true>(GenAbs{x}, n, dzero, false, ConsWrite{out}, sc, err, st);
  }
  exact::free_chain(sc, st);
  fricc_free(dzero, st);
  fricc_free(err, st);
  return rc;
}

// The chunk walks, the chunk draws (in chunk order), the decisions and the
// scans of each chunk, S assembled in the reference's order.
static int fricc_parallel_sample_finish(const double* q, int64_t n, int64_t n_sample, std::vector<SegInfo>& seg,
                                        unsigned* glibc_hist, int64_t* S_out, int64_t* n_draws, int64_t used,
                                        unsigned* err, cudaStream_t st) {
  const int T = (int)seg.size();
  double *P = nullptr, *A = nullptr, *R = nullptr;
  unsigned char* code = nullptr;
  unsigned* Sseg = nullptr;
  SegInfo* dseg = nullptr;
  Ctl* ctl = nullptr;
  int64_t *tlast = nullptr, *tcnt = nullptr;
  std::vector<Ctl> hc((size_t)T);
  std::vector<int64_t> dbase((size_t)T + 1, 0);
  unsigned e = 0;
  int64_t maxlen = 0;
  for (auto& g : seg) maxlen = g.len > maxlen ? g.len : maxlen;
  const int64_t ntile_max = fricc_cdiv(maxlen, PV_TILE);
  int rc = fricc_alloc_t(&P, n, st);
  if (!rc) rc = fricc_alloc_t(&A, n, st);
  if (!rc) rc = fricc_alloc_t(&code, n, st);
  if (!rc) rc = fricc_alloc_t(&Sseg, n_sample > 0 ? n_sample : 1, st);
  if (!rc) rc = fricc_alloc_t(&dseg, T, st);
  if (!rc) rc = fricc_alloc_t(&ctl, T, st);
  if (!rc) rc = fricc_alloc_t(&tlast, ntile_max, st);
  if (!rc) rc = fricc_alloc_t(&tcnt, ntile_max, st);
  if (!rc) {
    for (int j = 0; j < T; ++j) {
      std::memset(&hc[(size_t)j], 0, sizeof(Ctl));
      hc[(size_t)j].mp = seg[(size_t)j].g;
    }
    cudaError_t ce = cudaMemcpyAsync(P, q, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(dseg, seg.data(), sizeof(SegInfo) * T, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(ctl, hc.data(), sizeof(Ctl) * T, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) {
      k_seg_chain<<<(unsigned)T, 32, 0, st>>>(dseg, P, A, code, ctl);
      fricc_note_launch();
      ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(hc.data(), ctl, sizeof(Ctl) * T, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) rc = fricc_cuda_fail(ce, "parallel_sample walk", __FILE__, __LINE__);
  }
  if (!rc) {
    // chunk j consumes one draw per element it visits after its first
    for (int j = 0; j < T; ++j) dbase[(size_t)j + 1] = dbase[(size_t)j] + (seg[(size_t)j].len >= 2 ? hc[(size_t)j].jend : 0);
    const int64_t total = dbase[(size_t)T];
    if (total > 0) {
      rc = fricc_alloc_t(&R, total, st);
      if (!rc && glibc_hist) {
        rc = fricc_glibc_uniforms_device(glibc_hist, total, R, st);
      } else if (!rc) {
        std::vector<double> h((size_t)total);
        for (auto& r : h) r = (double)rand() / RAND_MAX;
        rc = fricc_cuda_check(cudaMemcpyAsync(R, h.data(), sizeof(double) * total, cudaMemcpyHostToDevice, st),
                              "draws");
        if (!rc) rc = fricc_cuda_check(cudaStreamSynchronize(st), "draws");
      }
    }
    used += total;
  }
  if (!rc) {
    int64_t lb = 0;
    for (int j = 0; j < T && !rc; ++j) {
      const SegInfo& g = seg[(size_t)j];
      Ctl* cj = ctl + j;
      const int64_t nt = fricc_cdiv(g.len, PV_TILE);
      if (hc[(size_t)j].jend > 0)
        k_piv_decide<<<grid_for(hc[(size_t)j].jend, 256), 256, 0, st>>>(P + g.lo, A + g.lo, code + g.lo,
                                                                        R + dbase[(size_t)j], cj, err);
      k_piv_tiles<<<(unsigned)nt, PV_NT, 0, st>>>(code + g.lo, cj, tlast, tcnt);
      k_piv_carry<<<1, 1024, 0, st>>>(tlast, tcnt, nt, cj);
      k_piv_emit<<<(unsigned)nt, PV_NT, 0, st>>>(code + g.lo, tlast, tcnt, cj, Sseg + lb);
      k_piv_final<<<1, 1, 0, st>>>(A + g.lo, g.len, cj, Sseg + lb, err);
      if (g.g > 0) k_s_to_flat<<<grid_for(g.g, 256), 256, 0, st>>>(Sseg + lb, g.g, g.lo, S_out + lb);
      fricc_note_launch(6);
      lb += g.g;
      rc = fricc_cuda_check(cudaGetLastError(), "parallel_sample");
    }
  }
  if (!rc) rc = fricc_cuda_check(cudaMemcpyAsync(&e, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "err");
  if (!rc) rc = fricc_cuda_check(cudaStreamSynchronize(st), "parallel_sample");
  if (!rc) rc = dev_status(e);
  if (!rc && n_draws) *n_draws = used;
  fricc_free(P, st);
  fricc_free(A, st);
  fricc_free(R, st);
  fricc_free(code, st);
  fricc_free(Sseg, st);
  fricc_free(dseg, st);
  fricc_free(ctl, st);
  fricc_free(tlast, st);
  fricc_free(tcnt, st);
  fricc_free(err, st);
  return rc;
}

// parallel_sample with T chunks over q (device, n doubles): S (device, n_sample
// int64) in the reference's order; draws from glibc_hist (host, advanced) or
// from this process's rand(), taken in chunk order.  *n_draws: draws used.
int fricc_parallel_sample_device(const double* q, int64_t n, int64_t n_sample, int T, unsigned* glibc_hist,
                                 int64_t* S_out, int64_t* n_draws, cudaStream_t st) {
  if (!q || !S_out || n <= 0 || n_sample < 0 || T < 1 || n < T || n >= 0xffffffffLL) {
    fricc_set_error("parallel_sample: bad arguments (need 1 <= chunks <= n, n < 2^32)");
    return FRICC_ERR_ARG;
  }
  const int64_t step = n / T;
  std::vector<SegInfo> seg((size_t)T);
  std::vector<double> frac((size_t)T);
  int rc = FRICC_OK;
  double *d_norm = nullptr, *dzero = nullptr;
  unsigned* err = nullptr;
  exact::ChainScratch sc;
  int64_t used = 0;
#define PTRY(x)           \
  do {                    \
    rc = (x);             \
    if (rc) goto pdone;   \
  } while (0)
  {
    // norms: exact sequential sums (the reference's one_norm at one thread)
    PTRY(fricc_alloc_t(&d_norm, T + 1, st));
    PTRY(fricc_alloc_t(&dzero, 1, st));
    PTRY(fricc_alloc_t(&err, 1, st));
    PTRY(fricc_cuda_check(cudaMemsetAsync(dzero, 0, sizeof(double), st), "memset"));
    PTRY(fricc_cuda_check(cudaMemsetAsync(err, 0, sizeof(unsigned), st), "memset"));
    for (int j = 0; j <= T; ++j) {
      const int64_t lo = j < T ? j * step : 0, hi = j < T ? ((j + 1 == T) ? n : lo + step) : n;
      PTRY((exact::run_chain<GenAbs, exact::ConsNull, false, false>(GenAbs{q + lo}, hi - lo, dzero, false,
                                                                     exact::ConsNull{}, sc, err, st)));
      PTRY(fricc_cuda_check(cudaMemcpyAsync(d_norm + j, sc.cstart + fricc_cdiv(hi - lo, exact::CH), sizeof(double),
                                            cudaMemcpyDeviceToDevice, st), "norm"));
    }
    std::vector<double> hn((size_t)T + 1);
    PTRY(fricc_cuda_check(cudaMemcpyAsync(hn.data(), d_norm, sizeof(double) * (T + 1), cudaMemcpyDeviceToHost, st),
                          "norms"));
    PTRY(fricc_cuda_check(cudaStreamSynchronize(st), "norms"));
    const double q_norm = hn[(size_t)T];
    uint64_t c = (uint64_t)n_sample;
    for (int j = 0; j < T; ++j) {
      SegInfo& g = seg[(size_t)j];
      g.lo = j * step;
      g.len = (j + 1 == T) ? n - g.lo : step;
      g.qn = hn[(size_t)j];
      g.a = (double)(uint64_t)n_sample * g.qn / q_norm;
      g.t = g.a - std::floor(g.a);
      g.g = (int)std::floor(g.a);
      frac[(size_t)j] = g.t;
      c -= (uint64_t)(int64_t)(int)g.g;
    }
    if (c > (uint64_t)T) {
      fricc_set_error("ERROR IN PIVOTAL SAMPLING: chunk counts exceed n_sample");
      PTRY(FRICC_ERR_PIVOTAL);
    }
    // the fraction sample decides which chunks give one more; its draws come
    // first, one at a time, from the same stream
    std::vector<int64_t> sp;
    int64_t uf = 0;
    auto draw = [&]() { return glibc_hist ? host_glibc_uniform(glibc_hist) : (double)rand() / RAND_MAX; };
    rc = host_pivotal((int64_t)c, frac, draw, sp, &uf);
    if (rc) {
      fricc_set_error("ERROR IN PIVOTAL SAMPLING (chunk fractions)");
      goto pdone;
    }
    used += uf;
    for (int64_t k : sp) seg[(size_t)k].g += 1;
    for (auto& g : seg)
      if (g.g < 0 || g.g > g.len) {
        fricc_set_error("ERROR IN PIVOTAL SAMPLING: a chunk cannot give its %lld samples", (long long)g.g);
        PTRY(FRICC_ERR_PIVOTAL);
      }
  }
pdone:
#undef PTRY
  exact::free_chain(sc, st);
  fricc_free(d_norm, st);
  fricc_free(dzero, st);
  if (rc) {
    fricc_free(err, st);
    return rc;
  }
  return fricc_parallel_sample_finish(q, n, n_sample, seg, glibc_hist, S_out, n_draws, used, err, st);
}
