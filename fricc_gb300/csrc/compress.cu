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
#include <vector>

#include "exactsum.cuh"
#include "radix.cuh"
#include "sparse.cuh"

namespace {

constexpr int DIG_BITS = 12;                 // first select digit: |x| bits [62:51]
constexpr int DIG_SHIFT = 63 - DIG_BITS;
constexpr int NDIG = 1 << DIG_BITS;

__device__ __forceinline__ unsigned long long abs_key(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

__global__ void __launch_bounds__(256) k_hist12(const double* __restrict__ x, int64_t n, unsigned* __restrict__ hist) {
  __shared__ unsigned h[NDIG];
  for (int i = threadIdx.x; i < NDIG; i += 256) h[i] = 0;
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * 256;
  for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += stride)
    atomicAdd(&h[abs_key(x[i]) >> DIG_SHIFT], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < NDIG; i += 256)
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
                                                 unsigned long long* tstate, unsigned* ticket, unsigned* err) {
  constexpr int NT = 256, ITEMS = 16, TILE = NT * ITEMS;
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
    if (i < n && (unsigned)(key[k] >> DIG_SHIFT) >= dmin) ++cnt;
  }
  int64_t tot;
  const int64_t excl = block_excl_sum(cnt, sm, &tot);
  if (threadIdx.x == 0) {
    int64_t pre = 0;
    if (tile == 0) {
      atomicExch(&tstate[0], ST_INCL | (unsigned long long)tot);
    } else {
      atomicExch(&tstate[tile], ST_AGG | (unsigned long long)tot);
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
    if (i < n && (unsigned)(key[k] >> DIG_SHIFT) >= dmin) {
      ckey[o] = key[k];
      cidx[o] = (unsigned)i;
      ++o;
    }
  }
}

struct GenAbs {
  const double* x;
  __device__ __forceinline__ double operator()(int64_t i) const { return fabs(x[i]); }
};

struct GenSorted {
  const unsigned long long* keys;
  __device__ __forceinline__ double operator()(int64_t i) const { return __longlong_as_double((long long)keys[i]); }
};

// p_i of make_probability_vector (src/fri_utils.cpp:375,378-381); D membership
// is "at or before the last kept element in (|x| desc, index asc) order".
struct GenP {
  const double* x;
  const Ctl* c;
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

// get_d_largest's acceptance test for every position d of the sorted list.
struct ConsAccept {
  int64_t m;
  double* Rb;                    // [m+1]: R before element d (Rb[m]: after the last)
  unsigned long long* first_fail;
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
  __device__ __forceinline__ void operator()(int64_t j, double lo, double hi, double p) const {
    if (!c->sample || !(p > 0.0)) return;
    const double rn = c->rn;
    const int64_t mp = c->mp;
    const int64_t k0 = count_below(lo, rn, mp);
    const int64_t k1 = count_below(hi, rn, mp);
    for (int64_t k = k0; k < k1; ++k) S[k] = (unsigned)j;
  }
};

// The select digit: the largest d with count(digit >= d) >= m (one thread).
__global__ void k_select_digit(const unsigned* __restrict__ hist, int64_t m, Ctl* c) {
  int64_t cum = 0;
  int d = NDIG - 1;
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
                           Ctl* c) {
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
                        const Ctl* __restrict__ c, int64_t* __restrict__ flat, double* __restrict__ vals) {
  const int64_t nd = c ? c->nd : nd_max;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned j = sidx[i];
    flat[i] = j;
    vals[i] = x[j];
  }
}

// S part: flat = S_k, value = x / p (src/fri_utils.cpp:495,502-504)
__global__ void k_out_s(GenP gp, const unsigned* __restrict__ S, int64_t* __restrict__ flat,
                        double* __restrict__ vals) {
  const int64_t mp = gp.c->mp, nd = gp.c->nd;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < mp; k += (int64_t)gridDim.x * blockDim.x) {
    const unsigned j = S[k];
    flat[nd + k] = j;
    vals[nd + k] = __ddiv_rn(gp.x[j], gp.value(j));
  }
}

__global__ void k_unpack(const int64_t* __restrict__ flat, int64_t m, int64_t d0, int64_t d1, int64_t d2, int64_t d3,
                         int* __restrict__ slots, unsigned* err) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m; s += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long f = (unsigned long long)flat[s];
    const unsigned long long D1 = d1, D2 = d2, D3 = d3;
    const unsigned long long i0 = f / (D1 * D2 * D3);
    const unsigned long long i1 = f % (D1 * D2 * D3) / (D2 * D3);
    const unsigned long long i2 = f % (D2 * D3) / D3;
    const unsigned long long i3 = f % D3;
    if (i0 >= (unsigned long long)d0) atomicOr(err, FRICC_DEV_INDEX);
    slots[4 * s + 0] = (int)i0;
    slots[4 * s + 1] = (int)i1;
    slots[4 * s + 2] = (int)i2;
    slots[4 * s + 3] = (int)i3;
  }
}

__global__ void k_set_u64(unsigned long long* p, unsigned long long v) { *p = v; }
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
  exact::free_chain(s.chain, st);
}

static int dev_status(unsigned e) {
  if (e & FRICC_DEV_P_GT_ONE) {
    fricc_set_error("ERROR MAKING PROBABILITY VECTOR: a sampling probability exceeds 1");
    return FRICC_ERR_P_GT_ONE;
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
int fricc_compress_device(const double* x, int64_t n, int64_t m, int mode, double rn, cudaStream_t st,
                          int64_t* flat, double* vals, int64_t* n_largest) {
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
    TRY(fricc_alloc_t(&s.tstate, ntile, st));
    TRY(fricc_alloc_t(&s.ticket, 1, st));
    TRY(fricc_alloc_t(&s.rhist, radix::hist_words(n), st));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.hist, 0, NDIG * sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.err, 0, sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.tstate, 0, ntile * sizeof(unsigned long long), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(s.ticket, 0, sizeof(unsigned), st), "memset"));
    TRY(fricc_cuda_check(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st), "memset"));
    {
      // the draw goes through a device word (a pageable-source copy completes
      // before cudaMemcpyAsync returns, so a stack value is safe)
      const double rn_h = rn;
      TRY(fricc_cuda_check(cudaMemcpyAsync(&ctl->rn, &rn_h, sizeof(double), cudaMemcpyHostToDevice, st), "rn"));
    }

    // 1-2. select digit, candidates, sort (argsort, src/fri_utils.cpp:11-36)
    k_hist12<<<grid_for(n, 256), 256, 0, st>>>(x, n, s.hist);
    k_select_digit<<<1, 1, 0, st>>>(s.hist, m, ctl);
    k_compact<<<(unsigned)ntile, 256, 0, st>>>(x, n, ctl, s.ckey, s.cidx, s.tstate, s.ticket, s.err);
    fricc_note_launch(3);
    TRY(radix::sort_pairs(s.ckey, s.cidx, s.ktmp, s.vtmp, n, 64, true, s.rhist, st, &ctl->ncand));

    if (mode == 1) {  // "largest": argsort(x, m) with unscaled values
      k_out_d<<<grid_for(m, 256), 256, 0, st>>>(x, s.cidx, m, nullptr, flat, vals);
      fricc_note_launch();
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

    // 5. probabilities, the p > 1 check, exact partial sums, systematic samples
    GenP gp{x, ctl};
    TRY(fricc_alloc_t(&s.S, m, st));
    k_zero_u32<<<grid_for(m, 256), 256, 0, st>>>(s.S, m);
    fricc_note_launch();
    // with m' = 0 every p is 0 (or NaN); with R <= 0 or not finite no
    // interval matches (ConsSample checks ctl->sample): in both cases all
    // samples keep index 0, as in the reference
    ConsSample cs{ctl, s.S};
    TRY((exact::run_chain<GenP, ConsSample, true, true>(gp, n, s.dzero, false, cs, s.chain, s.err, st)));

    // 6. output
    k_out_d<<<grid_for(m, 256), 256, 0, st>>>(x, s.cidx, m, ctl, flat, vals);
    k_out_s<<<grid_for(m, 256), 256, 0, st>>>(gp, s.S, flat, vals);
    fricc_note_launch(2);
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
  return rc;
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
