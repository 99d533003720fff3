// Exact, parallel reproduction of a SEQUENTIAL left-to-right FP64 sum of
// non-negative addends (or of a chain of subtractions of them), i.e. the
// bits of
//     s_0 = s_init;  s_{i+1} = fl(s_i + a_i)   (or fl(s_i - a_i))
// for i = 0..len-1, as a single CPU thread computes them.
//
// FRI compression needs three such chains bit for bit (fri-cc
// src/fri_utils.cpp): one_norm (:164-171), the remaining-norm chain
// R -= |x_(d)| of get_d_largest (:411-421), and std::partial_sum(p) of
// sample_systematic (:142-143).  A parallel reduction rounds differently,
// so instead:
//
// * Inside one binade [2^e, 2^(e+1)) every double is n * ulp with an
//   integer n in [2^52, 2^53] (the bottom binade, which includes the
//   subnormals, is [0, 2^-1021) with n in [0, 2^53]).  Adding a >= 0 moves
//   n by q = floor(a/ulp) plus a rounding carry that depends only on the
//   remainder class of a (0, <1/2, =1/2, >1/2) and, for exact ties, on the
//   parity of n.  A step is therefore a map n -> n + (n odd ? d1 : d0),
//   and such maps compose associatively: the chain inside a binade is a
//   parallel scan over pairs of int64.
// * The binade of the running sum is predicted from an approximate
//   (parallel) prefix sum with a safety margin; chunks whose predicted
//   range stays inside one binade are "clean".
// * A single-block walk applies the chunk maps to the exact running value,
//   verifies every assumption (start in the predicted binade, end inside
//   it) and, where a chunk crosses a binade or was mispredicted, processes
//   that chunk exactly: scan under the current binade, find the first
//   element whose step would leave it, perform that one step with a real
//   FP64 add, continue.  Correctness never depends on the prediction.
#pragma once
#include <climits>
#include <type_traits>
#include <utility>

#include "common.cuh"

namespace exact {

// Replica batches: a chain can run for R independent sequences at once
// (blockIdx.y, or blockIdx.x for the one-block kernels, is the replica).  A
// generator or consumer with a method at(r) gives replica r's copy (its
// pointers moved to that replica's data); one without is shared by all.
template <class G, class = void>
struct has_at : std::false_type {};
template <class G>
struct has_at<G, std::void_t<decltype(std::declval<const G&>().at(0))>> : std::true_type {};
template <class G>
__device__ __forceinline__ G replica_of(const G& g, int r) {
  if constexpr (has_at<G>::value) return g.at(r);
  else return g;
}

// Per-replica strides of a chain's device arguments (elements); the
// scratch arrays always hold nch + 1 entries per replica.
struct ChainStride {
  int64_t s_init = 0;  // the start values
  int64_t err = 0;     // the error words
};

constexpr int64_t TWO52 = 1LL << 52;
constexpr int64_t TWO53 = 1LL << 53;
constexpr int64_t SAT = 1LL << 60;
constexpr double SUB_STOP = 1e-14;  // get_d_largest stops once R <= 1e-14
constexpr int CH = 4096;            // chunk length (elements)

struct Map {
  int64_t d0, d1;  // n -> n + (n odd ? d1 : d0)
};

__device__ __forceinline__ Map map_id() { return Map{0, 0}; }
__device__ __forceinline__ int64_t sat(int64_t x) { return x > SAT ? SAT : (x < -SAT ? -SAT : x); }

// f then g
__device__ __forceinline__ Map compose(Map f, Map g) {
  Map r;
  r.d0 = sat(f.d0 + ((f.d0 & 1) ? g.d1 : g.d0));
  r.d1 = sat(f.d1 + ((f.d1 & 1) ? g.d0 : g.d1));
  return r;
}

__device__ __forceinline__ int64_t apply(Map f, int64_t n) { return n + ((n & 1) ? f.d1 : f.d0); }

// binade id b = max(biased exponent, 1); ulp of binade b is 2^(b-1075)
__device__ __forceinline__ int binade_of(double s) {
  const int ef = (int)(((unsigned long long)__double_as_longlong(s) >> 52) & 0x7ff);
  return ef < 1 ? 1 : ef;
}
__device__ __forceinline__ int64_t n_of(double s, int b) {
  return (int64_t)((unsigned long long)__double_as_longlong(s) - ((unsigned long long)(b - 1) << 52));
}
__device__ __forceinline__ double s_of(int b, int64_t n) {
  return __longlong_as_double((long long)(((unsigned long long)(b - 1) << 52) + (unsigned long long)n));
}

// a >= 0 measured in ulps of binade b: q = floor(a/ulp), cls = remainder class
// (0: exact, 1: below half, 2: exactly half, 3: above half).
__device__ __forceinline__ void decomp(double a, int b, int64_t& q, int& cls) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
  const int ef = (int)(bits >> 52);
  unsigned long long M = bits & ((1ull << 52) - 1);
  if (ef) M |= 1ull << 52;
  const int efp = ef < 1 ? 1 : ef;
  const int shift = b - efp;
  if (shift < 0) { q = SAT; cls = 0; return; }  // a itself is beyond the binade
  if (shift == 0) { q = (int64_t)M; cls = 0; return; }
  if (shift >= 63) { q = 0; cls = M ? 1 : 0; return; }
  q = (int64_t)(M >> shift);
  const unsigned long long r = M & ((1ull << shift) - 1);
  const unsigned long long half = 1ull << (shift - 1);
  cls = r == 0 ? 0 : (r < half ? 1 : (r == half ? 2 : 3));
}

__device__ __forceinline__ Map map_of(int64_t q, int cls, bool sub) {
  const int64_t inc_e = (cls == 3) | ((cls == 2) & (int)(q & 1));
  const int64_t inc_o = (cls == 3) | ((cls == 2) & (int)((q & 1) ^ 1));
  return sub ? Map{-(q + inc_e), -(q + inc_o)} : Map{q + inc_e, q + inc_o};
}

__device__ __forceinline__ Map elem_map(double a, int b, bool sub) {
  int64_t q;
  int cls;
  decomp(a, b, q, cls);
  return map_of(q, cls, sub);
}

// One step of the model from n, with exactness check.
__device__ __forceinline__ bool step(int64_t n, double a, int b, bool sub, int64_t& n_out) {
  int64_t q;
  int cls;
  decomp(a, b, q, cls);
  if (!sub) {
    n_out = apply(map_of(q, cls, false), n);
    return n_out <= TWO53;  // result inside binade b, or exactly at its top
  }
  const int64_t lower = b >= 2 ? TWO52 : 0;
  if (q >= SAT || n - q < lower + (cls != 0)) return false;  // exact result leaves binade b
  n_out = apply(map_of(q, cls, true), n);
  return true;
}

// A conservative test that a whole composite step from n0 stayed exact.
__device__ __forceinline__ bool run_valid(int64_t n_end, int b, bool sub) {
  if (!sub) return n_end <= TWO53;
  return n_end >= (b >= 2 ? TWO52 + 1 : 1);
}

// Block-wide exclusive scan of maps in thread order; *total = composite of all.
template <int NT>
__device__ __forceinline__ Map block_excl_scan_map(Map v, Map* smem, Map* total) {
  constexpr int NW = NT / 32;
  Map incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    Map w;
    w.d0 = __shfl_up_sync(0xffffffffu, incl.d0, o);
    w.d1 = __shfl_up_sync(0xffffffffu, incl.d1, o);
    if ((int)lane_id() >= o) incl = compose(w, incl);
  }
  Map wex;
  wex.d0 = __shfl_up_sync(0xffffffffu, incl.d0, 1);
  wex.d1 = __shfl_up_sync(0xffffffffu, incl.d1, 1);
  if (lane_id() == 0) wex = map_id();
  __syncthreads();
  if (lane_id() == 31) smem[warp_id()] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    Map run = map_id();
    for (int w = 0; w < NW; ++w) {
      Map t = smem[w];
      smem[w] = run;
      run = compose(run, t);
    }
    smem[NW] = run;
  }
  __syncthreads();
  Map r = compose(smem[warp_id()], wex);
  *total = smem[NW];
  __syncthreads();
  return r;
}

struct ChunkSmem {
  Map maps[33];
  int imin[32];
  double s;
};

struct ConsNull {
  __device__ __forceinline__ void operator()(int64_t, double, double, double) const {}
};

// Exact processing of one chunk by the whole block.  Thread t owns the
// contiguous elements [t*ITEMS, t*ITEMS+ITEMS).  cons(i, before, after, a)
// is called once for every element, in no particular order.  Returns the
// exact running value after the chunk (the same in every thread).
template <int NT, int ITEMS, class Gen, class Cons>
__device__ double block_exact_chunk(const Gen& gen, int64_t base, int n_in, double s_start, bool sub,
                                    const Cons& cons, ChunkSmem& sm) {
  double a[ITEMS];
  const int t = threadIdx.x;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int i = t * ITEMS + k;
    a[k] = i < n_in ? gen(base + i) : 0.0;
  }
  double s = s_start;
  int p = 0;
  for (int round = 0; round <= NT * ITEMS && p < n_in; ++round) {
    if (sub && !(s > SUB_STOP)) {  // the remaining-norm chain is over: R stays put
#pragma unroll
      for (int k = 0; k < ITEMS; ++k) {
        const int i = t * ITEMS + k;
        if (i >= p && i < n_in) cons(base + i, s, s, a[k]);
      }
      p = n_in;
      break;
    }
    const int b = binade_of(s);
    const int64_t n0 = n_of(s, b);
    Map agg = map_id();
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const int i = t * ITEMS + k;
      if (i >= p && i < n_in) agg = compose(agg, elem_map(a[k], b, sub));
    }
    Map tot;
    const Map pre = block_excl_scan_map<NT>(agg, sm.maps, &tot);
    int64_t n = apply(pre, n0);
    int first_bad = INT_MAX;
    int64_t n_bad = 0;
    int k_bad = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const int i = t * ITEMS + k;
      if (i >= p && i < n_in && first_bad == INT_MAX) {
        int64_t nn;
        if (step(n, a[k], b, sub, nn)) {
          n = nn;
        } else {
          first_bad = i;
          n_bad = n;
          k_bad = k;
        }
      }
    }
    const int istar = block_min<int>(first_bad, sm.imin);
    n = apply(pre, n0);
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const int i = t * ITEMS + k;
      if (i >= p && i < n_in && i < istar) {
        int64_t nn;
        step(n, a[k], b, sub, nn);
        cons(base + i, s_of(b, n), s_of(b, nn), a[k]);
        n = nn;
      }
    }
    if (istar == INT_MAX) {
      s = s_of(b, apply(tot, n0));
      p = n_in;
      break;
    }
    if (first_bad == istar) {
      const double sb = s_of(b, n_bad);
      const double sa = sub ? __dsub_rn(sb, a[k_bad]) : __dadd_rn(sb, a[k_bad]);
      cons(base + istar, sb, sa, a[k_bad]);
      sm.s = sa;
    }
    __syncthreads();
    s = sm.s;
    p = istar + 1;
    __syncthreads();
  }
  return s;
}

// ---------------------------------------------------------------- kernels

// K_A: approximate sum of each chunk (fixed reduction tree).  With CHECK_P,
// any addend above 1 sets FRICC_DEV_P_GT_ONE (make_probability_vector's check).
template <class Gen, bool CHECK_P>
__global__ void __launch_bounds__(256) k_chunk_sums(Gen gen0, int64_t len, double* csum, unsigned* err,
                                                    ChainStride cs) {
  const int rep = blockIdx.y;
  const Gen gen = replica_of(gen0, rep);
  csum += (int64_t)rep * (fricc_cdiv(len, CH) + 1);
  err += rep * cs.err;
  __shared__ double red[32];
  const int64_t base = (int64_t)blockIdx.x * CH;
  double acc = 0.0;
  bool bad = false;
  for (int r = 0; r < CH / 256; ++r) {
    const int64_t i = base + r * 256 + threadIdx.x;
    if (i < len) {
      const double v = gen(i);
      if (CHECK_P && v > 1.0) bad = true;
      acc += v;
    }
  }
  if (CHECK_P && bad) atomicOr(err, FRICC_DEV_P_GT_ONE);
  const double tot = block_sum_det(acc, red);
  if (threadIdx.x == 0) csum[blockIdx.x] = tot;
}

// K_B (one block of 1024): approximate prefix of the chunk sums and the
// per-chunk binade prediction: cbin[c] = binade if clean, 0 if not.
static __global__ void __launch_bounds__(1024) k_classify(const double* csum, int64_t nch, const double* s_init_dev,
                                                   int sub, int* cbin, ChainStride cs) {
  const int rep = blockIdx.x;
  csum += (int64_t)rep * (nch + 1);
  cbin += (int64_t)rep * (nch + 1);
  const double s_init = s_init_dev[rep * cs.s_init];
  __shared__ double part[1024];
  __shared__ double red[32];
  const int64_t per = fricc_cdiv(nch, 1024);
  const int64_t c0 = threadIdx.x * per;
  const int64_t c1 = c0 + per < nch ? c0 + per : nch;
  double loc = 0.0;
  for (int64_t c = c0; c < c1; ++c) loc += csum[c];
  part[threadIdx.x] = loc;
  const double total = block_sum_det(loc, red);
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0.0;
    for (int w = 0; w < 1024; ++w) {
      const double v = part[w];
      part[w] = run;
      run += v;
    }
  }
  __syncthreads();
  const double scale = fabs(s_init) + total;
  double pre = part[threadIdx.x];
  for (int64_t c = c0; c < c1; ++c) {
    const double P0 = sub ? s_init - pre : s_init + pre;
    pre += csum[c];
    const double P1 = sub ? s_init - pre : s_init + pre;
    const double margin = scale * ((double)(c + 1) * CH * 0x1p-50 + 0x1p-44);
    const double lo = (sub ? P1 : P0) - margin;
    const double hi = (sub ? P0 : P1) + margin;
    int b = 0;
    if (lo > (sub ? SUB_STOP : 0.0) && hi < 1e300) {
      const int b_lo = binade_of(lo), b_hi = binade_of(hi);
      if (b_lo == b_hi) b = b_lo;
    }
    cbin[c] = b;
  }
}

// K_C: composite map of each clean chunk under its predicted binade.
template <class Gen>
__global__ void __launch_bounds__(256) k_chunk_maps(Gen gen0, int64_t len, int sub, const int* cbin, Map* cmap) {
  constexpr int NT = 256, ITEMS = CH / NT;
  const int rep = blockIdx.y;
  const Gen gen = replica_of(gen0, rep);
  cbin += (int64_t)rep * (fricc_cdiv(len, CH) + 1);
  cmap += (int64_t)rep * (fricc_cdiv(len, CH) + 1);
  __shared__ Map smaps[33];
  const int b = cbin[blockIdx.x];
  if (b == 0) return;  // uniform per block
  const int64_t base = (int64_t)blockIdx.x * CH;
  Map agg = map_id();
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int64_t i = base + threadIdx.x * ITEMS + k;
    if (i < len) agg = compose(agg, elem_map(gen(i), b, sub != 0));
  }
  Map tot;
  block_excl_scan_map<NT>(agg, smaps, &tot);
  if (threadIdx.x == 0) cmap[blockIdx.x] = tot;
}

// K_D (one block of 1024): the exact chain over chunks.  cstart[c] receives
// the exact running value at the start of chunk c, cstart[nch] the total.
template <class Gen>
__global__ void __launch_bounds__(1024) k_walk(Gen gen0, int64_t len, const double* s_init_dev, int sub,
                                               const int* cbin, const Map* cmap, double* cstart, ChainStride cs) {
  const int rep = blockIdx.x;
  const Gen gen = replica_of(gen0, rep);
  {
    const int64_t st = (int64_t)rep * (fricc_cdiv(len, CH) + 1);
    cbin += st;
    cmap += st;
    cstart += st;
  }
  const double s_init = s_init_dev[rep * cs.s_init];
  constexpr int NT = 1024;
  __shared__ Map smaps[33];
  __shared__ int simin[32];
  __shared__ ChunkSmem csm;
  const int64_t nch = fricc_cdiv(len, CH);
  double s = s_init;
  int64_t c = 0;
  for (int64_t guard = 0; guard <= nch && c < nch; ++guard) {
    if (sub && !(s > SUB_STOP)) break;
    const int b = binade_of(s);
    const int64_t n0 = n_of(s, b);
    const int64_t ct = c + threadIdx.x;
    const bool ok = ct < nch && cbin[ct] == b;
    const int L = block_min<int>(ok ? INT_MAX : (int)threadIdx.x, simin);
    const Map mine = (ok && (int)threadIdx.x < L) ? cmap[ct] : map_id();
    Map tot;
    const Map pre = block_excl_scan_map<NT>(mine, smaps, &tot);
    const Map incl = compose(pre, mine);
    const int64_t n_end = apply(incl, n0);
    const bool bad = (int)threadIdx.x < L && !run_valid(n_end, b, sub != 0);
    int J = block_min<int>(bad ? (int)threadIdx.x : INT_MAX, simin);
    if (J > L) J = L;
    if (J > NT) J = NT;
    if ((int)threadIdx.x < J) cstart[ct] = s_of(b, apply(pre, n0));
    if (J > 0) {
      // the thread J-1 holds the end value; every thread can recompute it
      // from the block data only through smem, so pass it along.
      if ((int)threadIdx.x == J - 1) csm.s = s_of(b, n_end);
      __syncthreads();
      s = csm.s;
      __syncthreads();
      c += J;
      continue;
    }
    if (threadIdx.x == 0) cstart[c] = s;
    const int64_t base = c * CH;
    const int n_in = (int)(len - base < CH ? len - base : CH);
    s = block_exact_chunk<NT, CH / NT>(gen, base, n_in, s, sub != 0, ConsNull{}, csm);
    c += 1;
  }
  // chunks after an exhausted remaining-norm chain keep the final value
  for (int64_t cc = c + threadIdx.x; cc < nch; cc += NT) cstart[cc] = s;
  if (threadIdx.x == 0) cstart[nch] = s;
}

// K_E: every element's exact before/after values, from the exact chunk starts.
template <class Gen, class Cons>
__global__ void __launch_bounds__(256) k_emit(Gen gen0, Cons cons0, int64_t len, int sub, const double* cstart) {
  constexpr int NT = 256;
  const int rep = blockIdx.y;
  const Gen gen = replica_of(gen0, rep);
  const Cons cons = replica_of(cons0, rep);
  cstart += (int64_t)rep * (fricc_cdiv(len, CH) + 1);
  __shared__ ChunkSmem csm;
  const int64_t base = (int64_t)blockIdx.x * CH;
  const int n_in = (int)(len - base < CH ? len - base : CH);
  block_exact_chunk<NT, CH / NT>(gen, base, n_in, cstart[blockIdx.x], sub != 0, cons, csm);
}

struct ChainScratch {
  double* csum = nullptr;
  int* cbin = nullptr;
  Map* cmap = nullptr;
  double* cstart = nullptr;
  int64_t cap = 0;
};

// Runs the chain over gen(0..len-1) from s_init.  On return (stream order)
// scratch.cstart[nch] holds the exact final value; with EMIT, cons has seen
// every element.
template <class Gen, class Cons, bool CHECK_P, bool EMIT>
int run_chain(const Gen& gen, int64_t len, const double* s_init_dev, bool sub, const Cons& cons,
              ChainScratch& sc, unsigned* dev_err, cudaStream_t st, int R = 1, ChainStride cs = ChainStride{}) {
  const int64_t nch = fricc_cdiv(len, CH);
  if (nch > INT_MAX / 2 || R < 1 || R > 65535) return FRICC_ERR_ARG;
  if (R > 1) {  // the batch's scratch: nch + 1 entries per replica, sized by the caller
    if (sc.cap < R * (nch + 1)) return FRICC_ERR_ARG;
    if (nch == 0) return FRICC_ERR_ARG;
  } else if (sc.cap < nch + 1) {
    fricc_free(sc.csum, st);
    fricc_free(sc.cbin, st);
    fricc_free(sc.cmap, st);
    fricc_free(sc.cstart, st);
    int rc = fricc_alloc_t(&sc.csum, nch + 1, st);
    if (!rc) rc = fricc_alloc_t(&sc.cbin, nch + 1, st);
    if (!rc) rc = fricc_alloc_t(&sc.cmap, nch + 1, st);
    if (!rc) rc = fricc_alloc_t(&sc.cstart, nch + 1, st);
    if (rc) return rc;
    sc.cap = nch + 1;
  }
  if (nch == 0) {
    FRICC_CUDA(cudaMemcpyAsync(sc.cstart, s_init_dev, sizeof(double), cudaMemcpyDeviceToDevice, st));
    return FRICC_OK;
  }
  const dim3 gch((unsigned)nch, (unsigned)R);
  k_chunk_sums<Gen, CHECK_P><<<gch, 256, 0, st>>>(gen, len, sc.csum, dev_err, cs);
  k_classify<<<R, 1024, 0, st>>>(sc.csum, nch, s_init_dev, sub ? 1 : 0, sc.cbin, cs);
  k_chunk_maps<Gen><<<gch, 256, 0, st>>>(gen, len, sub ? 1 : 0, sc.cbin, sc.cmap);
  k_walk<Gen><<<R, 1024, 0, st>>>(gen, len, s_init_dev, sub ? 1 : 0, sc.cbin, sc.cmap, sc.cstart, cs);
  if (EMIT) k_emit<Gen, Cons><<<gch, 256, 0, st>>>(gen, cons, len, sub ? 1 : 0, sc.cstart);
  fricc_note_launch(EMIT ? 5 : 4);
  FRICC_LAUNCH_CHECK();
  return FRICC_OK;
}

inline void free_chain(ChainScratch& sc, cudaStream_t st) {
  fricc_free(sc.csum, st);
  fricc_free(sc.cbin, st);
  fricc_free(sc.cmap, st);
  fricc_free(sc.cstart, st);
  sc = ChainScratch{};
}

}  // namespace exact
