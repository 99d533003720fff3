// Stable LSD radix sort of (uint64 key, uint32 value) pairs, 8-bit digits.
//
// Used twice on the FRI path: to order the top-m candidates by descending
// |x| with ties in ascending flat index (the order a stable merge sort by
// |x| gives, fri-cc src/fri_utils.cpp:22-25), and to bucket the nonzeros
// of a SparseTensor4d by an index pair while keeping nonzero-slot order
// inside each bucket (the accumulation order of src/sparse_tensor.cpp).
#pragma once
#include "common.cuh"

namespace radix {

constexpr int NT = 256;
constexpr int IPT = 8;
constexpr int TILE = NT * IPT;

__device__ __forceinline__ unsigned digit(unsigned long long k, int shift, int desc) {
  const unsigned d = (unsigned)(k >> shift) & 255u;
  return desc ? 255u - d : d;
}

// n_dev (optional): the element count in device memory, overriding n; tiles
// past it count nothing (and scatter nothing), so a sort can be launched for
// a worst-case size without the host knowing the real one.
//
// Replica batches: blockIdx.y (blockIdx.x for k_scan_digits) is the replica;
// its keys and values start kv_stride elements after the previous one's,
// its histogram hist_stride words after, its n_dev n_stride int64s after.
struct Batch {
  int64_t kv_stride = 0, hist_stride = 0, n_stride = 0;
};

static __global__ void __launch_bounds__(NT) k_hist(const unsigned long long* __restrict__ keys, int64_t n, int shift,
                                             int desc, unsigned* __restrict__ hist, int64_t ntiles,
                                             const int64_t* __restrict__ n_dev, Batch bt) {
  const int rep = blockIdx.y;
  keys += rep * bt.kv_stride;
  hist += rep * bt.hist_stride;
  if (n_dev) n = n_dev[rep * bt.n_stride];
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * TILE;
#pragma unroll
  for (int r = 0; r < IPT; ++r) {
    const int64_t i = base + r * NT + threadIdx.x;
    if (i < n) atomicAdd(&h[digit(keys[i], shift, desc)], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of each digit's per-tile counts (one block per digit, in
// place); the digit's total goes to totals[d].
static __global__ void __launch_bounds__(256) k_scan_rows(unsigned* hist, int64_t ntiles, unsigned* totals, Batch bt) {
  hist += blockIdx.y * bt.hist_stride;
  totals += blockIdx.y * bt.hist_stride;
  __shared__ int64_t sm[33];
  unsigned* row = hist + (int64_t)blockIdx.x * ntiles;
  const int64_t per = fricc_cdiv(ntiles, 256);
  const int64_t b = threadIdx.x * per;
  const int64_t e = b + per < ntiles ? b + per : ntiles;
  int64_t loc = 0;
  for (int64_t i = b; i < e; ++i) loc += row[i];
  int64_t tot;
  int64_t run = block_excl_sum(loc, sm, &tot);
  for (int64_t i = b; i < e; ++i) {
    const unsigned c = row[i];
    row[i] = (unsigned)run;
    run += c;
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = (unsigned)tot;
}

// Exclusive scan of the 256 digit totals into base[d].
static __global__ void __launch_bounds__(256) k_scan_digits(const unsigned* totals, unsigned* base, Batch bt) {
  totals += blockIdx.x * bt.hist_stride;
  base += blockIdx.x * bt.hist_stride;
  __shared__ int64_t sm[33];
  int64_t tot;
  base[threadIdx.x] = (unsigned)block_excl_sum(totals[threadIdx.x], sm, &tot);
}

static __global__ void __launch_bounds__(NT) k_scatter(const unsigned long long* __restrict__ kin,
                                                const unsigned* __restrict__ vin,
                                                unsigned long long* __restrict__ kout, unsigned* __restrict__ vout,
                                                int64_t n, int shift, int desc, const unsigned* __restrict__ offs,
                                                int64_t ntiles, const unsigned* __restrict__ dbase,
                                                const int64_t* __restrict__ n_dev, Batch bt) {
  const int rep = blockIdx.y;
  kin += rep * bt.kv_stride;
  vin += rep * bt.kv_stride;
  kout += rep * bt.kv_stride;
  vout += rep * bt.kv_stride;
  offs += rep * bt.hist_stride;
  dbase += rep * bt.hist_stride;
  if (n_dev) n = n_dev[rep * bt.n_stride];
  if ((int64_t)blockIdx.x * TILE >= n) return;  // uniform per block
  constexpr int NW = NT / 32;
  __shared__ unsigned run[256];
  __shared__ unsigned wc[NW][256];
  run[threadIdx.x] = dbase[threadIdx.x] + offs[(int64_t)threadIdx.x * ntiles + blockIdx.x];
  unsigned lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
  const int w = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * TILE;
  for (int r = 0; r < IPT; ++r) {
#pragma unroll
    for (int k = 0; k < NW; ++k) wc[k][threadIdx.x] = 0;
    __syncthreads();
    const int64_t i = base + r * NT + threadIdx.x;
    const bool valid = i < n;
    unsigned long long key = 0;
    unsigned val = 0;
    unsigned d = 256;
    if (valid) {
      key = kin[i];
      val = vin[i];
      d = digit(key, shift, desc);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned lrank = __popc(peers & lt);
    if (valid && lrank == 0) wc[w][d] = __popc(peers);
    __syncthreads();
    {
      unsigned acc = run[threadIdx.x];
#pragma unroll
      for (int k = 0; k < NW; ++k) {
        const unsigned c = wc[k][threadIdx.x];
        wc[k][threadIdx.x] = acc;
        acc += c;
      }
      run[threadIdx.x] = acc;
    }
    __syncthreads();
    if (valid) {
      const unsigned pos = wc[w][d] + lrank;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
  }
}

// Sorts n pairs on key bits [0, bits) (or *n_dev <= n pairs, when given).
// The result ends in (keys, vals); the tmp buffers must hold n entries, hist
// hist_words(n) counts.
inline int64_t hist_words(int64_t n) { return 256 * fricc_cdiv(n, TILE) + 512; }

// With R > 1, R independent sorts of the replicas' arrays (kv_stride apart,
// each n long; hist holds R * hist_stride words, hist_stride >=
// hist_words(n)).
inline int sort_pairs(unsigned long long* keys, unsigned* vals, unsigned long long* ktmp, unsigned* vtmp,
                      int64_t n, int bits, bool desc, unsigned* hist, cudaStream_t st,
                      const int64_t* n_dev = nullptr, int R = 1, Batch bt = Batch{}) {
  if (n <= 1) return FRICC_OK;
  if (n > 0xffffffffLL || R < 1 || R > 65535) return FRICC_ERR_ARG;
  const int64_t ntiles = fricc_cdiv(n, TILE);
  unsigned long long *ka = keys, *kb = ktmp;
  unsigned *va = vals, *vb = vtmp;
  int passes = 0;
  for (int shift = 0; shift < bits; shift += 8, ++passes) {
    unsigned* totals = hist + 256 * ntiles;
    unsigned* base = totals + 256;
    k_hist<<<dim3((unsigned)ntiles, (unsigned)R), NT, 0, st>>>(ka, n, shift, desc ? 1 : 0, hist, ntiles, n_dev, bt);
    k_scan_rows<<<dim3(256, (unsigned)R), 256, 0, st>>>(hist, ntiles, totals, bt);
    k_scan_digits<<<R, 256, 0, st>>>(totals, base, bt);
    k_scatter<<<dim3((unsigned)ntiles, (unsigned)R), NT, 0, st>>>(ka, va, kb, vb, n, shift, desc ? 1 : 0, hist,
                                                                  ntiles, base, n_dev, bt);
    fricc_note_launch(4);
    unsigned long long* tk = ka;
    ka = kb;
    kb = tk;
    unsigned* tv = va;
    va = vb;
    vb = tv;
  }
  FRICC_LAUNCH_CHECK();
  if (passes & 1) {
    const int64_t span = R > 1 ? (int64_t)(R - 1) * bt.kv_stride + n : n;
    FRICC_CUDA(cudaMemcpyAsync(keys, ka, span * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
    FRICC_CUDA(cudaMemcpyAsync(vals, va, span * sizeof(unsigned), cudaMemcpyDeviceToDevice, st));
  }
  return FRICC_OK;
}

}  // namespace radix
