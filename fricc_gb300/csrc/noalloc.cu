// fricc_seq_cumsum_noalloc: the exact sequential running sum of
// fricc_seq_cumsum, with all of its scratch in one fixed device array that
// is part of the library image, so the call never allocates device memory.
//
// Why: some callers cannot allocate device memory at call time -- an
// application whose device memory is entirely reserved up front by its own
// allocator (a serving process that has divided HBM among resident solves
// and hands each call only its inputs and outputs), or a latency-critical
// loop that must not risk an out-of-memory failure or the device-wide
// synchronisation an allocation can bring.
//
// Limits and rules:
// * n <= FRICC_NOALLOC_MAX_N (2^26 = 67,108,864 elements, the largest
//   amplitude tensor of the o40v200 workload); larger n is rejected with
//   FRICC_ERR_ARG before any device work.
// * The scratch array (about 0.6 MB) is held by every GPU that loads the
//   library, until the process exits.
// * The first call on a device looks up the array's device address for
//   that device (cudaGetSymbolAddress, once per device, with that device
//   current; a failed lookup is retried by the next call); make that first
//   call before any stream capture begins.  The address is kept for the
//   life of the process: a process that resets a device
//   (cudaDeviceReset) must not call this entry point on it afterwards.
// * Every call uses the same array: two calls whose work overlaps on the
//   GPU (different streams, no ordering between them) race and corrupt
//   each other's results.  Calls ordered on one stream are safe.  Each call
//   clears the words that must start at zero; everything else it reads is
//   written earlier in the same call.
#include <mutex>

#include "exactsum.cuh"

namespace {

constexpr int64_t kMaxN = int64_t(1) << 26;
constexpr int64_t kMaxChunks = (kMaxN + exact::CH - 1) / exact::CH + 1;

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kOffZero = 0;                                   // double 0.0
constexpr size_t kOffErr = 256;                                  // unsigned error word
constexpr size_t kOffCsum = 512;
constexpr size_t kOffCbin = kOffCsum + align256(kMaxChunks * sizeof(double));
constexpr size_t kOffCmap = kOffCbin + align256(kMaxChunks * sizeof(int));
constexpr size_t kOffCstart = kOffCmap + align256(kMaxChunks * sizeof(exact::Map));
constexpr size_t kScratchBytes = kOffCstart + align256(kMaxChunks * sizeof(double));

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct GenAbsNA {
  const double* x;
  __device__ __forceinline__ double operator()(int64_t i) const { return fabs(x[i]); }
};

struct ConsWriteNA {
  double* out;
  __device__ __forceinline__ void operator()(int64_t i, double, double after, double) const { out[i] = after; }
};

std::mutex g_mu[64];
unsigned char* g_ptr[64] = {};

// Device address of g_scratch for the current device, looked up on the
// first successful call on that device and kept from then on.  A lookup
// that fails is not remembered: the next call tries again.
int scratch_for_current_device(unsigned char** p) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fricc_cuda_fail(e, "cudaGetDevice", __FILE__, __LINE__);
  if (dev < 0 || dev >= 64) {
    fricc_set_error("seq_cumsum_noalloc: device ordinal %d out of range", dev);
    return FRICC_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_mu[dev]);
  if (!g_ptr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_scratch);
    if (e != cudaSuccess) return fricc_cuda_fail(e, "cudaGetSymbolAddress(g_scratch)", __FILE__, __LINE__);
    if (!ptr) {
      fricc_set_error("seq_cumsum_noalloc: cudaGetSymbolAddress(g_scratch) gave a null address");
      return FRICC_ERR_CUDA;
    }
    g_ptr[dev] = static_cast<unsigned char*>(ptr);
  }
  *p = g_ptr[dev];
  return FRICC_OK;
}

}  // namespace

extern "C" int fricc_seq_cumsum_noalloc(const double* x, int64_t n, double* out, void* stream) {
  if (n < 0 || n > kMaxN) {
    fricc_set_error("seq_cumsum_noalloc: n = %lld is outside [0, %lld]; use fricc_seq_cumsum for larger inputs",
                    (long long)n, (long long)kMaxN);
    return FRICC_ERR_ARG;
  }
  if (n > 0 && (!x || !out)) {
    fricc_set_error("seq_cumsum_noalloc: null argument");
    return FRICC_ERR_ARG;
  }
  if (n == 0) return FRICC_OK;
  unsigned char* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  double* dzero = reinterpret_cast<double*>(base + kOffZero);
  unsigned* err = reinterpret_cast<unsigned*>(base + kOffErr);
  FRICC_CUDA(cudaMemsetAsync(dzero, 0, sizeof(double), st));
  FRICC_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
  exact::ChainScratch sc;
  sc.csum = reinterpret_cast<double*>(base + kOffCsum);
  sc.cbin = reinterpret_cast<int*>(base + kOffCbin);
  sc.cmap = reinterpret_cast<exact::Map*>(base + kOffCmap);
  sc.cstart = reinterpret_cast<double*>(base + kOffCstart);
  sc.cap = kMaxChunks;  // run_chain allocates only when cap is too small; it never is here
  return exact::run_chain<GenAbsNA, ConsWriteNA, false, true>(GenAbsNA{x}, n, dzero, false, ConsWriteNA{out}, sc,
                                                              err, st);
}
