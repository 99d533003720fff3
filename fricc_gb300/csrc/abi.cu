// extern "C" entry points of libfricc_gb300.so (declared in include/fricc_gb300.h).
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/fricc_gb300.h"
#include "common.cuh"
#include "sparse.cuh"

int fricc_compress_device(const double* x, int64_t n, int64_t m, int mode, double rn, cudaStream_t st, int64_t* flat,
                          double* vals, int64_t* n_largest, unsigned* glibc_hist, int64_t* n_draws,
                          unsigned long long* meta = nullptr, const double* rn_dev = nullptr,
                          const CompressPairOut* pair = nullptr);
int fricc_unpack_async(const int64_t* flat, int64_t m, const int64_t dims[4], int* slots, unsigned long long* meta,
                       cudaStream_t st);
int fricc_dev_status(unsigned e);
int fricc_parallel_sample_device(const double* q, int64_t n, int64_t n_sample, int T, unsigned* glibc_hist,
                                 int64_t* S_out, int64_t* n_draws, cudaStream_t st);
int fricc_glibc_uniforms_device(unsigned* hist, int64_t k, double* out, cudaStream_t st);
int fricc_seq_cumsum_device(const double* x, int64_t n, double* out, cudaStream_t st);
int fricc_unpack_device(const int64_t* flat, int64_t m, const int64_t dims[4], int* slots, cudaStream_t st);
int fricc_contract_device(const char* term, const double* W, const int64_t Wd[4], const int64_t Ws[4], FriccSparse* T,
                          double* out, const int64_t Od[4], const int64_t Os[4], cudaStream_t st);
double fricc_contract_flops_impl(const char* term, const FriccSparse* T);
int fricc_spmm_device(FriccSparse* T, int pa, int pb, int ka, int kb, double coef, const double* Wp, int64_t QS,
                      double* Op, cudaStream_t st);
int fricc_spmm_f2_device(FriccSparse* T, int pa, int pb, int ka, int kb, double coef, const float4* Wp, int64_t QS,
                         double* Op, cudaStream_t st);
int fricc_split_f2_device(const double* x, int64_t rows, int64_t qs, float4* out, cudaStream_t st);
int fricc_spmm_f1_device(FriccSparse* T, int pa, int pb, int ka, int kb, double coef, const float* W, int64_t QS,
                         int64_t ldw, double* Op, cudaStream_t st, bool fp32);
int fricc_densify_bf16x3_device(FriccSparse* T, int pa, int pb, int ka, int kb, double coef, void* Ap, int64_t kp,
                                cudaStream_t st);
int fricc_gemm_df_device(const double* A, const double* B, double* C, int64_t batch, int64_t M, int64_t N, int64_t K,
                         const int64_t sA[3], const int64_t sB[3], const int64_t sC[3], double alpha, double beta,
                         cudaStream_t st, int64_t batch2, const int64_t* s2);
int fricc_gemm_f64_device(const double* A, const double* B, double* C, int64_t batch, int64_t M, int64_t N,
                          int64_t K, const int64_t sA[3], const int64_t sB[3], const int64_t sC[3], double alpha,
                          double beta, cudaStream_t st, int64_t batch2, const int64_t* s2);
int fricc_combine_device(const int64_t dims[5], int n_in, const double* const* x, const int64_t* sx, int n_prod,
                         const double* const* p, const int64_t* sp, int n_out, double* const* out, const int64_t* so,
                         const double* coef, int accumulate, cudaStream_t st);
int fricc_combine4_device(const int64_t dims[4], int n_in, const double* const* x, const int64_t* sx, int n_prod,
                          const double* const* p, const int64_t* sp, int n_out, double* const* out, const int64_t* so,
                          const double* coef, int accumulate, cudaStream_t st);
int fricc_compress_pair_batch_device(const double* x, int64_t n, int64_t m, int R, const double* rn_dev,
                                     int64_t* flatA, double* valsA, unsigned long long* metaA, int64_t* flatB,
                                     double* valsB, unsigned long long* metaB, cudaStream_t st);
int fricc_unpack_batch_async(const int64_t* flat, int64_t m, int R, const int64_t dims[4], int* slots,
                             unsigned long long* meta, cudaStream_t st);
int fricc_batch_spmm_device(FriccSparseBatch* B, int which, int pa, int pb, int ka, int kb, double coef,
                            const void* Wp, int64_t w_stride, int64_t QS, double* Op, int64_t o_stride, bool f2,
                            cudaStream_t st);
int fricc_batch_densify_device(FriccSparseBatch* B, int which, int pa, int pb, int ka, int kb, double coef, void* Ap,
                               int64_t kp, cudaStream_t st);
int fricc_energy_update_batch_device(int R, const double* t1num, const double* t2num, const double* eia,
                                     const double* fov, const double* ovov, const double* t1old, const double* t2old,
                                     int64_t o, int64_t v, double* t1out, double* t2out, double* res,
                                     cudaStream_t st);
int fricc_energy_update_device(const double* t1num, const double* t2num, const double* eia, const double* fov,
                               const double* ovov, const double* t1old, const double* t2old, int64_t o, int64_t v,
                               double* t1out, double* t2out, double* res, cudaStream_t st, bool linear);

// ------------------------------------------------------------------ errors
static thread_local char g_err[512] = "";

void fricc_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int fricc_cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return FRICC_OK;
  fricc_set_error("CUDA error %s (%s) in %s", cudaGetErrorName(e), cudaGetErrorString(e), what);
  return FRICC_ERR_CUDA;
}

int fricc_cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  fricc_set_error("CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e), what, file, line);
  return FRICC_ERR_CUDA;
}

// ------------------------------------------------------------------ instrumentation
#include <atomic>
#include <vector>
static std::atomic<long long> g_launches{0};
static std::atomic<long long> g_allocs{0};
static std::atomic<bool> g_prof{false};
static std::mutex g_prof_mu;
// channel 0: the sparse contraction kernels; channel 1: the tensor-core
// GEMMs; channel 2: the FP64 GEMMs
constexpr int kProfChannels = 3;
static std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_prof_ev[kProfChannels];
static std::vector<double> g_prof_flops[kProfChannels];
static cudaEvent_t g_prof_pending[kProfChannels] = {nullptr, nullptr, nullptr};

void fricc_note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static thread_local int g_tune[FRICC_TUNE_KNOBS] = {-1, -1, -1, -1, -1, -1};
int fricc_tune_get(int knob) { return knob >= 0 && knob < FRICC_TUNE_KNOBS ? g_tune[knob] : -1; }
bool fricc_prof_on() { return g_prof.load(std::memory_order_relaxed); }

void fricc_prof_record(cudaStream_t st, bool start, double flops, int ch) {
  if (ch < 0 || ch >= kProfChannels) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, st);
  if (start) {
    if (g_prof_pending[ch]) cudaEventDestroy(g_prof_pending[ch]);
    g_prof_pending[ch] = e;
  } else if (g_prof_pending[ch]) {
    g_prof_ev[ch].emplace_back(g_prof_pending[ch], e);
    g_prof_flops[ch].push_back(flops);
    g_prof_pending[ch] = nullptr;
  } else {
    cudaEventDestroy(e);
  }
}

// ------------------------------------------------------------------ memory
static std::once_flag g_pool_once[64];

int fricc_alloc(void** p, size_t bytes, cudaStream_t s) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64) {
    std::call_once(g_pool_once[dev], [dev]() {
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;  // keep freed blocks cached in the pool
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
      }
    });
  }
  g_allocs.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 16, s);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fricc_cuda_fail(e, "cudaMallocAsync", __FILE__, __LINE__);
  }
  return FRICC_OK;
}

void fricc_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

static cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

static void free_sparse_arrays(FriccSparse* T, cudaStream_t st) {
  fricc_free(T->meta, st);
  T->meta = nullptr;
  fricc_free(T->flat, st);
  fricc_free(T->vals, st);
  fricc_free(T->slots, st);
  T->flat = nullptr;
  T->vals = nullptr;
  T->slots = nullptr;
  for (auto& b : T->buck) {
    fricc_free(b.bptr, st);
    fricc_free(b.order, st);
    b = Bucketing{};
  }
}

// after a re-compression: keep the arrays, rebuild on next use
static void stale_bucketings(FriccSparse* T) {
  for (auto& b : T->buck) b.valid = false;
}

static bool bad_dims(const int64_t dims[4]) {
  if (!dims) return true;
  for (int k = 0; k < 4; ++k)
    if (dims[k] <= 0 || dims[k] > 0x7fffffff) return true;
  return false;
}

// ------------------------------------------------------------------ API
extern "C" {

int fricc_version(void) { return 100; }

long long fricc_launch_count(void) { return g_launches.load(); }

long long fricc_alloc_count(void) { return g_allocs.load(); }

int fricc_tune_set(int knob, int value) {
  static const int lo[FRICC_TUNE_KNOBS] = {1, 0, 1, 1, 10, 1}, hi[FRICC_TUNE_KNOBS] = {4, 4, 16, 1 << 20, 13, 8};
  if (knob < 0 || knob >= FRICC_TUNE_KNOBS || (value != -1 && (value < lo[knob] || value > hi[knob]))) {
    fricc_set_error("tune_set: bad knob or value");
    return FRICC_ERR_ARG;
  }
  if (knob == FRICC_TUNE_SPMM_PPT && value == 3) {
    fricc_set_error("tune_set: pairs per thread is 1, 2 or 4");
    return FRICC_ERR_ARG;
  }
  g_tune[knob] = value;
  return FRICC_OK;
}

void fricc_prof_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.store(on != 0);
  for (int ch = 0; ch < kProfChannels; ++ch) {
    for (auto& pr : g_prof_ev[ch]) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
    g_prof_ev[ch].clear();
    g_prof_flops[ch].clear();
    if (g_prof_pending[ch]) cudaEventDestroy(g_prof_pending[ch]);
    g_prof_pending[ch] = nullptr;
  }
}

static int prof_read(int ch, double* ms, long long* launches, double* flops) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  double t = 0.0, f = 0.0;
  for (size_t k = 0; k < g_prof_ev[ch].size(); ++k) {
    float x = 0.f;
    cudaError_t e = cudaEventSynchronize(g_prof_ev[ch][k].second);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&x, g_prof_ev[ch][k].first, g_prof_ev[ch][k].second);
    if (e != cudaSuccess) return fricc_cuda_fail(e, "prof_read", __FILE__, __LINE__);
    t += x;
    f += g_prof_flops[ch][k];
  }
  if (ms) *ms = t;
  if (launches) *launches = (long long)g_prof_ev[ch].size();
  if (flops) *flops = f;
  return FRICC_OK;
}

int fricc_prof_read(double* ms, long long* launches, double* flops) { return prof_read(0, ms, launches, flops); }

int fricc_prof_read_tc(double* ms, long long* launches, double* flops) { return prof_read(1, ms, launches, flops); }

int fricc_prof_read_gemm(double* ms, long long* launches, double* flops) { return prof_read(2, ms, launches, flops); }

const char* fricc_last_error(void) { return g_err; }

// Read back the status block of an asynchronous compression (blocking).
static int settle(const fricc_sparse* Tc) {
  fricc_sparse* T = const_cast<fricc_sparse*>(Tc);
  if (!T->pending) return T->status;
  unsigned long long h[2] = {0, 0};
  cudaError_t e = cudaMemcpyAsync(h, T->meta, sizeof(h), cudaMemcpyDeviceToHost, T->owner_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(T->owner_stream);
  if (e != cudaSuccess) return fricc_cuda_fail(e, "compression status", __FILE__, __LINE__);
  // pending stays set: a re-compression replayed from a CUDA graph rewrites
  // the block without passing through the host
  T->n_largest = (int64_t)h[0];
  T->status = fricc_dev_status((unsigned)h[1]);
  return T->status;
}

// mode: 0 fri systematic (rn), 1 largest, 2 fri pivotal (hist / rand()).
// Modes 0 and 1 only enqueue work: |D| and any error are read back by the
// next blocking call on the handle (settle).
static int recompress(fricc_sparse* T, const double* t2, int mode, double rn, unsigned* hist, int64_t* n_draws,
                      void* stream, const double* rn_dev = nullptr) {
  cudaStream_t st = as_stream(stream);
  stale_bucketings(T);
  const int64_t n = T->dims[0] * T->dims[1] * T->dims[2] * T->dims[3];
  T->owner_stream = st;
  T->pending = false;
  T->status = FRICC_OK;
  FRICC_CUDA(cudaMemsetAsync(T->meta, 0, 2 * sizeof(unsigned long long), st));
  if (mode == 2) {
    int64_t nd = 0;
    int rc = fricc_compress_device(t2, n, T->m, mode, rn, st, T->flat, T->vals, &nd, hist, n_draws);
    if (rc) return rc;
    T->n_largest = nd;
    return fricc_unpack_device(T->flat, T->m, T->dims, T->slots, st);
  }
  int rc = fricc_compress_device(t2, n, T->m, mode, rn, st, T->flat, T->vals, nullptr, hist, n_draws, T->meta, rn_dev);
  if (!rc) rc = fricc_unpack_async(T->flat, T->m, T->dims, T->slots, T->meta, st);
  if (!rc) T->pending = true;
  return rc;
}

// Both handles from the same tensor with draws rn_a, rn_b (host values, or the
// two doubles at rn_dev): the shared phases run once and one sampling chain
// serves both (systematic FRI only; the handles must have t2's dims and
// equal m).  Stream-ordered like recompress.
static int recompress_pair(fricc_sparse* A, fricc_sparse* B, const double* t2, double rn_a, double rn_b,
                           const double* rn_dev, void* stream) {
  if (!A || !B || !t2 || A == B || A->m != B->m) {
    fricc_set_error("sp_recompress_pair: two distinct handles with the same m");
    return FRICC_ERR_ARG;
  }
  for (int k = 0; k < 4; ++k)
    if (A->dims[k] != B->dims[k]) {
      fricc_set_error("sp_recompress_pair: the handles' dims differ");
      return FRICC_ERR_ARG;
    }
  cudaStream_t st = as_stream(stream);
  stale_bucketings(A);
  stale_bucketings(B);
  const int64_t n = A->dims[0] * A->dims[1] * A->dims[2] * A->dims[3];
  for (fricc_sparse* T : {A, B}) {
    T->owner_stream = st;
    T->pending = false;
    T->status = FRICC_OK;
    FRICC_CUDA(cudaMemsetAsync(T->meta, 0, 2 * sizeof(unsigned long long), st));
  }
  const CompressPairOut pb{B->flat, B->vals, B->meta, rn_b, rn_dev ? rn_dev + 1 : nullptr};
  int rc = fricc_compress_device(t2, n, A->m, 0, rn_a, st, A->flat, A->vals, nullptr, nullptr, nullptr, A->meta,
                                 rn_dev, &pb);
  if (!rc) rc = fricc_unpack_async(A->flat, A->m, A->dims, A->slots, A->meta, st);
  if (!rc) rc = fricc_unpack_async(B->flat, B->m, B->dims, B->slots, B->meta, st);
  if (!rc) A->pending = B->pending = true;
  return rc;
}

int fricc_sp_recompress_pair(fricc_sparse* A, fricc_sparse* B, const double* t2, double rn_a, double rn_b,
                             void* stream) {
  return recompress_pair(A, B, t2, rn_a, rn_b, nullptr, stream);
}

int fricc_sp_recompress_pair_dev(fricc_sparse* A, fricc_sparse* B, const double* t2, const double* rn_dev,
                                 void* stream) {
  if (!rn_dev) {
    fricc_set_error("sp_recompress_pair_dev: null draws");
    return FRICC_ERR_ARG;
  }
  return recompress_pair(A, B, t2, 0.0, 0.0, rn_dev, stream);
}

int fricc_sp_status(const fricc_sparse* T) {
  if (!T) {
    fricc_set_error("sp_status: null handle");
    return FRICC_ERR_ARG;
  }
  return settle(T);
}

int fricc_sp_recompress(fricc_sparse* T, const double* t2, int compression, int sampling, double rn, void* stream) {
  if (!T || !t2) {
    fricc_set_error("sp_recompress: null argument");
    return FRICC_ERR_ARG;
  }
  if (compression != FRICC_COMPRESSION_FRI && compression != FRICC_COMPRESSION_LARGEST) {
    fricc_set_error("The compression method you chose isn't supported: compression must be 'largest' or 'fri'");
    return FRICC_ERR_ARG;
  }
  if (compression == FRICC_COMPRESSION_FRI && sampling == FRICC_SAMPLING_PIVOTAL) {
    // pivotal draws one uniform per element: its entry points take the stream
    fricc_set_error("pivotal sampling draws its uniforms itself: use fricc_sp_recompress_pivotal");
    return FRICC_ERR_ARG;
  }
  if (compression == FRICC_COMPRESSION_FRI && sampling != FRICC_SAMPLING_SYSTEMATIC) {
    fricc_set_error("sampling_method must be 'pivotal' or 'systematic'");
    return FRICC_ERR_ARG;
  }
  return recompress(T, t2, compression == FRICC_COMPRESSION_LARGEST ? 1 : 0, rn, nullptr, nullptr, stream);
}

int fricc_sp_recompress_dev(fricc_sparse* T, const double* t2, int compression, int sampling, const double* rn_dev,
                            void* stream) {
  if (!T || !t2 || (compression == FRICC_COMPRESSION_FRI && !rn_dev)) {
    fricc_set_error("sp_recompress_dev: null argument");
    return FRICC_ERR_ARG;
  }
  if (compression != FRICC_COMPRESSION_FRI && compression != FRICC_COMPRESSION_LARGEST) {
    fricc_set_error("The compression method you chose isn't supported: compression must be 'largest' or 'fri'");
    return FRICC_ERR_ARG;
  }
  if (compression == FRICC_COMPRESSION_FRI && sampling != FRICC_SAMPLING_SYSTEMATIC) {
    fricc_set_error("sp_recompress_dev: systematic sampling only (pivotal draws per element)");
    return FRICC_ERR_ARG;
  }
  return recompress(T, t2, compression == FRICC_COMPRESSION_LARGEST ? 1 : 0, 0.0, nullptr, nullptr, stream,
                    compression == FRICC_COMPRESSION_FRI ? rn_dev : nullptr);
}

int fricc_sp_recompress_pivotal(fricc_sparse* T, const double* t2, uint32_t* glibc_hist, void* stream,
                                int64_t* n_draws) {
  if (!T || !t2) {
    fricc_set_error("sp_recompress_pivotal: null argument");
    return FRICC_ERR_ARG;
  }
  return recompress(T, t2, 2, 0.0, glibc_hist, n_draws, stream);
}

static int create(const double* t2, const int64_t dims[4], int64_t m, int mode, double rn, unsigned* hist,
                  int64_t* n_draws, void* stream, fricc_sparse** out);

int fricc_sp_create_pivotal(const double* t2, const int64_t dims[4], int64_t m, uint32_t* glibc_hist, void* stream,
                            fricc_sparse** out, int64_t* n_draws) {
  return create(t2, dims, m, 2, 0.0, glibc_hist, n_draws, stream, out);
}

int fricc_sp_create(const double* t2, const int64_t dims[4], int64_t m, int compression, int sampling, double rn,
                    void* stream, fricc_sparse** out) {
  if (compression != FRICC_COMPRESSION_FRI && compression != FRICC_COMPRESSION_LARGEST) {
    fricc_set_error("The compression method you chose isn't supported: compression must be 'largest' or 'fri'");
    return FRICC_ERR_ARG;
  }
  if (compression == FRICC_COMPRESSION_FRI && sampling == FRICC_SAMPLING_PIVOTAL) {
    fricc_set_error("pivotal sampling draws its uniforms itself: use fricc_sp_create_pivotal");
    return FRICC_ERR_ARG;
  }
  if (compression == FRICC_COMPRESSION_FRI && sampling != FRICC_SAMPLING_SYSTEMATIC) {
    fricc_set_error("sampling_method must be 'pivotal' or 'systematic'");
    return FRICC_ERR_ARG;
  }
  return create(t2, dims, m, compression == FRICC_COMPRESSION_LARGEST ? 1 : 0, rn, nullptr, nullptr, stream, out);
}

static int create(const double* t2, const int64_t dims[4], int64_t m, int mode, double rn, unsigned* hist,
                  int64_t* n_draws, void* stream, fricc_sparse** out) {
  if (!out || !t2 || bad_dims(dims)) {
    fricc_set_error("sp_create: null pointer or non-positive dims");
    return FRICC_ERR_ARG;
  }
  *out = nullptr;
  const int64_t n = dims[0] * dims[1] * dims[2] * dims[3];
  if (m <= 0 || m > n) {
    fricc_set_error("Bad m_keep value! The following condition wasn't met 0 < m_keep <= t2.size (m=%lld, size=%lld)",
                    (long long)m, (long long)n);
    return FRICC_ERR_ARG;
  }
  cudaStream_t st = as_stream(stream);
  FriccSparse* T = new FriccSparse();
  for (int k = 0; k < 4; ++k) T->dims[k] = dims[k];
  T->m = m;
  cudaGetDevice(&T->device);
  int rc = fricc_alloc_t(&T->flat, m, st);
  if (!rc) rc = fricc_alloc_t(&T->vals, m, st);
  if (!rc) rc = fricc_alloc_t(&T->slots, 4 * m, st);
  if (!rc) rc = fricc_alloc_t(&T->meta, 2, st);
  if (!rc) rc = recompress(T, t2, mode, rn, hist, n_draws, stream);
  if (rc) {
    free_sparse_arrays(T, st);
    cudaStreamSynchronize(st);
    delete T;
    return rc;
  }
  *out = T;
  return FRICC_OK;
}

int fricc_sp_create_empty(const int64_t dims[4], int64_t nnz, void* stream, fricc_sparse** out) {
  if (!out || bad_dims(dims) || nnz < 0) {
    fricc_set_error("sp_create_empty: bad arguments");
    return FRICC_ERR_ARG;
  }
  cudaStream_t st = as_stream(stream);
  FriccSparse* T = new FriccSparse();
  for (int k = 0; k < 4; ++k) T->dims[k] = dims[k];
  T->m = nnz;
  cudaGetDevice(&T->device);
  int rc = fricc_alloc_t(&T->flat, nnz, st);
  if (!rc) rc = fricc_alloc_t(&T->vals, nnz, st);
  if (!rc) rc = fricc_alloc_t(&T->slots, 4 * nnz, st);
  if (!rc) rc = fricc_alloc_t(&T->meta, 2, st);
  if (!rc) {
    cudaMemsetAsync(T->meta, 0, 2 * sizeof(unsigned long long), st);
    cudaMemsetAsync(T->flat, 0, nnz * sizeof(int64_t), st);
    cudaMemsetAsync(T->vals, 0, nnz * sizeof(double), st);
    cudaMemsetAsync(T->slots, 0, 4 * nnz * sizeof(int), st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fricc_cuda_fail(e, "sp_create_empty", __FILE__, __LINE__);
  }
  if (rc) {
    free_sparse_arrays(T, st);
    delete T;
    return rc;
  }
  T->owner_stream = st;
  *out = T;
  return FRICC_OK;
}

int fricc_sp_destroy(fricc_sparse* T) {
  if (!T) return FRICC_OK;
  free_sparse_arrays(T, T->owner_stream);
  delete T;
  return FRICC_OK;
}

int fricc_sp_info(const fricc_sparse* T, int64_t dims[4], int64_t* m, int64_t* n_largest) {
  if (!T) {
    fricc_set_error("sp_info: null handle");
    return FRICC_ERR_ARG;
  }
  const int rc = settle(T);
  if (rc) return rc;
  if (dims)
    for (int k = 0; k < 4; ++k) dims[k] = T->dims[k];
  if (m) *m = T->m;
  if (n_largest) *n_largest = T->n_largest;
  return FRICC_OK;
}

int fricc_sp_get(const fricc_sparse* T, int64_t mi, int64_t idx[4], double* value) {
  if (!T || mi < 0 || mi >= T->m) {
    fricc_set_error("get_element: index %lld out of range", (long long)mi);
    return FRICC_ERR_ARG;
  }
  const int rc = settle(T);
  if (rc) return rc;
  int s[4];
  double v = 0.0;
  cudaError_t e = cudaStreamSynchronize(T->owner_stream);
  if (e == cudaSuccess) e = cudaMemcpy(s, T->slots + 4 * mi, sizeof(s), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&v, T->vals + mi, sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fricc_cuda_fail(e, "get_element", __FILE__, __LINE__);
  if (idx)
    for (int k = 0; k < 4; ++k) idx[k] = s[k];
  if (value) *value = v;
  return FRICC_OK;
}

int fricc_sp_export(const fricc_sparse* T, int64_t* flat_host, double* vals_host, void* stream) {
  if (!T) {
    fricc_set_error("sp_export: null handle");
    return FRICC_ERR_ARG;
  }
  const int rc = settle(T);  // also orders the copies after the compression
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
  if (flat_host) FRICC_CUDA(cudaMemcpyAsync(flat_host, T->flat, T->m * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  if (vals_host) FRICC_CUDA(cudaMemcpyAsync(vals_host, T->vals, T->m * sizeof(double), cudaMemcpyDeviceToHost, st));
  FRICC_CUDA(cudaStreamSynchronize(st));
  return FRICC_OK;
}

int fricc_sp_device_arrays(const fricc_sparse* T, const int64_t** flat, const double** vals, const int** slots) {
  if (!T) {
    fricc_set_error("sp_device_arrays: null handle");
    return FRICC_ERR_ARG;
  }
  if (flat) *flat = T->flat;
  if (vals) *vals = T->vals;
  if (slots) *slots = T->slots;
  return FRICC_OK;
}

int fricc_contract(const char* term, const double* W, const int64_t W_dims[4], const int64_t W_strides[4],
                   fricc_sparse* T, double* out, const int64_t out_dims[4], const int64_t out_strides[4],
                   void* stream) {
  if (!W_dims || !W_strides || !out_dims || !out_strides) {
    fricc_set_error("contract: null shape argument");
    return FRICC_ERR_ARG;
  }
  for (int k = 0; k < 4; ++k)
    if (W_strides[k] < 0 || out_strides[k] < 0 || W_dims[k] < 0 || out_dims[k] < 0) {
      fricc_set_error("contract: negative dims or strides are not supported");
      return FRICC_ERR_ARG;
    }
  cudaStream_t st = as_stream(stream);
  int rc = fricc_contract_device(term, W, W_dims, W_strides, T, out, out_dims, out_strides, st);
  if (!rc && T) T->owner_stream = st;
  return rc;
}

// the failing item's index in front of its own message
static int batch_item_error(const char* what, int64_t r, int rc) {
  char msg[sizeof(g_err)];
  snprintf(msg, sizeof(msg), "%s", g_err);
  fricc_set_error("%s item %lld: %s", what, (long long)r, msg);
  return rc;
}

int fricc_contract_batch(const char* term, int64_t count, const double* const* W, const int64_t* W_dims,
                         const int64_t* W_strides, fricc_sparse* const* T, double* const* out,
                         const int64_t* out_dims, const int64_t* out_strides, void* stream) {
  if (count < 0 || (count > 0 && (!W || !W_dims || !W_strides || !T || !out || !out_dims || !out_strides))) {
    fricc_set_error("contract_batch: negative count or null array");
    return FRICC_ERR_ARG;
  }
  for (int64_t r = 0; r < count; ++r) {
    const int rc = fricc_contract(term, W[r], W_dims + 4 * r, W_strides + 4 * r, T[r], out[r], out_dims + 4 * r,
                                  out_strides + 4 * r, stream);
    if (rc) return batch_item_error("contract_batch", r, rc);
  }
  return FRICC_OK;
}

int fricc_sp_recompress_batch(int64_t count, fricc_sparse* const* T, const double* const* t2, int compression,
                              int sampling, const double* rn, void* stream) {
  if (count < 0 || (count > 0 && (!T || !t2 || !rn))) {
    fricc_set_error("sp_recompress_batch: negative count or null array");
    return FRICC_ERR_ARG;
  }
  for (int64_t r = 0; r < count; ++r) {
    const int rc = fricc_sp_recompress(T[r], t2[r], compression, sampling, rn[r], stream);
    if (rc) return batch_item_error("sp_recompress_batch", r, rc);
  }
  return FRICC_OK;
}

int fricc_spmm(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, const double* Wp, int64_t QS,
               double* Op, void* stream) {
  cudaStream_t st = as_stream(stream);
  int rc = fricc_spmm_device(T, pa, pb, ka, kb, coef, Wp, QS, Op, st);
  if (!rc && T) T->owner_stream = st;
  return rc;
}

int fricc_spmm_f2(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, const float* Wp4, int64_t QS,
                  double* Op, void* stream) {
  cudaStream_t st = as_stream(stream);
  int rc = fricc_spmm_f2_device(T, pa, pb, ka, kb, coef, reinterpret_cast<const float4*>(Wp4), QS, Op, st);
  if (!rc && T) T->owner_stream = st;
  return rc;
}

int fricc_spmm_f1(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, const float* W, int64_t QS,
                  int64_t ldw, double* Op, void* stream) {
  cudaStream_t st = as_stream(stream);
  int rc = fricc_spmm_f1_device(T, pa, pb, ka, kb, coef, W, QS, ldw, Op, st, false);
  if (!rc && T) T->owner_stream = st;
  return rc;
}

int fricc_densify_bf16x3(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, void* Ap, int64_t kp,
                         void* stream) {
  cudaStream_t st = as_stream(stream);
  int rc = fricc_densify_bf16x3_device(T, pa, pb, ka, kb, coef, Ap, kp, st);
  if (!rc && T) T->owner_stream = st;
  return rc;
}

int fricc_spmm_f32(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, const float* W, int64_t QS,
                   int64_t ldw, double* Op, void* stream) {
  cudaStream_t st = as_stream(stream);
  int rc = fricc_spmm_f1_device(T, pa, pb, ka, kb, coef, W, QS, ldw, Op, st, true);
  if (!rc && T) T->owner_stream = st;
  return rc;
}

int fricc_split_f2(const double* x, int64_t rows, int64_t qs, float* out4, void* stream) {
  return fricc_split_f2_device(x, rows, qs, reinterpret_cast<float4*>(out4), as_stream(stream));
}

int fricc_gemm_df(const double* A, const double* B, double* C, int64_t batch, int64_t M, int64_t N, int64_t K,
                  const int64_t sA[3], const int64_t sB[3], const int64_t sC[3], double alpha, double beta,
                  void* stream) {
  if (!sA || !sB || !sC) {
    fricc_set_error("gemm_df: null stride array");
    return FRICC_ERR_ARG;
  }
  return fricc_gemm_df_device(A, B, C, batch, M, N, K, sA, sB, sC, alpha, beta, as_stream(stream), 1, nullptr);
}

int fricc_gemm_f64(const double* A, const double* B, double* C, int64_t batch, int64_t M, int64_t N, int64_t K,
                  const int64_t sA[3], const int64_t sB[3], const int64_t sC[3], double alpha, double beta,
                  void* stream) {
  if (!sA || !sB || !sC) {
    fricc_set_error("gemm_f64: null stride array");
    return FRICC_ERR_ARG;
  }
  return fricc_gemm_f64_device(A, B, C, batch, M, N, K, sA, sB, sC, alpha, beta, as_stream(stream), 1, nullptr);
}

int fricc_combine(const int64_t dims[4], int n_in, const double* const* x, const int64_t* sx, int n_prod,
                  const double* const* p, const int64_t* sp, int n_out, double* const* out, const int64_t* so,
                  const double* coef, int accumulate, void* stream) {
  return fricc_combine4_device(dims, n_in, x, sx, n_prod, p, sp, n_out, out, so, coef, accumulate, as_stream(stream));
}

int fricc_gemm_f64_b2(const double* A, const double* B, double* C, int64_t batch, int64_t batch2, int64_t M,
                      int64_t N, int64_t K, const int64_t sA[4], const int64_t sB[4], const int64_t sC[4], double alpha,
                      double beta, void* stream) {
  if (!sA || !sB || !sC) {
    fricc_set_error("gemm_f64_b2: null stride array");
    return FRICC_ERR_ARG;
  }
  const int64_t s2[3] = {sA[3], sB[3], sC[3]};
  return fricc_gemm_f64_device(A, B, C, batch, M, N, K, sA, sB, sC, alpha, beta, as_stream(stream), batch2, s2);
}

int fricc_gemm_df_b2(const double* A, const double* B, double* C, int64_t batch, int64_t batch2, int64_t M, int64_t N,
                     int64_t K, const int64_t sA[4], const int64_t sB[4], const int64_t sC[4], double alpha,
                     double beta, void* stream) {
  if (!sA || !sB || !sC) {
    fricc_set_error("gemm_df_b2: null stride array");
    return FRICC_ERR_ARG;
  }
  const int64_t s2[3] = {sA[3], sB[3], sC[3]};
  return fricc_gemm_df_device(A, B, C, batch, M, N, K, sA, sB, sC, alpha, beta, as_stream(stream), batch2, s2);
}

int fricc_combine5(const int64_t dims[5], int n_in, const double* const* x, const int64_t* sx, int n_prod,
                   const double* const* p, const int64_t* sp, int n_out, double* const* out, const int64_t* so,
                   const double* coef, int accumulate, void* stream) {
  return fricc_combine_device(dims, n_in, x, sx, n_prod, p, sp, n_out, out, so, coef, accumulate, as_stream(stream));
}

int fricc_spb_create(int R, const int64_t dims[4], int64_t m, void* stream, fricc_spbatch** out) {
  if (!out || R < 1 || R > 65535 || bad_dims(dims) || m <= 0) {
    fricc_set_error("spb_create: bad arguments");
    return FRICC_ERR_ARG;
  }
  *out = nullptr;
  const int64_t n = dims[0] * dims[1] * dims[2] * dims[3];
  if (m > n || n >= 0xffffffffLL) {
    fricc_set_error("Bad m_keep value: need 0 < m <= tensor size < 2^32 (m=%lld, size=%lld)", (long long)m,
                    (long long)n);
    return FRICC_ERR_ARG;
  }
  cudaStream_t st = as_stream(stream);
  auto* B = new FriccSparseBatch();
  B->R = R;
  for (int k = 0; k < 4; ++k) B->dims[k] = dims[k];
  B->m = m;
  B->owner_stream = st;
  cudaGetDevice(&B->device);
  int rc = FRICC_OK;
  for (int w = 0; w < 2 && !rc; ++w) {
    rc = fricc_alloc_t(&B->flat[w], (size_t)R * m, st);
    if (!rc) rc = fricc_alloc_t(&B->vals[w], (size_t)R * m, st);
    if (!rc) rc = fricc_alloc_t(&B->slots[w], (size_t)R * m * 4, st);
    if (!rc) rc = fricc_alloc_t(&B->meta[w], (size_t)R * 2, st);
    if (!rc) rc = fricc_cuda_check(cudaMemsetAsync(B->meta[w], 0, (size_t)R * 2 * sizeof(unsigned long long), st),
                                   "memset");
  }
  if (rc) {
    fricc_spb_destroy(B);
    return rc;
  }
  *out = B;
  return FRICC_OK;
}

int fricc_spb_destroy(fricc_spbatch* B) {
  if (!B) return FRICC_OK;
  cudaStream_t st = B->owner_stream;
  for (int w = 0; w < 2; ++w) {
    fricc_free(B->flat[w], st);
    fricc_free(B->vals[w], st);
    fricc_free(B->slots[w], st);
    fricc_free(B->meta[w], st);
    for (auto& b : B->buck[w]) {
      fricc_free(b.bptr, st);
      fricc_free(b.order, st);
    }
  }
  cudaStreamSynchronize(st);
  delete B;
  return FRICC_OK;
}

int fricc_spb_recompress_pair(fricc_spbatch* B, const double* t2, const double* rn_dev, void* stream) {
  if (!B || !t2 || !rn_dev) {
    fricc_set_error("spb_recompress_pair: null argument");
    return FRICC_ERR_ARG;
  }
  cudaStream_t st = as_stream(stream);
  const int64_t n = B->dims[0] * B->dims[1] * B->dims[2] * B->dims[3];
  // the status words start clean: each compression ORs its error bits in
  int rc = fricc_cuda_check(cudaMemsetAsync(B->meta[0], 0, (size_t)B->R * 2 * sizeof(unsigned long long), st), "meta");
  if (!rc) rc = fricc_cuda_check(cudaMemsetAsync(B->meta[1], 0, (size_t)B->R * 2 * sizeof(unsigned long long), st),
                                 "meta");
  if (!rc) rc = fricc_compress_pair_batch_device(t2, n, B->m, B->R, rn_dev, B->flat[0], B->vals[0], B->meta[0],
                                                 B->flat[1], B->vals[1], B->meta[1], st);
  for (int w = 0; w < 2 && !rc; ++w)
    rc = fricc_unpack_batch_async(B->flat[w], B->m, B->R, B->dims, B->slots[w], B->meta[w], st);
  for (auto& bw : B->buck)
    for (auto& b : bw) b.valid = false;
  if (!rc) B->compressed = true;
  return rc;
}

int fricc_spb_status(fricc_spbatch* B, int* replica) {
  if (!B) {
    fricc_set_error("spb_status: null batch");
    return FRICC_ERR_ARG;
  }
  if (replica) *replica = -1;
  std::vector<unsigned long long> h((size_t)B->R * 4);
  FRICC_CUDA(cudaMemcpyAsync(h.data(), B->meta[0], (size_t)B->R * 2 * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, B->owner_stream));
  FRICC_CUDA(cudaMemcpyAsync(h.data() + 2 * B->R, B->meta[1], (size_t)B->R * 2 * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, B->owner_stream));
  FRICC_CUDA(cudaStreamSynchronize(B->owner_stream));
  for (int k = 0; k < 2 * B->R; ++k) {
    const unsigned e = (unsigned)h[2 * (size_t)k + 1];
    if (e) {
      if (replica) *replica = k % B->R;
      return fricc_dev_status(e);
    }
  }
  return FRICC_OK;
}

int fricc_spb_export(fricc_spbatch* B, int which, int r, int64_t* flat_host, double* vals_host, void* stream) {
  if (!B || which < 0 || which > 1 || r < 0 || r >= B->R || !B->compressed) {
    fricc_set_error("spb_export: bad arguments (or nothing compressed yet)");
    return FRICC_ERR_ARG;
  }
  cudaStream_t st = as_stream(stream);
  const size_t off = (size_t)r * B->m;
  if (flat_host)
    FRICC_CUDA(cudaMemcpyAsync(flat_host, B->flat[which] + off, B->m * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  if (vals_host)
    FRICC_CUDA(cudaMemcpyAsync(vals_host, B->vals[which] + off, B->m * sizeof(double), cudaMemcpyDeviceToHost, st));
  FRICC_CUDA(cudaStreamSynchronize(st));
  return FRICC_OK;
}

int fricc_spb_spmm(fricc_spbatch* B, int which, int pa, int pb, int ka, int kb, double coef, const double* Wp,
                   int64_t w_stride, int64_t QS, double* Op, int64_t o_stride, void* stream) {
  return fricc_batch_spmm_device(B, which, pa, pb, ka, kb, coef, Wp, w_stride, QS, Op, o_stride, false,
                                 as_stream(stream));
}

int fricc_spb_spmm_f2(fricc_spbatch* B, int which, int pa, int pb, int ka, int kb, double coef, const void* W2,
                      int64_t w2_stride, int64_t QS, double* Op, int64_t o_stride, void* stream) {
  return fricc_batch_spmm_device(B, which, pa, pb, ka, kb, coef, W2, w2_stride, QS, Op, o_stride, true,
                                 as_stream(stream));
}

int fricc_spb_densify_bf16x3(fricc_spbatch* B, int which, int pa, int pb, int ka, int kb, double coef, void* Ap,
                             int64_t kp, void* stream) {
  return fricc_batch_densify_device(B, which, pa, pb, ka, kb, coef, Ap, kp, as_stream(stream));
}

int fricc_energy_update_batch(int R, const double* t1num, const double* t2num, const double* eia, const double* fov,
                              const double* ovov, const double* t1old, const double* t2old, int64_t o, int64_t v,
                              double* t1out, double* t2out, double* res, void* stream) {
  if (!t1num || !t2num || !eia || !fov || !ovov || !t1old || !t2old || !t1out || !t2out || !res) {
    fricc_set_error("energy_update_batch: null argument");
    return FRICC_ERR_ARG;
  }
  return fricc_energy_update_batch_device(R, t1num, t2num, eia, fov, ovov, t1old, t2old, o, v, t1out, t2out, res,
                                          as_stream(stream));
}

int fricc_zero(void* p, int64_t bytes, void* stream) {
  if (bytes < 0 || (!p && bytes > 0)) {
    fricc_set_error("zero: bad arguments");
    return FRICC_ERR_ARG;
  }
  if (bytes == 0) return FRICC_OK;
  FRICC_CUDA(cudaMemsetAsync(p, 0, (size_t)bytes, as_stream(stream)));
  return FRICC_OK;
}

double fricc_contract_flops(const char* term, const fricc_sparse* T) {
  return fricc_contract_flops_impl(term, T);
}

int fricc_compress(const double* x, int64_t n, int64_t m, int compression, double rn, int64_t* flat, double* vals,
                   int64_t* n_largest, void* stream) {
  if (!x || !flat || !vals) {
    fricc_set_error("compress: null argument");
    return FRICC_ERR_ARG;
  }
  if (compression != FRICC_COMPRESSION_FRI && compression != FRICC_COMPRESSION_LARGEST) {
    fricc_set_error("compress: compression must be 'largest' or 'fri'");
    return FRICC_ERR_ARG;
  }
  return fricc_compress_device(x, n, m, compression == FRICC_COMPRESSION_LARGEST ? 1 : 0, rn, as_stream(stream), flat,
                               vals, n_largest, nullptr, nullptr);
}

int fricc_compress_pivotal(const double* x, int64_t n, int64_t m, uint32_t* glibc_hist, int64_t* flat, double* vals,
                           int64_t* n_largest, int64_t* n_draws, void* stream) {
  if (!x || !flat || !vals) {
    fricc_set_error("compress_pivotal: null argument");
    return FRICC_ERR_ARG;
  }
  return fricc_compress_device(x, n, m, 2, 0.0, as_stream(stream), flat, vals, n_largest, glibc_hist, n_draws);
}

int fricc_stream_create(void** out) {
  if (!out) {
    fricc_set_error("stream_create: null argument");
    return FRICC_ERR_ARG;
  }
  cudaStream_t s = nullptr;
  FRICC_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *out = (void*)s;
  return FRICC_OK;
}

int fricc_stream_destroy(void* stream) {
  if (stream) FRICC_CUDA(cudaStreamDestroy(as_stream(stream)));
  return FRICC_OK;
}

int fricc_parallel_sample(const double* q, int64_t n, int64_t n_sample, int chunks, uint32_t* glibc_hist,
                          int64_t* S, int64_t* n_draws, void* stream) {
  return fricc_parallel_sample_device(q, n, n_sample, chunks, glibc_hist, S, n_draws, as_stream(stream));
}

int fricc_glibc_uniforms(uint32_t* hist, int64_t k, double* out, void* stream) {
  return fricc_glibc_uniforms_device(hist, k, out, as_stream(stream));
}

static int energy_update(const double* t1num, const double* t2num, const double* eia, const double* fov,
                         const double* ovov, const double* t1old, const double* t2old, int64_t nocc, int64_t nvir,
                         double* t1out, double* t2out, double* res, void* stream, bool linear) {
  if (!t1num || !t2num || !eia || !fov || !ovov || !t1old || !t2old || !t1out || !t2out || !res) {
    fricc_set_error("energy_update: null argument");
    return FRICC_ERR_ARG;
  }
  return fricc_energy_update_device(t1num, t2num, eia, fov, ovov, t1old, t2old, nocc, nvir, t1out, t2out, res,
                                    as_stream(stream), linear);
}

int fricc_energy_update(const double* t1num, const double* t2num, const double* eia, const double* fov,
                        const double* ovov, const double* t1old, const double* t2old, int64_t nocc, int64_t nvir,
                        double* t1out, double* t2out, double* res, void* stream) {
  return energy_update(t1num, t2num, eia, fov, ovov, t1old, t2old, nocc, nvir, t1out, t2out, res, stream, false);
}

int fricc_energy_update_lin(const double* t1num, const double* t2num, const double* eia, const double* fov,
                            const double* ovov, const double* t1old, const double* t2old, int64_t nocc, int64_t nvir,
                            double* t1out, double* t2out, double* res, void* stream) {
  return energy_update(t1num, t2num, eia, fov, ovov, t1old, t2old, nocc, nvir, t1out, t2out, res, stream, true);
}

int fricc_seq_cumsum(const double* x, int64_t n, double* out, void* stream) {
  return fricc_seq_cumsum_device(x, n, out, as_stream(stream));
}

}  // extern "C"
