/*
 * fricc_gb300.h -- C ABI of the GB300 (sm_103a) FRI-CCSD hot path.
 *
 * Plain pointers and sizes only.  Every function returns an int status:
 * FRICC_OK (0) or one of the FRICC_ERR_* codes, with a message available
 * from fricc_last_error() (thread-local).  The reference terminates the
 * process instead (exit(EXIT_FAILURE)); these entry points never do.
 *
 * Device pointers are CUDA global-memory addresses on the current device.
 * `stream` is a cudaStream_t (NULL = the legacy default stream).  Functions
 * are stream-ordered unless stated; those that return host values
 * synchronise the stream they are given.  Strides are in ELEMENTS.
 *
 * Reference interfaces replaced (fri-cc, by file:line):
 *   fricc_sp_create        SparseTensor4d(tensor_arr, dims, m, compression,
 *                          sampling_method, verbose)  include/sparse_tensor.hpp:33-77,
 *                          binding src/py_rccsd.cpp:34-39
 *   fricc_sp_create_empty  SparseTensor4d(dims, nnz)  include/sparse_tensor.hpp:27-31,
 *                          binding src/py_rccsd.cpp:33
 *   fricc_sp_get           SparseTensor4d::get_element  include/sparse_tensor.hpp:138-143,
 *                          binding src/py_rccsd.cpp:40-46
 *   fricc_sp_export        (bulk get_element; the reference has none)
 *   fricc_contract         contract_SparseTensor4d_wrapper  src/sparse_tensor.cpp:349-382,
 *                          binding "contract_DTSpT" src/py_rccsd.cpp:50-51
 *   fricc_compress         fri_compression  src/fri_utils.cpp:439-522 (systematic) and
 *                          argsort-based "largest" include/sparse_tensor.hpp:46-56
 *   fricc_seq_cumsum       the running sums of one_norm src/fri_utils.cpp:164-171 and of
 *                          std::partial_sum in sample_systematic :142-143
 *   fricc_energy_update    the denominator update of update_amps fricc/friccsd.py:281-284,
 *                          the CCSD energy and the step norm of kernel :418-427
 */
#ifndef FRICC_GB300_H
#define FRICC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FRICC_OK 0
#define FRICC_ERR_ARG 1          /* bad argument (sizes, m, dims, null) */
#define FRICC_ERR_TERM 2         /* unknown contraction term */
#define FRICC_ERR_P_GT_ONE 3     /* a sampling probability exceeded 1 */
#define FRICC_ERR_CUDA 4         /* a CUDA runtime call failed */
#define FRICC_ERR_TIMEOUT 5      /* a bounded device-side wait gave up */
#define FRICC_ERR_INDEX 6        /* an index fell outside dims */
#define FRICC_ERR_UNSUPPORTED 7  /* mode not implemented on this path */
#define FRICC_ERR_PIVOTAL 8      /* pivotal sampling failed as the reference's does (acceptance outside
                                    [0,1], leftover weight, wrong sample count) */

#define FRICC_COMPRESSION_FRI 0
#define FRICC_COMPRESSION_LARGEST 1
#define FRICC_SAMPLING_SYSTEMATIC 0
#define FRICC_SAMPLING_PIVOTAL 1

typedef struct FriccSparse fricc_sparse; /* opaque device-resident SparseTensor4d */
typedef struct FriccSparseBatch fricc_spbatch; /* opaque: R compressed tensors of one shape, two per replica */

/* Library version (major*10000 + minor*100 + patch). */
int fricc_version(void);

/* Message of the last failing call on this thread ("" if none). */
const char* fricc_last_error(void);

/* Compress the dense C-order tensor t2 (device, dims[0]*dims[1]*dims[2]*dims[3]
 * doubles) keeping m nonzeros.  compression: FRICC_COMPRESSION_FRI (sampling
 * must be FRICC_SAMPLING_SYSTEMATIC; rn is the one uniform draw
 * rand()/RAND_MAX the reference consumes) or FRICC_COMPRESSION_LARGEST (rn
 * unused).  Entries come out in the reference's slot order: the exactly kept
 * largest entries in descending |t| (ties by ascending flat index), then the
 * sampled ones in ascending flat index.  Stream-ordered and asynchronous:
 * the call returns once the work is enqueued on `stream`; |D| and the
 * compression's own failures (a probability above 1) are read back by the
 * next blocking call on the handle (fricc_sp_status, fricc_sp_info,
 * fricc_sp_get, fricc_sp_export), which then returns the error. */
int fricc_sp_create(const double* t2, const int64_t dims[4], int64_t m, int compression, int sampling, double rn,
                    void* stream, fricc_sparse** out);

/* Re-compress into an existing handle (same dims and m), reusing its memory;
 * asynchronous like fricc_sp_create. */
int fricc_sp_recompress(fricc_sparse* T, const double* t2, int compression, int sampling, double rn, void* stream);

/* fricc_sp_recompress with the uniform draw read from device memory
 * (rn_dev, one double; unused for "largest"), so that the whole call is
 * stream-ordered device work: with the handle created (and its bucketings
 * built) beforehand, it allocates only scratch that it frees again, and can
 * be captured into a CUDA graph.  Systematic or "largest" only. */
int fricc_sp_recompress_dev(fricc_sparse* T, const double* t2, int compression, int sampling, const double* rn_dev,
                            void* stream);

/* The two compressions one iteration makes of the same T2 (fricc/friccsd.py:
 * 100-117: the T2-term and W-intermediate compressions, draws rn_a then
 * rn_b), into handles A and B at once: the norm, the top-m select, the
 * largest-set walk and the probabilities run once and one partial-sum chain
 * serves both samplers.  Each handle ends bit-identical to
 * fricc_sp_recompress(A, t2, FRI, SYSTEMATIC, rn_a) and (B, ..., rn_b).
 * Systematic FRI only; A and B distinct, with t2's dims and equal m.  The
 * _dev form reads the two draws from device memory (rn_dev[0], rn_dev[1]). */
int fricc_sp_recompress_pair(fricc_sparse* A, fricc_sparse* B, const double* t2, double rn_a, double rn_b,
                             void* stream);
int fricc_sp_recompress_pair_dev(fricc_sparse* A, fricc_sparse* B, const double* t2, const double* rn_dev,
                                 void* stream);

/* Wait for the handle's last compression and return its status (FRICC_OK,
 * FRICC_ERR_P_GT_ONE, FRICC_ERR_TIMEOUT, FRICC_ERR_INDEX).  No reference
 * counterpart: the reference exits inside the constructor. */
int fricc_sp_status(const fricc_sparse* T);

/* "fri" compression with pivotal sampling (src/fri_utils.cpp:63-127, the
 * binding's default sampling_method), which draws one uniform
 * rand()/RAND_MAX per element it visits.  glibc_hist: the state of the
 * glibc rand() stream to draw from, as its 31-word history (the words
 * r[k-31..k-1] of the recurrence r[k] = r[k-31] + r[k-3] mod 2^32, oldest
 * first; host memory), advanced past the draws on return; NULL draws from
 * this process's own rand(), exactly as the reference does.  *n_draws
 * (optional) receives the number of draws consumed.  S keeps the order the
 * sampler emits it.  Synchronises `stream`.  Failures of the reference's
 * sampler (its exits) return FRICC_ERR_PIVOTAL. */
int fricc_sp_create_pivotal(const double* t2, const int64_t dims[4], int64_t m, uint32_t* glibc_hist, void* stream,
                            fricc_sparse** out, int64_t* n_draws);
int fricc_sp_recompress_pivotal(fricc_sparse* T, const double* t2, uint32_t* glibc_hist, void* stream,
                                int64_t* n_draws);

/* An all-zero tensor of nnz entries (index 0, value 0). */
int fricc_sp_create_empty(const int64_t dims[4], int64_t nnz, void* stream, fricc_sparse** out);

int fricc_sp_destroy(fricc_sparse* T);

/* dims, number of entries, and |D| (entries kept exactly, FRI only). */
int fricc_sp_info(const fricc_sparse* T, int64_t dims[4], int64_t* m, int64_t* n_largest);

/* Entry mi: unpacked index and value (synchronous device-to-host read). */
int fricc_sp_get(const fricc_sparse* T, int64_t mi, int64_t idx[4], double* value);

/* All entries to host memory: flat C-order index and value (either may be NULL). */
int fricc_sp_export(const fricc_sparse* T, int64_t* flat_host, double* vals_host, void* stream);

/* Device arrays of the handle: flat[m] (int64), vals[m] (double), slots[m][4] (int32). */
int fricc_sp_device_arrays(const fricc_sparse* T, const int64_t** flat, const double** vals, const int** slots);

/* out (device, any strides) += the term's contraction of W (device, any
 * strides) with T.  term is one of "0101", "2323", "1302", "1202", "1303",
 * "1203", "1323", "0112", "0113", "0313", "0312".  Each term reads
 * W'[key0,key1,q0,q1] and out'[p0,p1,q0,q1], where (p0,p1) are the two
 * index slots the reference's outer loop fixes, (key0,key1) the slots that
 * index W and (q0,q1) the inner dense loop; e.g. "2323" reads W as (c,d,a,b)
 * and out as (i,j,a,b).  A W or out whose strides already give that
 * contiguous layout is used in place; any other layout is gathered into a
 * permuted copy (and out scattered back).  Stream-ordered. */
int fricc_contract(const char* term, const double* W, const int64_t W_dims[4], const int64_t W_strides[4],
                   fricc_sparse* T, double* out, const int64_t out_dims[4], const int64_t out_strides[4],
                   void* stream);

/* Batched forms for R independent replicas or solves (no reference
 * counterpart: the reference runs one solve per process).  Item r is exactly
 * fricc_contract(term, W[r], W_dims + 4r, W_strides + 4r, T[r], out[r],
 * out_dims + 4r, out_strides + 4r, stream), respectively
 * fricc_sp_recompress(T[r], t2[r], compression, sampling, rn[r], stream),
 * issued in order on `stream`; the first failing item stops the batch and its
 * index leads the message.  count = 0 does nothing. */
int fricc_contract_batch(const char* term, int64_t count, const double* const* W, const int64_t* W_dims,
                         const int64_t* W_strides, fricc_sparse* const* T, double* const* out,
                         const int64_t* out_dims, const int64_t* out_strides, void* stream);
int fricc_sp_recompress_batch(int64_t count, fricc_sparse* const* T, const double* const* t2, int compression,
                              int sampling, const double* rn, void* stream);

/* The kernel behind every term, in general form (no reference counterpart;
 * each contract_DTSpT term is one instance of it):
 *   Op[P][q] += coef * sum over nonzeros e with P_e == P of Wp[key_e][q] * value_e
 * for q < QS, where P_e = slot[pa]*dims[pb] + slot[pb] and
 * key_e = slot[ka]*dims[kb] + slot[kb] (slots 0..3 = the tensor's four
 * indices).  Wp is contiguous [dims[ka]*dims[kb]][QS], Op contiguous
 * [dims[pa]*dims[pb]][QS].  Each Op element receives its contributions in
 * nonzero-slot order.  Stream-ordered. */
int fricc_spmm(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, const double* Wp, int64_t QS,
               double* Op, void* stream);

/* fricc_spmm in FP32-pair arithmetic (no reference counterpart): Wp4 is W'
 * split by fricc_split_f2 into its q-pair layout (16-byte aligned); every
 * product and sum carries ~48 significand bits (relative error per output
 * ~1e-14) and runs on the FP32 pipe, two outputs per packed instruction.
 * Op stays FP64. */
int fricc_spmm_f2(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, const float* Wp4, int64_t QS,
                  double* Op, void* stream);

/* x [rows][qs] (FP64, contiguous) split into float pairs, hi the top 24
 * significand bits of x and lo the rest rounded to 24 bits
 * (|x - hi - lo| < 2^-47 |x|; outside 2^-74 <= |x| < 2^128, hi = (float)x,
 * lo = (float)(x - hi)), in the q-pair
 * layout fricc_spmm_f2 reads: for row r and pair t < ceil(qs/2), the four
 * floats out4[4(r ceil(qs/2) + t) ..] = hi[r][2t], hi[r][2t+1], lo[r][2t],
 * lo[r][2t+1] (an odd qs padded with zero).  out4 holds
 * 4 rows ceil(qs/2) floats, 16-byte aligned.  Stream-ordered. */
int fricc_split_f2(const double* x, int64_t rows, int64_t qs, float* out4, void* stream);

/* fricc_spmm against an FP32 W (rows of ldw floats, ldw even, 8-byte
 * aligned base): the O^2V^4 term of the split-precision form, whose (vv|vv)
 * block is rebuilt in FP32 by fricc_vvvv_rebuild_bf16x3.  T's values enter
 * as float pairs and the sums are float-pair sums, as in fricc_spmm_f2. */
int fricc_spmm_f1(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, const float* W, int64_t QS,
                  int64_t ldw, double* Op, void* stream);

/* fricc_spmm_f1 in plain FP32: T values rounded to FP32, one FP32 sum per
 * output added to the FP64 output at the end (~2^-24 per product, the sum's
 * rounding on top).  For the split-precision form only, whose integrals
 * carry ~2^-16 relative error from the BF16x3 rebuild. */
int fricc_spmm_f32(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, const float* W, int64_t QS,
                   int64_t ldw, double* Op, void* stream);

/* The compressed T as a dense [dims[pa]*dims[pb]][R] matrix (R =
 * dims[ka]*dims[kb]; row P = (pa,pb) pair, column r = (ka,kb) pair) of
 * coef * value, split into BF16 hi + lo and written as the tensor-core A
 * operand [hi | hi | lo] (rows of kp >= 3R elements; everything else zero):
 * the split-precision form contracts it with fricc_gemm_bf16_tn_strided
 * against the split W^T.  Stream-ordered. */
int fricc_densify_bf16x3(fricc_sparse* T, int pa, int pb, int ka, int kb, double coef, void* Ap, int64_t kp,
                         void* stream);

/* Strided batched GEMM, FP64 in and out, products and sums in FP32 pairs
 * (no reference counterpart; it runs the dense O^2V^3 contractions of the
 * iteration):  C[b] = alpha * A[b] @ B[b] + beta * C[b], b < batch.
 * sA = {row, col, batch} element strides of the M x K matrix A, likewise sB
 * for K x N and sC for M x N.  Deterministic (a long K is split and the
 * partials summed in a fixed order).  Stream-ordered. */
int fricc_gemm_df(const double* A, const double* B, double* C, int64_t batch, int64_t M, int64_t N, int64_t K,
                  const int64_t sA[3], const int64_t sB[3], const int64_t sC[3], double alpha, double beta,
                  void* stream);

/* The same contract in FP64 arithmetic on the FP64 FMA pipe: the dense
 * O^2V^3 / O^3V^2 contractions of the FP64 iteration, which the reference
 * leaves to PySCF's einsums (fricc/friccsd.py:144-192,211,238-241 through
 * pyscf.cc.rintermediates).  Each output is one FMA chain in k order (a
 * long K with few output tiles is split and the partials summed in slice
 * order), so results are deterministic.  Stream-ordered. */
int fricc_gemm_f64(const double* A, const double* B, double* C, int64_t batch, int64_t M, int64_t N, int64_t K,
                   const int64_t sA[3], const int64_t sB[3], const int64_t sC[3], double alpha, double beta,
                   void* stream);

/* Strided elementwise combination over a 4-D index space, one pass (no
 * reference counterpart; it runs the permuted copies, linear combinations,
 * broadcast products and diagonal updates that fricc/friccsd.py:144-301 and
 * :309-376 write as NumPy expressions).  For every i < dims (i3 fastest):
 *   r_k(i) = sum_{t<n_in} coef[k*nc+t] x_t(i)
 *            + coef[k*nc+n_in] * p_0(i) * ... * p_{n_prod-1}(i)   (if n_prod > 0)
 *   out_k(i) = r_k(i), or out_k(i) + r_k(i) when accumulate != 0,
 * nc = n_in + (n_prod > 0), each operand addressed through its own four
 * element strides (sx[4t..4t+3], sp[4s..], so[4k..]; 0 broadcasts).  Terms
 * are summed in the order given, a zero coefficient drops its term.  Up to
 * FRICC_COMBINE_MAX_IN inputs, FRICC_COMBINE_MAX_PROD product factors and
 * FRICC_COMBINE_MAX_OUT outputs; outputs must not overlap the inputs.
 * Stream-ordered. */
#define FRICC_COMBINE_MAX_IN 5
#define FRICC_COMBINE_MAX_PROD 3
#define FRICC_COMBINE_MAX_OUT 3
int fricc_combine(const int64_t dims[4], int n_in, const double* const* x, const int64_t* sx, int n_prod,
                  const double* const* p, const int64_t* sp, int n_out, double* const* out, const int64_t* so,
                  const double* coef, int accumulate, void* stream);

/* Phase timing of the calling thread's compressions (the reference's
 * verbose table of fri_compression, src/fri_utils.cpp:509-519, and of the
 * SparseTensor4d constructor's verbose flag, include/sparse_tensor.hpp:33-77):
 * fricc_phase_timing_set(1) records CUDA events at the phase boundaries of
 * every later compression on this thread (0 stops);
 * fricc_phase_timing_read waits for the last one and writes the seconds of
 * its phases: sec[0] "Sorting" (the largest elements and the remaining
 * norm), sec[1] "P vector", sec[2] "Sampling", sec[3] "Wrap up" (the
 * outputs), sec[4] "Total". */
int fricc_phase_timing_set(int on);
int fricc_phase_timing_read(double sec[5]);

/* ---- Replica batches (no reference counterpart: the reference runs one
 * FRI replica per process; fricc/__init__.py:8-11 aggregates replicas'
 * energies afterwards).  R independent replicas of one system, each kernel
 * launched once for all R: the replica is one more grid dimension.  Each
 * replica's results are bit for bit those of its own single calls. ---- */

/* The batched GEMMs: batch2 groups of `batch` products; element strides
 * s*[0..2] as in fricc_gemm_f64 / fricc_gemm_df, s*[3] between groups
 * (0 = shared by all groups). */
int fricc_gemm_f64_b2(const double* A, const double* B, double* C, int64_t batch, int64_t batch2, int64_t M,
                      int64_t N, int64_t K, const int64_t sA[4], const int64_t sB[4], const int64_t sC[4], double alpha,
                      double beta, void* stream);
int fricc_gemm_df_b2(const double* A, const double* B, double* C, int64_t batch, int64_t batch2, int64_t M, int64_t N,
                     int64_t K, const int64_t sA[4], const int64_t sB[4], const int64_t sC[4], double alpha,
                     double beta, void* stream);

/* fricc_combine over a 5-D index space (five strides per operand). */
int fricc_combine5(const int64_t dims[5], int n_in, const double* const* x, const int64_t* sx, int n_prod,
                   const double* const* p, const int64_t* sp, int n_out, double* const* out, const int64_t* so,
                   const double* coef, int accumulate, void* stream);

/* A batch of R replicas' compressed T2s (dims, m kept each), two
 * compressions per replica and iteration (which = 0: the one the T2 terms
 * contract, fricc/friccsd.py:100-107; which = 1: the one the W intermediates
 * contract, :108-117). */
int fricc_spb_create(int R, const int64_t dims[4], int64_t m, void* stream, fricc_spbatch** out);
int fricc_spb_destroy(fricc_spbatch* B);
/* Both systematic FRI compressions of every replica's T2 (t2: R tensors of
 * dims, stacked) with the draws rn_dev[2r], rn_dev[2r+1] (device memory),
 * as fricc_sp_recompress_pair does for one replica (fri_compression,
 * src/fri_utils.cpp:439-522).  Stream-ordered; the status is read by
 * fricc_spb_status. */
int fricc_spb_recompress_pair(fricc_spbatch* B, const double* t2, const double* rn_dev, void* stream);
/* Waits for the last compression; FRICC_OK or its error, *replica the
 * first failing replica (-1 if none). */
int fricc_spb_status(fricc_spbatch* B, int* replica);
/* Replica r's entries of compression `which` to host memory (synchronous). */
int fricc_spb_export(fricc_spbatch* B, int which, int r, int64_t* flat_host, double* vals_host, void* stream);
/* The generic sparse term of fricc_spmm (FP64) / fricc_spmm_f2 (FP32 pairs,
 * W' in the q-pair layout) for every replica: W'_r = Wp + r w_stride
 * (w_stride 0: one W' for all replicas; in float4 units for the pair form),
 * out'_r = Op + r o_stride.  Stream-ordered. */
int fricc_spb_spmm(fricc_spbatch* B, int which, int pa, int pb, int ka, int kb, double coef, const double* Wp,
                   int64_t w_stride, int64_t QS, double* Op, int64_t o_stride, void* stream);
int fricc_spb_spmm_f2(fricc_spbatch* B, int which, int pa, int pb, int ka, int kb, double coef, const void* W2,
                      int64_t w2_stride, int64_t QS, double* Op, int64_t o_stride, void* stream);
/* fricc_densify_bf16x3 for every replica of a batch: replica r's
 * compression `which` into rows [r nP, (r+1) nP) of A' ([R][nP][kp], zeroed
 * here).  Stream-ordered. */
int fricc_spb_densify_bf16x3(fricc_spbatch* B, int which, int pa, int pb, int ka, int kb, double coef, void* Ap,
                             int64_t kp, void* stream);
/* fricc_gemm_bf16_tn_strided for `reps` replicas of one shape in one launch:
 * replica r reads A' from row r a_rep (a_rep = 0: one A' for all replicas;
 * else a_rep >= M), B' from row r b_rep (likewise) and writes C + r c_rep.
 * Each replica's tiles, K split and sums are those of its single call. */
int fricc_gemm_bf16_tn_strided_b(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N,
                                 int64_t K, double* C, int64_t mi, int64_t ni, int64_t sro, int64_t sri, int64_t sco,
                                 int64_t sci, double alpha, double beta, int ksplit, int reps, int64_t a_rep,
                                 int64_t b_rep, int64_t c_rep, unsigned* status, void* stream);
/* fricc_symadd for R replicas: out [R][o][o][v][v] (C order), X with
 * strides {replica, i, j, a, b}. */
int fricc_symadd_b(double* out, const double* X, int64_t R, int64_t nocc, int64_t nvir, const int64_t strides[5],
                   double coef, void* stream);
/* fricc_energy_update for R replicas (t1/t2 arrays stacked, res [R][4];
 * eia, fov and ovov shared).  Stream-ordered. */
int fricc_energy_update_batch(int R, const double* t1num, const double* t2num, const double* eia, const double* fov,
                              const double* ovov, const double* t1old, const double* t2old, int64_t o, int64_t v,
                              double* t1out, double* t2out, double* res, void* stream);

/* Zero `bytes` bytes of device memory at p (no reference counterpart; the
 * np.zeros of the reference's scratch outputs).  Stream-ordered. */
int fricc_zero(void* p, int64_t bytes, void* stream);

/* Floating-point operations of one contract call (2 per multiply-add). */
double fricc_contract_flops(const char* term, const fricc_sparse* T);

/* The bare FRI compression of n doubles: flat[m] (int64) and vals[m] to device
 * memory, |D| to *n_largest (host).  Synchronises `stream`. */
int fricc_compress(const double* x, int64_t n, int64_t m, int compression, double rn, int64_t* flat, double* vals,
                   int64_t* n_largest, void* stream);

/* fri_compression with pivotal sampling on flat device arrays (see
 * fricc_sp_create_pivotal for glibc_hist and n_draws). */
int fricc_compress_pivotal(const double* x, int64_t n, int64_t m, uint32_t* glibc_hist, int64_t* flat, double* vals,
                           int64_t* n_largest, int64_t* n_draws, void* stream);

/* parallel_sample (src/fri_utils.cpp:176-362) over the probability vector q
 * (device, n doubles) with `chunks` chunks (the reference uses one per
 * OpenMP thread): S (device, n_sample int64) in the reference's order.  Each
 * chunk's adjustment and pivotal walk runs on its own warp.  Draws come
 * from glibc_hist (as for fricc_sp_create_pivotal) or from this process's
 * rand(): first the chunk-fraction sample, then chunk 0, 1, ... (the
 * reference's threads share rand() concurrently; this order is its outcome
 * when they run one after another, and at one chunk the two coincide).
 * *n_draws (optional) receives the draws consumed.  Synchronises `stream`. */
int fricc_parallel_sample(const double* q, int64_t n, int64_t n_sample, int chunks, uint32_t* glibc_hist,
                          int64_t* S, int64_t* n_draws, void* stream);

/* k uniforms rand()/RAND_MAX of the glibc stream with history hist[31]
 * (host, oldest first) into out (device); hist is advanced past them.  The
 * device form of the draws the reference makes with rand() (no reference
 * counterpart as a function).  Synchronises `stream`. */
int fricc_glibc_uniforms(uint32_t* hist, int64_t k, double* out, void* stream);

/* out[i] = fl(out[i-1] + |x[i]|) with out[-1] = 0 (device arrays of n
 * doubles): the exact bits a single CPU thread's left-to-right FP64 sum
 * produces, computed in parallel.  Stream-ordered. */
int fricc_seq_cumsum(const double* x, int64_t n, double* out, void* stream);

/* The same exact running sum, for callers that cannot allocate device memory
 * (an application whose device memory is reserved up front by its own
 * allocator, or a latency-critical loop that must not enter the CUDA
 * allocator).  No counterpart in the reference.  It allocates nothing: its
 * scratch (about 0.6 MB) is a fixed array inside the library, held by every
 * GPU that loads it until exit.  n <= 2^26 (67,108,864), larger n fails
 * with FRICC_ERR_ARG.  The first call on a device looks up the array's
 * address for that device; make it before any stream capture begins.  All
 * calls share the array: calls that overlap on the GPU (unordered streams)
 * race; calls ordered on one stream are safe.  Stream-ordered. */
int fricc_seq_cumsum_noalloc(const double* x, int64_t n, double* out, void* stream);

/* t1 = t1num/eia, t2 = t2num/(eia_ia + eia_jb); res[0] = E_corr of (t1, t2),
 * res[1] = || (t1,t2) - (t1old,t2old) || in packed form.  All device, C order:
 * t1* (o,v), t2* (o,o,v,v), eia (o,v), fov (o,v), ovov (o,v,o,v); res holds 4
 * doubles.  t1out/t2out may alias t1num/t2num.  Stream-ordered. */
int fricc_energy_update(const double* t1num, const double* t2num, const double* eia, const double* fov,
                        const double* ovov, const double* t1old, const double* t2old, int64_t nocc, int64_t nvir,
                        double* t1out, double* t2out, double* res, void* stream);

/* The same update with the linearised energy of FRI-LCCSD,
 * E = 2 sum f_ia t1_ia + sum t2_ijab (2 (ia|jb) - (ib|ja)): replaces the
 * denominators of fricc/frilccsd.py:241-244 and lin_cc_energy :504-522. */
int fricc_energy_update_lin(const double* t1num, const double* t2num, const double* eia, const double* fov,
                            const double* ovov, const double* t1old, const double* t2old, int64_t nocc,
                            int64_t nvir, double* t1out, double* t2out, double* res, void* stream);

/* out[i,j,a,b] += coef * (X[i,j,a,b] + X[j,i,b,a]) in one pass: the
 * symmetrised additions of the T2 residual (fricc/friccsd.py:245-267,
 * "tmp + tmp.transpose(1,0,3,2)").  out: contiguous [nocc][nocc][nvir][nvir];
 * X: any [nocc][nocc][nvir][nvir] view given by its element strides, not
 * overlapping out.  Stream-ordered. */
int fricc_symadd(double* out, const double* X, int64_t nocc, int64_t nvir, const int64_t strides[4], double coef,
                 void* stream);

/* Split-precision integral rebuilds on the tcgen05 tensor cores (the
 * reference builds its dense integral blocks in FP64 through PySCF,
 * fricc/friccsd.py:325-331 for Wvvvv; the split-BF16x3 rebuild from a
 * Cholesky factor has no reference counterpart).
 *
 * fricc_gemm_bf16_tn: C[M][N] = A[M][K] B[N][K]^T with BF16 operands, both
 * K-major (row strides lda, ldb in elements: multiples of 8, base 16-byte
 * aligned), FP32 accumulation; C FP32 (or FP64 for the _f64 form, the FP32
 * sums widened exactly), row stride ldc.  Synchronises the stream and
 * returns FRICC_ERR_TIMEOUT if a bounded pipeline wait gave up.
 *
 * fricc_split_bf16x3: x [rows][ld] FP64 (first k columns) ->
 * A' = [hi | hi | lo], B' = [hi | lo | hi] ([rows][kp] BF16, kp >= 3k, the
 * columns past 3k zero), hi = bf16(x), lo = bf16(x - hi); A'_r . B'_s is
 * then the split-BF16x3 product of rows r and s.
 *
 * fricc_vvvv_rebuild_bf16x3: from the split operands of L_vv^T
 * ([v*v][kp], row c*v + a = L[:, a, c]), W[(c*v + d)*ldw + a*v + b] = (ac|bd)
 * in FP32 -- the O^2V^4 operand of fricc_spmm_f1.  With status == NULL it
 * synchronises like fricc_gemm_bf16_tn; otherwise it is stream-ordered (and
 * capturable into a CUDA graph) and a gave-up wait ORs FRICC_DEV_TIMEOUT (2)
 * into the device word *status. */
int fricc_gemm_bf16_tn(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N, int64_t K,
                       float* C, int64_t ldc, void* stream);
int fricc_gemm_bf16_tn_f64(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N, int64_t K,
                           double* C, int64_t ldc, void* stream);
int fricc_split_bf16x3(const double* x, int64_t rows, int64_t k, int64_t ld, int64_t kp, void* Ap, void* Bp,
                       void* stream);
int fricc_vvvv_rebuild_bf16x3(const void* Ap, const void* Bp, int64_t v, int64_t kp, float* W, int64_t ldw,
                              unsigned* status, void* stream);

/* fricc_vvvv_rebuild_split_b: the same rebuild written as the B operand of
 * the dense O^2V^4 GEMM: row q = a*v + b, K index k = c*v + d, (ac|bd) as
 * [hi | lo | hi] at k, v^2 + k, 2 v^2 + k (rows of kpo >= 3 v^2 elements, a
 * multiple of 8; the padding is zeroed).  status as above. */
int fricc_vvvv_rebuild_split_b(const void* Ap, const void* Bp, int64_t v, int64_t kp, void* Bout, int64_t kpo,
                               unsigned* status, void* stream);

/* The general forms behind the split-precision dense algebra.
 * fricc_split_bf16x3_strided: as fricc_split_bf16x3 for a strided view:
 * row r = (r / ri, r % ri) and column j < k of x at
 * (r / ri)*sro + (r % ri)*sri + j*sk (a transposed or batch-flattened
 * operand); either output may be NULL.
 * fricc_gemm_bf16_tn_strided: C = alpha (A B^T) + beta C, C FP64 with
 * element (r, c) at (r / mi)*sro + (r % mi)*sri + (c / ni)*sco + (c % ni)*sci
 * (beta == 0 does not read C); status as for fricc_vvvv_rebuild_bf16x3.
 * ksplit > 1 splits K into that many slices (for a long K and few output
 * tiles): FP32 partial sums per slice, then one reduction in slice order
 * (deterministic). */
int fricc_split_bf16x3_strided(const double* x, int64_t rows, int64_t k, int64_t ri, int64_t sro, int64_t sri,
                               int64_t sk, int64_t kp, void* Ap, void* Bp, void* stream);
int fricc_gemm_bf16_tn_strided(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int64_t N,
                               int64_t K, double* C, int64_t mi, int64_t ni, int64_t sro, int64_t sri, int64_t sco,
                               int64_t sci, double alpha, double beta, int ksplit, unsigned* status, void* stream);

/* A dedicated non-blocking stream of the current device, and its release
 * (no reference counterpart).  Solvers that overlap or capture work need
 * streams no other solver shares; torch's own streams come from a small
 * shared pool. */
int fricc_stream_create(void** out);
int fricc_stream_destroy(void* stream);

/* Launch-configuration overrides for an autotuner (no reference
 * counterpart), thread-local; value -1 restores the built-in choice.
 * knob 0: output pairs per thread of the float-pair sparse kernel (1, 2, 4);
 * knob 1: tile of the FP32-pair GEMM (0 = 64x64, 1 = 128x32, 2 = 32x128,
 * 3 = 32x160, 4 = 32x32; the FP64 GEMM's candidate set too); knob 2: CTAs per SM the
 * FP32-pair and FP64 GEMMs' split K aims for (1..16); knob 3 (a test of the
 * error path, 1..2^20): in every later compression on this thread, one
 * tile of the candidate compaction first polls a device word that nothing
 * sets, gives up after that many polls and reports FRICC_ERR_TIMEOUT
 * through the compression's status (its results stay valid: the
 * compaction then runs as usual); knob 4: the width in bits (10..13,
 * default 12) of a compression's first select digit -- how many candidates
 * the exact sort of the top-m selection (argsort / get_d_largest,
 * src/fri_utils.cpp:11-36,400-437) takes; every width keeps the same
 * entries; knob 5: the float-pair sparse kernel as a persistent launch of
 * this many CTAs per SM (1..8) taking its (bucket, q tile) items in
 * q-tile-major order (unset: one CTA per item).  No knob changes a
 * result's arithmetic except the GEMMs' tile and split, which reorder
 * their sums. */
int fricc_tune_set(int knob, int value);

/* Instrumentation (no reference counterpart): the number of kernels this
 * library has launched so far; and CUDA-event timing of every sparse
 * contraction kernel launched while enabled (fricc_prof_enable(1) clears
 * the record; fricc_prof_read synchronises on the recorded events and
 * returns total milliseconds, launches and algorithmic flops). */
long long fricc_launch_count(void);
/* The number of device allocations (stream-ordered cudaMallocAsync) this
 * library has made so far (no reference counterpart). */
long long fricc_alloc_count(void);
void fricc_prof_enable(int on);
int fricc_prof_read(double* ms, long long* launches, double* flops);
/* The same record for the tensor-core GEMM launches (fricc_gemm_bf16_*,
 * the rebuilds; flops = 2 M N K' of the BF16 products). */
int fricc_prof_read_tc(double* ms, long long* launches, double* flops);
/* The same record for the FP64 GEMM launches (fricc_gemm_f64; flops =
 * 2 batch M N K). */
int fricc_prof_read_gemm(double* ms, long long* launches, double* flops);

#ifdef __cplusplus
}
#endif
#endif /* FRICC_GB300_H */
