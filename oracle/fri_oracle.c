/*
 * fri_oracle.c -- CPU restatement of fri-cc's FRI compression and of its
 * eleven sparse-T2 x dense-W contraction terms.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the tests, the smoke
 * check and the CPU-baseline leg of bench.py load it to CHECK the CUDA path
 * or to time the reference algorithm on the host cores.  The product
 * (fricc_gb300/) never loads it.
 *
 * Parity pin: the outputs of this file are checked bit for bit against the
 * reference's own C++ (compiled from its sources into oracle/_ref/ by
 * oracle/Makefile) through the golden vectors in tests/golden/.
 *
 * Semantics follow the reference at OMP_NUM_THREADS=1 (the only setting in
 * which the reference is deterministic: its one_norm is an OpenMP
 * reduction).  Every floating-point expression keeps the reference's
 * operation order; the file is compiled with -ffp-contract=off so no
 * multiply-add is fused on any host.
 *
 * Status codes: 0 ok, 1 bad argument, 3 probability > 1 (the reference
 * exits with "ERROR MAKING PROBABILITY VECTOR"), 6 unpacked index out of
 * range (the reference exits in SparseTensor4d::unpack_idx), 7 an exit of
 * sample_pivotal ("ERROR IN PIVOTAL SAMPLING", "Wrong number of elements").
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define FO_OK 0
#define FO_BAD_ARG 1
#define FO_P_GT_ONE 3
#define FO_INDEX_RANGE 6
#define FO_PIVOTAL 7 /* sample_pivotal's own exits: acceptance outside [0,1],
                        a leftover weight |a-1| >= 1e-5, or a wrong count */

typedef struct {
  double key; /* |x_i| */
  int64_t idx;
} fo_pair;

/* Order used by argsort (src/fri_utils.cpp:22-25): descending |x|; the
 * stable merge keeps equal magnitudes in ascending flat-index order. */
static inline int fo_before(const fo_pair* a, const fo_pair* b) {
  if (a->key != b->key) return a->key > b->key;
  return a->idx < b->idx;
}

static void fo_merge(const fo_pair* src, fo_pair* dst, int64_t lo, int64_t mid,
                     int64_t hi) {
  int64_t i = lo, j = mid, k = lo;
  while (i < mid && j < hi) dst[k++] = fo_before(&src[j], &src[i]) ? src[j++] : src[i++];
  while (i < mid) dst[k++] = src[i++];
  while (j < hi) dst[k++] = src[j++];
}

static void fo_insertion(fo_pair* a, int64_t lo, int64_t hi) {
  for (int64_t i = lo + 1; i < hi; ++i) {
    fo_pair v = a[i];
    int64_t j = i - 1;
    while (j >= lo && fo_before(&v, &a[j])) { a[j + 1] = a[j]; --j; }
    a[j + 1] = v;
  }
}

/* Bottom-up merge sort of all n pairs, parallel over runs (the reference
 * sorts the whole array with a parallel merge sort, src/fri_utils.cpp:11-36).
 * The order is total, so any thread count gives the same permutation. */
static void fo_sort_pairs(fo_pair* a, int64_t n) {
  const int64_t RUN = 32;
  fo_pair* tmp = (fo_pair*)malloc(sizeof(fo_pair) * (size_t)(n > 0 ? n : 1));
#pragma omp parallel for schedule(static)
  for (int64_t lo = 0; lo < n; lo += RUN) fo_insertion(a, lo, lo + RUN < n ? lo + RUN : n);
  fo_pair* src = a;
  fo_pair* dst = tmp;
  for (int64_t w = RUN; w < n; w *= 2) {
#pragma omp parallel for schedule(static)
    for (int64_t lo = 0; lo < n; lo += 2 * w) {
      int64_t mid = lo + w < n ? lo + w : n;
      int64_t hi = lo + 2 * w < n ? lo + 2 * w : n;
      fo_merge(src, dst, lo, mid, hi);
    }
    fo_pair* t = src; src = dst; dst = t;
  }
  if (src != a) memcpy(a, src, sizeof(fo_pair) * (size_t)n);
  free(tmp);
}

/* one_norm, src/fri_utils.cpp:164-171, at one thread: index order. */
double fo_one_norm(const double* x, int64_t n) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += fabs(x[i]);
  return s;
}

/* argsort, src/fri_utils.cpp:11-36: the first m flat indices of x sorted
 * by descending |x| (ties: ascending index). */
int fo_argsort(const double* x, int64_t n, int64_t m, int64_t* out) {
  if (n < 0 || m < 0 || m > n) return FO_BAD_ARG;
  fo_pair* p = (fo_pair*)malloc(sizeof(fo_pair) * (size_t)(n > 0 ? n : 1));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) { p[i].key = fabs(x[i]); p[i].idx = i; }
  fo_sort_pairs(p, n);
  for (int64_t i = 0; i < m; ++i) out[i] = p[i].idx;
  free(p);
  return FO_OK;
}

/* get_d_largest, src/fri_utils.cpp:400-437.  sorted: the m largest indices.
 * Returns |D|; D is sorted[0..|D|); *remaining receives the final R. */
int64_t fo_get_d_largest(const double* x, int64_t n, int64_t m,
                         const int64_t* sorted, double* remaining) {
  double R = fo_one_norm(x, n);
  int64_t d = 0;
  for (int64_t i = 0; i < m; ++i) {
    double xi = fabs(x[sorted[i]]);
    /* (n_sample - d) is a size_t converted to double */
    if ((double)(uint64_t)(m - d) * xi >= R - xi && R > 1e-14) {
      ++d;
      R -= xi;
    } else {
      break;
    }
  }
  *remaining = R;
  return d;
}

/* make_probability_vector, src/fri_utils.cpp:367-398:
 *   p_i = |x_i| / R * n_sample, p_D = 0, error if any p_i > 1. */
int fo_make_probability_vector(const double* x, int64_t n, int64_t n_sample,
                               const int64_t* D, int64_t nd, double R, double* p) {
  const double ns = (double)(uint64_t)n_sample;
  for (int64_t i = 0; i < n; ++i) p[i] = fabs(x[i]) / R * ns;
  for (int64_t i = 0; i < nd; ++i) p[D[i]] = 0.0;
  for (int64_t i = 0; i < n; ++i)
    if (p[i] > 1.) return FO_P_GT_ONE;
  return FO_OK;
}

/* sample_systematic, src/fri_utils.cpp:129-159, with the single uniform
 * draw rn = rand()/RAND_MAX of lin_space_add_const (:45-58) passed in.
 *   u_k = k * 1.0 + rn, intervals = [0, partial_sum(p)], forward search.
 * A u_k that falls in no interval leaves S[k] = 0, as in the reference. */
void fo_sample_systematic(int64_t n_sample, const double* p, int64_t n, double rn,
                          int64_t* S) {
  double* I = (double*)malloc(sizeof(double) * (size_t)(n + 1));
  const double step = (double)(uint64_t)n_sample / (double)(uint64_t)n_sample;
  I[0] = 0.0;
  if (n > 0) {
    double acc = p[0]; /* std::partial_sum copies the first element */
    I[1] = acc;
    for (int64_t j = 1; j < n; ++j) { acc = acc + p[j]; I[j + 1] = acc; }
  }
  int64_t last = 0;
  for (int64_t k = 0; k < n_sample; ++k) {
    double u = (double)(uint64_t)k * step + rn;
    S[k] = 0;
    for (int64_t j = last; j < n; ++j) {
      if (u >= I[j] && u < I[j + 1]) { S[k] = j; last = j; break; }
    }
  }
  free(I);
}

/* sample_pivotal, src/fri_utils.cpp:63-127.  One uniform per element
 * j = 1, 2, ... (rand()/RAND_MAX): from draws[] when given (at most n_avail
 * of them), else from libc rand() itself.  The carried weight a = p_0,
 * a += p_j; below 1 the pivot i moves to j with probability p_j / a; at or
 * above 1, a -= 1 and one index is emitted: the pivot (which then moves to
 * j) with probability (1 - p_j) / (1 - a), else j.  Stops once n_sample
 * indices are out; a run that reaches the last element with |a - 1| < 1e-5
 * emits the pivot.  *n_used receives the draws consumed. */
int fo_sample_pivotal(int64_t n_sample, const double* p, int64_t n, const double* draws, int64_t n_avail,
                      int64_t* S, int64_t* n_used) {
  int64_t ns = 0, i = 0, used = 0;
  double a = n > 0 ? p[0] : 0.0;
  for (int64_t j = 1; j < n; ++j) {
    a += p[j];
    double rn;
    if (draws) {
      if (used >= n_avail) return FO_BAD_ARG;
      rn = draws[used];
    } else {
      rn = (double)rand() / RAND_MAX;
    }
    ++used;
    if (a < 1.) {
      if (rn < p[j] / a) i = j;
    } else {
      a -= 1.;
      const double prob_accept = (1. - p[j]) / (1. - a);
      if (prob_accept > 1 || prob_accept < 0) { *n_used = used; return FO_PIVOTAL; }
      if (rn < prob_accept) { S[ns++] = i; i = j; }
      else S[ns++] = j;
    }
    if (ns == n_sample) break;
    if (j == n - 1) {
      if (fabs(a - 1.) < 1e-5) S[ns++] = i;
      else { *n_used = used; return FO_PIVOTAL; }
    }
  }
  *n_used = used;
  return ns == n_sample ? FO_OK : FO_PIVOTAL;
}

/* parallel_sample, src/fri_utils.cpp:176-362, with T chunks (the reference
 * uses T = omp_get_max_threads()).  q is cut into T contiguous chunks (the
 * last takes the remainder); chunk j expects a_j = n * |q_j| / |q| samples,
 * floor(a_j) surely and one more with probability frac(a_j), decided by a
 * pivotal sample over the fractions; each chunk's probabilities are then
 * pushed towards its integer count (the reference's two capped loops) and
 * sampled pivotally, indices shifted by the chunk offset.  The reference
 * runs the chunk samplers on concurrent threads sharing rand(); here the
 * draws are taken in chunk order (the fraction sample, then chunk 0, 1, ...),
 * which is the reference's outcome when its threads run one after another;
 * at T = 1 the two coincide.  The norms are sequential sums (the reference's
 * one_norm at one thread).  *n_used: draws consumed. */
int fo_parallel_sample(int64_t n_sample, const double* q, int64_t n, int T, const double* draws,
                       int64_t n_avail, int64_t* S, int64_t* n_used) {
  if (T < 1 || n < T) return FO_BAD_ARG;
  const int64_t step = n / T, rem = n % T;
  double q_norm = 0.0;
  for (int64_t i = 0; i < n; ++i) q_norm += fabs(q[i]);
  double* t = (double*)malloc(sizeof(double) * T);
  double* a = (double*)malloc(sizeof(double) * T);
  double* qn = (double*)malloc(sizeof(double) * T);
  int* g = (int*)malloc(sizeof(int) * T);
  double* qj = (double*)malloc(sizeof(double) * (size_t)(step + rem));
  int64_t* Sj = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n_sample > 0 ? n_sample : 1));
  uint64_t c = (uint64_t)n_sample;
  for (int j = 0; j < T; ++j) {
    const int64_t lo = j * step, hi = (j + 1 == T) ? n : lo + step;
    double nj = 0.0;
    for (int64_t i = lo; i < hi; ++i) nj += fabs(q[i]);
    qn[j] = nj;
    a[j] = (double)(uint64_t)n_sample * qn[j] / q_norm;
    t[j] = a[j] - floor(a[j]);
    g[j] = (int)floor(a[j]);
    c -= (uint64_t)(int64_t)g[j];
  }
  int64_t used = 0, u = 0;
  int st = FO_OK;
  /* the fractions' pivotal sample picks which chunks get one more */
  int64_t* sp = (int64_t*)malloc(sizeof(int64_t) * (size_t)(T > 0 ? T : 1));
  if (c > (uint64_t)T) { st = FO_PIVOTAL; goto out; }
  st = fo_sample_pivotal((int64_t)c, t, T, draws, n_avail, sp, &u);
  used += u;
  if (st) goto out;
  for (uint64_t k = 0; k < c; ++k) g[sp[k]] += 1;
  {
    double chunk_lb = 0.0;
    for (int j = 0; j < T; ++j) {
      const int64_t lo = j * step, hi = (j + 1 == T) ? n : lo + step, len = hi - lo;
      for (int64_t i = 0; i < len; ++i) qj[i] = q[lo + i];
      double sj = qn[j];
      if ((double)g[j] > a[j]) {
        for (int64_t i = 0; i < len; ++i) {
          const double y = fmin(1., qj[i] / t[j]);
          sj += y - qj[i];
          qj[i] = y;
          if (sj >= (double)g[j]) { qj[i] = y + (double)g[j] - sj; break; }
        }
      } else if ((double)g[j] < a[j]) {
        for (int64_t i = 0; i < len; ++i) {
          const double y = fmax(0., (qj[i] - t[j]) / (1. - t[j]));
          sj += y - qj[i];
          qj[i] = y;
          if (sj <= (double)g[j]) { qj[i] = y + (double)g[j] - sj; break; }
        }
      }
      const int64_t lb = (int64_t)chunk_lb;
      chunk_lb += (double)g[j];
      if (g[j] < 0 || lb + g[j] > n_sample) { st = FO_PIVOTAL; goto out; }
      st = fo_sample_pivotal(g[j], qj, len, draws ? draws + used : NULL, draws ? n_avail - used : 0, Sj, &u);
      used += u;
      if (st) goto out;
      for (int64_t k = 0; k < g[j]; ++k) S[lb + k] = Sj[k] + lo;
    }
  }
out:
  *n_used = used;
  free(t); free(a); free(qn); free(g); free(qj); free(Sj); free(sp);
  return st;
}

/* fri_compression, src/fri_utils.cpp:439-522, pivotal sampling (S in the
 * order sample_pivotal emits it). */
int fo_fri_compression_pivotal(const double* x, int64_t n, int64_t m, const double* draws, int64_t n_avail,
                               int64_t* idx, double* val, int64_t* n_largest, int64_t* n_used) {
  if (n < 0 || m < 0 || m > n) return FO_BAD_ARG;
  int64_t* sorted = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
  fo_argsort(x, n, m, sorted);
  double R;
  int64_t nd = fo_get_d_largest(x, n, m, sorted, &R);
  double* p = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  int st = fo_make_probability_vector(x, n, m - nd, sorted, nd, R, p);
  *n_used = 0;
  if (st != FO_OK) { free(sorted); free(p); return st; }
  int64_t* S = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m - nd > 0 ? m - nd : 1));
  st = fo_sample_pivotal(m - nd, p, n, draws, n_avail, S, n_used);
  if (st == FO_OK) {
    for (int64_t i = 0; i < nd; ++i) { idx[i] = sorted[i]; val[i] = x[sorted[i]]; }
    for (int64_t k = 0; k < m - nd; ++k) {
      idx[nd + k] = S[k];
      val[nd + k] = x[S[k]] / p[S[k]];
    }
    if (n_largest) *n_largest = nd;
  }
  free(sorted); free(p); free(S);
  return st;
}

/* fri_compression, src/fri_utils.cpp:439-522, systematic sampling.
 * idx/val receive m entries: D in sorted order, then S in ascending order.
 * *n_largest receives |D|. */
int fo_fri_compression(const double* x, int64_t n, int64_t m, double rn,
                       int64_t* idx, double* val, int64_t* n_largest) {
  if (n < 0 || m < 0 || m > n) return FO_BAD_ARG;
  int64_t* sorted = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
  fo_argsort(x, n, m, sorted);
  double R;
  int64_t nd = fo_get_d_largest(x, n, m, sorted, &R);
  double* p = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  int st = fo_make_probability_vector(x, n, m - nd, sorted, nd, R, p);
  if (st != FO_OK) { free(sorted); free(p); return st; }
  int64_t* S = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m - nd > 0 ? m - nd : 1));
  fo_sample_systematic(m - nd, p, n, rn, S);
  for (int64_t i = 0; i < nd; ++i) { idx[i] = sorted[i]; val[i] = x[sorted[i]]; }
  for (int64_t k = 0; k < m - nd; ++k) {
    idx[nd + k] = S[k];
    val[nd + k] = x[S[k]] / p[S[k]];
  }
  if (n_largest) *n_largest = nd;
  free(sorted); free(p); free(S);
  return FO_OK;
}

/* "largest" compression, include/sparse_tensor.hpp:46-56: the first m of
 * argsort with unscaled values. */
int fo_largest(const double* x, int64_t n, int64_t m, int64_t* idx, double* val) {
  int st = fo_argsort(x, n, m, idx);
  if (st != FO_OK) return st;
  for (int64_t i = 0; i < m; ++i) val[i] = x[idx[i]];
  return FO_OK;
}

/* SparseTensor4d::unpack_idx, include/sparse_tensor.hpp:108-125. */
int fo_unpack(const int64_t* flat, int64_t m, const int64_t dims[4], int64_t* idx4) {
  const uint64_t d1 = (uint64_t)dims[1], d2 = (uint64_t)dims[2], d3 = (uint64_t)dims[3];
  for (int64_t s = 0; s < m; ++s) {
    uint64_t f = (uint64_t)flat[s];
    uint64_t i0 = f / (d1 * d2 * d3);
    uint64_t i1 = f % (d1 * d2 * d3) / (d2 * d3);
    uint64_t i2 = f % (d2 * d3) / d3;
    uint64_t i3 = f % d3;
    if (i0 >= (uint64_t)dims[0] || i1 >= d1 || i2 >= d2 || i3 >= d3) return FO_INDEX_RANGE;
    idx4[4 * s + 0] = (int64_t)i0; idx4[4 * s + 1] = (int64_t)i1;
    idx4[4 * s + 2] = (int64_t)i2; idx4[4 * s + 3] = (int64_t)i3;
  }
  return FO_OK;
}

/* ------------------------------------------------------------------------
 * Contractions, src/sparse_tensor.cpp:12-346.
 *
 * Each term loops over two output indices (the "outer pair"), scans all m
 * nonzeros for those whose two index slots match, and accumulates W*value
 * into the output in place.  For every output element the contributions
 * therefore arrive in nonzero-slot order; this file keeps that order.
 * W and out are addressed through element strides (the reference reads
 * them through pybind11 unchecked<4> views, which honour strides).
 *
 * outer_begin/outer_end/outer_step restrict the flattened outer-pair loop to
 * begin, begin + step, ... < end, so that a bounded sample of a large
 * contraction, spread evenly over all its outer pairs, can be timed.
 * ------------------------------------------------------------------------ */
#define W4(a, b, c, d) W[(a) * ws[0] + (b) * ws[1] + (c) * ws[2] + (d) * ws[3]]
#define O4(a, b, c, d) out[(a) * os[0] + (b) * os[1] + (c) * os[2] + (d) * os[3]]

enum {
  T0101 = 0, T2323, T1302, T1202, T1303, T1203, T1323, T0112, T0113, T0313, T0312, TN
};

static const char* fo_term_names[TN] = {"0101", "2323", "1302", "1202", "1303", "1203",
                                        "1323", "0112", "0113", "0313", "0312"};

int fo_term_id(const char* name) {
  for (int t = 0; t < TN; ++t)
    if (strcmp(name, fo_term_names[t]) == 0) return t;
  return -1;
}

/* number of outer pairs of a term (the collapse(2) loop of the reference) */
int64_t fo_outer_size(int term, const int64_t tdims[4], const int64_t wdims[4]) {
  const int64_t no = tdims[0], nv = tdims[2];
  switch (term) {
    case T0101: return nv * nv;
    case T2323: return tdims[0] * tdims[1];
    case T1302: case T1202: case T1303: return nv * no;
    case T1203: return nv * no;
    case T1323: return no * no;
    case T0112: case T0113: case T0313: case T0312: return nv * no;
  }
  (void)wdims;
  return -1;
}

int fo_contract(int term, const double* W, const int64_t wdims[4], const int64_t ws[4],
                const int64_t* idx4, const double* vals, int64_t m, const int64_t tdims[4],
                double* out, const int64_t os[4], int64_t outer_begin, int64_t outer_end,
                int64_t outer_step) {
  const int64_t no = tdims[0], nv = tdims[2];
  int64_t n_outer = fo_outer_size(term, tdims, wdims);
  if (n_outer < 0) return FO_BAD_ARG;
  if (outer_begin < 0) outer_begin = 0;
  if (outer_end < 0 || outer_end > n_outer) outer_end = n_outer;
  if (outer_step < 1) outer_step = 1;
  const int64_t n_iter = outer_end > outer_begin ? (outer_end - outer_begin + outer_step - 1) / outer_step : 0;

  switch (term) {
    case T0101: /* out(i,j,a,b) += W(k,l,i,j) * T(k,l,a,b); outer (a,b) */
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t a = p / nv, b = p % nv;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[2] == a && id[3] == b) {
            const int64_t k = id[0], l = id[1];
            const double v = vals[s];
            for (int64_t i = 0; i < no; ++i)
              for (int64_t j = 0; j < no; ++j) O4(i, j, a, b) += W4(k, l, i, j) * v;
          }
        }
      }
      break;
    case T2323: { /* out(i,j,a,b) += W(a,b,c,d) * T(i,j,c,d); outer (i,j) */
      const int64_t dj = tdims[1], da = wdims[0], db = wdims[1];
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t i = p / dj, j = p % dj;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[0] == i && id[1] == j) {
            const int64_t c = id[2], d = id[3];
            const double v = vals[s];
            for (int64_t a = 0; a < da; ++a)
              for (int64_t b = 0; b < db; ++b) O4(i, j, a, b) += W4(a, b, c, d) * v;
          }
        }
      }
      break;
    }
    case T1302: /* out(i,j,a,b) += 2*W(a,k,i,c)*T(k,j,c,b); outer (b,j) */
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t b = p / no, j = p % no;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[3] == b && id[1] == j) {
            const int64_t k = id[0], c = id[2];
            const double v = vals[s];
            for (int64_t i = 0; i < no; ++i)
              for (int64_t a = 0; a < nv; ++a) O4(i, j, a, b) += 2 * W4(a, k, i, c) * v;
          }
        }
      }
      break;
    case T1202: /* out(i,j,a,b) -= W(a,k,c,i)*T(k,j,c,b); outer (b,j) */
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t b = p / no, j = p % no;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[3] == b && id[1] == j) {
            const int64_t k = id[0], c = id[2];
            const double v = vals[s];
            for (int64_t i = 0; i < no; ++i)
              for (int64_t a = 0; a < nv; ++a) O4(i, j, a, b) -= W4(a, k, c, i) * v;
          }
        }
      }
      break;
    case T1303: /* out(i,j,a,b) += W(a,k,i,c)*T(k,j,b,c); outer (b,j) */
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t b = p / no, j = p % no;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[2] == b && id[1] == j) {
            const int64_t k = id[0], c = id[3];
            const double v = vals[s];
            for (int64_t i = 0; i < no; ++i)
              for (int64_t a = 0; a < nv; ++a) O4(i, j, a, b) += W4(a, k, i, c) * v;
          }
        }
      }
      break;
    case T1203: /* out(i,j,a,b) += W(b,k,c,i)*T(k,j,a,c); outer (a,j) */
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t a = p / no, j = p % no;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[2] == a && id[1] == j) {
            const int64_t k = id[0], c = id[3];
            const double v = vals[s];
            for (int64_t i = 0; i < no; ++i)
              for (int64_t b = 0; b < nv; ++b) O4(i, j, a, b) += W4(b, k, c, i) * v;
          }
        }
      }
      break;
    case T1323: /* out(k,l,i,j) += ovov(k,c,l,d)*T(i,j,c,d); outer (i,j) */
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t i = p / no, j = p % no;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[0] == i && id[1] == j) {
            const int64_t c = id[2], d = id[3];
            const double v = vals[s];
            for (int64_t k = 0; k < no; ++k)
              for (int64_t l = 0; l < no; ++l) O4(k, l, i, j) += W4(k, c, l, d) * v;
          }
        }
      }
      break;
    case T0112: /* out(a,k,i,c) -= 0.5*ovov(l,d,k,c)*T(i,l,d,a); outer (a,i) */
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t a = p / no, i = p % no;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[3] == a && id[0] == i) {
            const int64_t l = id[1], d = id[2];
            const double v = vals[s];
            for (int64_t k = 0; k < no; ++k)
              for (int64_t c = 0; c < nv; ++c) O4(a, k, i, c) -= 0.5 * W4(l, d, k, c) * v;
          }
        }
      }
      break;
    case T0313: /* out(a,k,i,c) -= 0.5*ovov(l,c,k,d)*T(i,l,a,d); outer (a,i) */
#pragma omp parallel for schedule(dynamic, 16)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t a = p / no, i = p % no;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[2] == a && id[0] == i) {
            const int64_t l = id[1], d = id[3];
            const double v = vals[s];
            for (int64_t k = 0; k < no; ++k)
              for (int64_t c = 0; c < nv; ++c) O4(a, k, i, c) -= 0.5 * W4(l, c, k, d) * v;
          }
        }
      }
      break;
    case T0113: /* out(a,k,i,c) += ovov(l,d,k,c)*T(i,l,a,d); outer (a,i) */
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t a = p / no, i = p % no;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[2] == a && id[0] == i) {
            const int64_t l = id[1], d = id[3];
            const double v = vals[s];
            for (int64_t k = 0; k < no; ++k)
              for (int64_t c = 0; c < nv; ++c) O4(a, k, i, c) += W4(l, d, k, c) * v;
          }
        }
      }
      break;
    case T0312: /* out(a,k,c,i) -= 0.5*ovov(l,c,k,d)*T(i,l,d,a); outer (a,i) */
#pragma omp parallel for schedule(dynamic)
      for (int64_t q = 0; q < n_iter; ++q) {
        const int64_t p = outer_begin + q * outer_step;
        const int64_t a = p / no, i = p % no;
        for (int64_t s = 0; s < m; ++s) {
          const int64_t* id = idx4 + 4 * s;
          if (id[3] == a && id[0] == i) {
            const int64_t l = id[1], d = id[2];
            const double v = vals[s];
            for (int64_t k = 0; k < no; ++k)
              for (int64_t c = 0; c < nv; ++c) O4(a, k, c, i) -= 0.5 * W4(l, c, k, d) * v;
          }
        }
      }
      break;
    default:
      return FO_BAD_ARG;
  }
  return FO_OK;
}

int fo_max_threads(void) { return omp_get_max_threads(); }
void fo_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }
