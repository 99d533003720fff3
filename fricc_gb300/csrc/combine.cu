// Strided elementwise combinations over a 5-D index space (the 4-D entry
// point is the 5-D one with a leading extent 1; the fifth dimension is the
// replica of a replica batch):
//
//   r_k(i) = sum_t c[k][t] x_t(i) + c[k][n_in] p_0(i) p_1(i) ... (product term)
//   out_k(i) = r_k(i)               (accumulate = 0)
//   out_k(i) = out_k(i) + r_k(i)    (accumulate = 1)
//
// for every i = (i0, .., i4) < dims, where every operand is a view
// x_t(i) = x_t[i0 s0 + .. + i4 s4] with its own element strides
// (0 broadcasts).  The permuted copies, linear combinations, broadcast
// products and diagonal updates of an FRI-CCSD iteration's intermediates
// (fricc/friccsd.py:144-301 and the W builds :309-376) run here, so every
// elementwise pass of the iteration is a launch of this library.
//
// The index space runs i4 fastest; callers order it so that the first
// output is contiguous along i4.  Inputs contiguous along i4 (or
// broadcast, or scattered) are read directly; an input contiguous along
// another dimension d (a transposed view) is read through 32 x 32 shared-
// memory tiles of the plane (d, 4), so that its reads and the outputs'
// accesses both coalesce.  Inputs are grouped by that layout and each group
// is one pass (the first writes or accumulates as asked, later ones
// accumulate), so a result is r_k summed group by group: deterministic for
// given layouts, within an FP64 rounding of any other summation order.
//
// Index arithmetic is 32-bit when every element count and offset fits,
// with divisions by the dimensions done as a multiply-high by a
// precomputed reciprocal (Granlund and Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994): for 1 <= d < 2^31 and
// p = 31 + ceil(log2 d), m = ceil(2^p / d), every n < 2^31 has
// n / d = umulhi(n, m) >> (p - 32).
#include "common.cuh"

namespace {

constexpr int kMaxIn = FRICC_COMBINE_MAX_IN, kMaxProd = FRICC_COMBINE_MAX_PROD, kMaxOut = FRICC_COMBINE_MAX_OUT;

struct FastDiv {
  unsigned d, m, s;  // d == 1: m = 0, s = 0
  __host__ void set(unsigned dd) {
    d = dd;
    if (dd <= 1) {
      m = 0;
      s = 0;
      return;
    }
    unsigned l = 0;
    while ((1ull << l) < dd) ++l;                 // ceil(log2 d)
    const unsigned p = 31 + l;
    m = (unsigned)(((1ull << p) + dd - 1) / dd);  // < 2^32 for d >= 2
    s = p - 32;
  }
  __device__ __forceinline__ unsigned div(unsigned n) const { return m ? (__umulhi(n, m) >> s) : n; }
};

constexpr int D = 5;

struct CombineArgs {
  int64_t d[D];
  int64_t n;                // product of the dims
  FastDiv f1, f2, f3, f4;   // dims[1..4] (32-bit path)
  const double* x[kMaxIn];
  int64_t sx[kMaxIn][D];
  const double* p[kMaxProd];
  int64_t sp[kMaxProd][D];
  double* out[kMaxOut];
  int64_t so[kMaxOut][D];
  double c[kMaxOut][kMaxIn + 1];
  // each coefficient's kind, decided on the host: 0 (the term is left out),
  // 1 (+x), -1 (-x), 2 (c x).  GB300's FP64 unit is slow enough that
  // comparing the coefficients per element in FP64 bounded these passes.
  signed char cc[kMaxOut][kMaxIn + 1];
  int acc[kMaxOut];  // per output: add to its current value (1) or overwrite it (0)
};

inline signed char coef_kind(double c) { return c == 0.0 ? 0 : (c == 1.0 ? 1 : (c == -1.0 ? -1 : 2)); }

template <typename I>
__device__ __forceinline__ I off5(const int64_t s[D], I i0, I i1, I i2, I i3, I i4) {
  return i0 * (I)s[0] + i1 * (I)s[1] + i2 * (I)s[2] + i3 * (I)s[3] + i4 * (I)s[4];
}

// -x by flipping the sign bit (an integer operation: an FP64 negation would
// occupy GB300's slow FP64 unit)
__device__ __forceinline__ double neg_bits(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}

// r_k from the loaded values; old[k] is out_k's value before the call
// (read only with accumulate)
template <int NIN, int NPROD, int NOUT>
__device__ __forceinline__ void finish(const CombineArgs& a, const double* xv, double pv, const double* old,
                                       double* const* o) {
#pragma unroll
  for (int k = 0; k < NOUT; ++k) {
    double acc = 0.0;
    bool first = true;
#pragma unroll
    for (int s = 0; s < NIN; ++s) {
      const int kind = a.cc[k][s];
      if (kind != 0) {
        const double term = kind == 1 ? xv[s] : (kind == -1 ? neg_bits(xv[s]) : a.c[k][s] * xv[s]);
        acc = first ? term : acc + term;
        first = false;
      }
    }
    if (NPROD > 0 && a.cc[k][NIN] != 0) {
      const int kind = a.cc[k][NIN];
      const double term = kind == 1 ? pv : (kind == -1 ? neg_bits(pv) : a.c[k][NIN] * pv);
      acc = first ? term : acc + term;
    }
    *o[k] = a.acc[k] ? old[k] + acc : acc;
  }
}

// Inputs read directly: each thread takes E elements a grid stride apart,
// loading all of them before storing any.
template <int NIN, int NPROD, int NOUT, typename I>
__global__ void __launch_bounds__(256) k_combine(const CombineArgs a) {
  constexpr int E = 4, NX = NIN > 0 ? NIN : 1;
  const I n = (I)a.n;
  const I stride = (I)gridDim.x * blockDim.x;
  for (I base = (I)blockIdx.x * blockDim.x + threadIdx.x; base < n; base += E * stride) {
    double xv[E][NX];
    double pv[E];
    double old[E][NOUT];
    double* op[E][NOUT];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const I t = base + (I)e * stride;
      pv[e] = 0.0;
      if (t >= n) continue;
      I r, i4, i3, i2, i1;
      if constexpr (sizeof(I) == 4) {
        r = a.f4.div(t);
        i4 = t - r * (I)a.d[4];
        I r2 = a.f3.div(r);
        i3 = r - r2 * (I)a.d[3];
        r = a.f2.div(r2);
        i2 = r2 - r * (I)a.d[2];
        r2 = a.f1.div(r);
        i1 = r - r2 * (I)a.d[1];
        r = r2;
      } else {
        i4 = t % a.d[4];
        r = t / a.d[4];
        i3 = r % a.d[3];
        r /= a.d[3];
        i2 = r % a.d[2];
        r /= a.d[2];
        i1 = r % a.d[1];
        r /= a.d[1];
      }
#pragma unroll
      for (int k = 0; k < NOUT; ++k) {
        op[e][k] = a.out[k] + off5<I>(a.so[k], r, i1, i2, i3, i4);
        old[e][k] = a.acc[k] ? *op[e][k] : 0.0;
      }
#pragma unroll
      for (int s = 0; s < NIN; ++s) xv[e][s] = __ldg(a.x[s] + off5<I>(a.sx[s], r, i1, i2, i3, i4));
      if (NPROD > 0) {
        double q = __ldg(a.p[0] + off5<I>(a.sp[0], r, i1, i2, i3, i4));
#pragma unroll
        for (int s = 1; s < NPROD; ++s) q = q * __ldg(a.p[s] + off5<I>(a.sp[s], r, i1, i2, i3, i4));
        pv[e] = q;
      }
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if (base + (I)e * stride >= n) continue;
      finish<NIN, NPROD, NOUT>(a, xv[e], pv[e], old[e], op[e]);
    }
  }
}

// Inputs contiguous along dimension 3 (the host moves the transposed
// dimension there): 32 x 32 tiles of the plane (3, 4).  Thread (x, y) of
// 32 x 8 stages element (i3 = x, i4 = y + 8 r) of every input and computes
// element (i4 = x, i3 = y + 8 r), r < 4.  Dimensions 0..2 run over
// blockIdx.y.
struct TileArgs {
  int64_t nt4;        // tiles along dimension 4
  int64_t ntiles;     // tiles in the (3, 4) plane
  int64_t nrest;      // dims[0] * dims[1] * dims[2]
};

template <int NIN, int NOUT, typename I>
__global__ void __launch_bounds__(256) k_combine_t(const CombineArgs a, const TileArgs ta) {
  extern __shared__ double sm[];  // [NIN][32][33]
  const int x = threadIdx.x & 31, y = threadIdx.x >> 5;
  const unsigned nt4 = (unsigned)ta.nt4;  // tiles along 4: a few (32-bit division)
  const I t4 = (I)(blockIdx.x % nt4), t3 = (I)(blockIdx.x / nt4);
  const I d3 = (I)a.d[3], d4 = (I)a.d[4];
  for (int64_t rest = blockIdx.y; rest < ta.nrest; rest += gridDim.y) {
    I i0, i1, i2;
    if constexpr (sizeof(I) == 4) {  // multiply-high divisions (every index < 2^31)
      const unsigned rr = (unsigned)rest;
      const unsigned q2 = a.f2.div(rr);
      i2 = rr - q2 * (unsigned)a.d[2];
      i0 = a.f1.div(q2);
      i1 = q2 - i0 * (unsigned)a.d[1];
    } else {
      i2 = (I)(rest % a.d[2]);
      const int64_t r01 = rest / a.d[2];
      i1 = (I)(r01 % a.d[1]);
      i0 = (I)(r01 / a.d[1]);
    }
    __syncthreads();  // the previous tile's reads of shared memory are done
    double v[NIN][4];
#pragma unroll
    for (int s = 0; s < NIN; ++s)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const I i3 = t3 * 32 + x, i4 = t4 * 32 + y + 8 * r;
        v[s][r] = (i3 < d3 && i4 < d4) ? __ldg(a.x[s] + off5<I>(a.sx[s], i0, i1, i2, i3, i4)) : 0.0;
      }
#pragma unroll
    for (int s = 0; s < NIN; ++s)
#pragma unroll
      for (int r = 0; r < 4; ++r) sm[(s * 32 + x) * 33 + y + 8 * r] = v[s][r];
    // the outputs' old values (with accumulate) are read before any store
    double old[4][NOUT];
    double* op[4][NOUT];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const I i4 = t4 * 32 + x, i3 = t3 * 32 + y + 8 * r;
      const bool in = i4 < d4 && i3 < d3;
#pragma unroll
      for (int k = 0; k < NOUT; ++k) {
        op[r][k] = a.out[k] + (in ? off5<I>(a.so[k], i0, i1, i2, i3, i4) : (I)0);
        old[r][k] = (a.acc[k] && in) ? *op[r][k] : 0.0;
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const I i4 = t4 * 32 + x, i3 = t3 * 32 + y + 8 * r;
      if (i4 >= d4 || i3 >= d3) continue;
      double xv[NIN];
#pragma unroll
      for (int s = 0; s < NIN; ++s) xv[s] = sm[(s * 32 + y + 8 * r) * 33 + x];
      finish<NIN, 0, NOUT>(a, xv, 0.0, old[r], op[r]);
    }
  }
}

template <int NIN, int NPROD, typename I>
void launch_direct(const CombineArgs& a, int n_out, unsigned grid, cudaStream_t st) {
  switch (n_out) {
    case 1: k_combine<NIN, NPROD, 1, I><<<grid, 256, 0, st>>>(a); break;
    case 2: k_combine<NIN, NPROD, 2, I><<<grid, 256, 0, st>>>(a); break;
    default: k_combine<NIN, NPROD, 3, I><<<grid, 256, 0, st>>>(a); break;
  }
}

template <int NIN, typename I>
void launch_direct_p(const CombineArgs& a, int n_prod, int n_out, unsigned grid, cudaStream_t st) {
  switch (n_prod) {
    case 0: launch_direct<NIN, 0, I>(a, n_out, grid, st); break;
    case 1: launch_direct<NIN, 1, I>(a, n_out, grid, st); break;
    case 2: launch_direct<NIN, 2, I>(a, n_out, grid, st); break;
    default: launch_direct<NIN, 3, I>(a, n_out, grid, st); break;
  }
}

template <typename I>
void launch_direct_all(const CombineArgs& a, int n_in, int n_prod, int n_out, unsigned grid, cudaStream_t st) {
  switch (n_in) {
    case 0: launch_direct_p<0, I>(a, n_prod, n_out, grid, st); break;
    case 1: launch_direct_p<1, I>(a, n_prod, n_out, grid, st); break;
    case 2: launch_direct_p<2, I>(a, n_prod, n_out, grid, st); break;
    case 3: launch_direct_p<3, I>(a, n_prod, n_out, grid, st); break;
    case 4: launch_direct_p<4, I>(a, n_prod, n_out, grid, st); break;
    default: launch_direct_p<5, I>(a, n_prod, n_out, grid, st); break;
  }
}

template <int NIN, typename I>
void launch_tiled_o(const CombineArgs& a, int n_out, const TileArgs& ta, cudaStream_t st) {
  const dim3 g((unsigned)ta.ntiles, (unsigned)(ta.nrest < 65535 ? ta.nrest : 65535));
  const size_t smem = (size_t)NIN * 32 * 33 * sizeof(double);
  switch (n_out) {
    case 1: k_combine_t<NIN, 1, I><<<g, 256, smem, st>>>(a, ta); break;
    case 2: k_combine_t<NIN, 2, I><<<g, 256, smem, st>>>(a, ta); break;
    default: k_combine_t<NIN, 3, I><<<g, 256, smem, st>>>(a, ta); break;
  }
}

template <typename I>
void launch_tiled(const CombineArgs& a, int n_in, int n_out, const TileArgs& ta, cudaStream_t st) {
  switch (n_in) {
    case 1: launch_tiled_o<1, I>(a, n_out, ta, st); break;
    case 2: launch_tiled_o<2, I>(a, n_out, ta, st); break;
    case 3: launch_tiled_o<3, I>(a, n_out, ta, st); break;
    case 4: launch_tiled_o<4, I>(a, n_out, ta, st); break;
    default: launch_tiled_o<5, I>(a, n_out, ta, st); break;
  }
}

// the largest element offset a view reaches (INT64_MAX for a negative
// stride, which the 32-bit path cannot take)
int64_t reach(const int64_t d[D], const int64_t s[D]) {
  int64_t r = 0;
  for (int k = 0; k < D; ++k) {
    if (s[k] < 0) return INT64_MAX;
    r += (d[k] - 1) * s[k];
  }
  return r;
}

}  // namespace

int fricc_combine_device(const int64_t dims[5], int n_in, const double* const* x, const int64_t* sx, int n_prod,
                         const double* const* p, const int64_t* sp, int n_out, double* const* out, const int64_t* so,
                         const double* coef, int accumulate, cudaStream_t st) {
  if (!dims || n_in < 0 || n_in > kMaxIn || n_prod < 0 || n_prod > kMaxProd || n_out < 1 || n_out > kMaxOut ||
      (n_in > 0 && (!x || !sx)) || (n_prod > 0 && (!p || !sp)) || !out || !so || !coef ||
      n_in + (n_prod > 0 ? 1 : 0) == 0) {
    fricc_set_error("combine: bad arguments");
    return FRICC_ERR_ARG;
  }
  int64_t n = 1;
  for (int d = 0; d < D; ++d) {
    if (dims[d] < 0) {
      fricc_set_error("combine: negative dimension");
      return FRICC_ERR_ARG;
    }
    n *= dims[d];
  }
  if (n == 0) return FRICC_OK;
  for (int s = 0; s < n_in; ++s)
    if (!x[s]) {
      fricc_set_error("combine: null input %d", s);
      return FRICC_ERR_ARG;
    }
  for (int s = 0; s < n_prod; ++s)
    if (!p[s]) {
      fricc_set_error("combine: null product factor %d", s);
      return FRICC_ERR_ARG;
    }
  for (int k = 0; k < n_out; ++k)
    if (!out[k]) {
      fricc_set_error("combine: null output %d", k);
      return FRICC_ERR_ARG;
    }
  const int nc = n_in + (n_prod > 0 ? 1 : 0);

  // group the inputs by layout: -1 read directly (contiguous along 4,
  // broadcast or scattered), d in 0..3 contiguous along d (tiled)
  int group[kMaxIn];
  for (int s = 0; s < n_in; ++s) {
    group[s] = -1;
    const int64_t* st5 = sx + D * s;
    if (st5[4] == 1 || st5[4] == 0 || dims[4] < 8) continue;
    for (int d = 0; d < 4; ++d)
      if (st5[d] == 1 && dims[d] >= 8) {
        group[s] = d;
        break;
      }
  }
  // Each output is written by the first pass that contributes to it
  // (added to, with accumulate) and added to by later ones; a pass leaves
  // out the outputs it contributes nothing to.  An output no input reaches
  // is zeroed (or left as it is, with accumulate) by the first pass.
  bool touched[kMaxOut];
  bool reached[kMaxOut];
  for (int k = 0; k < n_out; ++k) {
    touched[k] = accumulate != 0;
    reached[k] = false;
    for (int t = 0; t < nc; ++t) reached[k] = reached[k] || coef[k * nc + t] != 0.0;
  }
  bool first_pass = true;
  for (int gsel = -1; gsel < 4; ++gsel) {
    int members[kMaxIn], nm = 0;
    for (int s = 0; s < n_in; ++s)
      if (group[s] == gsel) members[nm++] = s;
    const bool with_prod = gsel == -1 && n_prod > 0;
    if (nm == 0 && !with_prod) continue;
    int outs[kMaxOut], no = 0;
    for (int k = 0; k < n_out; ++k) {
      bool contributes = with_prod && coef[k * nc + n_in] != 0.0;
      for (int j = 0; j < nm; ++j) contributes = contributes || coef[k * nc + members[j]] != 0.0;
      if (contributes || (first_pass && !reached[k] && !touched[k])) outs[no++] = k;
    }
    if (no == 0) continue;
    CombineArgs a{};
    // dimension order: the tiled dimension moves to position 3
    int order[D] = {0, 1, 2, 3, 4};
    if (gsel >= 0) {
      int nr = 0;
      for (int d = 0; d < 4; ++d)
        if (d != gsel) order[nr++] = d;
      order[3] = gsel;
      // the three remaining dimensions, walked by consecutive tiles, in the
      // first input's memory order (its smallest stride fastest; a
      // broadcast dimension, stride 0, slowest), so that tiles running at
      // once read neighbouring memory
      const int64_t* s0 = sx + D * members[0];
      auto key = [&](int d) { return s0[d] == 0 ? INT64_MAX : (s0[d] < 0 ? -s0[d] : s0[d]); };
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2 - a; ++b) {
          const int64_t sa = key(order[b]), sb = key(order[b + 1]);
          if (sa < sb) {
            const int t = order[b];
            order[b] = order[b + 1];
            order[b + 1] = t;
          }
        }
    }
    for (int d = 0; d < D; ++d) a.d[d] = dims[order[d]];
    a.n = n;
    for (int j = 0; j < nm; ++j) {
      a.x[j] = x[members[j]];
      for (int d = 0; d < D; ++d) a.sx[j][d] = sx[D * members[j] + order[d]];
    }
    if (with_prod)
      for (int s = 0; s < n_prod; ++s) {
        a.p[s] = p[s];
        for (int d = 0; d < D; ++d) a.sp[s][d] = sp[D * s + order[d]];
      }
    for (int q = 0; q < no; ++q) {
      const int k = outs[q];
      a.out[q] = out[k];
      for (int d = 0; d < D; ++d) a.so[q][d] = so[D * k + order[d]];
      for (int j = 0; j < nm; ++j) {
        a.c[q][j] = coef[k * nc + members[j]];
        a.cc[q][j] = coef_kind(a.c[q][j]);
      }
      if (with_prod) {
        a.c[q][nm] = coef[k * nc + n_in];
        a.cc[q][nm] = coef_kind(a.c[q][nm]);
      }
      a.acc[q] = touched[k] ? 1 : 0;
      touched[k] = true;
    }
    const int n_out_pass = no;
    // 32-bit index arithmetic when every count and offset fits
    bool narrow = n < (int64_t(1) << 31);
    for (int j = 0; j < nm && narrow; ++j) narrow = reach(a.d, a.sx[j]) < (int64_t(1) << 31);
    for (int s = 0; s < (with_prod ? n_prod : 0) && narrow; ++s) narrow = reach(a.d, a.sp[s]) < (int64_t(1) << 31);
    for (int q = 0; q < n_out_pass && narrow; ++q) narrow = reach(a.d, a.so[q]) < (int64_t(1) << 31);
    if (narrow) {
      a.f1.set((unsigned)a.d[1]);
      a.f2.set((unsigned)a.d[2]);
      a.f3.set((unsigned)a.d[3]);
      a.f4.set((unsigned)a.d[4]);
    }
    if (gsel < 0) {
      int64_t g = fricc_cdiv(n, 256 * 4);
      if (g > 152 * 32) g = 152 * 32;
      if (narrow) launch_direct_all<unsigned>(a, nm, with_prod ? n_prod : 0, n_out_pass, (unsigned)g, st);
      else launch_direct_all<int64_t>(a, nm, with_prod ? n_prod : 0, n_out_pass, (unsigned)g, st);
    } else {
      TileArgs ta{};
      ta.nt4 = fricc_cdiv(a.d[4], 32);
      ta.ntiles = ta.nt4 * fricc_cdiv(a.d[3], 32);
      ta.nrest = a.d[0] * a.d[1] * a.d[2];
      if (ta.ntiles > 0x7fffffff) {
        fricc_set_error("combine: tile grid too large");
        return FRICC_ERR_ARG;
      }
      if (narrow) launch_tiled<unsigned>(a, nm, n_out_pass, ta, st);
      else launch_tiled<int64_t>(a, nm, n_out_pass, ta, st);
    }
    fricc_note_launch();
    first_pass = false;
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FRICC_OK : fricc_cuda_fail(e, "combine", __FILE__, __LINE__);
}

// The 4-D form: a leading extent 1 and strides 0.
int fricc_combine4_device(const int64_t dims[4], int n_in, const double* const* x, const int64_t* sx, int n_prod,
                          const double* const* p, const int64_t* sp, int n_out, double* const* out, const int64_t* so,
                          const double* coef, int accumulate, cudaStream_t st) {
  if (!dims || n_in < 0 || n_in > kMaxIn || n_prod < 0 || n_prod > kMaxProd || n_out < 1 || n_out > kMaxOut ||
      (n_in > 0 && !sx) || (n_prod > 0 && !sp) || !so) {
    fricc_set_error("combine: bad arguments");
    return FRICC_ERR_ARG;
  }
  int64_t d5[D] = {1, dims[0], dims[1], dims[2], dims[3]};
  int64_t sx5[kMaxIn * D], sp5[kMaxProd * D], so5[kMaxOut * D];
  auto widen = [](const int64_t* s4, int64_t* s5, int cnt) {
    for (int t = 0; t < cnt; ++t) {
      s5[D * t] = 0;
      for (int d = 0; d < 4; ++d) s5[D * t + 1 + d] = s4[4 * t + d];
    }
  };
  widen(sx, sx5, n_in);
  widen(sp, sp5, n_prod);
  widen(so, so5, n_out);
  return fricc_combine_device(d5, n_in, x, sx5, n_prod, p, sp5, n_out, out, so5, coef, accumulate, st);
}
