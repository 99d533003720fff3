// Fused denominator update, correlation energy and step norm of one
// FRI-CCSD iteration:
//   t1 = t1num / eia,  t2 = t2num / (eia[i,a] + eia[j,b])   fri-cc fricc/friccsd.py:281-284
//   E  = 2 sum f_ia t1_ia + sum tau_ijab (2 (ia|jb) - (ib|ja)),  tau = t2 + t1 t1
//                                                             (CCSD energy, :427)
//        or, linearised (FRI-LCCSD, fricc/frilccsd.py:504-522), tau = t2
//   normt = || vec(t1,t2) - vec(t1old,t2old) ||, vec = t1 and the lower
//           triangle of t2 seen as an (ia, jb) matrix          (:418-420)
// One pass over t2num, ovov and t2old; (ib|ja) is read through a shared
// memory transpose so every global access is coalesced.  The reductions
// use a fixed tree, so results are run-to-run deterministic.
#include "common.cuh"

namespace {

constexpr int TB = 32;  // (a,b) tile edge

template <bool LIN>
__global__ void __launch_bounds__(256) k_t2_energy(const double* __restrict__ t2num, const double* __restrict__ t1,
                                                   const double* __restrict__ eia, const double* __restrict__ ovov,
                                                   const double* __restrict__ t2old, double* __restrict__ t2out,
                                                   int64_t o, int64_t v, double* __restrict__ part_e,
                                                   double* __restrict__ part_n, int64_t np = 0) {
  // replica batches: replica blockIdx.z's amplitudes follow o v (t1) and
  // o^2 v^2 (t2) elements after the previous replica's; np partial sums each
  {
    const int64_t r = blockIdx.z, n2 = o * o * v * v;
    t2num += r * n2;
    t1 += r * o * v;
    t2old += r * n2;
    t2out += r * n2;
    part_e += r * np;
    part_n += r * np;
  }
  __shared__ double xt[TB][TB + 1];  // xt[b][a] = (ib|ja)
  __shared__ double red[32];
  const int64_t ij = blockIdx.y;
  const int64_t i = ij / o, j = ij % o;
  const int64_t ntb = fricc_cdiv(v, TB);
  const int64_t a0 = (blockIdx.x / ntb) * TB, b0 = (blockIdx.x % ntb) * TB;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  // stage (ib|ja) for b in the tile rows, a in the tile columns
  for (int r = ty; r < TB; r += 8) {
    const int64_t b = b0 + r, a = a0 + tx;
    xt[r][tx] = (b < v && a < v) ? ovov[((i * v + b) * o + j) * v + a] : 0.0;
  }
  __syncthreads();
  double e_acc = 0.0, n_acc = 0.0;
  for (int r = ty; r < TB; r += 8) {
    const int64_t a = a0 + r, b = b0 + tx;
    if (a < v && b < v) {
      const int64_t idx = ((i * o + j) * v + a) * v + b;
      const double t2 = t2num[idx] / (eia[i * v + a] + eia[j * v + b]);
      t2out[idx] = t2;
      const double tau = LIN ? t2 : t2 + t1[i * v + a] * t1[j * v + b];
      const double iajb = ovov[((i * v + a) * o + j) * v + b];
      e_acc += tau * (2.0 * iajb - xt[tx][r]);
      if (i * v + a >= j * v + b) {
        const double d = t2 - t2old[idx];
        n_acc += d * d;
      }
    }
  }
  const double es = block_sum_det(e_acc, red);
  const double ns = block_sum_det(n_acc, red);
  if (threadIdx.x == 0) {
    const int64_t bid = blockIdx.y * gridDim.x + blockIdx.x;
    part_e[bid] = es;
    part_n[bid] = ns;
  }
}

__global__ void __launch_bounds__(256) k_t1(const double* __restrict__ t1num, const double* __restrict__ eia,
                                            const double* __restrict__ fov, const double* __restrict__ t1old,
                                            double* __restrict__ t1out, int64_t nov, double* __restrict__ res) {
  t1num += blockIdx.x * nov;  // replica blockIdx.x (one block per replica)
  t1old += blockIdx.x * nov;
  t1out += blockIdx.x * nov;
  res += 4 * blockIdx.x;
  __shared__ double red[32];
  double e = 0.0, n = 0.0;
  for (int64_t k = threadIdx.x; k < nov; k += 256) {
    const double t = t1num[k] / eia[k];
    t1out[k] = t;
    e += fov[k] * t;
    const double d = t - t1old[k];
    n += d * d;
  }
  const double es = block_sum_det(e, red);
  const double ns = block_sum_det(n, red);
  if (threadIdx.x == 0) {
    res[2] = 2.0 * es;
    res[3] = ns;
  }
}

__global__ void __launch_bounds__(256) k_final(const double* __restrict__ part_e, const double* __restrict__ part_n,
                                               int64_t np, double* __restrict__ res) {
  part_e += blockIdx.x * np;  // replica blockIdx.x (one block per replica)
  part_n += blockIdx.x * np;
  res += 4 * blockIdx.x;
  __shared__ double red[32];
  double e = 0.0, n = 0.0;
  for (int64_t k = threadIdx.x; k < np; k += 256) {
    e += part_e[k];
    n += part_n[k];
  }
  const double es = block_sum_det(e, red);
  const double ns = block_sum_det(n, red);
  if (threadIdx.x == 0) {
    res[0] = res[2] + es;       // E_corr
    res[1] = sqrt(res[3] + ns);  // normt
  }
}

}  // namespace

// res (device, 4 doubles): [E_corr, normt, scratch, scratch].  t1out/t2out
// may alias t1num/t2num.
int fricc_energy_update_device(const double* t1num, const double* t2num, const double* eia, const double* fov,
                               const double* ovov, const double* t1old, const double* t2old, int64_t o, int64_t v,
                               double* t1out, double* t2out, double* res, cudaStream_t st, bool linear) {
  if (o <= 0 || v <= 0) {
    fricc_set_error("energy_update: empty system");
    return FRICC_ERR_ARG;
  }
  const int64_t ntb = fricc_cdiv(v, TB);
  const int64_t gx = ntb * ntb, gy = o * o;
  if (gy > 65535) {
    fricc_set_error("energy_update: nocc too large");
    return FRICC_ERR_ARG;
  }
  double* part = nullptr;
  int rc = fricc_alloc_t(&part, 2 * gx * gy, st);
  if (rc) return rc;
  k_t1<<<1, 256, 0, st>>>(t1num, eia, fov, t1old, t1out, o * v, res);
  const dim3 grid((unsigned)gx, (unsigned)gy);
  if (linear)
    k_t2_energy<true><<<grid, 256, 0, st>>>(t2num, t1out, eia, ovov, t2old, t2out, o, v, part, part + gx * gy);
  else
    k_t2_energy<false><<<grid, 256, 0, st>>>(t2num, t1out, eia, ovov, t2old, t2out, o, v, part, part + gx * gy);
  k_final<<<1, 256, 0, st>>>(part, part + gx * gy, gx * gy, res);
  fricc_note_launch(3);
  cudaError_t e = cudaGetLastError();
  fricc_free(part, st);
  if (e != cudaSuccess) return fricc_cuda_fail(e, "energy_update", __FILE__, __LINE__);
  return FRICC_OK;
}

// R replicas at once: t1num/t1old/t1out [R][o][v], t2num/t2old/t2out
// [R][o][o][v][v], res [R][4]; eia, fov and ovov shared.  Each replica's
// arithmetic is that of its own call (the same reduction trees).
int fricc_energy_update_batch_device(int R, const double* t1num, const double* t2num, const double* eia,
                                     const double* fov, const double* ovov, const double* t1old, const double* t2old,
                                     int64_t o, int64_t v, double* t1out, double* t2out, double* res,
                                     cudaStream_t st) {
  if (o <= 0 || v <= 0 || R < 1 || R > 65535) {
    fricc_set_error("energy_update_batch: bad arguments");
    return FRICC_ERR_ARG;
  }
  const int64_t ntb = fricc_cdiv(v, TB);
  const int64_t gx = ntb * ntb, gy = o * o;
  if (gy > 65535) {
    fricc_set_error("energy_update_batch: nocc too large");
    return FRICC_ERR_ARG;
  }
  double* part = nullptr;
  const int64_t np = gx * gy;
  int rc = fricc_alloc_t(&part, (size_t)2 * np * R, st);
  if (rc) return rc;
  k_t1<<<R, 256, 0, st>>>(t1num, eia, fov, t1old, t1out, o * v, res);
  const dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)R);
  k_t2_energy<false><<<grid, 256, 0, st>>>(t2num, t1out, eia, ovov, t2old, t2out, o, v, part, part + np * R, np);
  k_final<<<R, 256, 0, st>>>(part, part + np * R, np, res);
  fricc_note_launch(3);
  cudaError_t e = cudaGetLastError();
  fricc_free(part, st);
  if (e != cudaSuccess) return fricc_cuda_fail(e, "energy_update_batch", __FILE__, __LINE__);
  return FRICC_OK;
}
