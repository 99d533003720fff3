// Arithmetic peaks of the GPU that the library's roofline figures divide by
// where the machine's measured peaks (HBM copy, cuBLAS BF16) have no entry:
// the FP64 FMA rate (the FP64 contraction kernel's bound), the FP32 FMA rate
// (the FP32-pair kernels' bound: 12 FP32 instructions per pair multiply-add)
// and, for scale, FP64 mma.sync and a plain copy.  Each kernel runs
// independent FMA chains (no data dependence between them) so the pipe, not
// latency, bounds it; times are CUDA events around one launch (five for the
// copy) after a warm-up launch.  One JSON object per line on stdout.
//
// Build and run: python -m fricc_gb300.peaks
#include <cstdio>
#include <cuda_runtime.h>

#define CK(x)                                                                        \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) {                                                         \
      printf("{\"error\": \"%s\", \"line\": %d}\n", cudaGetErrorString(e_), __LINE__); \
      return 1;                                                                      \
    }                                                                                \
  } while (0)

// 16 independent DFMA chains per thread
__global__ void k_dfma16(double* out, int iters, double b, double c) {
  double a[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// 8 independent FFMA chains per thread
__global__ void k_ffma8(float* out, int iters) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3f + k;
  const float b = 0.9999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], b, c);
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// 4 independent m8n8k4 FP64 mma.sync accumulators per warp
__global__ void k_dmma(double* out, int iters) {
  double a = threadIdx.x * 1e-3, b = 0.5;
  double c[4][2] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c[0][0] + c[0][1] + c[1][0] + c[1][1] + c[2][0] + c[2][1] + c[3][0] + c[3][1];
}

__global__ void k_copy(const double4* __restrict__ a, double4* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) b[i] = a[i];
}

// time `reps` launches after a warm-up launch; *ms = their total
template <class F>
static int time_launch(F launch, float* ms, int reps = 1) {
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  launch();  // warm-up
  CK(cudaDeviceSynchronize());
  CK(cudaEventRecord(e0));
  for (int r = 0; r < reps; ++r) launch();
  CK(cudaEventRecord(e1));
  CK(cudaEventSynchronize(e1));
  CK(cudaGetLastError());
  CK(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 0;
}

int main() {
  cudaDeviceProp p;
  CK(cudaGetDeviceProperties(&p, 0));
  const int nsm = p.multiProcessorCount;
  printf("{\"device\": \"%s\", \"sms\": %d, \"cc\": \"%d.%d\"}\n", p.name, nsm, p.major, p.minor);
  float ms = 0.f;
  const int iters = 20000;
  for (int tpb : {128, 256, 512}) {
    for (int bps : {4, 8, 16}) {
      const int blocks = nsm * bps;
      double* d = nullptr;
      CK(cudaMalloc(&d, (size_t)blocks * tpb * sizeof(double)));
      if (time_launch([&] { k_dfma16<<<blocks, tpb>>>(d, iters, 0.999999, 1e-7); }, &ms)) return 1;
      printf("{\"kernel\": \"dfma16\", \"threads\": %d, \"ctas_per_sm\": %d, \"tflops\": %.4f}\n", tpb, bps,
             2.0 * 16 * iters * (double)blocks * tpb / (ms * 1e-3) / 1e12);
      CK(cudaFree(d));
    }
  }
  {
    const int blocks = nsm * 8, tpb = 256;
    float* f = nullptr;
    CK(cudaMalloc(&f, (size_t)blocks * tpb * sizeof(float)));
    if (time_launch([&] { k_ffma8<<<blocks, tpb>>>(f, iters); }, &ms)) return 1;
    printf("{\"kernel\": \"ffma8\", \"threads\": %d, \"ctas_per_sm\": 8, \"tflops\": %.3f}\n", tpb,
           2.0 * 8 * iters * (double)blocks * tpb / (ms * 1e-3) / 1e12);
    CK(cudaFree(f));
    double* d = nullptr;
    const int it2 = 2000;
    CK(cudaMalloc(&d, (size_t)blocks * tpb * sizeof(double)));
    if (time_launch([&] { k_dmma<<<blocks, tpb>>>(d, it2); }, &ms)) return 1;
    // per warp and mma: 8 x 8 x 4 multiply-adds
    printf("{\"kernel\": \"dmma_m8n8k4\", \"threads\": %d, \"ctas_per_sm\": 8, \"tflops\": %.3f}\n", tpb,
           2.0 * 8 * 8 * 4 * 4 * it2 * (double)blocks * tpb / 32 / (ms * 1e-3) / 1e12);
    CK(cudaFree(d));
  }
  {
    const size_t n = (size_t)1 << 26;  // 2 GiB per buffer
    double4 *a = nullptr, *b = nullptr;
    CK(cudaMalloc(&a, n * sizeof(double4)));
    CK(cudaMalloc(&b, n * sizeof(double4)));
    CK(cudaMemset(a, 0, n * sizeof(double4)));
    if (time_launch([&] { k_copy<<<nsm * 4, 512>>>(a, b, n); }, &ms, 5)) return 1;
    printf("{\"kernel\": \"copy\", \"gbs\": %.1f}\n", 5 * 2.0 * n * sizeof(double4) / (ms * 1e-3) / 1e9);
    CK(cudaFree(a));
    CK(cudaFree(b));
  }
  return 0;
}
