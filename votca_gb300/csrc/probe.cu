// FP64 FMA throughput probe: the FP64 roofline denominator (MEASURED_PEAKS has
// only HBM and bf16 figures).  Each thread runs 8 independent FMA chains in
// registers; one store per thread keeps the work alive.
#include "common.cuh"

namespace vgb {

namespace {
__global__ void fma64_kernel(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
         x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

double probe_fp64_tflops() {
  const int blocks = sm_count() * 8, threads = 256, iters = 1 << 13;
  DeviceBuffer<double> out((size_t)blocks * threads);
  cudaStream_t s;
  VGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  fma64_kernel<<<blocks, threads, 0, s>>>(out.get(), 64, 0.999, 0.001);
  VGB_LAUNCH_CHECK();
  cudaEvent_t e0, e1;
  VGB_CUDA(cudaEventCreate(&e0));
  VGB_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    VGB_CUDA(cudaEventRecord(e0, s));
    fma64_kernel<<<blocks, threads, 0, s>>>(out.get(), iters, 0.999, 0.001);
    VGB_LAUNCH_CHECK();
    VGB_CUDA(cudaEventRecord(e1, s));
    VGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    VGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace vgb
