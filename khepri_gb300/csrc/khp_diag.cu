// Diagnostics of libkhp: a process-wide count of kernel launches made by the library, and a
// probe of the FP64 FMA pipe's throughput (the roofline denominator for FP64-bound kernels).
#include <cuda_runtime.h>

#include <atomic>

#include "khepri_gb300.h"
#include "khp_launch.h"

namespace khp {

static std::atomic<long long> g_launches{0};

void count_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

namespace {
__global__ void k_fp64_fma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace
}  // namespace khp

extern "C" {

long long khp_launch_count(void) { return khp::g_launches.load(std::memory_order_relaxed); }

double khp_probe_fp64_tflops(double* scratch, int64_t scratch_doubles, void* stream) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
  const int grid = sms * 4, block = 256, iters = 8192;
  if (!scratch || scratch_doubles < (int64_t)grid * block) return -1.0;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -1.0;
  if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return -1.0; }
  khp::k_fp64_fma<<<grid, block, 0, s>>>(scratch, 64, 0.999, 1e-3);
  cudaEventRecord(e0, s);
  khp::k_fp64_fma<<<grid, block, 0, s>>>(scratch, iters, 0.999, 1e-3);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
  return 2.0 * 8.0 * iters * (double)grid * block / (ms * 1e-3) / 1e12;
}

}  // extern "C"
