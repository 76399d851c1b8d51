// Diagnostics of libkhp: a process-wide count of kernel launches made by the library, probes of
// the FP64 and FP32 FMA pipes' throughput (roofline denominators), and per-stage device timing.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <utility>
#include <vector>

#include "khepri_gb300.h"
#include "khp_launch.h"

namespace khp {

static std::atomic<long long> g_launches{0};

void count_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

namespace {
struct StageRecord {
  cudaEvent_t open = nullptr;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> done;
  double ms = 0.0;
  long long marks = 0;
};
std::atomic<bool> g_timing{false};
std::mutex g_stage_mu;
StageRecord g_stages[KHP_NUM_STAGES];

void drop_events(StageRecord& r) {
  if (r.open) cudaEventDestroy(r.open);
  for (auto& pr : r.done) {
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  r = StageRecord{};
}
}  // namespace

void stage_begin(int stage, cudaStream_t s) {
  if (!g_timing.load(std::memory_order_relaxed) || stage < 0 || stage >= KHP_NUM_STAGES) return;
  std::lock_guard<std::mutex> lk(g_stage_mu);
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, s);
  StageRecord& r = g_stages[stage];
  if (r.open) cudaEventDestroy(r.open);  // a begin without its end (an error return) is dropped
  r.open = e;
}

void stage_end(int stage, cudaStream_t s) {
  if (!g_timing.load(std::memory_order_relaxed) || stage < 0 || stage >= KHP_NUM_STAGES) return;
  std::lock_guard<std::mutex> lk(g_stage_mu);
  StageRecord& r = g_stages[stage];
  if (!r.open) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, s);
  r.done.emplace_back(r.open, e);
  r.open = nullptr;
}

namespace {
__global__ void k_fp32_fma(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
        x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

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

double khp_probe_fp32_tflops(float* scratch, int64_t scratch_floats, void* stream) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
  const int grid = sms * 8, block = 256, iters = 16384;
  if (!scratch || scratch_floats < (int64_t)grid * block) return -1.0;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -1.0;
  if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return -1.0; }
  khp::k_fp32_fma<<<grid, block, 0, s>>>(scratch, 64, 0.999f, 1e-3f);
  cudaEventRecord(e0, s);
  khp::k_fp32_fma<<<grid, block, 0, s>>>(scratch, iters, 0.999f, 1e-3f);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
  return 2.0 * 8.0 * iters * (double)grid * block / (ms * 1e-3) / 1e12;
}

int khp_stage_timing(int32_t enable) {
  std::lock_guard<std::mutex> lk(khp::g_stage_mu);
  for (auto& r : khp::g_stages) khp::drop_events(r);
  khp::g_timing.store(enable != 0);
  return KHP_OK;
}

int khp_stage_timing_read(int32_t stage, double* ms, int64_t* marks) {
  if (stage < 0 || stage >= KHP_NUM_STAGES || !ms || !marks) return KHP_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(khp::g_stage_mu);
  khp::StageRecord& r = khp::g_stages[stage];
  int code = KHP_OK;
  for (auto& pr : r.done) {
    float t = 0.f;
    if (cudaEventSynchronize(pr.second) != cudaSuccess || cudaEventElapsedTime(&t, pr.first, pr.second) != cudaSuccess)
      code = KHP_ERR_CUDA;
    else {
      r.ms += t;
      r.marks += 1;
    }
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  r.done.clear();
  *ms = r.ms;
  *marks = r.marks;
  return code;
}

}  // extern "C"
