// Star product for callers that cannot allocate device memory.
//
// Every other libkhp entry point takes its scratch from the caller (`workspace`).  Some callers
// cannot provide one: a host application whose device memory is fully partitioned up front
// (a fixed budget per solver instance, with no allocator it may call at solve time), or a
// latency-critical loop where a cudaMalloc/cudaFree pair, which can synchronise the whole
// device, is not allowed.  khp_star_product_noalloc serves them: its scratch is the
// file-scope device array below, of fixed size KHP_NOALLOC_SCRATCH_BYTES, which every GPU that
// loads libkhp holds until the process exits.  The call itself allocates nothing.
#include <cuda_runtime.h>

#include <mutex>

#include "khepri_gb300.h"

namespace {

static __device__ __align__(256) unsigned char g_star_scratch[KHP_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of g_star_scratch on the current device.  In host code the symbol's name is
// only a host-side stand-in, so the address is looked up once per device (with that device
// current) and cached.
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KHP_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return KHP_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_star_scratch) != cudaSuccess || !p) return KHP_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return KHP_OK;
}

}  // namespace

extern "C" int khp_star_product_noalloc(int64_t batch, int32_t n, const double* SA, int64_t sa_stride,
                                        const double* SB, int64_t sb_stride, double* S, int32_t* status,
                                        void* stream) {
  if (batch < 0 || n < 1 || !SA || !SB || !S || !status || sa_stride < 0 || sb_stride < 0) return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  if (khp_star_product_workspace(batch, n) > (size_t)KHP_NOALLOC_SCRATCH_BYTES) return KHP_ERR_TOO_LARGE;
  void* scratch = nullptr;
  const int st = scratch_address(&scratch);
  if (st != KHP_OK) return st;
  // The scratch needs no clearing: the star product writes every scratch element (identity,
  // products, pivots) before reading it.
  return khp_star_product(batch, n, SA, sa_stride, SB, sb_stride, S, status, scratch,
                          (size_t)KHP_NOALLOC_SCRATCH_BYTES, stream);
}
