// Band structure from a scattering matrix: the generalized eigenproblem Sl v = w Sr v of
// khepri/eigentricks.py:5-55 (scattering_splitlr, scattering_det, scattering_eigenvalues).
//
// With S = [[S11, S12], [S21, S22]] in blocks of h = 2 ng (the [p, m] split of the reference),
//   Sl = [[S11, 0], [S21, -I]],   Sr = [[I, -S12], [0, -S22]],
// Sr is block upper triangular, invertible with S22, and
//   Sr^-1 Sl = [[S11 - S12 S22^-1 S21, S12 S22^-1], [-S22^-1 S21, S22^-1]],
// so the pencil's eigenpairs are those of this N x N matrix (N = 4 ng): one blocked inverse of
// S22, three products and one batched eigensolve instead of the QZ iteration of scipy's
// eig(Sl, Sr).  The reference's determinant, det(S11 - S12 S22^-1 S21) det(S22), reuses the
// Schur complement block.  A singular S22 (an infinite eigenvalue of the pencil) sets status
// SINGULAR for that problem.
#include <cuda_runtime.h>

#include <algorithm>

#include "khepri_gb300.h"
#include "khp_core.cuh"
#include "khp_launch.h"

namespace khp {
namespace {

using cd = cplx<double>;

struct EigPlan {
  cd *A, *Z, *W, *Di, *lu, *schur;
  int* piv;
};

struct EArena {
  char* base;
  size_t cap;
  size_t off = 0;
  bool ok = true;
  template <typename U>
  U* take(size_t count) {
    const size_t bytes = (count * sizeof(U) + 255) & ~size_t(255);
    U* p = base ? reinterpret_cast<U*>(base + off) : nullptr;
    off += bytes;
    if (base && off > cap) ok = false;
    return p;
  }
};

EigPlan plan_eig(EArena& a, int64_t batch, int ng) {
  const size_t N = 4 * (size_t)ng, h = 2 * (size_t)ng;
  EigPlan p;
  p.A = a.take<cd>(batch * N * N);
  p.Z = a.take<cd>(batch * N * N);
  p.W = a.take<cd>(batch * N * N);
  p.Di = a.take<cd>(batch * h * h);
  p.lu = a.take<cd>(batch * h * h);
  p.schur = a.take<cd>(batch * h * h);
  p.piv = a.take<int>(batch * N);
  return p;
}

// out[b] (*)= det of the LU factors: product of U's diagonal, sign from the row interchanges.
__global__ void k_det_from_lu(int64_t batch, int n, const cd* __restrict__ lu, int64_t bs, const int* __restrict__ piv,
                              cd* out, int multiply) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x) {
    cd d = mk(1.0);
    bool odd = false;
    const cd* L = lu + b * bs;
    for (int i = 0; i < n; ++i) {
      d = d * L[(int64_t)i * n + i];
      if (piv[b * n + i] != i) odd = !odd;
    }
    if (odd) d = -d;
    out[b] = multiply ? out[b] * d : d;
  }
}

// Non-finite entries anywhere in S (the reference returns None for NaN in Sl or Sr): status bit.
__global__ void k_flag_nonfinite(int64_t batch, int64_t count, const cd* __restrict__ S, int64_t bs, int* status) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / count;
    const cd v = S[b * bs + e % count];
    if (!isfinite(v.re) || !isfinite(v.im)) atomicOr(status + b, KHP_BIT_NONFINITE);
  }
}

inline unsigned blocks_for(int64_t total) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 32));
}

#define ET_TRY(x)       \
  do {                  \
    const int _s = (x); \
    if (_s) return _s;  \
  } while (0)

}  // namespace
}  // namespace khp

using namespace khp;

extern "C" {

size_t khp_scattering_eig_workspace(int64_t batch, int32_t ng) {
  if (batch < 0 || ng < 1) return 0;
  EArena a{nullptr, 0};
  plan_eig(a, batch, ng);
  return a.off;
}

int khp_scattering_eig(int64_t batch, int32_t ng, const double* S, int64_t s_stride, double* w, double* v,
                       double* det, int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (batch < 0 || ng < 1 || !S || !w || !status || s_stride < 16 * (int64_t)ng * ng) return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  EArena a{static_cast<char*>(workspace), ws_bytes};
  EigPlan p = plan_eig(a, batch, ng);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int N = 4 * ng, h = 2 * ng;
  const int64_t NN = (int64_t)N * N, hh = (int64_t)h * h;
  const cd* Sb = reinterpret_cast<const cd*>(S);
  const cd* S11 = Sb;
  const cd* S12 = Sb + h;
  const cd* S21 = Sb + (int64_t)h * N;
  const cd* S22 = Sb + (int64_t)h * N + h;
  const cd one = mk(1.0), mone = mk(-1.0), zero = mk(0.0);
  k_flag_nonfinite<<<blocks_for(batch * NN), 256, 0, s>>>(batch, NN, Sb, s_stride, status);
  count_launches(1);
  ET_TRY(cuda_status());
  // Di = S22^-1 (lu keeps the factors for det(S22))
  ET_TRY(launch_copy<double>(batch, h, h, S22, N, s_stride, p.lu, h, hh, s));
  ET_TRY(launch_inverse_blocked<double>(batch, h, p.lu, h, hh, p.Di, h, hh, p.piv, status, s));
  cd* A = p.A;
  cd* Atl = A;
  cd* Atr = A + h;
  cd* Abl = A + (int64_t)h * N;
  cd* Abr = A + (int64_t)h * N + h;
  ET_TRY(launch_gemm<double>(batch, h, h, h, one, S12, N, s_stride, p.Di, h, hh, zero, Atr, N, NN, s));   // X = S12 Di
  ET_TRY(launch_gemm<double>(batch, h, h, h, mone, p.Di, h, hh, S21, N, s_stride, zero, Abl, N, NN, s));  // -Di S21
  ET_TRY(launch_copy<double>(batch, h, h, S11, N, s_stride, Atl, N, NN, s));
  ET_TRY(launch_gemm<double>(batch, h, h, h, mone, Atr, N, NN, S21, N, s_stride, one, Atl, N, NN, s));   // S11 - X S21
  ET_TRY(launch_copy<double>(batch, h, h, p.Di, h, hh, Abr, N, NN, s));
  if (det) {
    cd* D = reinterpret_cast<cd*>(det);
    k_det_from_lu<<<blocks_for(batch), 256, 0, s>>>(batch, h, p.lu, hh, p.piv, D, 0);  // det(S22)
    count_launches(1);
    ET_TRY(cuda_status());
    ET_TRY(launch_copy<double>(batch, h, h, Atl, N, NN, p.schur, h, hh, s));
    ET_TRY(launch_getrf_blocked<double>(batch, h, p.schur, h, hh, p.piv, status, s));
    k_det_from_lu<<<blocks_for(batch), 256, 0, s>>>(batch, h, p.schur, hh, p.piv, D, 1);
    count_launches(1);
    ET_TRY(cuda_status());
  }
  cd* W = v ? reinterpret_cast<cd*>(v) : p.W;
  ET_TRY(launch_geev<double>(batch, N, A, N, NN, p.Z, W, N, NN, reinterpret_cast<cd*>(w), N, status, s));
  return KHP_OK;
}

}  // extern "C"
