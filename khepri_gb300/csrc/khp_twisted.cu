// Twisted bilayers (extended RCWA over a product expansion): R and T from the base solves.
//
// Reference path: Expansion.__add__ / rotate (khepri/expansion.py:52-73), ExtendedLayer.solve and
// joint_subspace (khepri/extension.py:10-111), then the ordinary chain and fluxes of the
// extended crystal (crystal.py:180-206, 363-396) at 2 N^2 unknowns per side.
//
// Here the chain is re-associated (star products are associative): every layer on the first
// expansion e1 (incidence half-space, lower layers, and the uniform layers of the product
// expansion, whose S-matrices are diagonal per harmonic) is block-diagonal in the "kind 1"
// ordering and is chained at base size 2N per shift; every layer on e2 (upper layers, emergence
// half-space) likewise in the "kind 0" ordering.  With A = left chain and B = right chain
// (extended, block-diagonal in the two orderings), only the final product is dense:
//   t = B21 (I - A22 B11)^-1 A21 c,   r = A11 c + A12 B11 (I - A22 B11)^-1 A21 c
// (the two source columns c at the centre harmonic).  Because A22 and B11 are block-diagonal in
// orthogonal orderings, every entry of A22 B11 is a sum of two products (O(n^2) to form); the
// one O(n^3) step is the LU of D = I - A22 B11, n = 2 N^2.
//
// Extended index of (polarisation s, e1 harmonic p, e2 harmonic q): s N^2 + p N + q
// (expansion.py:60-74: the left operand's vectors vary slowest).  Base index: s N + a.
//   A (kind 1): A_ext[(s,p,q)][(s',p',q)] = A_q[s N + p][s' N + p']   (q: shift of the e1 solves)
//   B (kind 0): B_ext[(s,p,q)][(s',p,q')] = B_p[s N + q][s' N + q']   (p: shift of the e2 solves)
#include <cuda_runtime.h>

#include <algorithm>

#include "khepri_gb300.h"
#include "khp_gamma_kernels.cuh"
#include "khp_launch.h"

namespace khp {
namespace {

// One base S-matrix block (row-major [2][2][nb][nb], nb = 2N) of shift m of problem b.
__device__ __forceinline__ const cd* sblk(const cd* S, int64_t b, int N, int m, int blk) {
  const int64_t nb = 2 * (int64_t)N;
  return S + ((b * N + m) * 4 + blk) * nb * nb;
}

// D = I - A22 B11 (extended), one thread per element.
__global__ void k_twist_d(int64_t batch, int N, const cd* __restrict__ A, const cd* __restrict__ B, cd* D) {
  const int64_t NN = (int64_t)N * N, n = 2 * NN, nn = n * n, nb = 2 * (int64_t)N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int64_t rc = e % nn;
    const int64_t r = rc / n, c = rc % n;
    const int s = (int)(r / NN), p = (int)((r % NN) / N), q = (int)(r % N);
    const int s2 = (int)(c / NN), p2 = (int)((c % NN) / N), q2 = (int)(c % N);
    const cd* A22 = sblk(A, b, N, q, 3);
    const cd* B11 = sblk(B, b, N, p2, 0);
    cd acc = mk(0.0);
    for (int s1 = 0; s1 < 2; ++s1)
      acc += A22[(s * N + p) * nb + s1 * N + p2] * B11[(s1 * N + q) * nb + s2 * N + q2];
    D[e] = (r == c ? mk(1.0) : mk(0.0)) - acc;
  }
}

// X = A21 c for the two unit sources at the centre (columns: x, y polarisation), [batch][n][2].
__global__ void k_twist_rhs(int64_t batch, int N, const cd* __restrict__ A, cd* X) {
  const int64_t NN = (int64_t)N * N, n = 2 * NN, nb = 2 * (int64_t)N;
  const int cen = (N - 1) / 2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n * 2; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / (n * 2);
    const int64_t r = (e / 2) % n;
    const int col = (int)(e % 2);
    const int s = (int)(r / NN), p = (int)((r % NN) / N), q = (int)(r % N);
    cd v = mk(0.0);
    if (q == cen) v = sblk(A, b, N, cen, 2)[(s * N + p) * nb + col * N + cen];
    X[e] = v;
  }
}

// U = B_blk X (block blk of the right chain, kind 0), two columns.
__global__ void k_twist_bx(int64_t batch, int N, const cd* __restrict__ B, int blk, const cd* __restrict__ X, cd* U) {
  const int64_t NN = (int64_t)N * N, n = 2 * NN, nb = 2 * (int64_t)N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n * 2; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / (n * 2);
    const int64_t r = (e / 2) % n;
    const int col = (int)(e % 2);
    const int s = (int)(r / NN), p = (int)((r % NN) / N), q = (int)(r % N);
    const cd* Bp = sblk(B, b, N, p, blk);
    const cd* xb = X + b * n * 2;
    cd acc = mk(0.0);
    for (int s1 = 0; s1 < 2; ++s1)
      for (int q1 = 0; q1 < N; ++q1) acc += Bp[(s * N + q) * nb + s1 * N + q1] * xb[(s1 * NN + p * N + q1) * 2 + col];
    U[e] = acc;
  }
}

// R = A11 c + A12 U (left chain, kind 1), two columns.
__global__ void k_twist_r(int64_t batch, int N, const cd* __restrict__ A, const cd* __restrict__ U, cd* Rv) {
  const int64_t NN = (int64_t)N * N, n = 2 * NN, nb = 2 * (int64_t)N;
  const int cen = (N - 1) / 2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n * 2; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / (n * 2);
    const int64_t r = (e / 2) % n;
    const int col = (int)(e % 2);
    const int s = (int)(r / NN), p = (int)((r % NN) / N), q = (int)(r % N);
    const cd* A12 = sblk(A, b, N, q, 1);
    const cd* ub = U + b * n * 2;
    cd acc = q == cen ? sblk(A, b, N, cen, 0)[(s * N + p) * nb + col * N + cen] : mk(0.0);
    for (int s1 = 0; s1 < 2; ++s1)
      for (int p1 = 0; p1 < N; ++p1) acc += A12[(s * N + p) * nb + s1 * N + p1] * ub[(s1 * NN + p1 * N + q) * 2 + col];
    Rv[e] = acc;
  }
}

struct TwistPlan {
  cd *D, *X, *U, *Rv, *Tv;
  int* piv;
};

template <class Arena>
TwistPlan plan_twist(Arena& a, int64_t batch, int N) {
  const size_t n = 2 * (size_t)N * N;
  TwistPlan p;
  p.D = a.template take<cd>(batch * n * n);
  p.X = a.template take<cd>(batch * n * 2);
  p.U = a.template take<cd>(batch * n * 2);
  p.Rv = a.template take<cd>(batch * n * 2);
  p.Tv = a.template take<cd>(batch * n * 2);
  p.piv = a.template take<int>(batch * n);
  return p;
}

struct TArena {
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

#define TW_TRY(x)        \
  do {                   \
    const int _s = (x);  \
    if (_s) return _s;   \
  } while (0)
#define TW_EW(kernel, total, ...)                                        \
  do {                                                                   \
    kernel<<<grid_for(total), 256, 0, s>>>(__VA_ARGS__);                 \
    count_launches(1);                                                   \
    TW_TRY(cuda_status());                                               \
  } while (0)

}  // namespace
}  // namespace khp

using namespace khp;

extern "C" {

size_t khp_twisted_rt_workspace(int64_t batch, int32_t nbase) {
  if (batch < 0 || nbase < 1) return 0;
  TArena a{nullptr, 0};
  plan_twist(a, batch, nbase);
  return a.off;
}

int khp_twisted_rt(int64_t batch, int32_t nbase, const double* s_left, const double* s_right, const double* gx,
                   const double* gy, const double* kp, const double* k0, int32_t npol, const double* te,
                   const double* tm, double epsi_re, double epsi_im, double epse_re, double epse_im, double* R,
                   double* T, double* rv, double* tv, int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (batch < 0 || nbase < 1 || npol < 1 || !s_left || !s_right || !gx || !gy || !kp || !k0 || !te || !tm || !R ||
      !T || !status)
    return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  TArena a{static_cast<char*>(workspace), ws_bytes};
  TwistPlan p = plan_twist(a, batch, nbase);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int N = nbase;
  const int n = 2 * N * N;
  const int64_t nn = (int64_t)n * n;
  const cd* A = reinterpret_cast<const cd*>(s_left);
  const cd* B = reinterpret_cast<const cd*>(s_right);
  TW_EW(k_twist_d, batch * nn, batch, N, A, B, p.D);
  TW_EW(k_twist_rhs, batch * n * 2, batch, N, A, p.X);
  TW_TRY(launch_getrf_blocked<double>(batch, n, p.D, n, nn, p.piv, status, s));
  TW_TRY(launch_getrs_blocked<double>(batch, n, p.D, n, nn, p.piv, p.X, 2, (int64_t)n * 2, 2, s));
  cd* Tv = tv ? reinterpret_cast<cd*>(tv) : p.Tv;
  cd* Rv = rv ? reinterpret_cast<cd*>(rv) : p.Rv;
  TW_EW(k_twist_bx, batch * n * 2, batch, N, B, 2, p.X, Tv);   // t = B21 x
  TW_EW(k_twist_bx, batch * n * 2, batch, N, B, 0, p.X, p.U);  // u = B11 x
  TW_EW(k_twist_r, batch * n * 2, batch, N, A, p.U, Rv);       // r = A11 c + A12 u
  k_flux_cols<double><<<(unsigned)batch, 128, 0, s>>>(N * N, npol, Rv, Tv, gx, gy, kp, k0,
                                                       reinterpret_cast<const cd*>(te), reinterpret_cast<const cd*>(tm),
                                                       mk(epsi_re, epsi_im), mk(epse_re, epse_im), R, T);
  count_launches(1);
  return cuda_status();
}

}  // extern "C"
