// Batched dense complex kernels: one CTA per matrix for the factorisations and the eigensolver
// (team algorithms of khp_dense.cuh), a tiled kernel for the products, element-wise helpers.
#include <algorithm>

#include "khp_dense.cuh"
#include "khp_launch.h"

namespace khp {

namespace {

constexpr int kTeamThreads = 256;
constexpr int64_t kMaxGridY = 65535;

template <typename T>
__global__ void __launch_bounds__(kTeamThreads) k_getrf(int n, cplx<T>* A, int64_t lda, int64_t bsA, int* piv,
                                                         int* info) {
  __shared__ TeamShared sh;
  TeamCta t;
  const int64_t b = blockIdx.x;
  const int st = team_getrf(t, A + b * bsA, lda, n, piv + b * n, &sh);
  if (threadIdx.x == 0 && st) info[b] |= st;
}

template <typename T>
__global__ void __launch_bounds__(kTeamThreads) k_getrs(int n, const cplx<T>* A, int64_t lda, int64_t bsA,
                                                         const int* piv, cplx<T>* B, int64_t ldb, int64_t bsB,
                                                         int m) {
  TeamCta t;
  const int64_t b = blockIdx.x;
  team_getrs(t, A + b * bsA, lda, n, piv + b * n, B + b * bsB, ldb, m);
}

template <typename T>
__global__ void __launch_bounds__(kTeamThreads) k_geev(int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Z,
                                                        cplx<T>* W, int64_t ldw, int64_t bsW, cplx<T>* lam,
                                                        int64_t bsLam, int* info) {
  __shared__ TeamShared sh;
  __shared__ cplx<T> win[(KHP_HQR_WIN + 2) * (KHP_HQR_WIN + 2)];
  __shared__ cplx<T> rs[KHP_HQR_WIN];
  __shared__ T rc[KHP_HQR_WIN];
  extern __shared__ unsigned char dyn[];
  cplx<T>* vbuf = reinterpret_cast<cplx<T>*>(dyn);
  TeamCta t;
  const int64_t b = blockIdx.x;
  const int st = team_geev(t, A + b * bsA, lda, n, Z + b * (int64_t)n * n, n, W + b * bsW, ldw, lam + b * bsLam,
                           vbuf, win, rc, rs, &sh);
  if (threadIdx.x == 0 && st) info[b] |= st;
}

// Tiled product: CTA tile BM x BN, 256 threads as 16 x 16, each thread TM x TN outputs
// strided by 16 (conflict-free shared-memory reads).
template <typename T, int BM, int BN, int BK>
__global__ void __launch_bounds__(256) k_gemm(int n, int m, int k, cplx<T> alpha, const cplx<T>* __restrict__ A,
                                              int64_t lda, int64_t bsA, const cplx<T>* __restrict__ B, int64_t ldb,
                                              int64_t bsB, cplx<T> beta, cplx<T>* C, int64_t ldc, int64_t bsC,
                                              int64_t boff, const int* __restrict__ aidx) {
  constexpr int TM = BM / 16, TN = BN / 16;
  __shared__ cplx<T> As[BK][BM];
  __shared__ cplx<T> Bs[BK][BN];
  const int64_t b = blockIdx.z + boff;
  A += (aidx ? (int64_t)aidx[b] : b) * bsA;
  B += b * bsB;
  C += b * bsC;
  const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  cplx<T> acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = mk(T(0));
  for (int k0 = 0; k0 < k; k0 += BK) {
    for (int e = threadIdx.x; e < BM * BK; e += 256) {
      const int r = e / BK, c = e % BK;
      const int gr = row0 + r, gc = k0 + c;
      As[c][r] = (gr < n && gc < k) ? A[(int64_t)gr * lda + gc] : mk(T(0));
    }
    for (int e = threadIdx.x; e < BK * BN; e += 256) {
      const int r = e / BN, c = e % BN;
      const int gr = k0 + r, gc = col0 + c;
      Bs[r][c] = (gr < k && gc < m) ? B[(int64_t)gr * ldb + gc] : mk(T(0));
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      cplx<T> a[TM], bb[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) bb[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) fma_acc(acc[i][j], a[i], bb[j]);
    }
    __syncthreads();
  }
  const bool use_beta = !(beta.re == T(0) && beta.im == T(0));
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int r = row0 + ty + 16 * i;
    if (r >= n) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int c = col0 + tx + 16 * j;
      if (c >= m) continue;
      cplx<T> v = alpha * acc[i][j];
      if (use_beta) v += beta * C[(int64_t)r * ldc + c];
      C[(int64_t)r * ldc + c] = v;
    }
  }
}

template <typename T>
__global__ void k_copy(int n, int m, const cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* B, int64_t ldb,
                       int64_t bsB, int64_t boff) {
  const int64_t b = blockIdx.y + boff;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)n * m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / m), j = (int)(e % m);
    B[b * bsB + i * ldb + j] = A[b * bsA + i * lda + j];
  }
}

template <typename T>
__global__ void k_identity(int n, int m, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T> diag, int64_t boff) {
  const int64_t b = blockIdx.y + boff;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)n * m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / m), j = (int)(e % m);
    A[b * bsA + i * lda + j] = (i == j) ? diag : mk(T(0));
  }
}

template <typename T>
__global__ void k_axpby(int n, int m, cplx<T> a, const cplx<T>* A, int64_t lda, int64_t bsA, cplx<T> bcoef,
                        const cplx<T>* B, int64_t ldb, int64_t bsB, cplx<T>* C, int64_t ldc, int64_t bsC,
                        int64_t boff) {
  const int64_t b = blockIdx.y + boff;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)n * m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / m), j = (int)(e % m);
    C[b * bsC + i * ldc + j] = a * A[b * bsA + i * lda + j] + bcoef * B[b * bsB + i * ldb + j];
  }
}

inline int ew_blocks(int n, int m) {
  const int64_t e = (int64_t)n * m;
  return (int)std::min<int64_t>((e + 255) / 256, 64);
}

}  // namespace

template <typename T>
int launch_getrf(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, int* piv, int* info, cudaStream_t s) {
  if (batch <= 0) return KHP_OK;
  k_getrf<T><<<(unsigned)batch, kTeamThreads, 0, s>>>(n, A, lda, bsA, piv, info);
  count_launches(1);
  return cuda_status();
}

template <typename T>
int launch_getrs(int64_t batch, int n, const cplx<T>* A, int64_t lda, int64_t bsA, const int* piv, cplx<T>* B,
                 int64_t ldb, int64_t bsB, int m, cudaStream_t s) {
  if (batch <= 0) return KHP_OK;
  k_getrs<T><<<(unsigned)batch, kTeamThreads, 0, s>>>(n, A, lda, bsA, piv, B, ldb, bsB, m);
  count_launches(1);
  return cuda_status();
}

template <typename T>
int launch_gemm(int64_t batch, int n, int m, int k, cplx<T> alpha, const cplx<T>* A, int64_t lda, int64_t bsA,
                const cplx<T>* B, int64_t ldb, int64_t bsB, cplx<T> beta, cplx<T>* C, int64_t ldc, int64_t bsC,
                cudaStream_t s, const int* aidx) {
  if (batch <= 0 || n <= 0 || m <= 0) return KHP_OK;
  constexpr int BM = 32, BN = 32, BK = 16;
  for (int64_t off = 0; off < batch; off += kMaxGridY) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
    dim3 grid((m + BN - 1) / BN, (n + BM - 1) / BM, nb);
    k_gemm<T, BM, BN, BK><<<grid, 256, 0, s>>>(n, m, k, alpha, A, lda, bsA, B, ldb, bsB, beta, C, ldc, bsC, off,
                                                aidx);
    count_launches(1);
  }
  return cuda_status();
}

template <typename T>
int launch_geev(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Z, cplx<T>* W, int64_t ldw,
                int64_t bsW, cplx<T>* lam, int64_t bsLam, int* info, cudaStream_t s) {
  if (batch <= 0) return KHP_OK;
  const size_t smem = sizeof(cplx<T>) * (size_t)n;
  k_geev<T><<<(unsigned)batch, kTeamThreads, smem, s>>>(n, A, lda, bsA, Z, W, ldw, bsW, lam, bsLam, info);
  count_launches(1);
  return cuda_status();
}

template <typename T>
int launch_copy(int64_t batch, int n, int m, const cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* B, int64_t ldb,
                int64_t bsB, cudaStream_t s) {
  for (int64_t off = 0; off < batch; off += kMaxGridY) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
    k_copy<T><<<dim3(ew_blocks(n, m), nb), 256, 0, s>>>(n, m, A, lda, bsA, B, ldb, bsB, off);
    count_launches(1);
  }
  return cuda_status();
}

template <typename T>
int launch_identity(int64_t batch, int n, int m, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T> diag, cudaStream_t s) {
  for (int64_t off = 0; off < batch; off += kMaxGridY) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
    k_identity<T><<<dim3(ew_blocks(n, m), nb), 256, 0, s>>>(n, m, A, lda, bsA, diag, off);
    count_launches(1);
  }
  return cuda_status();
}

template <typename T>
int launch_axpby(int64_t batch, int n, int m, cplx<T> a, const cplx<T>* A, int64_t lda, int64_t bsA, cplx<T> b,
                 const cplx<T>* B, int64_t ldb, int64_t bsB, cplx<T>* C, int64_t ldc, int64_t bsC, cudaStream_t s) {
  for (int64_t off = 0; off < batch; off += kMaxGridY) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
    k_axpby<T><<<dim3(ew_blocks(n, m), nb), 256, 0, s>>>(n, m, a, A, lda, bsA, b, B, ldb, bsB, C, ldc, bsC, off);
    count_launches(1);
  }
  return cuda_status();
}

template <typename T>
int launch_inverse(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Ainv, int64_t ldi,
                   int64_t bsI, int* piv, int* info, cudaStream_t s) {
  int st = launch_identity<T>(batch, n, n, Ainv, ldi, bsI, mk(T(1)), s);
  if (st) return st;
  st = launch_getrf<T>(batch, n, A, lda, bsA, piv, info, s);
  if (st) return st;
  return launch_getrs<T>(batch, n, A, lda, bsA, piv, Ainv, ldi, bsI, n, s);
}

#define KHP_INSTANTIATE(T)                                                                                       \
  template int launch_getrf<T>(int64_t, int, cplx<T>*, int64_t, int64_t, int*, int*, cudaStream_t);             \
  template int launch_getrs<T>(int64_t, int, const cplx<T>*, int64_t, int64_t, const int*, cplx<T>*, int64_t,   \
                               int64_t, int, cudaStream_t);                                                     \
  template int launch_gemm<T>(int64_t, int, int, int, cplx<T>, const cplx<T>*, int64_t, int64_t, const cplx<T>*, \
                              int64_t, int64_t, cplx<T>, cplx<T>*, int64_t, int64_t, cudaStream_t, const int*); \
  template int launch_geev<T>(int64_t, int, cplx<T>*, int64_t, int64_t, cplx<T>*, cplx<T>*, int64_t, int64_t,  \
                              cplx<T>*, int64_t, int*, cudaStream_t);                                           \
  template int launch_copy<T>(int64_t, int, int, const cplx<T>*, int64_t, int64_t, cplx<T>*, int64_t, int64_t,  \
                              cudaStream_t);                                                                    \
  template int launch_identity<T>(int64_t, int, int, cplx<T>*, int64_t, int64_t, cplx<T>, cudaStream_t);        \
  template int launch_axpby<T>(int64_t, int, int, cplx<T>, const cplx<T>*, int64_t, int64_t, cplx<T>,           \
                               const cplx<T>*, int64_t, int64_t, cplx<T>*, int64_t, int64_t, cudaStream_t);     \
  template int launch_inverse<T>(int64_t, int, cplx<T>*, int64_t, int64_t, cplx<T>*, int64_t, int64_t, int*,    \
                                 int*, cudaStream_t);

KHP_INSTANTIATE(double)
KHP_INSTANTIATE(float)

}  // namespace khp
