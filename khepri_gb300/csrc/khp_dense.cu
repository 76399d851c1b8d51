// Batched dense complex kernels: one CTA per matrix for the factorisations and the eigensolver
// (team algorithms of khp_dense.cuh), a tiled kernel for the products, element-wise helpers.
#include <algorithm>

#include "khepri_gb300.h"
#include "khp_dense.cuh"
#include "khp_launch.h"

namespace khp {

namespace {

constexpr int kTeamThreads = 256;
constexpr int64_t kMaxGridY = 65535;

// Threads per eigensolver CTA by matrix size (khp_tune; 0 = kTeamThreads).  Small matrices leave
// most of a 256-thread team idle, and smaller teams let more matrices share an SM.
constexpr int kTuneMaxN = 4096;
int g_eig_threads[kTuneMaxN + 1] = {0};

int eig_threads(int n) {
  const int v = n <= kTuneMaxN ? g_eig_threads[n] : 0;
  return v > 0 ? v : kTeamThreads;
}

}  // namespace

// Smallest matrix size whose FP32 products in the mixed solve's recursion run as 3xTF32 on the
// tensor cores (khp_tune KHP_TUNE_TF32_MIN_N; 0 = never).  Below it the 128-row tiles are mostly
// padding and the SIMT product is faster.
int g_tf32_min_n = 128;
bool use_tf32_products(int n) { return g_tf32_min_n > 0 && n >= g_tf32_min_n; }

// Digits per operand of the eigen-refinement steps' M W products (khp_tune KHP_TUNE_MODE_DIGITS).
int g_mode_digits = 8;
int mode_step_digits() { return g_mode_digits; }

namespace {

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

// Hessenberg reduction, Q in Z: blocked (panels of KHP_GEHRD_NB reflectors, scratch in W) when
// the matrix is large enough for it, else one reflector at a time.
template <typename T>
__global__ void __launch_bounds__(kTeamThreads, 3) k_gehrd(int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Z,
                                                         int blocked) {
  __shared__ TeamShared sh;
  extern __shared__ unsigned char dyn[];
  TeamCta t;
  const int64_t b = blockIdx.x;
  if (blocked)
    team_gehrd_blocked(t, A + b * bsA, lda, n, Z + b * (int64_t)n * n, n, reinterpret_cast<cplx<T>*>(dyn), &sh);
  else
    team_gehrd(t, A + b * bsA, lda, n, Z + b * (int64_t)n * n, n, reinterpret_cast<cplx<T>*>(dyn), &sh);
}

// Schur form of the Hessenberg matrix and eigenvectors of the triangular factor (X left in A,
// Q in Z); the back-transform W = Z X runs afterwards as a batched tiled product.  With a log
// region (log_bytes per matrix at logbuf) Z's updates are logged and left for k_hqr_apply_log.
template <typename T>
__global__ void __launch_bounds__(kTeamThreads) k_geev_schur(int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Z,
                                                              cplx<T>* lam, int64_t bsLam, int* info,
                                                              unsigned char* logbuf, int64_t log_bytes) {
  __shared__ TeamShared sh;
  __shared__ cplx<T> win[(KHP_HQR_WIN + 2) * (KHP_HQR_WIN + 2)];
  __shared__ cplx<T> rs[KHP_HQR_WIN];
  __shared__ T rc[KHP_HQR_WIN];
  TeamCta t;
  const int64_t b = blockIdx.x;
  cplx<T>* Ab = A + b * bsA;
  cplx<T>* Zb = Z + b * (int64_t)n * n;
  int st;
  if (logbuf) {
    const HqrLog<T> L = hqr_log_view<T>(logbuf + b * log_bytes, log_bytes, n);
    st = team_hqr_win(t, Ab, lda, n, Zb, n, win, rc, rs, &sh, &L);
  } else {
    st = team_hqr_win(t, Ab, lda, n, Zb, n, win, rc, rs, &sh);
  }
  team_trevc(t, Ab, lda, n, lam + b * bsLam);
  if (threadIdx.x == 0 && st) info[b] |= st;
}

// The sweeps left in each matrix's rotation log applied to Z: a CTA of one warp holds
// kLogRows rows of Z in shared memory (one row per lane, row stride odd so the lanes' accesses
// fall in distinct banks) and rolls them through the logged rotations, which stream through a
// double-buffered shared-memory stage (cp.async, kLogChunk rotations per stage).  Every lane
// follows the same sweeps, so the control flow is uniform across the warp.
constexpr int kLogRows = 32;
constexpr int kLogChunk = 256;

template <typename T>
size_t apply_log_smem(int n) {
  return 2 * kLogChunk * sizeof(HqrRot<T>) + (size_t)kLogRows * (n | 1) * sizeof(cplx<T>);
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <typename T>
__global__ void __launch_bounds__(kLogRows) k_hqr_apply_log(int n, cplx<T>* Z, const unsigned char* logbuf,
                                                             int64_t log_bytes, int64_t boff) {
  extern __shared__ __align__(32) unsigned char dyn[];
  HqrRot<T>* stage = reinterpret_cast<HqrRot<T>*>(dyn);  // [2][kLogChunk]
  cplx<T>* rows = reinterpret_cast<cplx<T>*>(dyn + 2 * kLogChunk * sizeof(HqrRot<T>));
  const int lds = n | 1;
  const int64_t b = blockIdx.y + boff;
  const HqrLog<T> L = hqr_log_view<T>(const_cast<unsigned char*>(logbuf) + b * log_bytes, log_bytes, n);
  const int nsw = L.head[0], nrot = L.head[1];
  if (nsw <= 0) return;
  const int lane = threadIdx.x;
  const int r0 = blockIdx.x * kLogRows;
  const int nr = min(kLogRows, n - r0);
  cplx<T>* Zb = Z + b * (int64_t)n * n;
  for (int i = 0; i < nr; ++i)
    for (int j = lane; j < n; j += kLogRows) rows[i * lds + j] = Zb[(int64_t)(r0 + i) * n + j];
  // stage chunk c of the rotations into buffer c % 2 (16-byte pieces; past the end: not copied)
  constexpr int kPieces = (int)sizeof(HqrRot<T>) / 16;
  auto load_chunk = [&](int c) {
    const int q0 = c * kLogChunk;
    const int cnt = min(kLogChunk, nrot - q0);
    HqrRot<T>* dst = stage + (c & 1) * kLogChunk;
    for (int e = lane; e < cnt * kPieces; e += kLogRows)
      cp_async16(reinterpret_cast<char*>(dst) + 16 * (size_t)e, reinterpret_cast<const char*>(L.rot + q0) + 16 * (size_t)e);
    cp_async_commit();
  };
  const int nchunks = (nrot + kLogChunk - 1) / kLogChunk;
  load_chunk(0);
  if (nchunks > 1) load_chunk(1);
  else cp_async_commit();  // an empty group keeps the wait counts below uniform
  cp_async_wait<1>();
  __syncwarp();
  cplx<T>* row = rows + lane * lds;  // lanes past the last row roll a copy they never store
  int chunk = 0, q = 0, qend = min(kLogChunk, nrot);
  const HqrRot<T>* cur = stage;
  int nlo = L.sweeps[0], nhi = L.sweeps[1];
  for (int sw = 0; sw < nsw; ++sw) {
    const int lo = nlo, hi = nhi;
    if (sw + 1 < nsw) {  // the next sweep's bounds load while this one rolls
      nlo = L.sweeps[2 * sw + 2];
      nhi = L.sweeps[2 * sw + 3];
    }
    cplx<T> a = row[lo];
    int k = lo;
    while (k < hi) {
      if (q == qend) {  // next chunk: refill this buffer with chunk + 2, wait for chunk + 1
        __syncwarp();
        if (chunk + 2 < nchunks) load_chunk(chunk + 2);
        else cp_async_commit();
        ++chunk;
        cp_async_wait<1>();
        __syncwarp();
        cur = stage + (chunk & 1) * kLogChunk;
        qend = min(q + kLogChunk, nrot);
      }
      const int take = min(hi - k, qend - q);
      const HqrRot<T>* g = cur + (q - chunk * kLogChunk);
#pragma unroll 4
      for (int u = 0; u < take; ++u) {
        const HqrRot<T> r = g[u];
        const cplx<T> s = mk(r.sre, r.sim);
        const cplx<T> bb = row[k + u + 1];
        row[k + u] = r.c * a + mul_conj(bb, s);
        a = r.c * bb - s * a;
      }
      k += take;
      q += take;
    }
    row[hi] = a;
  }
  cp_async_wait<0>();
  __syncwarp();
  for (int i = 0; i < nr; ++i)
    for (int j = lane; j < n; j += kLogRows) Zb[(int64_t)(r0 + i) * n + j] = rows[i * lds + j];
}

// Scale every column of W to unit 2-norm (thread per column, coalesced along rows).
template <typename T>
__global__ void k_normalize_cols(int64_t batch, int n, cplx<T>* W, int64_t ldw, int64_t bsW) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / n;
    const int k = (int)(e % n);
    cplx<T>* w = W + b * bsW + k;
    T s = T(0);
    for (int i = 0; i < n; ++i) s += norm2(w[(int64_t)i * ldw]);
    const T inv = s > T(0) ? T(1) / sqrt(s) : T(1);
    for (int i = 0; i < n; ++i) w[(int64_t)i * ldw] = w[(int64_t)i * ldw] * inv;
  }
}

// Tiled product: CTA tile BM x BN, 256 threads as 16 x 16, each thread TM x TN outputs
// strided by 16 (conflict-free shared-memory reads).
template <typename T, int BM, int BN, int BK>
__global__ void __launch_bounds__(256) k_gemm(int n, int m, int k, cplx<T> alpha, const cplx<T>* __restrict__ A,
                                              int64_t lda, int64_t bsA, const cplx<T>* __restrict__ B, int64_t ldb,
                                              int64_t bsB, cplx<T> beta, cplx<T>* C, int64_t ldc, int64_t bsC,
                                              int64_t boff, const int* __restrict__ aidx,
                                              const int* __restrict__ bidx, cplx<T> bshift) {
  constexpr int TM = BM / 16, TN = BN / 16;
  constexpr int LA = BM * BK / 256, LB = BK * BN / 256;  // tile elements loaded per thread
  static_assert(LA * 256 == BM * BK && LB * 256 == BK * BN, "tile loads must split evenly over 256 threads");
  __shared__ cplx<T> As[BK][BM];
  __shared__ cplx<T> Bs[BK][BN];
  const int64_t b = blockIdx.z + boff;
  A += (aidx ? (int64_t)aidx[b] : b) * bsA;
  B += (bidx ? (int64_t)bidx[b] : b) * bsB;
  C += b * bsC;
  const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  cplx<T> acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = mk(T(0));
  // the next K-slice is loaded into registers while the current one is multiplied
  cplx<T> ra[LA], rb[LB];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < LA; ++q) {
      const int e = threadIdx.x + 256 * q, r = e / BK, c = e % BK;
      const int gr = row0 + r, gc = k0 + c;
      ra[q] = (gr < n && gc < k) ? A[(int64_t)gr * lda + gc] : mk(T(0));
    }
#pragma unroll
    for (int q = 0; q < LB; ++q) {
      const int e = threadIdx.x + 256 * q, r = e / BN, c = e % BN;
      const int gr = k0 + r, gc = col0 + c;
      rb[q] = (gr < k && gc < m) ? B[(int64_t)gr * ldb + gc] + (gr == gc ? bshift : mk(T(0))) : mk(T(0));
    }
  };
  auto stage = [&]() {
#pragma unroll
    for (int q = 0; q < LA; ++q) {
      const int e = threadIdx.x + 256 * q;
      As[e % BK][e / BK] = ra[q];
    }
#pragma unroll
    for (int q = 0; q < LB; ++q) {
      const int e = threadIdx.x + 256 * q;
      Bs[e / BN][e % BN] = rb[q];
    }
  };
  // FP32: prefetch (the products are latency-bound); FP64: load and stage in turn (the FP64 pipe
  // bounds them, and the prefetch registers would cost occupancy)
  constexpr bool kPrefetch = sizeof(T) == 4;
  if (kPrefetch && k > 0) load(0);
  for (int k0 = 0; k0 < k; k0 += BK) {
    if (!kPrefetch) load(k0);
    stage();
    __syncthreads();
    if (kPrefetch && k0 + BK < k) load(k0 + BK);
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

// ------------------------------------------------------------------------------------------
// Blocked LU / inverse: panels of KHP_NB columns factorised in shared memory, trailing updates
// and block-triangular solves as batched tiled products.
// ------------------------------------------------------------------------------------------
constexpr int KHP_NB = 32;

// Factor the panel A[kb:n, kb:kb+w] (w <= KHP_NB) with partial pivoting, in shared memory.
// piv[kb + jj] receives the global row swapped with row kb + jj (rows swapped inside the panel).
template <typename T>
__global__ void __launch_bounds__(256) k_panel_lu(int n, int kb, int w, cplx<T>* A, int64_t lda, int64_t bsA, int* piv,
                                                  int* info) {
  __shared__ TeamShared sh;
  extern __shared__ unsigned char dyn[];
  cplx<T>* P = reinterpret_cast<cplx<T>*>(dyn);  // (n - kb) x w, row-major, ld w
  TeamCta t;
  const int64_t b = blockIdx.x;
  cplx<T>* Ab = A + b * bsA;
  const int rows = n - kb;
  for (int e = t.tid(); e < rows * w; e += t.size()) P[e] = Ab[(int64_t)(kb + e / w) * lda + kb + e % w];
  t.sync();
  int st = 0;
  for (int jj = 0; jj < w; ++jj) {
    T best = T(-1);
    int bi = jj;
    for (int i = jj + t.tid(); i < rows; i += t.size()) {
      const T v = abs1(P[i * w + jj]);
      if (v > best) { best = v; bi = i; }
    }
    team_argmax(t, best, bi, &sh);
    if (t.tid() == 0) piv[b * n + kb + jj] = kb + bi;
    if (!(best > T(0))) {
      st |= (best == T(0)) ? KHP_BIT_SINGULAR : KHP_BIT_NONFINITE;
      t.sync();
      continue;
    }
    if (bi != jj)
      for (int c = t.tid(); c < w; c += t.size()) {
        const cplx<T> a = P[jj * w + c];
        P[jj * w + c] = P[bi * w + c];
        P[bi * w + c] = a;
      }
    t.sync();
    const cplx<T> pv = P[jj * w + jj];
    for (int i = jj + 1 + t.tid(); i < rows; i += t.size()) P[i * w + jj] = cdiv(P[i * w + jj], pv);
    t.sync();
    const int cw = w - jj - 1;
    for (int e = t.tid(); e < (rows - jj - 1) * cw; e += t.size()) {
      const int i = jj + 1 + e / cw, c = jj + 1 + e % cw;
      fms_acc(P[i * w + c], P[i * w + jj], P[jj * w + c]);
    }
    t.sync();
  }
  for (int e = t.tid(); e < rows * w; e += t.size()) Ab[(int64_t)(kb + e / w) * lda + kb + e % w] = P[e];
  if (threadIdx.x == 0 && st) info[b] |= st;
}

// The same panel factorisation with the panel in registers: thread i holds row kb + i (needs
// n - kb <= 256 and w <= KHP_NB).  Per column: a team argmax (ties to the lower row), the pivot
// row and row jj exchanged through shared memory, then each thread scales and updates its own
// row from the pivot row (a shared-memory broadcast).  Two barriers per column and no shared-memory
// traffic for the elimination itself.  Same pivots, same order of operations per element as
// k_panel_lu.
template <typename T>
__global__ void __launch_bounds__(256, 3) k_panel_lu_reg(int n, int kb, int w, cplx<T>* A, int64_t lda, int64_t bsA,
                                                         int* piv, int* info) {
  __shared__ cplx<T> prow[KHP_NB], srow[KHP_NB];
  __shared__ T wv[8];
  __shared__ int wi[8];
  const int64_t b = blockIdx.x;
  cplx<T>* Ab = A + b * bsA;
  const int rows = n - kb;
  const int i = threadIdx.x, lane = i & 31, warp = i >> 5;
  cplx<T> a[KHP_NB];
#pragma unroll
  for (int c = 0; c < KHP_NB; ++c) a[c] = (i < rows && c < w) ? Ab[(int64_t)(kb + i) * lda + kb + c] : mk(T(0));
  int st = 0;
  // a[] is only indexed by compile-time c (selects against jj), so it stays in registers
#pragma unroll 1
  for (int jj = 0; jj < KHP_NB; ++jj) {
    if (jj < w) {
      cplx<T> ajj = a[0];
#pragma unroll
      for (int c = 1; c < KHP_NB; ++c)
        if (c == jj) ajj = a[c];
      T v = T(-1);
      int bi = jj;
      if (i >= jj && i < rows) {
        const T x = abs1(ajj);
        if (x > v) { v = x; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const T ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > v || (ov == v && oi < bi)) { v = ov; bi = oi; }
      }
      if (lane == 0) { wv[warp] = v; wi[warp] = bi; }
      __syncthreads();
      T best = wv[0];
      int bsel = wi[0];
#pragma unroll
      for (int q = 1; q < 8; ++q)
        if (wv[q] > best || (wv[q] == best && wi[q] < bsel)) { best = wv[q]; bsel = wi[q]; }
      if (i == 0) piv[b * n + kb + jj] = kb + bsel;
      if (!(best > T(0))) {
        st |= (best == T(0)) ? KHP_BIT_SINGULAR : KHP_BIT_NONFINITE;
        __syncthreads();  // wv / wi are read before the next column writes them
      } else {
        if (i == bsel) {
#pragma unroll
          for (int c = 0; c < KHP_NB; ++c) prow[c] = a[c];
        } else if (i == jj) {
#pragma unroll
          for (int c = 0; c < KHP_NB; ++c) srow[c] = a[c];
        }
        __syncthreads();
        if (bsel != jj) {
          if (i == jj) {
#pragma unroll
            for (int c = 0; c < KHP_NB; ++c) a[c] = prow[c];
          } else if (i == bsel) {
#pragma unroll
            for (int c = 0; c < KHP_NB; ++c) a[c] = srow[c];
            ajj = srow[jj];  // this thread now holds the old row jj
          }
        }
        if (i > jj && i < rows) {
          const cplx<T> l = cdiv(ajj, prow[jj]);
#pragma unroll
          for (int c = 0; c < KHP_NB; ++c) {
            if (c == jj) a[c] = l;
            else if (c > jj && c < w) fms_acc(a[c], l, prow[c]);
            // keeps the compiler from hoisting all of prow into registers at once
            if ((c & 7) == 7) asm volatile("" ::: "memory");
          }
        }
      }
    }
  }
  if (i < rows)
#pragma unroll
    for (int c = 0; c < KHP_NB; ++c)
      if (c < w) Ab[(int64_t)(kb + i) * lda + kb + c] = a[c];
  if (threadIdx.x == 0 && st) info[b] |= st;
}

// B = P: the permutation matrix of the row interchanges piv[0:n) applied to the identity (one CTA
// per matrix; the permutation is resolved in shared memory by one thread, then written row-wise).
template <typename T>
__global__ void k_perm_matrix(int n, const int* __restrict__ piv, cplx<T>* B, int64_t ldb, int64_t bsB) {
  extern __shared__ int perm[];
  const int64_t b = blockIdx.x;
  for (int r = threadIdx.x; r < n; r += blockDim.x) perm[r] = r;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < n; ++k) {
      const int p = piv[b * n + k];
      if (p != k) {
        const int t = perm[k];
        perm[k] = perm[p];
        perm[p] = t;
      }
    }
  __syncthreads();
  cplx<T>* Bb = B + b * bsB;
  for (int64_t e = threadIdx.x; e < (int64_t)n * n; e += blockDim.x) {
    const int r = (int)(e / n), c = (int)(e % n);
    Bb[(int64_t)r * ldb + c] = (c == perm[r]) ? mk(T(1)) : mk(T(0));
  }
}

// X <- X P, P the permutation matrix of the row interchanges piv[0:n) (one CTA per matrix): the
// permutation and its inverse are resolved in shared memory, then the rows pass through a
// shared-memory buffer R at a time and come back with their columns gathered, X[i][c] =
// X[i][pinv[c]] (coalesced reads and writes).
template <typename T>
__global__ void k_col_perm(int n, int R, const int* __restrict__ piv, cplx<T>* X, int64_t ldx, int64_t bsX) {
  extern __shared__ __align__(16) unsigned char dyn_cp[];
  int* perm = reinterpret_cast<int*>(dyn_cp);
  int* pinv = perm + n;
  cplx<T>* buf = reinterpret_cast<cplx<T>*>(dyn_cp + ((2 * sizeof(int) * (size_t)n + 15) & ~size_t(15)));
  const int64_t b = blockIdx.x;
  for (int r = threadIdx.x; r < n; r += blockDim.x) perm[r] = r;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < n; ++k) {
      const int p = piv[b * n + k];
      if (p != k) {
        const int t = perm[k];
        perm[k] = perm[p];
        perm[p] = t;
      }
    }
  __syncthreads();
  for (int r = threadIdx.x; r < n; r += blockDim.x) pinv[perm[r]] = r;
  cplx<T>* Xb = X + b * bsX;
  for (int r0 = 0; r0 < n; r0 += R) {
    const int rows = min(R, n - r0);
    __syncthreads();  // pinv ready; the previous rows written back
    for (int e = threadIdx.x; e < rows * n; e += blockDim.x) buf[e] = Xb[(int64_t)(r0 + e / n) * ldx + e % n];
    __syncthreads();
    for (int e = threadIdx.x; e < rows * n; e += blockDim.x) {
      const int i = e / n, c = e % n;
      Xb[(int64_t)(r0 + i) * ldx + c] = buf[i * n + pinv[c]];
    }
  }
}

// Apply the row interchanges piv[k0:k1] to columns [c0, c1) of A (thread per column, in order).
template <typename T>
__global__ void k_laswp(int64_t batch, int n, int k0, int k1, int c0, int c1, cplx<T>* A, int64_t lda, int64_t bsA,
                        const int* piv) {
  const int nc = c1 - c0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nc; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nc;
    const int c = c0 + (int)(e % nc);
    cplx<T>* Ab = A + b * bsA;
    for (int k = k0; k < k1; ++k) {
      const int p = piv[b * n + k];
      if (p != k) {
        const cplx<T> a = Ab[(int64_t)k * lda + c];
        Ab[(int64_t)k * lda + c] = Ab[(int64_t)p * lda + c];
        Ab[(int64_t)p * lda + c] = a;
      }
    }
  }
}

// The row interchanges piv[kb:kb+w] of one panel applied to every column outside the panel
// [kb, kb+w).  The w sequential swaps are first resolved in shared memory into a permutation of
// the (at most 2w) rows they touch; then each thread (a column) loads all of the moved rows
// before it stores any, instead of one dependent round trip per swap.  CTA per (column chunk,
// problem), kSwpThreads threads; dynamic shared memory laswp_panel_smem<T>(n).
constexpr int kSwpThreads = 64;
template <typename T>
size_t laswp_panel_smem(int n) {
  // stage [2 NB][threads] complex, then content [n], touched [n], rows [2 NB] and the count
  return sizeof(cplx<T>) * 2 * KHP_NB * kSwpThreads + sizeof(int) * (2 * (size_t)n + 2 * KHP_NB + 1);
}
template <typename T>
__global__ void __launch_bounds__(kSwpThreads) k_laswp_panel(int n, int kb, int w, cplx<T>* A, int64_t lda,
                                                             int64_t bsA, const int* __restrict__ piv) {
  extern __shared__ unsigned char dyn_sw[];
  cplx<T>* stage = reinterpret_cast<cplx<T>*>(dyn_sw);         // [2 KHP_NB][kSwpThreads]
  int* content = reinterpret_cast<int*>(stage + 2 * KHP_NB * kSwpThreads);  // [n]: source row now at r
  int* touched = content + n;                                   // [n]: row already listed
  int* rows = touched + n;                                      // [<= 2 w]: the moved rows
  int* cnt = rows + 2 * KHP_NB;
  const int64_t b = blockIdx.y;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    content[r] = r;
    touched[r] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0;
    for (int k = kb; k < kb + w; ++k) {
      const int p = piv[b * n + k];
      if (p == k) continue;
      const int t = content[k];
      content[k] = content[p];
      content[p] = t;
      if (!touched[k]) { touched[k] = 1; rows[c++] = k; }
      if (!touched[p]) { touched[p] = 1; rows[c++] = p; }
    }
    *cnt = c;
  }
  __syncthreads();
  const int nr = *cnt;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;  // q-th column outside the panel
  if (nr == 0 || q >= n - w) return;
  const int col = q < kb ? q : q + w;
  cplx<T>* Ab = A + b * bsA + col;
  for (int i = 0; i < nr; ++i) stage[i * kSwpThreads + threadIdx.x] = Ab[(int64_t)content[rows[i]] * lda];
  for (int i = 0; i < nr; ++i) Ab[(int64_t)rows[i] * lda] = stage[i * kSwpThreads + threadIdx.x];
}

// B[r0:r0+w, 0:m] <- T^-1 B[r0:r0+w, 0:m] with T = the diagonal block A[d0:d0+w, d0:d0+w]
// (unit lower when lower, else upper with its diagonal).  Thread per column of B; T in smem.
template <typename T>
__global__ void k_trsm_block(int w, int d0, const cplx<T>* __restrict__ A, int64_t lda, int64_t bsA, int r0, int m,
                             cplx<T>* B, int64_t ldb, int64_t bsB, int lower, int64_t batch) {
  __shared__ cplx<T> Tb[KHP_NB * KHP_NB];
  __shared__ cplx<T> dinv[KHP_NB];  // reciprocals of the diagonal (upper)
  const int64_t b = blockIdx.y;
  const cplx<T>* Ab = A + b * bsA;
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) Tb[e] = Ab[(int64_t)(d0 + e / w) * lda + d0 + e % w];
  __syncthreads();
  if (!lower && threadIdx.x < w) dinv[threadIdx.x] = cdiv(mk(T(1)), Tb[threadIdx.x * w + threadIdx.x]);
  __syncthreads();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  cplx<T>* Bb = B + b * bsB + (int64_t)r0 * ldb + j;
  cplx<T> x[KHP_NB];
#pragma unroll
  for (int i = 0; i < KHP_NB; ++i)
    if (i < w) x[i] = Bb[(int64_t)i * ldb];
  if (lower) {
#pragma unroll
    for (int i = 0; i < KHP_NB; ++i) {
      if (i >= w) break;
      cplx<T> acc = x[i];
#pragma unroll
      for (int k = 0; k < KHP_NB; ++k)
        if (k < i) fms_acc(acc, Tb[i * w + k], x[k]);
      x[i] = acc;
    }
  } else {
#pragma unroll
    for (int ii = KHP_NB - 1; ii >= 0; --ii) {
      if (ii >= w) continue;
      cplx<T> acc = x[ii];
#pragma unroll
      for (int k = 0; k < KHP_NB; ++k)
        if (k > ii && k < w) fms_acc(acc, Tb[ii * w + k], x[k]);
      x[ii] = acc * dinv[ii];
    }
  }
#pragma unroll
  for (int i = 0; i < KHP_NB; ++i)
    if (i < w) Bb[(int64_t)i * ldb] = x[i];
}

// One block row of the substitutions, product and triangular solve fused:
//   B[r0:r0+w, tile] <- Tkk^-1 (B[r0:r0+w, tile] - A[r0:r0+w, k0:k0+K] B[k0:k0+K, tile])
// with Tkk = A[r0:r0+w, r0:r0+w] unit lower (lower) or upper with its diagonal.  A CTA per 128
// columns of one problem: the 32 x 128 product tile in registers (2 x 8 per thread), then staged in
// shared memory and solved a thread per column in place.  Dynamic shared memory:
// block_solve_smem<T>() bytes.
constexpr int kBsBM = 32, kBsBN = 128, kBsBK = 16;
template <typename T>
constexpr size_t block_solve_smem() {
  return sizeof(cplx<T>) * ((size_t)kBsBK * kBsBM + (size_t)kBsBK * kBsBN + (size_t)kBsBM * kBsBN +
                            (size_t)KHP_NB * KHP_NB + KHP_NB);
}
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) k_block_solve(int w, int r0, int k0, int K, int m, const cplx<T>* __restrict__ A,
                                                     int64_t lda, int64_t bsA, cplx<T>* B, int64_t ldb, int64_t bsB,
                                                     int lower) {
  constexpr int TM = kBsBM / 16, TN = kBsBN / 16;
  extern __shared__ unsigned char dyn_bs[];
  cplx<T>* As = reinterpret_cast<cplx<T>*>(dyn_bs);  // [BK][BM]
  cplx<T>* Bs = As + kBsBK * kBsBM;                    // [BK][BN]
  cplx<T>* Cs = Bs + kBsBK * kBsBN;                    // [BM][BN]
  cplx<T>* Tb = Cs + kBsBM * kBsBN;                    // [w][w]
  cplx<T>* dinv = Tb + KHP_NB * KHP_NB;                // [w]
  const int64_t b = blockIdx.y;
  const cplx<T>* Ab = A + b * bsA;
  cplx<T>* Bb = B + b * bsB;
  const int col0 = blockIdx.x * kBsBN;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  cplx<T> acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = mk(T(0));
  constexpr int LA = kBsBM * kBsBK / 256, LB = kBsBK * kBsBN / 256;
  cplx<T> ra[LA], rb[LB];  // the next K-slice, loaded while the current one is multiplied
  auto load = [&](int kk0) {
#pragma unroll
    for (int q = 0; q < LA; ++q) {
      const int e = threadIdx.x + 256 * q, r = e / kBsBK, c = e % kBsBK;
      ra[q] = (r < w && kk0 + c < K) ? Ab[(int64_t)(r0 + r) * lda + k0 + kk0 + c] : mk(T(0));
    }
#pragma unroll
    for (int q = 0; q < LB; ++q) {
      const int e = threadIdx.x + 256 * q, r = e / kBsBN, c = e % kBsBN;
      rb[q] = (kk0 + r < K && col0 + c < m) ? Bb[(int64_t)(k0 + kk0 + r) * ldb + col0 + c] : mk(T(0));
    }
  };
  constexpr bool kPrefetch = sizeof(T) == 4;  // as in k_gemm
  if (kPrefetch && K > 0) load(0);
  for (int kk0 = 0; kk0 < K; kk0 += kBsBK) {
    if (!kPrefetch) load(kk0);
#pragma unroll
    for (int q = 0; q < LA; ++q) {
      const int e = threadIdx.x + 256 * q;
      As[(e % kBsBK) * kBsBM + e / kBsBK] = ra[q];
    }
#pragma unroll
    for (int q = 0; q < LB; ++q) {
      const int e = threadIdx.x + 256 * q;
      Bs[(e / kBsBN) * kBsBN + e % kBsBN] = rb[q];
    }
    __syncthreads();
    if (kPrefetch && kk0 + kBsBK < K) load(kk0 + kBsBK);
#pragma unroll
    for (int kk = 0; kk < kBsBK; ++kk) {
      cplx<T> a[TM], bb[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk * kBsBM + ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) bb[j] = Bs[kk * kBsBN + tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) fma_acc(acc[i][j], a[i], bb[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int r = ty + 16 * i;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int c = tx + 16 * j;
      Cs[r * kBsBN + c] = (r < w && col0 + c < m) ? Bb[(int64_t)(r0 + r) * ldb + col0 + c] - acc[i][j] : mk(T(0));
    }
  }
  for (int e = threadIdx.x; e < w * w; e += 256) Tb[e] = Ab[(int64_t)(r0 + e / w) * lda + r0 + e % w];
  __syncthreads();
  if (!lower && threadIdx.x < w) dinv[threadIdx.x] = cdiv(mk(T(1)), Tb[threadIdx.x * w + threadIdx.x]);
  __syncthreads();
  // a thread per column solves in place in the shared tile (its own column only, no barriers)
  const int j = threadIdx.x;
  if (j >= kBsBN || col0 + j >= m) return;
  cplx<T>* xc = Cs + j;  // xc[i * kBsBN] = row i of this column
  if (lower) {
    for (int i = 1; i < w; ++i) {
      cplx<T> a = xc[i * kBsBN];
      for (int k = 0; k < i; ++k) fms_acc(a, Tb[i * w + k], xc[k * kBsBN]);
      xc[i * kBsBN] = a;
    }
  } else {
    for (int ii = w - 1; ii >= 0; --ii) {
      cplx<T> a = xc[ii * kBsBN];
      for (int k = ii + 1; k < w; ++k) fms_acc(a, Tb[ii * w + k], xc[k * kBsBN]);
      xc[ii * kBsBN] = a * dinv[ii];
    }
  }
  cplx<T>* out = Bb + (int64_t)r0 * ldb + col0 + j;
  for (int i = 0; i < w; ++i) out[(int64_t)i * ldb] = xc[i * kBsBN];
}

// Grid for a thread-per-column row interchange: one thread per column up to 8 CTAs per SM.
inline unsigned swp_blocks(int64_t columns) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((columns + 255) / 256, 152 * 8)); }

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
                cudaStream_t s, const int* aidx, const int* bidx, cplx<T> bshift) {
  if (batch <= 0 || n <= 0 || m <= 0) return KHP_OK;
  // 64 x 64 tiles (4 x 4 outputs per thread) once both output dimensions reach 64; 32 x 128
  // (2 x 8) for outputs of at most 32 rows and at least 128 columns (the block rows of the
  // substitutions); else 32 x 32
  const bool big = n >= 64 && m >= 64;
  const bool wide = !big && n <= 32 && m >= 128;
  const int BM = big ? 64 : 32, BN = big ? 64 : wide ? 128 : 32;
  for (int64_t off = 0; off < batch; off += kMaxGridY) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
    dim3 grid((m + BN - 1) / BN, (n + BM - 1) / BM, nb);
    if (wide)
      k_gemm<T, 32, 128, 16><<<grid, 256, 0, s>>>(n, m, k, alpha, A, lda, bsA, B, ldb, bsB, beta, C, ldc, bsC, off,
                                                  aidx, bidx, bshift);
    else if (big)
      k_gemm<T, 64, 64, 8><<<grid, 256, 0, s>>>(n, m, k, alpha, A, lda, bsA, B, ldb, bsB, beta, C, ldc, bsC, off,
                                                aidx, bidx, bshift);
    else
      k_gemm<T, 32, 32, 16><<<grid, 256, 0, s>>>(n, m, k, alpha, A, lda, bsA, B, ldb, bsB, beta, C, ldc, bsC, off,
                                                 aidx, bidx, bshift);
    count_launches(1);
  }
  return cuda_status();
}

template <typename T>
int launch_geev(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Z, cplx<T>* W, int64_t ldw,
                int64_t bsW, cplx<T>* lam, int64_t bsLam, int* info, cudaStream_t s, void* logbuf,
                int64_t log_bytes) {
  if (batch <= 0) return KHP_OK;
  // blocked reduction when panels pay off and their scratch fits in shared memory
  const size_t scratch = sizeof(cplx<T>) * (size_t)gehrd_blocked_scratch(n);
  const int blocked = (n >= 64 && scratch <= 200 * 1024) ? 1 : 0;
  // blocked: the panel's reflectors, Y, T; unblocked: one Householder vector
  const size_t smem = blocked ? scratch : sizeof(cplx<T>) * (size_t)n;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_gehrd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return KHP_ERR_CUDA;
  const int threads = eig_threads(n);
  // the blocked reduction keeps full 256-thread teams (its panel updates are parallel work; three
  // teams per SM already cover the SM), whatever team size suits the QR's serial window chase
  const int gthreads = blocked ? kTeamThreads : threads;
  k_gehrd<T><<<(unsigned)batch, gthreads, smem, s>>>(n, A, lda, bsA, Z, blocked);
  // Z through the rotation log when the region holds at least one full sweep per matrix
  unsigned char* lg = nullptr;
  if (logbuf && log_bytes % 32 == 0 && reinterpret_cast<uintptr_t>(logbuf) % 32 == 0 &&
      hqr_log_view<T>(logbuf, log_bytes, n).cap_rot >= n - 1)
    lg = static_cast<unsigned char*>(logbuf);
  k_geev_schur<T><<<(unsigned)batch, threads, 0, s>>>(n, A, lda, bsA, Z, lam, bsLam, info, lg, log_bytes);
  count_launches(2);
  int st = cuda_status();
  if (st) return st;
  if (lg) {
    const size_t lsm = apply_log_smem<T>(n);
    if (lsm > 48 * 1024 &&
        cudaFuncSetAttribute(k_hqr_apply_log<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsm) != cudaSuccess)
      return KHP_ERR_CUDA;
    for (int64_t off = 0; off < batch; off += kMaxGridY) {
      const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
      k_hqr_apply_log<T><<<dim3((n + kLogRows - 1) / kLogRows, nb), kLogRows, lsm, s>>>(n, Z, lg, log_bytes, off);
      count_launches(1);
    }
    st = cuda_status();
    if (st) return st;
  }
  // W = Z X (X unit upper triangular, stored in A) and unit columns
  st = launch_gemm<T>(batch, n, n, n, mk(T(1)), Z, n, (int64_t)n * n, A, lda, bsA, mk(T(0)), W, ldw, bsW, s);
  if (st) return st;
  const int64_t cols = batch * n;
  k_normalize_cols<T><<<(unsigned)std::min<int64_t>((cols + 127) / 128, 152 * 16), 128, 0, s>>>(batch, n, W, ldw, bsW);
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

template <typename T>
int launch_getrf_blocked(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, int* piv, int* info,
                         cudaStream_t s) {
  if (batch <= 0) return KHP_OK;
  constexpr size_t kPanelSmem = 200 * 1024;
  for (int kb = 0, w = 0; kb < n; kb += w) {
    // panel width: KHP_NB columns, fewer when the (n - kb) x w panel would not fit in shared memory
    w = (int)std::min<size_t>({(size_t)KHP_NB, (size_t)(n - kb), kPanelSmem / (sizeof(cplx<T>) * (size_t)(n - kb))});
    if (w < 1) return KHP_ERR_TOO_LARGE;
    bool reg_panel = false;
    if constexpr (sizeof(T) == 4) {
      if (n - kb <= 256) {
        // FP32 panels of up to 256 rows: one row per thread, in registers
        k_panel_lu_reg<T><<<(unsigned)batch, 256, 0, s>>>(n, kb, w, A, lda, bsA, piv, info);
        reg_panel = true;
      }
    }
    if (!reg_panel) {
      const size_t smem = sizeof(cplx<T>) * (size_t)(n - kb) * w;
      if (smem > 48 * 1024 &&
          cudaFuncSetAttribute(k_panel_lu<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return KHP_ERR_CUDA;
      k_panel_lu<T><<<(unsigned)batch, 256, smem, s>>>(n, kb, w, A, lda, bsA, piv, info);
    }
    count_launches(1);
    // row swaps of this panel to the columns left and right of it
    const int other = n - w;
    if (other > 0) {
      const size_t ssm = laswp_panel_smem<T>(n);
      if (ssm <= 48 * 1024) {
        for (int64_t off = 0; off < batch; off += kMaxGridY) {
          const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
          k_laswp_panel<T><<<dim3((other + kSwpThreads - 1) / kSwpThreads, nb), kSwpThreads, ssm, s>>>(
              n, kb, w, A + off * bsA, lda, bsA, piv + off * n);
          count_launches(1);
        }
      } else {
        if (kb > 0) {
          k_laswp<T><<<swp_blocks(batch * kb), 256, 0, s>>>(batch, n, kb, kb + w, 0, kb, A, lda, bsA, piv);
          count_launches(1);
        }
        if (kb + w < n) {
          k_laswp<T><<<swp_blocks(batch * (n - kb - w)), 256, 0, s>>>(batch, n, kb, kb + w, kb + w, n, A, lda,
                                                                      bsA, piv);
          count_launches(1);
        }
      }
    }
    const int rest = n - kb - w;
    if (rest > 0) {
      // U12 = L11^-1 A12, then A22 -= L21 U12
      for (int64_t off = 0; off < batch; off += kMaxGridY) {
        const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
        k_trsm_block<T><<<dim3((rest + 127) / 128, nb), 128, 0, s>>>(w, kb, A + off * bsA, lda, bsA, kb, rest,
                                                                    A + off * bsA + kb + w, lda, bsA, 1, nb);
        count_launches(1);
      }
      const int st = launch_gemm<T>(batch, rest, rest, w, mk(T(-1)), A + (int64_t)(kb + w) * lda + kb, lda, bsA,
                                    A + (int64_t)kb * lda + kb + w, lda, bsA, mk(T(1)),
                                    A + (int64_t)(kb + w) * lda + kb + w, lda, bsA, s);
      if (st) return st;
    }
  }
  return cuda_status();
}

// Block forward and backward substitution with launch_getrf_blocked's L and U (B already
// permuted): for 128 or more right-hand sides each block row is one fused product + solve
// (k_block_solve), for fewer a tiled product sized to m followed by the block solve.
// tri_rhs: B is lower triangular (the identity, for an inverse), so L Y = B keeps Y lower
// triangular and the forward sweep's block row kb only computes its first kb + w columns (the
// rest stay 0): a third of the forward work instead of all of it.
template <typename T>
int getrs_blocked_tri(int64_t batch, int n, const cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* B, int64_t ldb,
                      int64_t bsB, int m, cudaStream_t s, bool tri_rhs = false) {
  if (m < kBsBN) {
    // few right-hand sides: tiled product sized to m, then the block solve
    auto trsm = [&](int kb, int w, int lower) {
      for (int64_t off = 0; off < batch; off += kMaxGridY) {
        const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
        k_trsm_block<T><<<dim3((m + 127) / 128, nb), 128, 0, s>>>(w, kb, A + off * bsA, lda, bsA, kb, m,
                                                                 B + off * bsB, ldb, bsB, lower, nb);
        count_launches(1);
      }
    };
    for (int kb = 0; kb < n; kb += KHP_NB) {
      const int w = std::min(KHP_NB, n - kb);
      if (kb > 0) {
        const int st = launch_gemm<T>(batch, w, m, kb, mk(T(-1)), A + (int64_t)kb * lda, lda, bsA, B, ldb, bsB,
                                      mk(T(1)), B + (int64_t)kb * ldb, ldb, bsB, s);
        if (st) return st;
      }
      trsm(kb, w, 1);
    }
    const int last = ((n - 1) / KHP_NB) * KHP_NB;
    for (int kb = last; kb >= 0; kb -= KHP_NB) {
      const int w = std::min(KHP_NB, n - kb);
      const int rest = n - kb - w;
      if (rest > 0) {
        const int st = launch_gemm<T>(batch, w, m, rest, mk(T(-1)), A + (int64_t)kb * lda + kb + w, lda, bsA,
                                      B + (int64_t)(kb + w) * ldb, ldb, bsB, mk(T(1)), B + (int64_t)kb * ldb, ldb,
                                      bsB, s);
        if (st) return st;
      }
      trsm(kb, w, 0);
    }
    return cuda_status();
  }
  constexpr size_t smem = block_solve_smem<T>();
  if (cudaFuncSetAttribute(k_block_solve<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return KHP_ERR_CUDA;
  auto block = [&](int kb, int w, int k0, int K, int lower, int mc) {
    for (int64_t off = 0; off < batch; off += kMaxGridY) {
      const unsigned nb = (unsigned)std::min<int64_t>(batch - off, kMaxGridY);
      k_block_solve<T><<<dim3((mc + kBsBN - 1) / kBsBN, nb), 256, smem, s>>>(w, kb, k0, K, mc, A + off * bsA, lda,
                                                                            bsA, B + off * bsB, ldb, bsB, lower);
      count_launches(1);
    }
  };
  for (int kb = 0; kb < n; kb += KHP_NB) {  // L Y = B
    const int w = std::min(KHP_NB, n - kb);
    block(kb, w, 0, kb, 1, tri_rhs ? std::min(m, kb + w) : m);
  }
  const int last = ((n - 1) / KHP_NB) * KHP_NB;
  for (int kb = last; kb >= 0; kb -= KHP_NB) {  // U X = Y
    const int w = std::min(KHP_NB, n - kb);
    block(kb, w, kb + w, n - kb - w, 0, m);
  }
  return cuda_status();
}

// Solve A X = B (n x m) with launch_getrf_blocked's factors: pivots, then the block substitutions.
template <typename T>
int launch_getrs_blocked(int64_t batch, int n, const cplx<T>* A, int64_t lda, int64_t bsA, const int* piv, cplx<T>* B,
                         int64_t ldb, int64_t bsB, int m, cudaStream_t s) {
  if (batch <= 0) return KHP_OK;
  k_laswp<T><<<swp_blocks(batch * m), 256, 0, s>>>(batch, n, 0, n, 0, m, B, ldb, bsB, piv);
  count_launches(1);
  return getrs_blocked_tri<T>(batch, n, A, lda, bsA, B, ldb, bsB, m, s);
}

// A^-1 = U^-1 L^-1 P: the factors, the permutation matrix P written directly, the substitutions.
template <typename T>
int launch_inverse_blocked(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Ainv, int64_t ldi,
                           int64_t bsI, int* piv, int* info, cudaStream_t s) {
  if (batch <= 0) return KHP_OK;
  int st = launch_getrf_blocked<T>(batch, n, A, lda, bsA, piv, info, s);
  if (st) return st;
  const size_t psmem = sizeof(int) * (size_t)n;
  if (psmem > 48 * 1024) {
    st = launch_identity<T>(batch, n, n, Ainv, ldi, bsI, mk(T(1)), s);
    if (st) return st;
    return launch_getrs_blocked<T>(batch, n, A, lda, bsA, piv, Ainv, ldi, bsI, n, s);
  }
  // A^-1 = U^-1 L^-1 P: the substitutions on the identity (lower triangular, so the forward sweep
  // skips the zero columns), then the columns permuted; for few columns the permutation matrix
  // itself is the right-hand side
  const size_t head = (2 * sizeof(int) * (size_t)n + 15) & ~size_t(15);
  const size_t row_bytes = sizeof(cplx<T>) * (size_t)n;
  if (n < kBsBN || head + row_bytes > 48 * 1024) {
    k_perm_matrix<T><<<(unsigned)batch, 256, psmem, s>>>(n, piv, Ainv, ldi, bsI);
    count_launches(1);
    st = cuda_status();
    if (st) return st;
    return getrs_blocked_tri<T>(batch, n, A, lda, bsA, Ainv, ldi, bsI, n, s);
  }
  st = launch_identity<T>(batch, n, n, Ainv, ldi, bsI, mk(T(1)), s);
  if (!st) st = getrs_blocked_tri<T>(batch, n, A, lda, bsA, Ainv, ldi, bsI, n, s, true);
  if (st) return st;
  const int R = (int)std::min<size_t>(16, (48 * 1024 - head) / row_bytes);
  k_col_perm<T><<<(unsigned)batch, 256, head + row_bytes * R, s>>>(n, R, piv, Ainv, ldi, bsI);
  count_launches(1);
  return cuda_status();
}

#define KHP_INSTANTIATE(T)                                                                                       \
  template int launch_getrf<T>(int64_t, int, cplx<T>*, int64_t, int64_t, int*, int*, cudaStream_t);             \
  template int launch_getrs<T>(int64_t, int, const cplx<T>*, int64_t, int64_t, const int*, cplx<T>*, int64_t,   \
                               int64_t, int, cudaStream_t);                                                     \
  template int launch_gemm<T>(int64_t, int, int, int, cplx<T>, const cplx<T>*, int64_t, int64_t, const cplx<T>*, \
                              int64_t, int64_t, cplx<T>, cplx<T>*, int64_t, int64_t, cudaStream_t, const int*, \
                              const int*, cplx<T>);                                                             \
  template int launch_geev<T>(int64_t, int, cplx<T>*, int64_t, int64_t, cplx<T>*, cplx<T>*, int64_t, int64_t,  \
                              cplx<T>*, int64_t, int*, cudaStream_t, void*, int64_t);                           \
  template int launch_copy<T>(int64_t, int, int, const cplx<T>*, int64_t, int64_t, cplx<T>*, int64_t, int64_t,  \
                              cudaStream_t);                                                                    \
  template int launch_identity<T>(int64_t, int, int, cplx<T>*, int64_t, int64_t, cplx<T>, cudaStream_t);        \
  template int launch_axpby<T>(int64_t, int, int, cplx<T>, const cplx<T>*, int64_t, int64_t, cplx<T>,           \
                               const cplx<T>*, int64_t, int64_t, cplx<T>*, int64_t, int64_t, cudaStream_t);     \
  template int launch_inverse<T>(int64_t, int, cplx<T>*, int64_t, int64_t, cplx<T>*, int64_t, int64_t, int*,    \
                                 int*, cudaStream_t);                                                           \
  template int launch_getrf_blocked<T>(int64_t, int, cplx<T>*, int64_t, int64_t, int*, int*, cudaStream_t);     \
  template int launch_getrs_blocked<T>(int64_t, int, const cplx<T>*, int64_t, int64_t, const int*, cplx<T>*,    \
                                       int64_t, int64_t, int, cudaStream_t);                                    \
  template int launch_inverse_blocked<T>(int64_t, int, cplx<T>*, int64_t, int64_t, cplx<T>*, int64_t, int64_t,  \
                                         int*, int*, cudaStream_t);

KHP_INSTANTIATE(double)
KHP_INSTANTIATE(float)

}  // namespace khp

extern "C" {

int khp_tune(int32_t param, int32_t n, int32_t value) {
  using namespace khp;
  if (param == KHP_TUNE_TF32_MIN_N) {
    if (value < 0) return KHP_ERR_INVALID_ARG;
    g_tf32_min_n = value;
    return KHP_OK;
  }
  if (param == KHP_TUNE_MODE_DIGITS) {
    if (value != 6 && value != 8) return KHP_ERR_INVALID_ARG;
    g_mode_digits = value;
    return KHP_OK;
  }
  if (param != KHP_TUNE_EIG_THREADS || n < 1 || n > kTuneMaxN) return KHP_ERR_INVALID_ARG;
  if (value != 0 && (value < 32 || value > kTeamThreads || value % 32 != 0)) return KHP_ERR_INVALID_ARG;
  g_eig_threads[n] = value;
  return KHP_OK;
}

size_t khp_inverse_workspace(int64_t batch, int32_t n) {
  if (batch < 0 || n < 1) return 0;
  return sizeof(int) * (size_t)batch * n;  // pivots
}

int khp_inverse(int64_t batch, int32_t n, int32_t precision, void* A, int64_t a_stride, void* Ainv,
                int64_t inv_stride, int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  using namespace khp;
  if (batch < 0 || n < 1 || (precision != 0 && precision != 1) || !A || !Ainv || !status ||
      a_stride < (int64_t)n * n || inv_stride < (int64_t)n * n)
    return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  if (!workspace || ws_bytes < khp_inverse_workspace(batch, n)) return KHP_ERR_WORKSPACE;
  int* piv = static_cast<int*>(workspace);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (precision == 0)
    return launch_inverse_blocked<double>(batch, n, static_cast<cplx<double>*>(A), n, a_stride,
                                          static_cast<cplx<double>*>(Ainv), n, inv_stride, piv, status, s);
  return launch_inverse_blocked<float>(batch, n, static_cast<cplx<float>*>(A), n, a_stride,
                                       static_cast<cplx<float>*>(Ainv), n, inv_stride, piv, status, s);
}

}  // extern "C"
