// Internal C++ launch interface of libkhp (not part of the C-ABI): batched dense kernels over
// strided batches of row-major complex matrices, all asynchronous on the given stream.
#pragma once

#include <cuda_runtime.h>

#include "khp_core.cuh"

namespace khp {

// LU factorisation with partial pivoting of batch matrices A[b] (n x n); piv: batch x n ints.
// info[b] |= status bits (SINGULAR / NONFINITE).
template <typename T>
int launch_getrf(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, int* piv, int* info, cudaStream_t s);

// Solve A[b] X = B[b] with getrf factors; B (n x m) overwritten.
template <typename T>
int launch_getrs(int64_t batch, int n, const cplx<T>* A, int64_t lda, int64_t bsA, const int* piv, cplx<T>* B,
                 int64_t ldb, int64_t bsB, int m, cudaStream_t s);

// C = alpha A B + beta C (A n x k, B k x m).  A batch stride of 0 broadcasts one matrix;
// aidx / bidx (optional, device int[batch]) pick A[aidx[b]] / B[bidx[b]] for problem b.
template <typename T>
int launch_gemm(int64_t batch, int n, int m, int k, cplx<T> alpha, const cplx<T>* A, int64_t lda, int64_t bsA,
                const cplx<T>* B, int64_t ldb, int64_t bsB, cplx<T> beta, cplx<T>* C, int64_t ldc, int64_t bsC,
                cudaStream_t s, const int* aidx = nullptr, const int* bidx = nullptr, cplx<T> bshift = cplx<T>{});

// Eigen-decomposition A W = W diag(lam); A destroyed; Z: batch x n x n scratch (ld n).
// logbuf (optional, log_bytes per matrix, both multiples of 32): scratch for the QR's rotation
// log, which defers the updates of Z (used when it holds at least one full sweep).
template <typename T>
int launch_geev(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Z, cplx<T>* W, int64_t ldw,
                int64_t bsW, cplx<T>* lam, int64_t bsLam, int* info, cudaStream_t s, void* logbuf = nullptr,
                int64_t log_bytes = 0);

// Element-wise helpers on batches of n x m matrices.
template <typename T>
int launch_copy(int64_t batch, int n, int m, const cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* B, int64_t ldb,
                int64_t bsB, cudaStream_t s);
template <typename T>
int launch_identity(int64_t batch, int n, int m, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T> diag, cudaStream_t s);
// C = a A + b B (C may alias A or B)
template <typename T>
int launch_axpby(int64_t batch, int n, int m, cplx<T> a, const cplx<T>* A, int64_t lda, int64_t bsA, cplx<T> b,
                 const cplx<T>* B, int64_t ldb, int64_t bsB, cplx<T>* C, int64_t ldc, int64_t bsC, cudaStream_t s);

// Inverse: Ainv[b] = A[b]^-1 (A destroyed: holds the LU factors on return).
template <typename T>
int launch_inverse(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Ainv, int64_t ldi,
                   int64_t bsI, int* piv, int* info, cudaStream_t s);

// Blocked forms: panel LU in shared memory, trailing updates and off-diagonal blocks of the
// triangular solves as batched tiled products (fast for n >> 32).
template <typename T>
int launch_getrf_blocked(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, int* piv, int* info,
                         cudaStream_t s);
template <typename T>
int launch_getrs_blocked(int64_t batch, int n, const cplx<T>* A, int64_t lda, int64_t bsA, const int* piv, cplx<T>* B,
                         int64_t ldb, int64_t bsB, int m, cudaStream_t s);
template <typename T>
int launch_inverse_blocked(int64_t batch, int n, cplx<T>* A, int64_t lda, int64_t bsA, cplx<T>* Ainv, int64_t ldi,
                           int64_t bsI, int* piv, int* info, cudaStream_t s);

// FP64-accurate complex products on the bf16 tensor cores (error-free digit splitting; the
// result matches an FP64 product to its own rounding bound).  Scratch for the digit arrays:
// capacities in elements (bf16 digits) and entries (exponents); products over more problems
// than the capacities hold run in chunks.
struct OzakiWs {
  void* ad = nullptr;  // A digits
  size_t ad_elems = 0;
  int* ea = nullptr;   // A row exponents
  size_t ea_n = 0;
  void* bd = nullptr;  // B digits
  size_t bd_elems = 0;
  int* eb = nullptr;   // B column exponents
  size_t eb_n = 0;
  int* err = nullptr;  // one int: set when a tensor-core tile timed out (the tcgen05 path)
};
constexpr int64_t kOzakiMaxChunk = 256;  // problems per chunk (digit arrays: ~5.5 MB per 242 x 242 problem)
size_t ozaki_a_elems(int m, int k);  // per problem
size_t ozaki_b_elems(int k, int n);  // per problem
int ozaki_rows_padded(int m);
int64_t ozaki_chunk(int64_t batch);  // problems per chunk for a batch (even split, <= kOzakiMaxChunk)
// C[b] = A[aidx ? aidx[b] : b] B[b] (complex FP64; A m x k, B k x n; aidx optional, device).
// digits = 8: FP64-accurate (operands cut at 2^-56 of their row / column maximum); digits = 6:
// operands cut at 2^-42 (error ~2^-42 2k |A row| |B column|, for residuals that need ~1e-12).
int ozaki_zgemm(int64_t batch, int m, int n, int k, const cplx<double>* A, int64_t lda, int64_t bsA, const int* aidx,
                const cplx<double>* B, int64_t ldb, int64_t bsB, cplx<double>* C, int64_t ldc, int64_t bsC,
                const OzakiWs& w, cudaStream_t s, int digits = 8);

// The same exact digit products on tcgen05 with TMEM accumulators (7-bit digits, ND = 8 or 6 for
// an FP64 result, 4 for FP32): C = alpha A B + beta C, A[aidx[b]] and B[bidx[b]] optional gathers.
// Valid while 2k rounded up to 64 is at most tc_max_k2p(ND); digit arrays in OzakiWs sized by
// tc_a_elems / tc_b_elems (per problem), exponents by tc_rows_padded(m) and n.
int tc_max_k2p(int nd);
size_t tc_a_elems(int nd, int m, int k);
size_t tc_b_elems(int nd, int k, int n);
int tc_rows_padded(int m);
template <int ND, typename TI, typename TO>
int tc_product(int64_t batch, int m, int n, int k, const cplx<TI>* A, int64_t lda, int64_t bsA, const int* aidx,
               const cplx<TI>* B, int64_t ldb, int64_t bsB, const int* bidx, cplx<TO> alpha, cplx<TO> beta,
               cplx<TO>* C, int64_t ldc, int64_t bsC, const OzakiWs& w, cudaStream_t s);

// The refined FP64 modes a khp_solve_batched_mixed call left in its workspace (same batch and
// stack description as that call): W, V [slots][batch][n][n] and lam [slots][batch][n], one
// slot per distinct map in order of first use (all null when the stack has no patterned layer).
int mixed_modes_in_workspace(int64_t batch, int nh, int L, const int* kinds, const int* maps, const void* ws,
                             size_t ws_bytes, const cplx<double>** W, const cplx<double>** V,
                             const cplx<double>** lam);

// FP32-accurate complex products on the tcgen05 tensor cores, 3xTF32: operands split once into
// TF32 (hi, lo) planes (elements per problem: tf32x3_a_elems / tf32x3_b_elems), then
// C = alpha A B + beta C from the planes (err: one device int, set on a tensor-core time-out).
size_t tf32x3_a_elems(int m, int k);
size_t tf32x3_b_elems(int k, int n);
int tf32x3_split_a(int64_t batch, int m, int k, const cplx<float>* A, int64_t lda, int64_t bsA, const int* aidx,
                   float* planes, cudaStream_t s);
int tf32x3_split_b(int64_t batch, int k, int n, const cplx<float>* B, int64_t ldb, int64_t bsB, const int* bidx,
                   cplx<float> shift, float* planes, cudaStream_t s);  // planes of B + shift I
int tf32x3_from_planes(int64_t batch, int m, int n, int k, const float* Aplanes, const float* Bplanes,
                       cplx<float> alpha, cplx<float> beta, cplx<float>* C, int64_t ldc, int64_t bsC, int* err,
                       cudaStream_t s);

// Whether the mixed solve's n x n FP32 products take the 3xTF32 tensor-core path (khp_tune).
bool use_tf32_products(int n);
// Digits per operand of the mixed solve's eigen-refinement products (khp_tune).
int mode_step_digits();

inline int cuda_status() { return cudaGetLastError() == cudaSuccess ? KHP_OK : KHP_ERR_CUDA; }

// Adds k to the process-wide launch counter reported by khp_launch_count().
void count_launches(int k);

// Stage timing (khp_stage_timing): when enabled, a CUDA event is recorded on the stream at the
// begin and end marks of a stage (KHP_STAGE_* of the public header); no-ops otherwise.
void stage_begin(int stage, cudaStream_t s);
void stage_end(int stage, cudaStream_t s);

}  // namespace khp
